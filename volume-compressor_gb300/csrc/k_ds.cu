// 2x downscale on the device: the exporter's within-cell methods
// (tools/downscale.h:29-93). Every output voxel is a function of its own 2x2x2
// cell (odd boundaries edge-replicated):
//   DS_BOX   (sum + 4) >> 3, the float mean rounded half up, which is also the
//            codec's pyramid rule (src/vc/vc.c:1562-1577): with n in-bounds
//            children (a power of two) the replicated sum is 8/n times theirs
//   DS_CBOX  the mean pushed by alpha toward the cell's voxel of largest
//            deviation (first in (dz, dy, dx) order on ties), then clamped and
//            rounded half up. The push is evaluated as the reference's release
//            build (gcc -O3 -ffast-math -ffp-contract=fast -march=native) does:
//            one fused multiply-add, except in the 8-lane vector body of its
//            nz == 2 fast path (tools/downscale.h:62-79: the first
//            8 * floor(ox / 8) outputs of each row), where it multiplies and
//            adds separately
// HBM-bound: each level reads its input once and writes an eighth of it.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "ds_cell.cuh"
#include "k_ds.cuh"
#include "vc_device.h"

namespace vcg {

// nx a multiple of 32, in and out 16-byte aligned: one thread makes 16 output
// voxels of one output row from 32 bytes of each of its 4 input rows.
template <int M>
__global__ void __launch_bounds__(256) k_ds2x_vec(const uint8_t *__restrict__ in, uint32_t nx, uint32_t ny,
                                                  uint32_t nz, uint8_t *__restrict__ out, float alpha) {
    const uint32_t ox = nx / 2, oy = (ny + 1) / 2, oz = (nz + 1) / 2, cpr = ox / 16;
    const uint32_t vec_end = nz == 2 && ny % 2 == 0 ? ox & ~7u : 0;   // unfused below
    const uint64_t n = (uint64_t)cpr * oy * oz;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t k = (uint32_t)(i % cpr);
        const uint64_t row = i / cpr;
        const uint32_t y = (uint32_t)(row % oy), z = (uint32_t)(row / oy);
        const uint32_t y0 = 2 * y, y1 = 2 * y + 1 < ny ? 2 * y + 1 : ny - 1;
        const uint32_t z0 = 2 * z, z1 = 2 * z + 1 < nz ? 2 * z + 1 : nz - 1;
        const uint64_t rows[4] = {((uint64_t)z0 * ny + y0) * nx, ((uint64_t)z0 * ny + y1) * nx,
                                  ((uint64_t)z1 * ny + y0) * nx, ((uint64_t)z1 * ny + y1) * nx};
        uint32_t w[4][8];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint4 *p = reinterpret_cast<const uint4 *>(in + rows[j] + 32ull * k);
            const uint4 a = __ldcs(p), b = __ldcs(p + 1);
            w[j][0] = a.x; w[j][1] = a.y; w[j][2] = a.z; w[j][3] = a.w;
            w[j][4] = b.x; w[j][5] = b.y; w[j][6] = b.z; w[j][7] = b.w;
        }
        uint32_t r[8];   // r[q]: outputs 2q (bits 0-7) and 2q+1 (bits 16-23)
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            if (M == 0) {
                uint32_t p = 0;
#pragma unroll
                for (int j = 0; j < 4; ++j) p += (w[j][q] & 0x00FF00FFu) + ((w[j][q] >> 8) & 0x00FF00FFu);
                r[q] = ((p + 0x00040004u) >> 3) & 0x00FF00FFu;   // lanes <= 2044: no carry between them
            } else {
                uint32_t res = 0;
#pragma unroll
                for (int h = 0; h < 2; ++h) {   // output 2q + h: bytes 2h, 2h + 1 of word q of each row
                    uint32_t c[8];
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        c[2 * j] = (w[j][q] >> (16 * h)) & 0xFFu;
                        c[2 * j + 1] = (w[j][q] >> (16 * h + 8)) & 0xFFu;
                    }
                    res |= ds_cell<1>(c, alpha, 16 * k + 2 * q + h >= vec_end) << (16 * h);
                }
                r[q] = res;
            }
        }
        uint32_t o[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) o[m] = __byte_perm(r[2 * m], r[2 * m + 1], 0x6420);
        *reinterpret_cast<uint4 *>(out + ((uint64_t)z * oy + y) * ox + 16ull * k) = make_uint4(o[0], o[1], o[2], o[3]);
    }
}

// Any dims and alignment: one output voxel per thread, byte loads.
template <int M>
__global__ void __launch_bounds__(256) k_ds2x_any(const uint8_t *__restrict__ in, uint32_t nx, uint32_t ny,
                                                  uint32_t nz, uint8_t *__restrict__ out, float alpha) {
    const uint32_t ox = (nx + 1) / 2, oy = (ny + 1) / 2, oz = (nz + 1) / 2;
    const uint32_t vec_end = nz == 2 && nx % 2 == 0 && ny % 2 == 0 ? ox & ~7u : 0;   // unfused below
    const uint64_t n = (uint64_t)ox * oy * oz;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t x = (uint32_t)(i % ox), y = (uint32_t)((i / ox) % oy), z = (uint32_t)(i / ((uint64_t)ox * oy));
        const uint32_t xs[2] = {2 * x, 2 * x + 1 < nx ? 2 * x + 1 : nx - 1};
        const uint32_t ys[2] = {2 * y, 2 * y + 1 < ny ? 2 * y + 1 : ny - 1};
        const uint32_t zs[2] = {2 * z, 2 * z + 1 < nz ? 2 * z + 1 : nz - 1};
        uint32_t c[8];
#pragma unroll
        for (int dz = 0; dz < 2; ++dz)
#pragma unroll
            for (int dy = 0; dy < 2; ++dy) {
                const uint8_t *r = in + ((uint64_t)zs[dz] * ny + ys[dy]) * nx;
                c[dz * 4 + dy * 2] = r[xs[0]];
                c[dz * 4 + dy * 2 + 1] = r[xs[1]];
            }
        out[i] = (uint8_t)ds_cell<M>(c, alpha, x >= vec_end);
    }
}

void launch_ds2x(const uint8_t *in, uint32_t nx, uint32_t ny, uint32_t nz, uint8_t *out, int method, float alpha,
                 int num_sms, cudaStream_t s) {
    const uint32_t ox = (nx + 1) / 2, oy = (ny + 1) / 2, oz = (nz + 1) / 2;
    const bool vec = nx % 32 == 0 && ((uintptr_t)in & 15u) == 0 && ((uintptr_t)out & 15u) == 0;
    const uint64_t units = vec ? (uint64_t)(ox / 16) * oy * oz : (uint64_t)ox * oy * oz;
    if (!units) return;
    const uint64_t cap = (uint64_t)num_sms * 16;
    const unsigned blocks = (unsigned)((units + 255) / 256 < cap ? (units + 255) / 256 : cap);
    if (vec) {
        if (method == 1) k_ds2x_vec<1><<<blocks, 256, 0, s>>>(in, nx, ny, nz, out, alpha);
        else k_ds2x_vec<0><<<blocks, 256, 0, s>>>(in, nx, ny, nz, out, alpha);
    } else {
        if (method == 1) k_ds2x_any<1><<<blocks, 256, 0, s>>>(in, nx, ny, nz, out, alpha);
        else k_ds2x_any<0><<<blocks, 256, 0, s>>>(in, nx, ny, nz, out, alpha);
    }
}

}  // namespace vcg

using namespace vcg;

// Levels 1..levels of the cascade from `in` (device), level l into out[l-1]
// (device). With a host input / outputs (on_device == 0) the volume is staged
// through device scratch and every level copied back.
extern "C" int vcd_downscale(const uint8_t *in, int on_device, const uint32_t dims[3], int method, float alpha,
                             int levels, uint8_t *const *out) {
    vcd_ctx *c = vcd_thread_ctx();
    if (!c) return 4;
    cudaStream_t st = c->stream;
    uint64_t nvox[9];
    uint32_t d[9][3];
    memcpy(d[0], dims, sizeof d[0]);
    nvox[0] = (uint64_t)dims[0] * dims[1] * dims[2];
    uint64_t total = 0, off[9] = {0};
    for (int l = 1; l <= levels; ++l) {
        for (int k = 0; k < 3; ++k) d[l][k] = (d[l - 1][k] + 1) / 2;
        nvox[l] = (uint64_t)d[l][0] * d[l][1] * d[l][2];
        off[l] = total;
        total += (nvox[l] + 255) & ~255ull;
    }
    cudaError_t e;
    const uint8_t *src = in;
    uint8_t *stage = NULL;
    if (!on_device) {
        void *p_in, *p_out;
        if ((e = vcd_scratch(c, VCD_BUF_VOL, nvox[0] + 16, &p_in)) != cudaSuccess ||
            (e = vcd_scratch(c, VCD_BUF_PYR, total + 16, &p_out)) != cudaSuccess) {
            vcd_set_error("downscale buffers", e);
            return vcd_status_of(e);
        }
        cudaEventRecord(c->ev[0], st);
        cudaMemcpyAsync(p_in, in, nvox[0], cudaMemcpyHostToDevice, st);
        src = (const uint8_t *)p_in;
        stage = (uint8_t *)p_out;
    } else {
        cudaEventRecord(c->ev[0], st);
    }
    cudaEventRecord(c->ev[1], st);
    for (int l = 1; l <= levels; ++l) {
        uint8_t *dst = on_device ? out[l - 1] : stage + off[l];
        launch_ds2x(src, d[l - 1][0], d[l - 1][1], d[l - 1][2], dst, method, alpha, g_dev.num_sms, st);
        src = dst;
    }
    cudaEventRecord(c->ev[2], st);
    if (!on_device)
        for (int l = 1; l <= levels; ++l) cudaMemcpyAsync(out[l - 1], stage + off[l], nvox[l], cudaMemcpyDeviceToHost, st);
    cudaEventRecord(c->ev[3], st);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess || (e = cudaGetLastError()) != cudaSuccess) {
        vcd_set_error("downscale", e);
        return vcd_status_of(e);
    }
    c->last_ms = vcd_elapsed(c->ev[0], c->ev[3]);
    if (vcd_prof_on()) {
        uint64_t rd = 0, wr = 0;
        for (int l = 1; l <= levels; ++l) { rd += nvox[l - 1]; wr += nvox[l]; }
        vcd_prof_add(method == 1 ? "downscale_cbox" : "downscale_box", vcd_elapsed(c->ev[1], c->ev[2]),
                     (uint64_t)levels, rd, wr, wr);
    }
    return 0;
}

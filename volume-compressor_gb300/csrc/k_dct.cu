// Exact integer 3-D DCT-32 of whole atoms, in two forms (device + C ABI).
//
// The transform is the reference's (src/vc/vc.c:77-229): voxels minus a centre
// value, then along x, y and z the Q14 matrix CMATA with (acc + 2^13) >> 14
// after every pass and i32 sums with wrap-around; the inverse applies CMATA^T
// along x, y and z in the same way and adds the centre back, clamped to
// [0, 255]. The centre is one value for every atom, or each atom's dc, the
// rounded mean (sum + 16384) / 32768 of its voxels (src/vc/vc.c:603), as the
// codec uses it. Coefficients of an atom are 32768 i32 in (kz, ky, kx) raster
// order.
//
//   butterfly  CUDA cores: one CTA per atom, the recursive even/odd partial
//              butterfly of dct32.cuh per line (344 multiplies per line).
//   imma       int8 tensor cores (mma.sync m16n8k32, s8 x s8 -> s32): every
//              pass is OUT = C V over the atom's 1024 lines, 8 lines per MMA
//              tile. CMATA entries (|c| <= 4091) are split into two int8 pieces
//              c = 128 c1 + c0 (c0 = c & 127, c1 = c >> 7) and every pass input
//              into VP pieces v = sum_j 128^j v_j (v_j = (v >> 7j) & 127 below
//              the top piece, the top piece v >> 7(VP-1), signed). Products of
//              equal weight 128^(cp+j) share an s32 accumulator; the
//              accumulators are recombined by shift-add modulo 2^32, which is
//              the reference's i32 sum, so the rounded outputs are the same
//              bits. Intermediates stay in shared memory as int8 piece planes.
//              Forward inputs provably fit two pieces (|vox - centre| <= 255,
//              after one pass <= 2038, after two <= 16285 < 2^14); inverse
//              inputs take three (|v| < 2^21), and an atom whose values leave
//              that range in any pass is redone with the butterfly, so every
//              input gives the reference's result.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "../../include/vcg.h"
#include "dct32.cuh"
#include "imma.cuh"
#include "kernels.cuh"
#include "vc_device.h"

namespace vcg {

struct DctJob {
    const uint8_t *vol_in;     // forward input volume
    const int32_t *coef_in;    // inverse input coefficients
    int32_t *coef_out;         // forward output coefficients
    uint8_t *vol_out;          // inverse output volume
    uint64_t nx, ny, nz;       // volume dims (multiples of 32)
    uint32_t ax, ay;           // atoms along x and y
    uint64_t n_atoms;
    int32_t centre;            // >= 0: every atom's centre; < 0: each atom's dc
    uint8_t *dc;               // per atom: written by the forward, read by the inverse (centre < 0)
    uint32_t *redone;          // atoms the imma form redid with the butterfly
};

constexpr int kDctThreads = 256;

__device__ __forceinline__ void atom_xyz(const DctJob &J, uint64_t a, uint64_t &bx, uint64_t &by, uint64_t &bz) {
    bx = (a % J.ax) * 32;
    by = ((a / J.ax) % J.ay) * 32;
    bz = (a / ((uint64_t)J.ax * J.ay)) * 32;
}

__device__ __forceinline__ uint8_t clamp_u8(int32_t v) { return (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v)); }

// The 16-byte row pieces of atom a a thread loads: row i>>1 = (z, y), x0 = 16 (i & 1).
__device__ __forceinline__ void load_rows(const DctJob &J, uint64_t bx, uint64_t by, uint64_t bz, uint4 (&w)[8]) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int i = threadIdx.x + k * kDctThreads, row = i >> 1, z = row >> 5, y = row & 31;
        w[k] = *reinterpret_cast<const uint4 *>(J.vol_in + ((bz + z) * J.ny + by + y) * J.nx + bx + (i & 1) * 16);
    }
}

// Forward centre of atom a: the fixed centre, or the atom's dc from the voxels
// every thread holds (written to J.dc[a]). Called by the whole CTA.
__device__ int32_t fwd_centre(const DctJob &J, uint64_t a, const uint4 (&w)[8]) {
    if (J.centre >= 0) return J.centre;
    __shared__ uint32_t s_part[kDctThreads / 32];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        s = __dp4a(w[k].x, 0x01010101u, s);
        s = __dp4a(w[k].y, 0x01010101u, s);
        s = __dp4a(w[k].z, 0x01010101u, s);
        s = __dp4a(w[k].w, 0x01010101u, s);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = s;
    __syncthreads();
    uint32_t tot = 0;
#pragma unroll
    for (int i = 0; i < kDctThreads / 32; ++i) tot += s_part[i];
    const int32_t dc = (int32_t)((tot + 16384u) >> 15);   // src/vc/vc.c:603
    if (threadIdx.x == 0) J.dc[a] = (uint8_t)dc;
    __syncthreads();
    return dc;
}

__device__ __forceinline__ int32_t inv_centre(const DctJob &J, uint64_t a) {
    return J.centre >= 0 ? J.centre : (int32_t)J.dc[a];
}

// ------------------------------------------------------------------ butterfly
// One atom through the three passes with T as the padded 32 slabs x 32x32 i32
// tile of dct32.cuh: x and y per slab (warp per
// slab, lane per line), then z per column (thread per column) straight to the
// output. Starts and ends with the CTA converged.
template <bool INV>
__device__ void bf_atom(int32_t *T, const DctJob &J, uint64_t a) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint64_t bx, by, bz;
    atom_xyz(J, a, bx, by, bz);
    int32_t cen = 0;
    if (!INV) {
        uint4 w[8];
        load_rows(J, bx, by, bz, w);
        cen = fwd_centre(J, a, w);
#pragma unroll
        for (int k = 0; k < 8; ++k) {   // 16 voxels of row (z, y)
            const int i = tid + k * kDctThreads, row = i >> 1, x0 = (i & 1) * 16, z = row >> 5, y = row & 31;
            const uint32_t ws[4] = {w[k].x, w[k].y, w[k].z, w[k].w};
#pragma unroll
            for (int b = 0; b < 16; ++b)
                T[z * kSlabPitch + y * kRowPitch + x0 + b] = (int32_t)((ws[b >> 2] >> (8 * (b & 3))) & 0xFFu) - cen;
        }
    } else {
        cen = inv_centre(J, a);
        const int4 *src = reinterpret_cast<const int4 *>(J.coef_in + a * 32768);
        for (int i = tid; i < 8192; i += kDctThreads) {
            const int4 w = src[i];
            const int z = i >> 8, y = (i >> 3) & 31, x = (i & 7) * 4;
            int32_t *d = T + z * kSlabPitch + y * kRowPitch + x;
            d[0] = w.x;
            d[1] = w.y;
            d[2] = w.z;
            d[3] = w.w;
        }
    }
    __syncthreads();
    for (int z = warp; z < 32; z += kDctThreads / 32) {
        int32_t *S = T + z * kSlabPitch;
        int32_t *row = S + lane * kRowPitch, *col = S + lane;
        int32_t v[32], o[32];
#pragma unroll
        for (int x = 0; x < 32; ++x) v[x] = row[x];
        if (INV) idct32_line(v, o); else fdct32_line(v, o);
#pragma unroll
        for (int x = 0; x < 32; ++x) row[x] = o[x];
        __syncwarp();
#pragma unroll
        for (int y = 0; y < 32; ++y) v[y] = col[y * kRowPitch];
        if (INV) idct32_line(v, o); else fdct32_line(v, o);
#pragma unroll
        for (int y = 0; y < 32; ++y) col[y * kRowPitch] = o[y];
        __syncwarp();
    }
    __syncthreads();
    for (int c = tid; c < 1024; c += kDctThreads) {
        const int y = c >> 5, x = c & 31;
        int32_t v[32], o[32];
#pragma unroll
        for (int z = 0; z < 32; ++z) v[z] = T[z * kSlabPitch + y * kRowPitch + x];
        if (INV) {
            idct32_line(v, o);
#pragma unroll
            for (int z = 0; z < 32; ++z)
                J.vol_out[((bz + z) * J.ny + by + y) * J.nx + bx + x] = clamp_u8(o[z] + cen);
        } else {
            fdct32_line(v, o);
            int32_t *dst = J.coef_out + a * 32768 + y * 32 + x;
#pragma unroll
            for (int k = 0; k < 32; ++k) dst[k * 1024] = o[k];
        }
    }
    __syncthreads();
}

template <bool INV>
__global__ void __launch_bounds__(kDctThreads, 1) k_dct_bf(DctJob J) {
    extern __shared__ __align__(16) int32_t T[];
    for (uint64_t a = blockIdx.x; a < J.n_atoms; a += gridDim.x) bf_atom<INV>(T, J, a);
}

// ------------------------------------------------------------------ imma
template <bool INV, int VP>
__global__ void __launch_bounds__(kDctThreads, 1) k_dct_imma(DctJob J) {
    extern __shared__ __align__(16) uint8_t sm[];
    __shared__ int s_bad;
    const int tid = threadIdx.x;
    uint32_t A[2][2][4];
    imma_a_frags<INV>(A);
    auto plane = [&](int b, int j) -> uint8_t * { return imma_plane<VP>(sm, b, j); };

    for (uint64_t a = blockIdx.x; a < J.n_atoms; a += gridDim.x) {
        uint64_t bx, by, bz;
        atom_xyz(J, a, bx, by, bz);
        if (tid == 0) s_bad = 0;
        bool bad = false;
        // pass-0 input: line (z, y), element x
        int32_t cen = 0;
        if (!INV) {
            uint4 wv[8];
            load_rows(J, bx, by, bz, wv);
            cen = fwd_centre(J, a, wv);
#pragma unroll
            for (int kk = 0; kk < 8; ++kk) {
                const int i = tid + kk * kDctThreads, row = i >> 1, half = i & 1;
                const uint32_t ws[4] = {wv[kk].x, wv[kk].y, wv[kk].z, wv[kk].w};
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    uint32_t pk[VP];
#pragma unroll
                    for (int j = 0; j < VP; ++j) pk[j] = 0;
#pragma unroll
                    for (int i4 = 0; i4 < 4; ++i4) {
                        const int32_t v = (int32_t)((ws[q] >> (8 * i4)) & 0xFFu) - cen;
#pragma unroll
                        for (int j = 0; j < VP; ++j) pk[j] |= piece<VP>(v, j) << (8 * i4);
                    }
#pragma unroll
                    for (int j = 0; j < VP; ++j)
                        *reinterpret_cast<uint32_t *>(plane(0, j) + row * 32 + q * 8 + half * 4) = pk[j];
                }
            }
        } else {
            cen = inv_centre(J, a);
            const int4 *src = reinterpret_cast<const int4 *>(J.coef_in + a * 32768);
            for (int i = tid; i < 8192; i += kDctThreads) {
                const int4 w = src[i];
                const int row = i >> 3, n0 = (i & 7) * 4;
                const int32_t vs[4] = {w.x, w.y, w.z, w.w};
                uint32_t pk[VP];
#pragma unroll
                for (int j = 0; j < VP; ++j) pk[j] = 0;
#pragma unroll
                for (int i4 = 0; i4 < 4; ++i4) {
                    bad |= !fits<VP>(vs[i4]);
#pragma unroll
                    for (int j = 0; j < VP; ++j) pk[j] |= piece<VP>(vs[i4], j) << (8 * i4);
                }
#pragma unroll
                for (int j = 0; j < VP; ++j) *reinterpret_cast<uint32_t *>(plane(0, j) + row * 32 + ppos(n0)) = pk[j];
            }
        }
        __syncthreads();

#pragma unroll 1
        for (int pass = 0; pass < 3; ++pass) {
            imma_pass<VP, kDctThreads>(sm, A, pass, bad, [&](int k, int la, int lb, int32_t o0, int32_t o1) {
                if (!INV) {
                    *reinterpret_cast<int2 *>(J.coef_out + a * 32768 + (k * 32 + la) * 32 + lb) = make_int2(o0, o1);
                } else {
                    const uint32_t v2 = (uint32_t)clamp_u8(o0 + cen) | ((uint32_t)clamp_u8(o1 + cen) << 8);
                    *reinterpret_cast<uint16_t *>(J.vol_out + ((bz + k) * J.ny + by + la) * J.nx + bx + lb) =
                        (uint16_t)v2;
                }
            });
            if (bad) s_bad = 1;
            __syncthreads();
        }
        if (s_bad) {   // a value left the piece range: redo the atom exactly
            if (tid == 0) atomicAdd(J.redone, 1u);
            bf_atom<INV>(reinterpret_cast<int32_t *>(sm), J, a);
        }
        __syncthreads();
    }
}

}  // namespace vcg

using namespace vcg;

#define VC_API extern "C" __attribute__((visibility("default")))

static vc_status dct_run(const void *in, void *out, uint8_t *dc, vc_dims dims, int centre, int form, int inverse,
                         uint32_t *redone) {
    if (!in || !out || !dims.nx || !dims.ny || !dims.nz || (dims.nx | dims.ny | dims.nz) & 31u ||
        dims.nx > VC_MAX_DIM || dims.ny > VC_MAX_DIM || dims.nz > VC_MAX_DIM || centre < VCG_DCT_ATOM_DC ||
        centre > 255 || (centre == VCG_DCT_ATOM_DC && !dc) ||
        (form != VCG_DCT_BUTTERFLY && form != VCG_DCT_IMMA) || ((uintptr_t)in & 15u) || ((uintptr_t)out & 15u))
        return VC_ERR_RANGE;
    vcd_ctx *c = vcd_thread_ctx();
    if (!c) return VC_ERR_IO;
    cudaPointerAttributes pa, pb, pc;
    if (cudaPointerGetAttributes(&pa, in) != cudaSuccess || cudaPointerGetAttributes(&pb, out) != cudaSuccess ||
        pa.type != cudaMemoryTypeDevice || pb.type != cudaMemoryTypeDevice ||
        (centre == VCG_DCT_ATOM_DC &&
         (cudaPointerGetAttributes(&pc, dc) != cudaSuccess || pc.type != cudaMemoryTypeDevice))) {
        cudaGetLastError();
        return VC_ERR_RANGE;
    }
    void *p_red;
    cudaError_t e = vcd_scratch(c, VCD_BUF_RED, 64, &p_red);
    if (e != cudaSuccess) {
        vcd_set_error("dct scratch", e);
        return (vc_status)vcd_status_of(e);
    }
    DctJob J;
    memset(&J, 0, sizeof J);
    J.vol_in = inverse ? nullptr : (const uint8_t *)in;
    J.coef_in = inverse ? (const int32_t *)in : nullptr;
    J.coef_out = inverse ? nullptr : (int32_t *)out;
    J.vol_out = inverse ? (uint8_t *)out : nullptr;
    J.nx = dims.nx;
    J.ny = dims.ny;
    J.nz = dims.nz;
    J.ax = dims.nx / 32;
    J.ay = dims.ny / 32;
    J.n_atoms = (uint64_t)J.ax * J.ay * (dims.nz / 32);
    J.centre = centre;
    J.dc = centre == VCG_DCT_ATOM_DC ? dc : nullptr;
    J.redone = (uint32_t *)p_red;
    const unsigned grid = (unsigned)(J.n_atoms < (uint64_t)g_dev.num_sms ? J.n_atoms : (uint64_t)g_dev.num_sms);
    cudaStream_t st = c->stream;
    cudaMemsetAsync(p_red, 0, 4, st);
    cudaEventRecord(c->ev[0], st);
    const char *name;
    if (form == VCG_DCT_BUTTERFLY) {
        smem_attr((const void *)k_dct_bf<false>, (int)kTileBytes);
        smem_attr((const void *)k_dct_bf<true>, (int)kTileBytes);
        if (inverse) k_dct_bf<true><<<grid, kDctThreads, kTileBytes, st>>>(J);
        else k_dct_bf<false><<<grid, kDctThreads, kTileBytes, st>>>(J);
        name = inverse ? "dct_inverse_butterfly" : "dct_forward_butterfly";
    } else {
        // piece planes; an atom redone with the butterfly reuses them as its tile
        const size_t planes_fwd = 2 * 2 * 32768, planes_inv = 2 * 3 * 32768;
        const size_t fwd_smem = planes_fwd > kTileBytes ? planes_fwd : kTileBytes;
        const size_t inv_smem = planes_inv > kTileBytes ? planes_inv : kTileBytes;
        smem_attr((const void *)k_dct_imma<false, 2>, (int)fwd_smem);
        smem_attr((const void *)k_dct_imma<true, 3>, (int)inv_smem);
        if (inverse) k_dct_imma<true, 3><<<grid, kDctThreads, inv_smem, st>>>(J);
        else k_dct_imma<false, 2><<<grid, kDctThreads, fwd_smem, st>>>(J);
        name = inverse ? "dct_inverse_imma" : "dct_forward_imma";
    }
    cudaEventRecord(c->ev[1], st);
    uint32_t red = 0;
    cudaMemcpyAsync(&red, p_red, 4, cudaMemcpyDeviceToHost, st);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess || (e = cudaGetLastError()) != cudaSuccess) {
        vcd_set_error("dct kernels", e);
        return (vc_status)vcd_status_of(e);
    }
    c->last_ms = vcd_elapsed(c->ev[0], c->ev[1]);
    if (redone) *redone = red;
    if (vcd_prof_on()) {
        const uint64_t vox = J.n_atoms * 32768ull;
        vcd_prof_add(name, c->last_ms, 1, inverse ? 4 * vox : vox, inverse ? vox : 4 * vox, J.n_atoms);
    }
    return VC_OK;
}

VC_API vc_status vcg_dct_forward(const uint8_t *vol_dev, vc_dims dims, int centre, int form, int32_t *coef_dev,
                                 uint8_t *dc_dev, uint32_t *redone) {
    VCD_SCOPE();
    return dct_run(vol_dev, coef_dev, dc_dev, dims, centre, form, 0, redone);
}

VC_API vc_status vcg_dct_inverse(const int32_t *coef_dev, const uint8_t *dc_dev, vc_dims dims, int centre, int form,
                                 uint8_t *vol_dev, uint32_t *redone) {
    VCD_SCOPE();
    return dct_run(coef_dev, vol_dev, const_cast<uint8_t *>(dc_dev), dims, centre, form, 1, redone);
}

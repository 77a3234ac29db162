// CUDA implementation of the seeded synthetic volume generator (definition in
// synth_core.h; identical bytes to the host generator), plus the small
// device-memory helpers the vcg_* entry points expose. Generates z-slabs with
// a 3-plane halo so the float working set stays bounded for large volumes.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "synth_core.h"
#include "vc_device.h"

#define VC_API extern "C" __attribute__((visibility("default")))

namespace {

__device__ __forceinline__ uint32_t clampi(int64_t v, uint32_t n) {
    return v < 0 ? 0u : v >= (int64_t)n ? n - 1 : (uint32_t)v;
}

// pre-blur values of planes [h0, h1)
__global__ void k_syn_pre(const syn_cfg *c, uint32_t h0, uint32_t h1, float *a) {
    const uint64_t plane = (uint64_t)c->nx * c->ny, n = plane * (h1 - h0);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x = (uint32_t)(i % c->nx), y = (uint32_t)((i / c->nx) % c->ny), z = h0 + (uint32_t)(i / plane);
        int32_t k0, k1;
        syn_sheet_range(c, z, &k0, &k1);
        float surf[32];
        int32_t nk = k1 - k0 + 1;
        if (nk > 32) nk = 32;
        for (int32_t s = 0; s < nk; ++s) surf[s] = syn_surface(c, (uint32_t)(k0 + s), x, y);
        a[i] = syn_preblur(c, x, y, z, surf, k0, k0 + nk - 1);
    }
}

// axis 0: x, 1: y, 2: z (planes [h0,h1) in `src`, output planes [o0,o1))
__global__ void k_syn_blur(const syn_cfg *c, int axis, const float *src, float *dst, uint32_t h0, uint32_t o0,
                           uint32_t o1) {
    const uint32_t nx = c->nx, ny = c->ny;
    const uint64_t plane = (uint64_t)nx * ny, n = plane * (o1 - o0);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x = (uint32_t)(i % nx), y = (uint32_t)((i / nx) % ny), z = o0 + (uint32_t)(i / plane);
        float t[7];
        for (int d = -3; d <= 3; ++d) {
            uint32_t xx = x, yy = y, zz = z;
            if (axis == 0) xx = clampi((int64_t)x + d, nx);
            else if (axis == 1) yy = clampi((int64_t)y + d, ny);
            else zz = clampi((int64_t)z + d, c->nz);
            t[d + 3] = src[(uint64_t)(zz - h0) * plane + (uint64_t)yy * nx + xx];
        }
        dst[(uint64_t)(z - h0) * plane + (uint64_t)y * nx + x] = syn_blur7(t[0], t[1], t[2], t[3], t[4], t[5], t[6]);
    }
}

__global__ void k_syn_round(const float *src, uint64_t n, uint8_t *out) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = syn_round_u8(src[i]);
}

// byte-wise maximum into a word-addressed mask
__device__ __forceinline__ void byte_max(uint8_t *base, uint64_t off, uint32_t v) {
    uint32_t *w = reinterpret_cast<uint32_t *>(base + (off & ~3ull));
    uint32_t sh = (uint32_t)(off & 3u) * 8u;
    uint32_t old = *w, assumed;
    do {
        assumed = old;
        if (((assumed >> sh) & 0xFFu) >= v) return;
        old = atomicCAS(w, assumed, (assumed & ~(0xFFu << sh)) | (v << sh));
    } while (old != assumed);
}

__global__ void k_syn_incl(const syn_cfg *c, uint32_t z0, uint32_t z1, uint8_t *mask) {
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < c->n_incl;
         j += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t cx, cy, cz, rr, val;
        syn_inclusion(c, j, &cx, &cy, &cz, &rr, &val);
        if ((int64_t)cz + rr < (int64_t)z0 || (int64_t)cz - (int64_t)rr >= (int64_t)z1) continue;
        for (int32_t dz = -(int32_t)rr; dz <= (int32_t)rr; ++dz) {
            int64_t z = (int64_t)cz + dz;
            if (z < z0 || z >= z1) continue;
            for (int32_t dy = -(int32_t)rr; dy <= (int32_t)rr; ++dy) {
                int64_t y = (int64_t)cy + dy;
                if (y < 0 || y >= c->ny) continue;
                for (int32_t dx = -(int32_t)rr; dx <= (int32_t)rr; ++dx) {
                    int64_t x = (int64_t)cx + dx;
                    if (x < 0 || x >= c->nx) continue;
                    if ((uint32_t)(dx * dx + dy * dy + dz * dz) > rr * rr) continue;
                    byte_max(mask, ((uint64_t)(z - z0) * c->ny + (uint64_t)y) * c->nx + (uint64_t)x, val);
                }
            }
        }
    }
}

__global__ void k_syn_merge(const uint8_t *mask, uint64_t n, uint8_t *out) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        if (mask[i]) out[i] = mask[i];
}

}  // namespace

// Generate the whole volume described by *cfg_host into device memory out_dev.
VC_API int vcg_synth_device(const syn_cfg *cfg_host, uint8_t *out_dev) {
    VCD_SCOPE();
    if (vcd_init() != 0) return 4;
    vcd_ctx *cx = vcd_thread_ctx();
    if (!cx) return 4;
    cudaStream_t st = cx->stream;
    const uint64_t plane = (uint64_t)cfg_host->nx * cfg_host->ny;
    uint32_t slab = (uint32_t)((1ull << 28) / (plane ? plane : 1));   // ~1 GiB of floats per buffer
    if (slab < 8) slab = 8;
    if (slab > cfg_host->nz) slab = cfg_host->nz;
    syn_cfg *c = NULL;
    float *a = NULL, *b = NULL;
    uint8_t *mask = NULL;
    cudaError_t e = vcd_malloc((void **)&c, sizeof(syn_cfg));
    if (e == cudaSuccess) e = cudaMemcpyAsync(c, cfg_host, sizeof(syn_cfg), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = vcd_malloc((void **)&a, plane * (slab + 6) * sizeof(float));
    if (e == cudaSuccess) e = vcd_malloc((void **)&b, plane * (slab + 6) * sizeof(float));
    if (e == cudaSuccess) e = vcd_malloc((void **)&mask, plane * slab + 16);
    const int grid = g_dev.num_sms * 8;
    for (uint32_t z0 = 0; e == cudaSuccess && z0 < cfg_host->nz; z0 += slab) {
        uint32_t z1 = z0 + slab < cfg_host->nz ? z0 + slab : cfg_host->nz;
        uint32_t h0 = z0 >= 3 ? z0 - 3 : 0, h1 = z1 + 3 <= cfg_host->nz ? z1 + 3 : cfg_host->nz;
        k_syn_pre<<<grid, 256, 0, st>>>(c, h0, h1, a);
        k_syn_blur<<<grid, 256, 0, st>>>(c, 0, a, b, h0, h0, h1);
        k_syn_blur<<<grid, 256, 0, st>>>(c, 1, b, a, h0, h0, h1);
        k_syn_blur<<<grid, 256, 0, st>>>(c, 2, a, b, h0, z0, z1);
        uint8_t *o = out_dev + (uint64_t)z0 * plane;
        k_syn_round<<<grid, 256, 0, st>>>(b + (uint64_t)(z0 - h0) * plane, plane * (z1 - z0), o);
        cudaMemsetAsync(mask, 0, plane * (z1 - z0), st);
        k_syn_incl<<<grid, 256, 0, st>>>(c, z0, z1, mask);
        k_syn_merge<<<grid, 256, 0, st>>>(mask, plane * (z1 - z0), o);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaFree(c);
    cudaFree(a);
    cudaFree(b);
    cudaFree(mask);
    if (e != cudaSuccess) { vcd_set_error("synthetic volume", e); return vcd_status_of(e); }
    return 0;
}

// ---------------------------------------------------------------- device memory helpers
VC_API void *vcg_alloc(size_t bytes) {
    VCD_SCOPE();
    if (vcd_init() != 0) return NULL;
    void *p = NULL;
    return vcd_malloc((void **)&p, bytes ? bytes : 1) == cudaSuccess ? p : NULL;
}
VC_API void vcg_free(void *p) {
    VCD_SCOPE();
    if (p) cudaFree(p);
}
VC_API void *vcg_alloc_host(size_t bytes) {
    VCD_SCOPE();
    if (vcd_init() != 0) return NULL;
    void *p = NULL;
    return vcd_malloc_host((void **)&p, bytes ? bytes : 1) == cudaSuccess ? p : NULL;
}
VC_API void vcg_free_host(void *p) {
    VCD_SCOPE();
    if (p) cudaFreeHost(p);
}
VC_API int vcg_copy(void *dst, const void *src, size_t bytes) {
    VCD_SCOPE();
    if (vcd_init() != 0) return 4;
    return cudaMemcpy(dst, src, bytes, cudaMemcpyDefault) == cudaSuccess ? 0 : 4;
}
VC_API int vcg_memset(void *dst, int v, size_t bytes) {
    VCD_SCOPE();
    if (vcd_init() != 0) return 4;
    return cudaMemset(dst, v, bytes) == cudaSuccess ? 0 : 4;
}
VC_API int vcg_sync(void) {
    VCD_SCOPE();
    if (vcd_init() != 0) return 4;
    vcd_ctx *c = vcd_thread_ctx();
    if (c) cudaStreamSynchronize(c->stream);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : 4;
}
VC_API int vcg_device_info(int *num_sms, int *cc_major, int *cc_minor) {
    VCD_SCOPE();
    if (vcd_init() != 0) return 4;
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, g_dev.device) != cudaSuccess) return 4;
    if (num_sms) *num_sms = p.multiProcessorCount;
    if (cc_major) *cc_major = p.major;
    if (cc_minor) *cc_minor = p.minor;
    return 0;
}
VC_API const char *vcg_last_error(void) { return vcd_last_error(); }
VC_API int vcg_device_memory(size_t *free_bytes, size_t *total_bytes) {
    VCD_SCOPE();
    if (vcd_init() != 0) return 4;
    size_t f = 0, t = 0;
    if (cudaMemGetInfo(&f, &t) != cudaSuccess) return 4;
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
    return 0;
}

VC_API int vcg_synth_volume_device(uint32_t nx, uint32_t ny, uint32_t nz, uint64_t seed, uint8_t *out_dev) {
    VCD_SCOPE();
    if (!nx || !ny || !nz || !out_dev) return 2;
    syn_cfg *c = (syn_cfg *)calloc(1, sizeof(syn_cfg));
    if (!c) return 3;
    syn_setup(c, nx, ny, nz, seed);
    int rc = vcg_synth_device(c, out_dev);
    free(c);
    return rc;
}

// Host implementation of the seeded synthetic volume generator (definition in
// synth_core.h). Builds any z-slab of the volume independently, so large
// volumes are produced slab by slab in bounded memory; OpenMP over rows.
// Compiled with -ffp-contract=off so that x86-64 and AArch64 hosts give the
// same bytes as the CUDA generator.
#include <stdlib.h>
#include <string.h>

#include "synth_core.h"

#define VCS_API __attribute__((visibility("default")))

VCS_API size_t vcs_cfg_size(void) { return sizeof(syn_cfg); }

VCS_API void vcs_setup(syn_cfg *c, uint32_t nx, uint32_t ny, uint32_t nz, uint64_t seed) {
    memset(c, 0, sizeof *c);
    syn_setup(c, nx, ny, nz, seed);
}

static inline uint32_t clampi(int64_t v, uint32_t n) { return v < 0 ? 0u : v >= (int64_t)n ? n - 1 : (uint32_t)v; }

// planes [z0, z1) of the volume, x fastest, into out ((z1-z0) * ny * nx bytes)
VCS_API int vcs_generate_slab(const syn_cfg *c, uint32_t z0, uint32_t z1, uint8_t *out, int nthreads) {
    if (z0 >= z1 || z1 > c->nz) return 2;
    const uint32_t nx = c->nx, ny = c->ny;
    const uint32_t h0 = z0 >= 3 ? z0 - 3 : 0, h1 = z1 + 3 <= c->nz ? z1 + 3 : c->nz;
    const size_t plane = (size_t)nx * ny, np = h1 - h0;
    float *a = (float *)malloc(np * plane * sizeof(float));
    float *b = (float *)malloc(np * plane * sizeof(float));
    if (!a || !b) { free(a); free(b); return 3; }
    int32_t ka, kb, t0, t1;
    syn_sheet_range(c, h0, &ka, &t1);
    syn_sheet_range(c, h1 - 1, &t0, &kb);
    const int32_t nk = kb >= ka ? kb - ka + 1 : 0;
    if (nthreads < 1) nthreads = 1;

    // pre-blur values over the halo'd slab; sheet surfaces once per column
    #pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
    for (uint32_t y = 0; y < ny; ++y) {
        float *surf = (float *)malloc((size_t)(nk > 0 ? nk : 1) * nx * sizeof(float));
        for (uint32_t x = 0; x < nx; ++x)
            for (int32_t s = 0; s < nk; ++s) surf[(size_t)x * nk + s] = syn_surface(c, (uint32_t)(ka + s), x, y);
        for (uint32_t z = h0; z < h1; ++z) {
            int32_t k0, k1;
            syn_sheet_range(c, z, &k0, &k1);
            if (k0 < ka) k0 = ka;
            if (k1 > kb) k1 = kb;
            float *row = a + (size_t)(z - h0) * plane + (size_t)y * nx;
            for (uint32_t x = 0; x < nx; ++x)
                row[x] = syn_preblur(c, x, y, z, surf + (size_t)x * nk + (k0 - ka), k0, k1);
        }
        free(surf);
    }
    // blur x: a -> b
    #pragma omp parallel for schedule(static) num_threads(nthreads)
    for (size_t r = 0; r < np * ny; ++r) {
        const float *s = a + r * nx;
        float *d = b + r * nx;
        for (uint32_t x = 0; x < nx; ++x)
            d[x] = syn_blur7(s[clampi((int64_t)x - 3, nx)], s[clampi((int64_t)x - 2, nx)], s[clampi((int64_t)x - 1, nx)],
                             s[x], s[clampi((int64_t)x + 1, nx)], s[clampi((int64_t)x + 2, nx)], s[clampi((int64_t)x + 3, nx)]);
    }
    // blur y: b -> a
    #pragma omp parallel for schedule(static) num_threads(nthreads)
    for (size_t r = 0; r < np * ny; ++r) {
        size_t p = r / ny;
        uint32_t y = (uint32_t)(r % ny);
        const float *s = b + p * plane;
        float *d = a + p * plane + (size_t)y * nx;
        const float *r0 = s + (size_t)clampi((int64_t)y - 3, ny) * nx, *r1 = s + (size_t)clampi((int64_t)y - 2, ny) * nx,
                    *r2 = s + (size_t)clampi((int64_t)y - 1, ny) * nx, *r3 = s + (size_t)y * nx,
                    *r4 = s + (size_t)clampi((int64_t)y + 1, ny) * nx, *r5 = s + (size_t)clampi((int64_t)y + 2, ny) * nx,
                    *r6 = s + (size_t)clampi((int64_t)y + 3, ny) * nx;
        for (uint32_t x = 0; x < nx; ++x) d[x] = syn_blur7(r0[x], r1[x], r2[x], r3[x], r4[x], r5[x], r6[x]);
    }
    // blur z + round: a -> out (planes z0..z1-1; clamped neighbours lie inside the halo)
    #pragma omp parallel for schedule(static) num_threads(nthreads)
    for (size_t r = 0; r < (size_t)(z1 - z0) * ny; ++r) {
        uint32_t z = z0 + (uint32_t)(r / ny), y = (uint32_t)(r % ny);
        const float *p[7];
        for (int dd = -3; dd <= 3; ++dd)
            p[dd + 3] = a + (size_t)(clampi((int64_t)z + dd, c->nz) - h0) * plane + (size_t)y * nx;
        uint8_t *o = out + (size_t)(z - z0) * plane + (size_t)y * nx;
        for (uint32_t x = 0; x < nx; ++x)
            o[x] = syn_round_u8(syn_blur7(p[0][x], p[1][x], p[2][x], p[3][x], p[4][x], p[5][x], p[6][x]));
    }
    free(b);
    // inclusions: per voxel the largest covering value (reuse `a` as a byte mask)
    uint8_t *inc = (uint8_t *)a;
    memset(inc, 0, (size_t)(z1 - z0) * plane);
    for (uint64_t j = 0; j < c->n_incl; ++j) {
        uint32_t cx, cy, cz, rr, val;
        syn_inclusion(c, j, &cx, &cy, &cz, &rr, &val);
        if ((int64_t)cz + rr < (int64_t)z0 || (int64_t)cz - (int64_t)rr >= (int64_t)z1) continue;
        for (int32_t dz = -(int32_t)rr; dz <= (int32_t)rr; ++dz) {
            int64_t z = (int64_t)cz + dz;
            if (z < z0 || z >= z1) continue;
            for (int32_t dy = -(int32_t)rr; dy <= (int32_t)rr; ++dy) {
                int64_t y = (int64_t)cy + dy;
                if (y < 0 || y >= ny) continue;
                for (int32_t dx = -(int32_t)rr; dx <= (int32_t)rr; ++dx) {
                    int64_t x = (int64_t)cx + dx;
                    if (x < 0 || x >= nx) continue;
                    if ((uint32_t)(dx * dx + dy * dy + dz * dz) > rr * rr) continue;
                    uint8_t *m = inc + ((size_t)(z - z0) * ny + (size_t)y) * nx + (size_t)x;
                    if (val > *m) *m = (uint8_t)val;
                }
            }
        }
    }
    for (size_t i = 0; i < (size_t)(z1 - z0) * plane; ++i)
        if (inc[i]) out[i] = inc[i];
    free(a);
    return 0;
}

VCS_API int vcs_generate(const syn_cfg *c, uint8_t *out, int nthreads) {
    const uint32_t slab = 32;
    for (uint32_t z = 0; z < c->nz; z += slab) {
        uint32_t e = z + slab < c->nz ? z + slab : c->nz;
        int s = vcs_generate_slab(c, z, e, out + (size_t)z * c->nx * c->ny, nthreads);
        if (s) return s;
    }
    return 0;
}

// Seeded synthetic "scroll sheet" volume generator: the workload the benchmarks
// and parity tests feed the codec (stacked wavy bright sheets over a noisy dark
// background, Gaussian-blurred, with small bright inclusions). Shared verbatim
// by the host C library and the CUDA generator so both produce identical bytes:
// it uses only IEEE add/sub/mul/div/sqrt/floor on floats and 64-bit integer
// hashing, with no FMA contraction (host: -ffp-contract=off; device: explicit
// round-to-nearest intrinsics).
//
// Definition (all per-voxel randomness is counter-based, so any z-slab can be
// generated independently of the rest of the volume):
//   H(i)      = splitmix64 finaliser of (seed * 0x9E3779B97F4A7C15 + stream * 0xD1B54A32D192ED03 + i)
//   U(h)      = (h >> 40) * 2^-24
//   normal    = sqrt(-2 ln u1) * cos(2 pi u2), u1 = ((h1 >> 40) + 1) * 2^-24, u2 = U(h2)
//   sheets    K = max(1, nz / 12); sheet k: lx, ly ~ U[80,300], phases ~ U[0,1) turns,
//             thickness ~ U[3,7], intensity ~ U[110,170]; centre z0_k = (k + 0.5) nz / K;
//             surface z_k(x,y) = z0_k + 4 sin(2 pi (x/lx + px)) + 3 sin(2 pi (y/ly + py))
//   pre-blur  v = 18 + 5 n_bg; the first sheet k with |z - z_k| < thickness/2 sets
//             v = intensity_k + 10 n_sheet
//   blur      separable Gaussian sigma 0.8, radius 3, normalised, clamped edges,
//             passes x, then y, then z, taps accumulated from -3 to +3
//   round     u8 = clamp(rint(v), 0, 255)
//   inclusions round(1e-4 * nx*ny*nz) balls, centre uniform in the volume, radius
//             U{1,2,3}, value U{230..255}; a voxel inside one or more balls takes
//             the largest of their values
#ifndef VC_SYNTH_CORE_H
#define VC_SYNTH_CORE_H
#include <stdint.h>

#if defined(__CUDACC__)
#define SYN_FN __host__ __device__ static inline
#if defined(__CUDA_ARCH__)
#define SYN_ADD(a, b) __fadd_rn((a), (b))
#define SYN_SUB(a, b) __fsub_rn((a), (b))
#define SYN_MUL(a, b) __fmul_rn((a), (b))
#define SYN_DIV(a, b) __fdiv_rn((a), (b))
#define SYN_SQRT(a) __fsqrt_rn(a)
#define SYN_FLOOR(a) floorf(a)
#define SYN_RINT(a) rintf(a)
#endif
#else
#define SYN_FN static inline
#endif
#ifndef SYN_ADD
#include <math.h>
#define SYN_ADD(a, b) ((a) + (b))
#define SYN_SUB(a, b) ((a) - (b))
#define SYN_MUL(a, b) ((a) * (b))
#define SYN_DIV(a, b) ((a) / (b))
#define SYN_SQRT(a) sqrtf(a)
#define SYN_FLOOR(a) floorf(a)
#define SYN_RINT(a) rintf(a)
#endif

#define SYN_MAX_SHEETS 512

enum { SYN_STREAM_SHEET = 1, SYN_STREAM_BG = 2, SYN_STREAM_SHEETNOISE = 3, SYN_STREAM_INCL = 4 };

typedef struct {
    uint32_t nx, ny, nz, nsheets;
    uint64_t seed;
    uint64_t n_incl;
    float z0[SYN_MAX_SHEETS], ilx[SYN_MAX_SHEETS], ily[SYN_MAX_SHEETS];
    float px[SYN_MAX_SHEETS], py[SYN_MAX_SHEETS], half_th[SYN_MAX_SHEETS], inten[SYN_MAX_SHEETS];
} syn_cfg;

// Gaussian sigma 0.8, radius 3, normalised (float32 of the exact weights)
#define SYN_W0 0.49867644906044006f
#define SYN_W1 0.2283107191324234f
#define SYN_W2 0.02191031351685524f
#define SYN_W3 0.0004407433734741062f

SYN_FN uint64_t syn_mix(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
SYN_FN uint64_t syn_hash(uint64_t seed, uint32_t stream, uint64_t i) {
    return syn_mix(seed * 0x9E3779B97F4A7C15ull + (uint64_t)stream * 0xD1B54A32D192ED03ull + i);
}
SYN_FN float syn_u01(uint64_t h) { return (float)(uint32_t)(h >> 40) * (1.0f / 16777216.0f); }

// sin(2 pi t) for any t: reduce to [-1/2, 1/2), fold to [-1/4, 1/4], odd Taylor
// polynomial in x = 2 pi t through x^11 (|error| < 1e-7 on the folded range).
SYN_FN float syn_sin_turns(float t) {
    float r = SYN_SUB(t, SYN_FLOOR(SYN_ADD(t, 0.5f)));   // [-0.5, 0.5)
    if (r > 0.25f) r = SYN_SUB(0.5f, r);
    else if (r < -0.25f) r = SYN_SUB(-0.5f, r);
    float x = SYN_MUL(r, 6.28318530717958647692f);
    float x2 = SYN_MUL(x, x);
    float p = -2.50521083854417e-08f;                   // -1/11!
    p = SYN_ADD(SYN_MUL(p, x2), 2.75573192239859e-06f);  // 1/9!
    p = SYN_ADD(SYN_MUL(p, x2), -1.98412698412698e-04f); // -1/7!
    p = SYN_ADD(SYN_MUL(p, x2), 8.33333333333333e-03f);  // 1/5!
    p = SYN_ADD(SYN_MUL(p, x2), -1.66666666666667e-01f); // -1/3!
    p = SYN_MUL(SYN_MUL(p, x2), x);
    return SYN_ADD(x, p);
}
SYN_FN float syn_cos_turns(float t) { return syn_sin_turns(SYN_ADD(t, 0.25f)); }

// natural log of u in (0, 1]: u = m 2^e, m in [1,2); ln m = 2 atanh((m-1)/(m+1)).
SYN_FN float syn_ln(float u) {
    union { float f; uint32_t b; } v;
    v.f = u;
    int32_t e = (int32_t)((v.b >> 23) & 0xFFu) - 127;
    v.b = (v.b & 0x007FFFFFu) | 0x3F800000u;
    float m = v.f;
    float s = SYN_DIV(SYN_SUB(m, 1.0f), SYN_ADD(m, 1.0f));
    float s2 = SYN_MUL(s, s);
    float p = 0.0909090909f;                        // 1/11
    p = SYN_ADD(SYN_MUL(p, s2), 0.1111111111f);      // 1/9
    p = SYN_ADD(SYN_MUL(p, s2), 0.1428571429f);      // 1/7
    p = SYN_ADD(SYN_MUL(p, s2), 0.2f);               // 1/5
    p = SYN_ADD(SYN_MUL(p, s2), 0.3333333333f);      // 1/3
    p = SYN_ADD(SYN_MUL(p, s2), 1.0f);
    float lnm = SYN_MUL(SYN_MUL(2.0f, s), p);
    return SYN_ADD(lnm, SYN_MUL((float)e, 0.693147180559945309f));
}

SYN_FN float syn_normal(uint64_t seed, uint32_t stream, uint64_t i) {
    uint64_t h1 = syn_hash(seed, stream, 2 * i), h2 = syn_hash(seed, stream, 2 * i + 1);
    float u1 = (float)((uint32_t)(h1 >> 40) + 1u) * (1.0f / 16777216.0f);
    float u2 = syn_u01(h2);
    return SYN_MUL(SYN_SQRT(SYN_MUL(-2.0f, syn_ln(u1))), syn_cos_turns(u2));
}

// Sheet and inclusion parameters (host side, once per volume).
static inline void syn_setup(syn_cfg *c, uint32_t nx, uint32_t ny, uint32_t nz, uint64_t seed) {
    c->nx = nx; c->ny = ny; c->nz = nz; c->seed = seed;
    uint32_t k = nz / 12u;
    if (k < 1) k = 1;
    if (k > SYN_MAX_SHEETS) k = SYN_MAX_SHEETS;
    c->nsheets = k;
    for (uint32_t s = 0; s < k; ++s) {
        uint64_t b = 6ull * s;
        float lx = 80.0f + 220.0f * syn_u01(syn_hash(seed, SYN_STREAM_SHEET, b + 0));
        float ly = 80.0f + 220.0f * syn_u01(syn_hash(seed, SYN_STREAM_SHEET, b + 1));
        c->ilx[s] = 1.0f / lx;
        c->ily[s] = 1.0f / ly;
        c->px[s] = syn_u01(syn_hash(seed, SYN_STREAM_SHEET, b + 2));
        c->py[s] = syn_u01(syn_hash(seed, SYN_STREAM_SHEET, b + 3));
        c->half_th[s] = (3.0f + 4.0f * syn_u01(syn_hash(seed, SYN_STREAM_SHEET, b + 4))) * 0.5f;
        c->inten[s] = 110.0f + 60.0f * syn_u01(syn_hash(seed, SYN_STREAM_SHEET, b + 5));
        c->z0[s] = ((float)s + 0.5f) * (float)nz / (float)k;
    }
    uint64_t nvox = (uint64_t)nx * ny * nz;
    c->n_incl = (nvox + 5000u) / 10000u;
}

// Inclusion j: centre, radius, value.
SYN_FN void syn_inclusion(const syn_cfg *c, uint64_t j, uint32_t *x, uint32_t *y, uint32_t *z,
                          uint32_t *r, uint32_t *val) {
    *x = (uint32_t)(syn_hash(c->seed, SYN_STREAM_INCL, 5 * j + 0) % c->nx);
    *y = (uint32_t)(syn_hash(c->seed, SYN_STREAM_INCL, 5 * j + 1) % c->ny);
    *z = (uint32_t)(syn_hash(c->seed, SYN_STREAM_INCL, 5 * j + 2) % c->nz);
    *r = 1u + (uint32_t)(syn_hash(c->seed, SYN_STREAM_INCL, 5 * j + 3) % 3u);
    *val = 230u + (uint32_t)(syn_hash(c->seed, SYN_STREAM_INCL, 5 * j + 4) % 26u);
}

// Sheet surface height of sheet s over column (x, y).
SYN_FN float syn_surface(const syn_cfg *c, uint32_t s, uint32_t x, uint32_t y) {
    float a = syn_sin_turns(SYN_ADD(SYN_MUL((float)x, c->ilx[s]), c->px[s]));
    float b = syn_sin_turns(SYN_ADD(SYN_MUL((float)y, c->ily[s]), c->py[s]));
    return SYN_ADD(SYN_ADD(c->z0[s], SYN_MUL(4.0f, a)), SYN_MUL(3.0f, b));
}

// Range of sheets that can touch plane z (|z - z0| must be below 4+3+3.5).
SYN_FN void syn_sheet_range(const syn_cfg *c, uint32_t z, int32_t *k0, int32_t *k1) {
    float per = (float)c->nz / (float)c->nsheets;   // sheet spacing
    int32_t lo = (int32_t)(((float)z - 11.0f) / per) - 2;
    int32_t hi = (int32_t)(((float)z + 11.0f) / per) + 2;
    if (lo < 0) lo = 0;
    if (hi > (int32_t)c->nsheets - 1) hi = (int32_t)c->nsheets - 1;
    *k0 = lo; *k1 = hi;
}

// Pre-blur value of voxel (x,y,z); surf[s] = syn_surface(c, s, x, y) for s in [k0,k1].
SYN_FN float syn_preblur(const syn_cfg *c, uint32_t x, uint32_t y, uint32_t z, const float *surf,
                         int32_t k0, int32_t k1) {
    uint64_t i = ((uint64_t)z * c->ny + y) * c->nx + x;
    float v = SYN_ADD(18.0f, SYN_MUL(5.0f, syn_normal(c->seed, SYN_STREAM_BG, i)));
    float fz = (float)z;
    for (int32_t s = k0; s <= k1; ++s) {
        float d = SYN_SUB(fz, surf[s - k0]);
        if (d < 0.0f) d = -d;
        if (d < c->half_th[s]) {
            v = SYN_ADD(c->inten[s], SYN_MUL(10.0f, syn_normal(c->seed, SYN_STREAM_SHEETNOISE, i)));
            break;
        }
    }
    return v;
}

// 7-tap blur of samples v[-3..3] (already edge-clamped), taps summed left to right.
SYN_FN float syn_blur7(float a, float b, float cc, float d, float e, float f, float g) {
    float acc = SYN_MUL(SYN_W3, a);
    acc = SYN_ADD(acc, SYN_MUL(SYN_W2, b));
    acc = SYN_ADD(acc, SYN_MUL(SYN_W1, cc));
    acc = SYN_ADD(acc, SYN_MUL(SYN_W0, d));
    acc = SYN_ADD(acc, SYN_MUL(SYN_W1, e));
    acc = SYN_ADD(acc, SYN_MUL(SYN_W2, f));
    acc = SYN_ADD(acc, SYN_MUL(SYN_W3, g));
    return acc;
}

SYN_FN uint8_t syn_round_u8(float v) {
    float r = SYN_RINT(v);
    if (r < 0.0f) r = 0.0f;
    if (r > 255.0f) r = 255.0f;
    return (uint8_t)(int32_t)r;
}

#endif

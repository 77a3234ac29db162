// Exact integer DCT-32 line transforms (device).
//
// The reference transforms each 32-voxel line with the Q14 matrix CMATA
// (src/vc/vc.c:75-88) and rounds with (acc + 2^13) >> 14 after every pass
// (src/vc/vc.c:142-205). Sums are i32 with wrap-around. Because integer
// addition and multiplication modulo 2^32 are associative and commutative, any
// factorisation of the same sums gives identical bits; these use the full
// recursive even/odd partial butterfly (342-344 multiplies per 32-point line
// instead of 1024), which is valid because CMATA obeys the DCT-II mirror
// symmetries exactly at every level — asserted at compile time below.
#pragma once
#include <stdint.h>

#include "vc_release_tables.h"

namespace vcg {

constexpr int kCm[32][32] = VC_CMAT_INIT;

// The same in constant memory, for loops with a computed index (the int8
// tensor-core transform builds its matrix pieces from it).
static __constant__ int32_t c_cmat[32][32] = VC_CMAT_INIT;

// CMATA[k][n]; with constant indices (fully unrolled loops) it folds to an immediate.
__host__ __device__ constexpr int cmat(int k, int n) {
    constexpr int t[32][32] = VC_CMAT_INIT;
    return t[k][n];
}

// C[k][L-1-n] = (-1)^(k / (32/L)) C[k][n] for every k that is a multiple of 32/L,
// L = 32, 16, 8, 4, 2 (the recursive butterfly's precondition).
constexpr bool cmat_mirror_ok() {
    for (int L = 32, step = 1; L >= 2; L /= 2, step *= 2)
        for (int k = 0; k < 32; k += step)
            for (int n = 0; n < L / 2; ++n) {
                int s = ((k / step) & 1) ? -1 : 1;
                if (kCm[k][L - 1 - n] != s * kCm[k][n]) return false;
            }
    return true;
}
static_assert(cmat_mirror_ok(), "CMATA must satisfy the recursive DCT-II mirror symmetry");

__device__ __forceinline__ int32_t rnd14(int32_t acc) { return (acc + 8192) >> 14; }

// Inverse line: o[n] = rnd14(sum_k C[k][n] v[k]) for n = 0..31 (src/vc/vc.c:172-205).
__device__ __forceinline__ void idct32_line(const int32_t (&v)[32], int32_t (&o)[32]) {
    int32_t O[16], EO[8], EEO[4], EEEO[2], EEEE[2];
#pragma unroll
    for (int n = 0; n < 16; ++n) {
        int32_t a = 0;
#pragma unroll
        for (int k = 1; k < 32; k += 2) a += cmat(k, n) * v[k];
        O[n] = a;
    }
#pragma unroll
    for (int n = 0; n < 8; ++n) {
        int32_t a = 0;
#pragma unroll
        for (int k = 2; k < 32; k += 4) a += cmat(k, n) * v[k];
        EO[n] = a;
    }
#pragma unroll
    for (int n = 0; n < 4; ++n) {
        int32_t a = 0;
#pragma unroll
        for (int k = 4; k < 32; k += 8) a += cmat(k, n) * v[k];
        EEO[n] = a;
    }
#pragma unroll
    for (int n = 0; n < 2; ++n) {
        EEEO[n] = cmat(8, n) * v[8] + cmat(24, n) * v[24];
        EEEE[n] = cmat(0, n) * v[0] + cmat(16, n) * v[16];
    }
    int32_t EEE[4], EE[8], E[16];
#pragma unroll
    for (int n = 0; n < 2; ++n) { EEE[n] = EEEE[n] + EEEO[n]; EEE[3 - n] = EEEE[n] - EEEO[n]; }
#pragma unroll
    for (int n = 0; n < 4; ++n) { EE[n] = EEE[n] + EEO[n]; EE[7 - n] = EEE[n] - EEO[n]; }
#pragma unroll
    for (int n = 0; n < 8; ++n) { E[n] = EE[n] + EO[n]; E[15 - n] = EE[n] - EO[n]; }
#pragma unroll
    for (int n = 0; n < 16; ++n) { o[n] = rnd14(E[n] + O[n]); o[31 - n] = rnd14(E[n] - O[n]); }
}

// Forward line: o[k] = rnd14(sum_n C[k][n] v[n]) for k = 0..31 (src/vc/vc.c:142-171).
__device__ __forceinline__ void fdct32_line(const int32_t (&v)[32], int32_t (&o)[32]) {
    int32_t s[16], d[16];
#pragma unroll
    for (int n = 0; n < 16; ++n) { s[n] = v[n] + v[31 - n]; d[n] = v[n] - v[31 - n]; }
#pragma unroll
    for (int k = 1; k < 32; k += 2) {
        int32_t a = 0;
#pragma unroll
        for (int n = 0; n < 16; ++n) a += cmat(k, n) * d[n];
        o[k] = rnd14(a);
    }
    int32_t ss[8], sd[8];
#pragma unroll
    for (int n = 0; n < 8; ++n) { ss[n] = s[n] + s[15 - n]; sd[n] = s[n] - s[15 - n]; }
#pragma unroll
    for (int k = 2; k < 32; k += 4) {
        int32_t a = 0;
#pragma unroll
        for (int n = 0; n < 8; ++n) a += cmat(k, n) * sd[n];
        o[k] = rnd14(a);
    }
    int32_t sss[4], ssd[4];
#pragma unroll
    for (int n = 0; n < 4; ++n) { sss[n] = ss[n] + ss[7 - n]; ssd[n] = ss[n] - ss[7 - n]; }
#pragma unroll
    for (int k = 4; k < 32; k += 8) {
        int32_t a = 0;
#pragma unroll
        for (int n = 0; n < 4; ++n) a += cmat(k, n) * ssd[n];
        o[k] = rnd14(a);
    }
    int32_t s4[2], d4[2];
#pragma unroll
    for (int n = 0; n < 2; ++n) { s4[n] = sss[n] + sss[3 - n]; d4[n] = sss[n] - sss[3 - n]; }
    o[8] = rnd14(cmat(8, 0) * d4[0] + cmat(8, 1) * d4[1]);
    o[24] = rnd14(cmat(24, 0) * d4[0] + cmat(24, 1) * d4[1]);
    o[0] = rnd14(cmat(0, 0) * s4[0] + cmat(0, 1) * s4[1]);
    o[16] = rnd14(cmat(16, 0) * s4[0] + cmat(16, 1) * s4[1]);
}

// Atom tile in shared memory (i32): 32 slabs of 32 rows with a row pitch of 33
// ints, element (z, y, x) at z*kSlabPitch + y*kRowPitch + x. A warp that
// touches one row (lane = x), one column (lane = y) or one (y, x) line across
// slabs (lane = x) hits 32 distinct banks, and in unrolled loops every address
// is a base register plus a constant.
constexpr int kRowPitch = 33;
constexpr int kSlabPitch = 32 * kRowPitch;
constexpr int kTileInts = 32 * kSlabPitch;
constexpr size_t kTileBytes = (size_t)kTileInts * sizeof(int32_t);

__host__ __device__ __forceinline__ int tile_idx(uint32_t r) {   // raster (z, y, x) -> tile slot
    return (int)(r >> 10) * kSlabPitch + (int)((r >> 5) & 31u) * kRowPitch + (int)(r & 31u);
}

}  // namespace vcg

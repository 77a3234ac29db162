// Host build of the device's 2x2x2 cell values (volume-compressor_gb300/csrc/
// ds_cell.cuh: DS_BOX and DS_CBOX with the fused or separate push), with the
// float intrinsics as IEEE single-precision operations (compiled without
// contraction; fmaf for the fused multiply-add). Test infrastructure:
// tests/test_host_ds.py compares every cell with the oracle's orc_ds_cell.
//
//   host_ds <in> <out> <method 0|1> <alpha> <fused 0|1>
//   in: n x 8 cell bytes (dz, dy, dx order); out: n bytes
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <algorithm>
#include <vector>

#define __device__
#define __host__
#define __forceinline__ inline

static inline float __fmul_rn(float a, float b) { return a * b; }
static inline float __fsub_rn(float a, float b) { return a - b; }
static inline float __fadd_rn(float a, float b) { return a + b; }
static inline float __fmaf_rn(float a, float b, float c) { return fmaf(a, b, c); }
static inline float __uint2float_rn(uint32_t u) { return (float)u; }
static inline int __float2int_rz(float f) { return (int)f; }
static inline uint32_t max(uint32_t a, uint32_t b) { return std::max(a, b); }

#include "ds_cell.cuh"

int main(int argc, char **argv) {
    if (argc != 6) return 2;
    FILE *fi = fopen(argv[1], "rb"), *fo = fopen(argv[2], "wb");
    if (!fi || !fo) return 2;
    const int method = atoi(argv[3]);
    const float alpha = strtof(argv[4], nullptr);
    const bool fused = atoi(argv[5]) != 0;
    uint8_t b[8];
    while (fread(b, 1, 8, fi) == 8) {
        uint32_t c[8];
        for (int i = 0; i < 8; ++i) c[i] = b[i];
        const uint32_t v = method == 0 ? vcg::ds_cell<0>(c, alpha, fused) : vcg::ds_cell<1>(c, alpha, fused);
        fputc((int)v, fo);
    }
    fclose(fi);
    fclose(fo);
    return 0;
}

// Value of one 2x2x2 cell under the exporter's within-cell methods
// (tools/downscale.h:29-93), shared by the downscale kernels (k_ds.cu):
// DS_BOX (M = 0) and DS_CBOX (M = 1), see k_ds.cu for the rounding rules.
#pragma once
#include <stdint.h>

namespace vcg {

// The DS_CBOX value of one cell from its sum and its chosen voxel.
__device__ __forceinline__ uint32_t cbox_value(uint32_t sum, uint32_t best, float alpha, bool fused) {
    const float mean = __fmul_rn(__uint2float_rn(sum), 0.125f);
    const float d = __fsub_rn(__uint2float_rn(best), mean);
    const float v = fused ? __fmaf_rn(alpha, d, mean) : __fadd_rn(mean, __fmul_rn(alpha, d));
    if (v < 0.0f) return 0;
    if (v > 255.0f) return 255;
    return (uint32_t)__float2int_rz(__fadd_rn(v, 0.5f));   // 0 for an all-zero cell
}

template <int M>
__device__ __forceinline__ uint32_t ds_cell(const uint32_t (&c)[8], float alpha, bool fused) {
    uint32_t sum = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) sum += c[i];
    if (M == 0) return (sum + 4u) >> 3;   // 0 for an all-zero cell, as the reference's short-circuit
    // largest 8 |c - mean| (exact), the first in order on ties: one max over
    // keys deviation << 11 | (7 - i) << 8 | c
    uint32_t key = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i)
        key = max(key, (uint32_t)abs(8 * (int)c[i] - (int)sum) << 11 | (uint32_t)(7 - i) << 8 | c[i]);
    return cbox_value(sum, key & 0xFFu, alpha, fused);
}

}  // namespace vcg

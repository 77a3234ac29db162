// Exact integer DCT-32 passes on the int8 tensor cores (device), shared by the
// whole-atom transform and the batched decode.
//
// One pass is OUT = C V over an atom's 1024 lines (8 lines per
// mma.sync.m16n8k32 s8 x s8 -> s32 tile). CMATA (|c| <= 4091) is split into two
// int8 pieces c = 128 c1 + c0 (c0 = c & 127, c1 = c >> 7); a pass input v into
// VP pieces v = sum_j 128^j v_j (v_j = (v >> 7j) & 127 below the top piece, the
// top piece v >> 7(VP-1), signed). Products of equal weight 128^(cp+j) share an
// s32 accumulator; recombining the accumulators by shift-add modulo 2^32 gives
// the reference's i32 sum (src/vc/vc.c:142-205), then (s + 8192) >> 14.
// Values live in shared memory as VP int8 piece planes of 32 bytes per line,
// in two ping-pong buffers.
#pragma once
#include <stdint.h>

#include "dct32.cuh"
#include "vc_release_tables.h"

namespace vcg {

// Byte of element n in a 32-byte piece line, arranged so that lane (g, t) of
// an m16n8k32 B fragment finds its elements n = 4t..4t+3 and 16+4t..16+4t+3 as
// one aligned 8-byte word.
__device__ __forceinline__ int ppos(int n) { return (((n & 15) >> 2) << 3) | ((n >> 4) << 2) | (n & 3); }

__device__ __forceinline__ void mma_s8(int32_t (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+r"(d[0]), "+r"(d[1]), "+r"(d[2]), "+r"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// piece j of v (VP pieces): low pieces 7 bits, the top piece signed
template <int VP>
__device__ __forceinline__ uint32_t piece(int32_t v, int j) {
    return j < VP - 1 ? (uint32_t)(v >> (7 * j)) & 127u : (uint32_t)(v >> (7 * (VP - 1))) & 0xFFu;
}
template <int VP>
__device__ __forceinline__ bool fits(int32_t v) {
    const int32_t top = v >> (7 * (VP - 1));
    return top >= -128 && top <= 127;
}

// A fragments of the two coefficient pieces for this lane: rows g, g+8 (+16 per
// m-tile), columns 4t..4t+3 and 16+4t..16+4t+3; A = C (forward) or C^T (inverse).
template <bool INV>
__device__ __forceinline__ void imma_a_frags(uint32_t (&A)[2][2][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int cp = 0; cp < 2; ++cp)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int row = mt * 16 + g + (r & 1) * 8, col0 = (r >> 1) * 16 + t * 4;
                uint32_t w = 0;
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    const int32_t c = INV ? c_cmat[col0 + b][row] : c_cmat[row][col0 + b];
                    const uint32_t p = cp ? (uint32_t)(c >> 7) & 0xFFu : (uint32_t)c & 127u;
                    w |= p << (8 * b);
                }
                A[mt][cp][r] = w;
            }
}

// piece plane j of ping-pong buffer b (VP planes of 32 KiB per buffer)
template <int VP>
__device__ __forceinline__ uint8_t *imma_plane(uint8_t *sm, int b, int j) { return sm + (b * VP + j) * 32768; }

// Pass `pass` (0..2) over one atom: lines of buffer (pass & 1), 8 per MMA tile,
// tiles spread over the CTA's warps. The output of line (a, b) at row k is the
// reference's axis rotation: element b of line k*32 + a. On passes 0 and 1 it is
// written as pieces to buffer (pass & 1) ^ 1 (bad is set when a value leaves
// the VP-piece range); on pass 2 each pair of rounded outputs of rows k of lines
// (a, b), (a, b + 1) goes to fin(k, a, b, o0, o1).
template <int VP, int NT, class Fin>
__device__ __forceinline__ void imma_pass(uint8_t *sm, const uint32_t (&A)[2][2][4], int pass, bool &bad, Fin &&fin) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, g = lane >> 2, t = lane & 3;
    const int sb = pass & 1, db = sb ^ 1;
#pragma unroll 1
    for (int tile = warp; tile < 128; tile += NT / 32) {
        const int L0 = tile * 8;
        uint32_t B[VP][2];
#pragma unroll
        for (int j = 0; j < VP; ++j) {
            const uint2 w = *reinterpret_cast<const uint2 *>(imma_plane<VP>(sm, sb, j) + (L0 + g) * 32 + t * 8);
            B[j][0] = w.x;
            B[j][1] = w.y;
        }
        int32_t acc[2][VP + 1][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int w = 0; w <= VP; ++w)
#pragma unroll
                for (int r = 0; r < 4; ++r) acc[mt][w][r] = 0;
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int cp = 0; cp < 2; ++cp)
#pragma unroll
                for (int j = 0; j < VP; ++j) mma_s8(acc[mt][cp + j], A[mt][cp], B[j][0], B[j][1]);
        // lane holds rows k = 16 mt + 8 h + g of lines L0 + 2t, L0 + 2t + 1
        const int line = L0 + 2 * t, la = line >> 5, lb = line & 31;
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int k = mt * 16 + h * 8 + g;
                int32_t o[2];
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    uint32_t s = 0;
#pragma unroll
                    for (int w = 0; w <= VP; ++w) s += (uint32_t)acc[mt][w][h * 2 + e] << (7 * w);
                    o[e] = (int32_t)(s + 8192u) >> 14;
                }
                if (pass < 2) {
                    bad |= !fits<VP>(o[0]) || !fits<VP>(o[1]);
                    const int off = (k * 32 + la) * 32 + ppos(lb);
#pragma unroll
                    for (int j = 0; j < VP; ++j)
                        *reinterpret_cast<uint16_t *>(imma_plane<VP>(sm, db, j) + off) =
                            (uint16_t)(piece<VP>(o[0], j) | (piece<VP>(o[1], j) << 8));
                } else {
                    fin(k, la, lb, o[0], o[1]);
                }
            }
    }
}

}  // namespace vcg

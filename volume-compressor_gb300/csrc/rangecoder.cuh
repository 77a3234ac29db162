// Adaptive binary range coder and coefficient context coder, one GPU thread
// per atom (device).
//
// Bit-exact with the reference's coder (src/vc/vc.c:344-560): 12-bit P(0),
// shift-5 adaptation, LZMA-style carry-less low with a cached byte, 16-bit EOB
// in bypass bits, 8 significance contexts by frequency band + 12 unary
// magnitude contexts, EG0 escape tail and sign in bypass bits, contexts reset
// per atom. Two facts keep the per-bit work branch-light: a probability never
// leaves [31, 4065], so starting from range >= 2^24 one renormalisation byte
// always suffices (the reference's while-loops run at most once); and the scan
// order is sorted by frequency, so the significance band is non-decreasing
// along the scan and only one band context is live at a time.
#pragma once
#include <stdint.h>

namespace vcg {

constexpr uint32_t kTop = 1u << 24;

__device__ __forceinline__ void adapt(uint32_t &p, int bit) {
    p = bit ? p - (p >> 5) : p + ((4096u - p) >> 5);
}

// ---------------------------------------------------------------- decoder
struct RcDec {
    const uint8_t *buf;
    uint32_t len, pos, code, range;

    __device__ __forceinline__ uint32_t next_byte() {
        uint32_t b = pos < len ? (uint32_t)__ldg(buf + pos) : 0u;   // zeros past the end
        ++pos;
        return b;
    }
    __device__ __forceinline__ void init(const uint8_t *b, uint32_t n) {   // src/vc/vc.c:403-413
        buf = b; len = n; pos = 0; code = 0; range = 0xFFFFFFFFu;
#pragma unroll
        for (int i = 0; i < 5; ++i) code = (code << 8) | next_byte();
    }
    __device__ __forceinline__ int bit(uint32_t &p) {   // src/vc/vc.c:414-430
        uint32_t r0 = (uint32_t)(((uint64_t)range * p) >> 12);
        int b = code >= r0;
        if (b) { code -= r0; range -= r0; } else { range = r0; }
        adapt(p, b);
        if (range < kTop) { code = (code << 8) | next_byte(); range <<= 8; }
        return b;
    }
    __device__ __forceinline__ int bypass() {   // src/vc/vc.c:431-441
        range >>= 1;
        int b = code >= range;
        if (b) code -= range;
        if (range < kTop) { code = (code << 8) | next_byte(); range <<= 8; }
        return b;
    }
};

// Decode one atom's levels. Calls sink(scan_position, level) for every
// nonzero level in scan order. Returns 0, or 1 for a malformed stream (EG0
// escape prefix longer than 32 ones, which no encoder output contains).
template <class Sink>
__device__ __forceinline__ int rc_decode_levels(RcDec &d, const uint32_t *band_start, Sink &&sink) {
    uint32_t eob = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) eob = (eob << 1) | (uint32_t)d.bypass();
    if (eob > 32768u) eob = 32768u;   // src/vc/vc.c:549
    uint32_t mag[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) mag[k] = 2048u;
    uint32_t p = 0;
    for (int b = 0; b < 8 && p < eob; ++b) {
        uint32_t sig = 2048u;
        uint32_t end = band_start[b + 1] < eob ? band_start[b + 1] : eob;
        for (; p < end; ++p) {
            if (!d.bit(sig)) continue;
            uint32_t v = 0, m = 0;   // src/vc/vc.c:491-506
            bool done = false;
#pragma unroll
            for (int k = 0; k < 11; ++k) {
                if (!done) {
                    if (d.bit(mag[k])) ++v;
                    else { m = v + 1; done = true; }
                }
            }
            if (!done) {
                if (!d.bit(mag[11])) {
                    m = v + 1;
                } else {
                    uint32_t nb = 0;
                    while (d.bypass()) {
                        if (++nb > 32u) return 1;
                    }
                    uint32_t x = 1;
                    for (uint32_t i = 0; i < nb; ++i) x = (x << 1) | (uint32_t)d.bypass();
                    m = v + (x - 1u) + 1u;
                }
            }
            int neg = d.bypass();
            sink(p, (uint32_t)(neg ? 0u - m : m) & 0xFFFFu);
        }
    }
    return 0;
}

// ---------------------------------------------------------------- encoder
// WRITE = false only tracks the interval width: the byte count of the
// reference encoder equals its number of shift-low calls (renormalisation
// steps plus the 5 flush steps), which does not depend on `low`.
template <bool WRITE>
struct RcEnc {
    uint64_t low;
    uint32_t range, pending, nbytes;
    uint32_t cache;
    uint8_t *out;

    __device__ __forceinline__ void init(uint8_t *o) {
        low = 0; range = 0xFFFFFFFFu; pending = 1; nbytes = 0; cache = 0; out = o;
    }
    __device__ __forceinline__ void shift_low() {   // src/vc/vc.c:369-380
        if (!WRITE) { ++nbytes; return; }
        if ((uint32_t)(low >> 32) != 0u || low < 0xFF000000ull) {
            uint32_t carry = (uint32_t)(low >> 32);
            uint32_t c = cache;
            do {
                out[nbytes++] = (uint8_t)(c + carry);
                c = 0xFFu;
            } while (--pending);
            cache = (uint32_t)(low >> 24) & 0xFFu;
        }
        ++pending;
        low = (low << 8) & 0xFFFFFFFFull;
    }
    __device__ __forceinline__ void bit(uint32_t &p, int b) {   // src/vc/vc.c:381-393
        uint32_t r0 = (uint32_t)(((uint64_t)range * p) >> 12);
        if (b) { if (WRITE) low += r0; range -= r0; } else { range = r0; }
        adapt(p, b);
        if (range < kTop) { shift_low(); range <<= 8; }
    }
    __device__ __forceinline__ void bypass(int b) {   // src/vc/vc.c:394-398
        range >>= 1;
        if (WRITE && b) low += range;
        if (range < kTop) { shift_low(); range <<= 8; }
    }
    __device__ __forceinline__ void flush() {
#pragma unroll 1
        for (int i = 0; i < 5; ++i) shift_low();
    }
};

// Encode one atom from its nonzero levels in scan order: ent[i] = scan
// position | level << 16. Returns the range-coder byte count
// (src/vc/vc.c:471-490, 512-544).
template <bool WRITE>
__device__ __forceinline__ uint32_t rc_encode_levels(const uint32_t *ent, uint32_t nnz,
                                                     const uint32_t *band_start, uint8_t *out) {
    RcEnc<WRITE> e;
    e.init(out);
    uint32_t eob = nnz ? (ent[nnz - 1] & 0xFFFFu) + 1u : 0u;
#pragma unroll
    for (int i = 15; i >= 0; --i) e.bypass((eob >> i) & 1u);
    uint32_t mag[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) mag[k] = 2048u;
    uint32_t p = 0, sig = 2048u;
    int b = 0;
    uint32_t bend = band_start[1];
    for (uint32_t i = 0; i < nnz; ++i) {
        uint32_t w = ent[i];
        uint32_t pi = w & 0xFFFFu;
        int32_t lv = (int16_t)(w >> 16);
        while (p < pi) {   // zero run, crossing band boundaries
            if (p == bend) { ++b; bend = band_start[b + 1]; sig = 2048u; }
            uint32_t stop = pi < bend ? pi : bend;
            for (; p < stop; ++p) e.bit(sig, 0);
        }
        while (p >= bend) { ++b; bend = band_start[b + 1]; sig = 2048u; }
        e.bit(sig, 1);
        uint32_t v = (uint32_t)(lv < 0 ? -lv : lv) - 1u;
        bool done = false;
#pragma unroll
        for (int k = 0; k < 11; ++k) {
            if (!done) {
                if (v == 0) { e.bit(mag[k], 0); done = true; }
                else { e.bit(mag[k], 1); --v; }
            }
        }
        if (!done) {
            if (v == 0) {
                e.bit(mag[11], 0);
            } else {
                e.bit(mag[11], 1);
                uint32_t x1 = v + 1u;
                uint32_t nb = 31u - __clz(x1);
                for (uint32_t j = 0; j < nb; ++j) e.bypass(1);
                e.bypass(0);
                for (int j = (int)nb - 1; j >= 0; --j) e.bypass((x1 >> j) & 1u);
            }
        }
        e.bypass(lv < 0);
        ++p;
    }
    e.flush();
    return e.nbytes;
}

}  // namespace vcg

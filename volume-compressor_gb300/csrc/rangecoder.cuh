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

// ---------------------------------------------------------------- fast decoder
// Stream bytes through a 64-bit window refilled from aligned 32-bit words, with
// the next word always already in flight, so a renormalisation never waits on
// memory. Words are big-endian-ordered; bytes outside [0, len) read as zero and
// words wholly outside the stream are never loaded.
struct StreamWin {
    const uint32_t *wp;   // aligned word containing stream byte 0
    int32_t lim0;         // len + misalignment: bytes of the stream + lead-in
    uint32_t wi;          // index of the word in `pf`
    uint64_t win;         // valid bytes at the top
    int32_t wb;           // valid bits in win
    uint32_t pf;          // prefetched word wi

    __device__ __forceinline__ uint32_t word(uint32_t i) const {
        int32_t lim = lim0 - 4 * (int32_t)i;   // stream bytes (from the front) in word i
        uint32_t raw = lim > 0 ? __ldg(wp + i) : 0u;
        uint32_t w = __byte_perm(raw, 0, 0x0123);
        return lim >= 4 ? w : (lim <= 0 ? 0u : w & (0xFFFFFFFFu << (8 * (4 - lim))));
    }
    __device__ __forceinline__ void init(const uint8_t *p, uint32_t len) {
        uintptr_t a = (uintptr_t)p;
        int32_t mis = (int32_t)(a & 3u);
        wp = reinterpret_cast<const uint32_t *>(a - (uintptr_t)mis);
        lim0 = (int32_t)len + mis;
        win = ((uint64_t)word(0) << 32) << (8 * mis);
        wb = 32 - 8 * mis;
        win |= (uint64_t)word(1) << (32 - wb);
        wb += 32;
        wi = 2;
        pf = word(2);
    }
    __device__ __forceinline__ uint32_t byte() {
        uint32_t b = (uint32_t)(win >> 56);
        win <<= 8;
        wb -= 8;
        if (wb <= 32) {
            win |= (uint64_t)pf << (32 - wb);
            wb += 32;
            pf = word(++wi);
        }
        return b;
    }
    // Branch-free variant: consumes the top byte only when `take`; the refill
    // is predicated too, so the lanes of a warp stay converged.
    __device__ __forceinline__ uint32_t byte_if(bool take) {
        const uint32_t b = (uint32_t)(win >> 56);
        win = take ? win << 8 : win;
        wb = take ? wb - 8 : wb;
        const bool need = wb <= 32;
        win |= need ? (uint64_t)pf << (32 - wb) : 0ull;
        wb = need ? wb + 32 : wb;
        wi = need ? wi + 1 : wi;
        if (need) pf = word(wi);
        return b;
    }
};

// One binary decision per loop iteration for every lane (no divergence between
// significance, magnitude, escape and sign decisions). Phases below PH_EOB use
// an adaptive context; the 12 magnitude contexts live in this thread's column
// of a shared-memory array (ctx[j * stride], j = 0..11) so that selecting one
// by index costs a single load.
enum : uint32_t { PH_SIG = 0, PH_MAG, PH_EOB, PH_EGP, PH_EGS, PH_SIGN, PH_DONE };

// Calls sink(scan_position, level) for every nonzero level in scan order;
// returns 0, or 1 for a malformed stream (escape prefix longer than 32 ones).
template <class Sink>
__device__ __forceinline__ int rc_decode_levels_fast(const uint8_t *src, uint32_t len, const uint32_t *band_start,
                                                     uint32_t *ctx, int stride, Sink &&sink) {
    StreamWin s;
    s.init(src, len);
    uint32_t code = 0, range = 0xFFFFFFFFu;
#pragma unroll
    for (int i = 0; i < 5; ++i) code = (code << 8) | s.byte();
#pragma unroll
    for (int j = 0; j < 12; ++j) ctx[j * stride] = 2048u;
    uint32_t phase = PH_EOB, cnt = 16, eob = 0, p = 0, k = 0, x = 0, m = 0, sig = 2048u;
    uint32_t band = 0, bend = band_start[1];
    int bad = 0;
    while (phase != PH_DONE) {
        const uint32_t cv = ctx[k * stride];
        const bool isSIG = phase == PH_SIG, isMAG = phase == PH_MAG, isEOB = phase == PH_EOB;
        const bool isEGP = phase == PH_EGP, isEGS = phase == PH_EGS, isSIGN = phase == PH_SIGN;
        const bool adaptive = phase < PH_EOB;
        const uint32_t pr = isSIG ? sig : cv;
        const uint32_t rm = (uint32_t)(((uint64_t)range * pr) >> 12);
        const uint32_t r0 = adaptive ? rm : (range >> 1);
        const bool bit = code >= r0;
        code = bit ? code - r0 : code;
        range = (bit && adaptive) ? range - r0 : r0;
        const bool ren = range < kTop;
        const uint32_t nbyte = s.byte_if(ren);
        code = ren ? (code << 8) | nbyte : code;
        range = ren ? range << 8 : range;
        const uint32_t npr = bit ? pr - (pr >> 5) : pr + ((4096u - pr) >> 5);
        sig = isSIG ? npr : sig;
        if (isMAG) ctx[k * stride] = npr;
        if (isSIGN) sink(p, (bit ? 0u - m : m) & 0xFFFFu);
        // next state, all as selects
        const uint32_t cnt0 = cnt, k0 = k;
        const uint32_t x2 = (x << 1) | (uint32_t)bit;
        const bool egs_end = isEGS && cnt0 == 1u;
        const bool eob_end = isEOB && cnt0 == 1u;
        const bool egp_over = isEGP && bit && cnt0 + 1u > 32u;
        const uint32_t eob2 = (eob << 1) | (uint32_t)bit;
        eob = isEOB ? ((eob_end && eob2 > 32768u) ? 32768u : eob2) : eob;
        m = (isMAG && !bit) ? k0 + 1u : m;
        m = (isEGP && !bit && cnt0 == 0u) ? 12u : m;
        m = egs_end ? 11u + x2 : m;
        x = isEGS ? x2 : (isEGP ? 1u : x);
        bad |= egp_over ? 1 : 0;
        cnt = (isEOB || isEGS) ? cnt0 - 1u : cnt0;
        cnt = (isEGP && bit) ? cnt0 + 1u : cnt;
        cnt = (isMAG && bit && k0 == 11u) ? 0u : cnt;
        k = (isSIG && bit) ? 0u : k0;
        k = (isMAG && bit && k0 < 11u) ? k0 + 1u : k;
        const bool adv = (isSIG && !bit) || isSIGN;
        p = adv ? p + 1u : p;
        uint32_t nph = phase;
        nph = isSIG ? (bit ? PH_MAG : PH_SIG) : nph;
        nph = isMAG ? (!bit ? PH_SIGN : (k0 == 11u ? PH_EGP : PH_MAG)) : nph;
        nph = isEGP ? (bit ? (egp_over ? PH_DONE : PH_EGP) : (cnt0 == 0u ? PH_SIGN : PH_EGS)) : nph;
        nph = egs_end ? PH_SIGN : nph;
        nph = isSIGN ? PH_SIG : nph;
        nph = eob_end ? (eob ? PH_SIG : PH_DONE) : nph;
        nph = (adv && p >= eob) ? PH_DONE : nph;
        phase = nph;
        const bool bsw = adv && p == bend;
        band = bsw ? band + 1u : band;
        if (bsw) bend = band_start[band < 8u ? band + 1u : 8u];
        sig = bsw ? 2048u : sig;
    }
    return bad;
}

// ---------------------------------------------------------------- lockstep decoder
// All lanes of a warp walk the scan positions together, each lane decoding its
// own atom. The significance band and the unary-magnitude index are then
// warp-uniform, so every context is a register with a static index and every
// decision is the same instruction stream for all lanes; a lane with nothing to
// decode at a step (past its EOB, or a zero at this position during the
// magnitude steps) runs along predicated off, and warp votes end the magnitude
// steps as soon as no lane needs another one.
constexpr uint32_t kFull = 0xFFFFFFFFu;

__device__ __forceinline__ bool dec_ctx(bool on, uint32_t &code, uint32_t &range, uint32_t &prob, StreamWin &s) {
    const uint32_t r0 = (uint32_t)(((uint64_t)range * prob) >> 12);
    const bool b = code >= r0;
    const uint32_t nrange = b ? range - r0 : r0;
    const uint32_t ncode = b ? code - r0 : code;
    const uint32_t nprob = b ? prob - (prob >> 5) : prob + ((4096u - prob) >> 5);
    const bool ren = on && nrange < kTop;
    const uint32_t byte = s.byte_if(ren);
    code = on ? (ren ? (ncode << 8) | byte : ncode) : code;
    range = on ? (ren ? nrange << 8 : nrange) : range;
    prob = on ? nprob : prob;
    return b;
}

__device__ __forceinline__ bool dec_byp(bool on, uint32_t &code, uint32_t &range, StreamWin &s) {
    const uint32_t r0 = range >> 1;
    const bool b = code >= r0;
    const uint32_t ncode = b ? code - r0 : code;
    const bool ren = on && r0 < kTop;
    const uint32_t byte = s.byte_if(ren);
    code = on ? (ren ? (ncode << 8) | byte : ncode) : code;
    range = on ? (ren ? r0 << 8 : r0) : range;
    return b;
}

// Every lane of the warp must call this together. `active` lanes decode the
// stream src[0..len); the others take part predicated off. Calls sink(scan
// position, level) for each nonzero level of an active lane; returns 1 for a
// malformed stream (escape prefix longer than 32 ones), else 0.
template <class Sink>
__device__ __forceinline__ int rc_decode_levels_warp(const uint8_t *src, uint32_t len, bool active,
                                                     const uint32_t *band_start, Sink &&sink) {
    StreamWin s;
    s.init(active ? src : nullptr, active ? len : 0u);
    uint32_t code = 0, range = 0xFFFFFFFFu;
#pragma unroll
    for (int i = 0; i < 5; ++i) code = (code << 8) | s.byte_if(true);
    uint32_t eob = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) eob = (eob << 1) | (uint32_t)dec_byp(active, code, range, s);
    if (!active) eob = 0;
    if (eob > 32768u) eob = 32768u;
    const uint32_t eob_max = __reduce_max_sync(kFull, eob);
    uint32_t mag[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) mag[k] = 2048u;
    bool bad = false;
    for (int b = 0; b < 8; ++b) {
        uint32_t sig = 2048u;
        const uint32_t pend = band_start[b + 1] < eob_max ? band_start[b + 1] : eob_max;
        for (uint32_t p = band_start[b]; p < pend; ++p) {
            const bool on = p < eob && !bad;
            const bool nz = dec_ctx(on, code, range, sig, s) && on;
            if (!__any_sync(kFull, nz)) continue;
            uint32_t m = 0;
            bool go = nz;
#pragma unroll
            for (int k = 0; k < 12; ++k) {
                if (!__any_sync(kFull, go)) break;
                const bool one = dec_ctx(go, code, range, mag[k], s);
                m = (go && !one) ? (uint32_t)k + 1u : m;
                go = go && one;
            }
            if (__any_sync(kFull, go)) {   // escape: EG0 tail in bypass bits (rare)
                uint32_t nb = 0, x = 1, rem = 0;
                bool pre = go, suf = false;
                while (__any_sync(kFull, pre || suf)) {
                    const bool one = dec_byp(pre || suf, code, range, s);
                    if (pre) {
                        if (one) {
                            if (++nb > 32u) { bad = true; pre = false; }
                        } else {
                            pre = false;
                            suf = nb != 0;
                            rem = nb;
                        }
                    } else if (suf) {
                        x = (x << 1) | (uint32_t)one;
                        suf = --rem != 0;
                    }
                }
                m = go ? 11u + x : m;
            }
            const bool emit = nz && !bad;
            const bool neg = dec_byp(emit, code, range, s);
            if (emit) sink(p, (neg ? 0u - m : m) & 0xFFFFu);
        }
    }
    return bad ? 1 : 0;
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

// Same output as rc_encode_levels, one decision per loop iteration for every
// lane, magnitude contexts in shared memory as in the decoder; the coefficient
// list is read four entries at a time with the next four already in flight
// (ent must be 16-byte aligned).
template <bool WRITE>
__device__ __forceinline__ uint32_t rc_encode_levels_fast(const uint32_t *ent, uint32_t nnz,
                                                          const uint32_t *band_start, uint32_t *ctx, int stride,
                                                          uint8_t *out) {
    RcEnc<WRITE> e;
    e.init(out);
    auto load4 = [&](uint32_t j) -> uint4 {
        return j < nnz ? __ldg(reinterpret_cast<const uint4 *>(ent + j)) : make_uint4(0, 0, 0, 0);
    };
    const uint32_t eob = nnz ? (ent[nnz - 1] & 0xFFFFu) + 1u : 0u;
    uint4 g = load4(0), gn = load4(4);
    uint32_t gi = 0, cur = g.x;
#pragma unroll
    for (int j = 0; j < 12; ++j) ctx[j * stride] = 2048u;
    uint32_t phase = PH_EOB, cnt = 16, p = 0, i = 0, k = 0, v = 0, nb = 0, x1 = 0, sig = 2048u;
    uint32_t band = 0, bend = band_start[1];
    while (phase != PH_DONE) {
        const uint32_t cv = ctx[k * stride];
        const bool isSIG = phase == PH_SIG, isMAG = phase == PH_MAG, isEOB = phase == PH_EOB;
        const bool isEGP = phase == PH_EGP, isEGS = phase == PH_EGS, isSIGN = phase == PH_SIGN;
        const bool adaptive = phase < PH_EOB;
        const uint32_t pr = isSIG ? sig : cv;
        const uint32_t sh = (isEOB || isEGS) ? cnt - 1u : 0u;
        const uint32_t bits_src = isEOB ? eob : x1;
        bool bit = ((bits_src >> sh) & 1u) != 0;   // PH_EOB / PH_EGS
        bit = isSIG ? p == (cur & 0xFFFFu) : bit;
        bit = isMAG ? v != 0 : bit;
        bit = isEGP ? nb > cnt : bit;
        bit = isSIGN ? (cur >> 31) != 0 : bit;
        const uint32_t rm = (uint32_t)(((uint64_t)e.range * pr) >> 12);
        const uint32_t r0 = adaptive ? rm : (e.range >> 1);
        if (WRITE) e.low += bit ? r0 : 0u;
        e.range = (bit && adaptive) ? e.range - r0 : r0;
        const bool ren = e.range < kTop;
        if (WRITE) {
            if (ren) e.shift_low();
        } else {
            e.nbytes += ren ? 1u : 0u;
        }
        e.range = ren ? e.range << 8 : e.range;
        const uint32_t npr = bit ? pr - (pr >> 5) : pr + ((4096u - pr) >> 5);
        sig = isSIG ? npr : sig;
        if (isMAG) ctx[k * stride] = npr;
        // next state, all as selects
        const uint32_t cnt0 = cnt, k0 = k;
        const int32_t lv = (int16_t)(cur >> 16);
        const uint32_t vnew = (uint32_t)(lv < 0 ? -lv : lv) - 1u;
        const bool mag_esc = isMAG && bit && k0 == 11u;
        const uint32_t x1n = v + 1u;
        x1 = mag_esc ? x1n : x1;
        nb = mag_esc ? 31u - __clz(x1n) : nb;
        v = (isSIG && bit) ? vnew : ((isMAG && bit && k0 < 11u) ? v - 1u : v);
        k = (isSIG && bit) ? 0u : ((isMAG && bit && k0 < 11u) ? k0 + 1u : k0);
        cnt = (isEOB || isEGS) ? cnt0 - 1u : cnt0;
        cnt = mag_esc ? 0u : cnt;
        cnt = isEGP ? (bit ? cnt0 + 1u : nb) : cnt;
        const bool adv = (isSIG && !bit) || isSIGN;
        uint32_t nph = phase;
        nph = isSIG ? (bit ? PH_MAG : PH_SIG) : nph;
        nph = isMAG ? (!bit ? PH_SIGN : (k0 == 11u ? PH_EGP : PH_MAG)) : nph;
        nph = isEGP ? (bit ? PH_EGP : (nb ? PH_EGS : PH_SIGN)) : nph;
        nph = (isEGS && cnt0 == 1u) ? PH_SIGN : nph;
        nph = isSIGN ? PH_SIG : nph;
        nph = (isEOB && cnt0 == 1u) ? (eob ? PH_SIG : PH_DONE) : nph;
        // the list advances past an entry after its sign
        i = isSIGN ? i + 1u : i;
        const uint32_t gi1 = isSIGN ? gi + 1u : gi;
        const bool refill = gi1 == 4u;
        g = refill ? gn : g;
        if (refill) gn = load4(i + 4u);
        gi = refill ? 0u : gi1;
        cur = gi == 0u ? g.x : gi == 1u ? g.y : gi == 2u ? g.z : g.w;
        p = adv ? p + 1u : p;
        nph = (adv && p >= eob) ? PH_DONE : nph;
        phase = nph;
        const bool bsw = adv && p == bend;
        band = bsw ? band + 1u : band;
        if (bsw) bend = band_start[band < 8u ? band + 1u : 8u];
        sig = bsw ? 2048u : sig;
    }
    e.flush();
    return e.nbytes;
}

// ---------------------------------------------------------------- lockstep encoder
template <bool WRITE>
__device__ __forceinline__ void enc_ctx(bool on, bool bit, RcEnc<WRITE> &e, uint32_t &prob) {
    const uint32_t r0 = (uint32_t)(((uint64_t)e.range * prob) >> 12);
    if (WRITE && on && bit) e.low += r0;
    const uint32_t nrange = bit ? e.range - r0 : r0;
    const uint32_t nprob = bit ? prob - (prob >> 5) : prob + ((4096u - prob) >> 5);
    const bool ren = on && nrange < kTop;
    if (WRITE) {
        if (ren) e.shift_low();
    } else {
        e.nbytes += ren ? 1u : 0u;
    }
    e.range = on ? (ren ? nrange << 8 : nrange) : e.range;
    prob = on ? nprob : prob;
}

template <bool WRITE>
__device__ __forceinline__ void enc_byp(bool on, bool bit, RcEnc<WRITE> &e) {
    const uint32_t r0 = e.range >> 1;
    if (WRITE && on && bit) e.low += r0;
    const bool ren = on && r0 < kTop;
    if (WRITE) {
        if (ren) e.shift_low();
    } else {
        e.nbytes += ren ? 1u : 0u;
    }
    e.range = on ? (ren ? r0 << 8 : r0) : e.range;
}

// Every lane of the warp must call this together; `active` lanes encode their
// list ent[0..nnz) (scan position | level << 16, 16-byte aligned) and return
// the coder byte count (inactive lanes return 0). Same output as
// rc_encode_levels.
template <bool WRITE>
__device__ __forceinline__ uint32_t rc_encode_levels_warp(const uint32_t *ent, uint32_t nnz, bool active,
                                                          const uint32_t *band_start, uint8_t *out) {
    RcEnc<WRITE> e;
    e.init(out);
    if (!active) nnz = 0;
    auto load4 = [&](uint32_t j) -> uint4 {
        return j < nnz ? __ldg(reinterpret_cast<const uint4 *>(ent + j)) : make_uint4(0, 0, 0, 0);
    };
    const uint32_t eob = nnz ? (ent[nnz - 1] & 0xFFFFu) + 1u : 0u;
#pragma unroll
    for (int i = 15; i >= 0; --i) enc_byp(active, (eob >> i) & 1u, e);
    const uint32_t eob_max = __reduce_max_sync(kFull, eob);
    uint4 g = load4(0), gn = load4(4);
    uint32_t gi = 0, i = 0, cur = g.x;
    uint32_t mag[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) mag[k] = 2048u;
    for (int b = 0; b < 8; ++b) {
        uint32_t sig = 2048u;
        const uint32_t pend = band_start[b + 1] < eob_max ? band_start[b + 1] : eob_max;
        for (uint32_t p = band_start[b]; p < pend; ++p) {
            const bool on = p < eob;
            const bool nz = on && p == (cur & 0xFFFFu);
            enc_ctx(on, nz, e, sig);
            if (!__any_sync(kFull, nz)) continue;
            const int32_t lv = (int16_t)(cur >> 16);
            const uint32_t m = (uint32_t)(lv < 0 ? -lv : lv);
            bool go = nz;
#pragma unroll
            for (int k = 0; k < 12; ++k) {
                if (!__any_sync(kFull, go)) break;
                const bool one = m > (uint32_t)k + 1u;   // unary: 1 while more remains
                enc_ctx(go, one, e, mag[k]);
                go = go && one;
            }
            if (__any_sync(kFull, go)) {   // escape: EG0 of m - 12 in bypass bits (rare)
                const uint32_t x1 = go ? m - 11u : 2u;
                const uint32_t nb = 31u - __clz(x1);
                uint32_t step = 0;
                const uint32_t total = go ? 2u * nb + 1u : 0u;
                while (__any_sync(kFull, step < total)) {
                    const bool on2 = step < total;
                    const bool one = step < nb ? true : (step == nb ? false : ((x1 >> (2u * nb - step)) & 1u) != 0);
                    enc_byp(on2, one, e);
                    ++step;
                }
            }
            enc_byp(nz, lv < 0, e);
            // the lane's list advances past this entry
            i = nz ? i + 1u : i;
            const uint32_t gi1 = nz ? gi + 1u : gi;
            const bool refill = gi1 == 4u;
            g = refill ? gn : g;
            if (refill) gn = load4(i + 4u);
            gi = refill ? 0u : gi1;
            cur = gi == 0u ? g.x : gi == 1u ? g.y : gi == 2u ? g.z : g.w;
        }
    }
    if (active) e.flush();
    return active ? e.nbytes : 0u;
}

}  // namespace vcg

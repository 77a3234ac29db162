// Adaptive binary range coder and coefficient context coder (device): one
// atom per GPU thread, either alone in its warp (latency path) or in a warp of
// atoms decoded in lockstep (throughput path).
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

// ---------------------------------------------------------------- decoder
// Stream bytes of one lane: up to four unconsumed bytes at the top of `cur`
// (`nb` bits), refilled from the next aligned word `pf`, which is always
// already loaded, so a renormalisation never waits on memory. Words are read
// big-endian-ordered; bytes outside [0, len) read as zero and words wholly
// outside the stream are never loaded. A decision consumes at most one byte,
// so refilling whenever cur runs empty keeps a byte ready for the next one.
struct ByteStream {
    const uint32_t *wp;   // aligned word containing stream byte 0
    int32_t lim0;         // len + misalignment: bytes of the stream + lead-in
    uint32_t wi;          // index of the word in pf
    uint32_t cur, pf;
    uint32_t nb;          // valid bits in cur

    __device__ __forceinline__ uint32_t word(uint32_t i) const {
        const int32_t lim = lim0 - 4 * (int32_t)i;   // stream bytes (from the front) in word i
        const uint32_t raw = lim > 0 ? __ldg(wp + i) : 0u;
        const uint32_t w = __byte_perm(raw, 0, 0x0123);
        return lim >= 4 ? w : (lim <= 0 ? 0u : w & (0xFFFFFFFFu << (8 * (4 - lim))));
    }
    __device__ __forceinline__ void init(const uint8_t *p, uint32_t len) {
        const uintptr_t a = (uintptr_t)p;
        const uint32_t mis = (uint32_t)(a & 3u);
        wp = reinterpret_cast<const uint32_t *>(a - (uintptr_t)mis);
        lim0 = (int32_t)(len + mis);
        cur = word(0) << (8 * mis);
        nb = 32u - 8u * mis;
        wi = 1;
        pf = word(1);
    }
    // code = code << sh | next sh bits of the stream (sh = 0 or 8)
    __device__ __forceinline__ void shift(uint32_t &code, uint32_t sh) {
        code = __funnelshift_l(cur, code, sh);
        cur <<= sh;
        nb -= sh;
    }
    __device__ __forceinline__ void refill() {
        cur = pf;
        nb = 32u;
        pf = word(++wi);
    }
    __device__ __forceinline__ void refill_if(bool need) {
        cur = need ? pf : cur;
        nb = need ? 32u : nb;
        wi = need ? wi + 1u : wi;
        if (need) pf = word(wi);
    }
};

// Adaptive decision with P(0) = prob / 4096 (src/vc/vc.c:414-430): the split
// point (range * prob) >> 12 is the high word of range * (prob << 20), and the
// two adaptation rules are one: prob += ((bit ? 31 : 4096) - prob) >> 5 with an
// arithmetic shift (for bit = 1 it equals -(prob >> 5)). A bypass decision
// (src/vc/vc.c:431-441) is the split range >> 1 without adaptation.
__device__ __forceinline__ uint32_t rc_split(uint32_t range, uint32_t prob) { return __umulhi(range, prob << 20); }
__device__ __forceinline__ uint32_t rc_adapt(uint32_t prob, bool bit) {
    return prob + (uint32_t)((int32_t)((bit ? 31u : 4096u) - prob) >> 5);
}

// One atom per thread, for warps that decode a single atom (latency path):
// plain branches, contexts in registers. Calls sink(scan_position, level) for
// every nonzero level in scan order (src/vc/vc.c:545-560); returns 0, or 1 for
// a malformed stream (escape prefix longer than 32 ones, which no encoder
// output contains).
template <class Sink>
__device__ __forceinline__ int rc_decode_levels_lane(const uint8_t *src, uint32_t len, const uint32_t *band_start,
                                                     Sink &&sink) {
    ByteStream s;
    s.init(src, len);
    uint32_t code = 0, range = 0xFFFFFFFFu;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        s.shift(code, 8);
        if (s.nb == 0) s.refill();
    }
    auto renorm = [&]() {
        if (range < kTop) {
            range <<= 8;
            s.shift(code, 8);
            if (s.nb == 0) s.refill();
        }
    };
    auto bit = [&](uint32_t &prob) -> bool {
        const uint32_t r0 = rc_split(range, prob);
        const bool b = code >= r0;
        code = b ? code - r0 : code;
        range = b ? range - r0 : r0;
        prob = rc_adapt(prob, b);
        renorm();
        return b;
    };
    auto bypass = [&]() -> bool {
        range >>= 1;
        const bool b = code >= range;
        code = b ? code - range : code;
        renorm();
        return b;
    };
    uint32_t eob = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) eob = (eob << 1) | (uint32_t)bypass();
    if (eob > 32768u) eob = 32768u;   // src/vc/vc.c:549
    uint32_t mag[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) mag[k] = 2048u;
    for (int b = 0; b < 8; ++b) {
        const uint32_t beg = band_start[b];
        if (beg >= eob) break;
        const uint32_t end = band_start[b + 1] < eob ? band_start[b + 1] : eob;
        uint32_t sig = 2048u;
        for (uint32_t p = beg; p < end; ++p) {
            if (!bit(sig)) continue;
            uint32_t m = 0;   // unary magnitude, then EG0 escape (src/vc/vc.c:491-506)
#pragma unroll
            for (int k = 0; k < 12; ++k) {
                if (!bit(mag[k])) {
                    m = (uint32_t)k + 1u;
                    break;
                }
            }
            if (m == 0) {
                uint32_t ones = 0;
                while (bypass()) {
                    if (++ones > 32u) return 1;
                }
                uint32_t x = 1;
                for (uint32_t i = 0; i < ones; ++i) x = (x << 1) | (uint32_t)bypass();
                m = 11u + x;
            }
            const bool neg = bypass();
            sink(p, (neg ? 0u - m : m) & 0xFFFFu);
        }
    }
    return 0;
}

// ---------------------------------------------------------------- lockstep decoder
// The lanes of a warp walk the scan positions together, each lane decoding its
// own atom. The significance band and the unary-magnitude index are then
// warp-uniform, so every context is a register with a static index and every
// decision is the same instruction stream for all lanes. The significance step
// runs unpredicated (a lane past its EOB decodes garbage that is never used;
// its reads stay inside its stream); magnitude, escape and sign steps are
// predicated on the lanes that need them, and warp votes end them as soon as no
// lane needs another one.
constexpr uint32_t kFull = 0xFFFFFFFFu;

__device__ __forceinline__ bool ls_ctx(bool on, uint32_t &code, uint32_t &range, uint32_t &prob, ByteStream &s) {
    const uint32_t r0 = rc_split(range, prob);
    const bool b = code >= r0;
    const uint32_t nr = b ? range - r0 : r0;
    const uint32_t nc = b ? code - r0 : code;
    const uint32_t np = rc_adapt(prob, b);
    range = on ? nr : range;
    code = on ? nc : code;
    prob = on ? np : prob;
    const uint32_t sh = (on && nr < kTop) ? 8u : 0u;
    range <<= sh;
    s.shift(code, sh);
    return b;
}

__device__ __forceinline__ bool ls_byp(bool on, uint32_t &code, uint32_t &range, ByteStream &s) {
    const uint32_t r0 = range >> 1;
    const bool b = code >= r0;
    code = (on && b) ? code - r0 : code;
    range = on ? r0 : range;
    const uint32_t sh = (on && r0 < kTop) ? 8u : 0u;
    range <<= sh;
    s.shift(code, sh);
    return b;
}

__device__ __forceinline__ void ls_keep(ByteStream &s) { s.refill_if(s.nb == 0); }

// Every lane of the warp must call this together. `active` lanes decode the
// stream src[0..len); the others take part predicated off. Same results as
// rc_decode_levels_lane for each active lane.
template <class Sink>
__device__ __forceinline__ int rc_decode_levels_warp(const uint8_t *src, uint32_t len, bool active,
                                                     const uint32_t *band_start, Sink &&sink) {
    ByteStream s;
    s.init(active ? src : nullptr, active ? len : 0u);
    uint32_t code = 0, range = 0xFFFFFFFFu;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        s.shift(code, 8);
        s.refill_if(s.nb == 0);
    }
    uint32_t eob = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        eob = (eob << 1) | (uint32_t)ls_byp(true, code, range, s);
        s.refill_if(s.nb == 0);
    }
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
            const uint32_t r0 = rc_split(range, sig);
            const bool one = code >= r0;
            code = one ? code - r0 : code;
            range = one ? range - r0 : r0;
            sig = rc_adapt(sig, one);
            const uint32_t sh = range < kTop ? 8u : 0u;
            range <<= sh;
            s.shift(code, sh);
            const bool nz = one && p < eob && !bad;
            ls_keep(s);
            if (!__any_sync(kFull, nz)) continue;
            // unary magnitude: every lane with a nonzero takes step 0, so it needs
            // no vote; the escape vote is taken with the last step
            uint32_t m = 0;
            bool go = nz, esc = false;
#pragma unroll
            for (int k = 0; k < 12; ++k) {
                if (k > 0 && !__any_sync(kFull, go)) break;
                const bool more = ls_ctx(go, code, range, mag[k], s);
                m = (go && !more) ? (uint32_t)k + 1u : m;
                go = go && more;
                ls_keep(s);
                if (k == 11) esc = __any_sync(kFull, go);
            }
            if (esc) {   // escape: EG0 tail in bypass bits (rare)
                uint32_t ones = 0, x = 1, rem = 0;
                bool pre = go, suf = false;
                while (__any_sync(kFull, pre || suf)) {
                    const bool bit = ls_byp(pre || suf, code, range, s);
                    ls_keep(s);
                    if (pre) {
                        if (bit) {
                            if (++ones > 32u) { bad = true; pre = false; }
                        } else {
                            pre = false;
                            suf = ones != 0;
                            rem = ones;
                        }
                    } else if (suf) {
                        x = (x << 1) | (uint32_t)bit;
                        suf = --rem != 0;
                    }
                }
                m = go ? 11u + x : m;
            }
            const bool emit = nz && !bad;
            const bool neg = ls_byp(emit, code, range, s);
            ls_keep(s);
            if (emit) sink(p, (neg ? 0u - m : m) & 0xFFFFu);
        }
    }
    return bad ? 1 : 0;
}

// ---------------------------------------------------------------- per-lane decoder
// Each lane of a warp decodes its own atom and every step is one binary
// decision of that atom, whatever its kind: the lanes of a warp are at
// different points of their streams, and no lane waits for another (unlike the
// lockstep decoder, whose warps run every magnitude step as long as any lane
// needs it). The decision kind is the lane's state:
//   0        significance bit of scan position p (band context, a register)
//   1..12    unary magnitude step c - 1 (context mag[c - 1] in shared memory)
//   13       escape: exponential-Golomb prefix of ones (bypass)
//   14       bypass run: the escape suffix bits, then the sign bit
//   15       done
// (src/vc/vc.c:491-506, 545-560). A bypass bit is the adaptive split with
// probability 2048 and no adaptation, except that the range becomes the half
// for both bit values (src/vc/vc.c:431-441). The magnitude context of the next
// step is loaded from shared memory one step ahead. Stream bytes are fetched
// one at a time, one byte ahead of the renormalisation that consumes them;
// bytes past the end read as zero. Probabilities are kept unscaled (12 bits).
__device__ __forceinline__ uint32_t ld_u8_if(bool on, const uint8_t *ptr, uint32_t old) {
#ifdef __CUDA_ARCH__
    uint32_t v = old;
    asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q ld.global.nc.u8 %0, [%1];\n\t}"
                 : "+r"(v) : "l"(ptr), "r"((uint32_t)on));
    return v;
#else
    return on ? *ptr : old;
#endif
}
__device__ __forceinline__ void st_u32_if(bool on, uint32_t *ptr, uint32_t v) {
#ifdef __CUDA_ARCH__
    asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q st.global.u32 [%0], %1;\n\t}"
                 :: "l"(ptr), "r"(v), "r"((uint32_t)on) : "memory");
#else
    if (on) *ptr = v;
#endif
}

constexpr uint32_t kLaneDone = 15u;

struct RcLane {
    const uint8_t *src;
    uint32_t pos, len;     // next byte to fetch; stream length
    uint32_t nxt;          // the byte at pos (0 past the end)
    uint32_t code, range;
    uint32_t c, r, m;      // state; escape / run count; magnitude so far
    uint32_t p, eob, bend, bi;   // scan position, EOB, end of the current band, band
    uint32_t sigp, magp;   // context of the current band; magnitude context of the next step
    uint32_t *dst;         // coefficient list (scan position | level << 16)
    uint32_t n, cap, bad;  // entries decoded (all, also past cap); list capacity; malformed

    // bstart: the 9-entry band table followed by a copy of its last entry (a
    // lane that ends at the last band's end loads the entry after it).
    // S: this lane's 12 magnitude contexts at S[0], S[st], ..., S[11 * st]
    __device__ __forceinline__ void init(const uint8_t *s, uint32_t l, bool active, const uint32_t *bstart,
                                         uint32_t *S, uint32_t st, uint32_t *d, uint32_t cp) {
        src = s;
        len = active ? l : 0u;
        uint32_t cd = 0;
#pragma unroll
        for (uint32_t i = 0; i < 5; ++i) cd = (cd << 8) | (i < len ? (uint32_t)__ldg(src + i) : 0u);
        pos = 5;
        nxt = 5 < len ? __ldg(src + 5) : 0u;
        uint32_t rg = 0xFFFFFFFFu, e = 0;
#pragma unroll
        for (int i = 0; i < 16; ++i) {   // 16-bit EOB in bypass bits (src/vc/vc.c:520-525)
            rg >>= 1;
            const bool b = cd >= rg;
            cd = b ? cd - rg : cd;
            e = (e << 1) | (b ? 1u : 0u);
            if (rg < kTop) {
                rg <<= 8;
                cd = (cd << 8) | nxt;
                ++pos;
                nxt = pos < len ? __ldg(src + pos) : 0u;
            }
        }
        if (e > 32768u) e = 32768u;   // src/vc/vc.c:549
        code = cd;
        range = rg;
        eob = e;
        p = 0;
        bi = 0;
        bend = bstart[1];
        sigp = 2048u;
        magp = 2048u;
#pragma unroll
        for (int k = 0; k < 12; ++k) S[k * st] = 2048u;
        c = (active && e) ? 0u : kLaneDone;
        r = 0;
        m = 0;
        dst = d;
        n = 0;
        cap = cp;
        bad = 0;
    }

    __device__ __forceinline__ void step(const uint32_t *bstart, uint32_t *S, uint32_t st) {
        const uint32_t s0 = c;
        const bool isA = s0 < 13u, isPre = s0 == 13u, isRun = s0 == 14u, isSig = s0 == 0u;
        const uint32_t nmag = S[(s0 < 11u ? s0 : 11u) * st];   // context of step s0 + 1 if this bit is a one
        const uint32_t pc = isSig ? sigp : magp;
        const uint32_t pr = isA ? pc : 2048u;
        const uint32_t r0 = __umulhi(range, pr << 20);
        const bool b = code >= r0;
        const uint32_t one = b ? 1u : 0u;
        code = b ? code - r0 : code;
        const uint32_t nr = (b && isA) ? range - r0 : r0;
        const uint32_t pa = rc_adapt(pc, b);
        if (s0 - 1u < 12u) S[(s0 - 1u) * st] = pa;
        sigp = isSig ? pa : sigp;
        magp = nmag;
        // renormalisation: one byte at most
        const bool ren = nr < kTop;
        range = ren ? nr << 8 : nr;
        code = ren ? (code << 8) | nxt : code;
        const uint32_t np_ = pos + (ren ? 1u : 0u);
        pos = np_;
        nxt = ld_u8_if(ren && np_ < len, src + np_, ren ? 0u : nxt);
        // the sign bit ends a run of one: emit the level
        const uint32_t r_ = r, m_ = m;
        const bool last = isRun && r_ == 1u;
        const uint32_t sm = b ? 0u - m_ : m_;
        st_u32_if(last && n < cap, dst + n, (sm << 16) | p);
        n += last ? 1u : 0u;
        // next state: a one climbs the ladder (12 -> 13 is the escape); a zero at
        // significance moves on, a zero on the ladder ends the magnitude (run of
        // one: the sign); the prefix ends with a zero (run of ones + 1 bits)
        const uint32_t cA = b ? s0 + 1u : (isSig ? 0u : 14u);
        const uint32_t cB = isPre ? 14u - one : (last ? 0u : 14u);
        uint32_t nc = isA ? cA : (s0 == kLaneDone ? kLaneDone : cB);
        r = isA ? one ^ 1u : (isPre ? r_ + 1u : r_ - 1u);
        // magnitude: the ladder step that ended it, or 11 + the suffix value
        m = isA ? s0 : (isPre ? 12u : 2u * m_ + one - 11u);
        const bool malformed = isPre && b && r_ == 32u;   // a prefix of 33 ones: no level needs it
        bad |= malformed ? 1u : 0u;
        const bool adv = (isSig && !b) || last;
        const uint32_t pn = p + (adv ? 1u : 0u);
        p = pn;
        const bool cross = adv && pn == bend;   // next band: fresh context
        nc = (malformed || (adv && pn == eob)) ? kLaneDone : nc;
        const uint32_t nbi = bi + (cross ? 1u : 0u);
        bi = nbi;
        bend = cross ? bstart[nbi + 1u] : bend;
        sigp = cross ? 2048u : sigp;
        c = nc;
    }
};

// ---------------------------------------------------------------- latency decoder
// One atom on one lane when few atoms share the GPU, so that the dependency
// chain of one decision is all that counts: both outcomes of a decision (the
// new range renormalised, the adapted probability) are computed before the
// compare, which then only selects; the byte fetch is predicated, not
// branched; and a significance decision takes one branch (a one, or the end of
// the band). Same results as rc_decode_levels_lane; measured on GB300 with one
// atom per SM sub-partition 44 ns per decision against 57 ns. With several
// warps per sub-partition its extra instructions make it slower, so it serves
// only the latency-bound case.
struct RcIn {
    const uint8_t *src;
    uint32_t pos, len, nxt;   // next byte to fetch (nxt: its value, 0 past the end)
};

__device__ __forceinline__ uint32_t rc_take_if(bool ren, uint32_t c1, RcIn &in) {
    const uint32_t nx = in.nxt;
    const uint32_t np = in.pos + (ren ? 1u : 0u);
    in.pos = np;
    in.nxt = ld_u8_if(ren && np < in.len, in.src + np, ren ? 0u : nx);
    return ren ? (c1 << 8) | nx : c1;
}

__device__ __forceinline__ bool rc_bit_lat(uint32_t &code, uint32_t &range, uint32_t &p, RcIn &in) {
    const uint32_t r0 = __umulhi(range, p << 20);
    const uint32_t p0 = p + ((4096u - p) >> 5), p1 = p - (p >> 5);
    const uint32_t n1 = range - r0;
    const bool ren0 = r0 < kTop, ren1 = n1 < kTop;
    const uint32_t rr0 = ren0 ? r0 << 8 : r0, rr1 = ren1 ? n1 << 8 : n1;
    const bool b = code >= r0;
    const uint32_t c1 = b ? code - r0 : code;
    range = b ? rr1 : rr0;
    p = b ? p1 : p0;
    code = rc_take_if(b ? ren1 : ren0, c1, in);
    return b;
}

__device__ __forceinline__ bool rc_bypass_lat(uint32_t &code, uint32_t &range, RcIn &in) {
    const uint32_t r0 = range >> 1;
    const bool b = code >= r0;
    const uint32_t c1 = b ? code - r0 : code;
    const bool ren = r0 < kTop;
    range = ren ? r0 << 8 : r0;
    code = rc_take_if(ren, c1, in);
    return b;
}

template <class Sink>
__device__ __forceinline__ int rc_decode_levels_lat(const uint8_t *src, uint32_t len, const uint32_t *band_start,
                                                    Sink &&sink) {
    RcIn in;
    in.src = src;
    in.len = len;
    uint32_t code = 0;
#pragma unroll
    for (uint32_t i = 0; i < 5; ++i) code = (code << 8) | (i < len ? (uint32_t)__ldg(src + i) : 0u);
    in.pos = 5;
    in.nxt = 5 < len ? __ldg(src + 5) : 0u;
    uint32_t range = 0xFFFFFFFFu, eob = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) eob = (eob << 1) | (rc_bypass_lat(code, range, in) ? 1u : 0u);
    if (eob > 32768u) eob = 32768u;   // src/vc/vc.c:549
    uint32_t mag[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) mag[k] = 2048u;
    for (int bnd = 0; bnd < 8; ++bnd) {
        uint32_t p = band_start[bnd];
        if (p >= eob) break;
        const uint32_t lim = band_start[bnd + 1] < eob ? band_start[bnd + 1] : eob;
        uint32_t sig = 2048u;
        for (;;) {
            const bool one = rc_bit_lat(code, range, sig, in);
            if (!(one | (p + 1u == lim))) {
                ++p;
                continue;
            }
            if (one) {
                uint32_t m = 0;   // unary magnitude, then EG0 escape (src/vc/vc.c:491-506)
#pragma unroll
                for (int k = 0; k < 12; ++k) {
                    if (!rc_bit_lat(code, range, mag[k], in)) {
                        m = (uint32_t)k + 1u;
                        break;
                    }
                }
                if (m == 0) {
                    uint32_t ones = 0;
                    while (rc_bypass_lat(code, range, in)) {
                        if (++ones > 32u) return 1;
                    }
                    uint32_t x = 1;
                    for (uint32_t i = 0; i < ones; ++i) x = (x << 1) | (rc_bypass_lat(code, range, in) ? 1u : 0u);
                    m = 11u + x;
                }
                const bool neg = rc_bypass_lat(code, range, in);
                sink(p, (neg ? 0u - m : m) & 0xFFFFu);
            }
            if (++p == lim) break;
        }
    }
    return 0;
}

// ---------------------------------------------------------------- latency decoder, staged stream
// The same decisions with the stream first copied to shared memory (a zero
// byte after it), for one atom on one thread. A decision's outcome selects by
// masks, not predicates (a predicate read right after it is written costs more
// latency than the mask arithmetic): the 33-bit difference code - r0 gives the
// mask of a zero bit. The renormalisation shift is clz(range) & 8: a split
// leaves at least 2^16 (the probability stays in [31, 4065] and the range at
// least 2^24), so clz < 16 and bit 3 of clz says range < 2^24. The next four
// stream bytes sit in a window that funnel shifts feed into the code; the byte
// after them is read from shared memory every decision (clamped to the zero
// byte). The adaptation is one formula for both outcomes: p - ((p - 4065) >> 5)
// (arithmetic shift) is p + (4096 - p) / 32 rounded down, p - (p >> 5) the
// other. Measured on GB300, one atom: 42 ns per decision against 50 ns for
// rc_decode_levels_lat.
struct RcSm {
    const uint8_t *s;     // stream bytes, s[len] == 0
    uint32_t len, pos;    // pos: stream index of the window's first byte
    uint32_t w;           // bytes pos .. pos + 3, the first in the top byte
};

__device__ __forceinline__ uint32_t rcs_clz(uint32_t x) {
#ifdef __CUDA_ARCH__
    return (uint32_t)__clz(x);
#else
    return x ? (uint32_t)__builtin_clz(x) : 32u;
#endif
}

__device__ __forceinline__ uint32_t rcs_fsl(uint32_t lo, uint32_t hi, uint32_t sh) {
#ifdef __CUDA_ARCH__
    return __funnelshift_l(lo, hi, sh);
#else
    return (uint32_t)(((((uint64_t)hi << 32) | lo) << (sh & 31u)) >> 32);
#endif
}

__device__ __forceinline__ void rcs_norm(uint32_t &code, uint32_t &range, uint32_t c1, uint32_t nr, RcSm &in) {
    const uint32_t s = rcs_clz(nr) & 8u;
    const uint32_t q = in.pos + 4u;
    const uint32_t b4 = (uint32_t)in.s[q < in.len ? q : in.len] << 24;
    range = nr << s;
    code = rcs_fsl(in.w, c1, s);
    in.w = rcs_fsl(b4, in.w, s);
    in.pos += s >> 3;
}

// adaptive decision; returns all ones for a zero bit, 0 for a one
__device__ __forceinline__ uint32_t rcs_bit(uint32_t &code, uint32_t &range, uint32_t &p, RcSm &in) {
    const uint32_t r0 = __umulhi(range, p << 20);
    const uint64_t dd = (uint64_t)code - (uint64_t)r0;
    const uint32_t z = (uint32_t)(dd >> 32);
    const uint32_t c1 = (code & z) | ((uint32_t)dd & ~z);
    const uint32_t nr = (r0 & z) | ((range - r0) & ~z);
    p = p - (uint32_t)((int32_t)(p - (z & 4065u)) >> 5);
    rcs_norm(code, range, c1, nr, in);
    return z;
}

__device__ __forceinline__ uint32_t rcs_bypass(uint32_t &code, uint32_t &range, RcSm &in) {
    const uint32_t r0 = range >> 1;
    const uint64_t dd = (uint64_t)code - (uint64_t)r0;
    const uint32_t z = (uint32_t)(dd >> 32);
    const uint32_t c1 = (code & z) | ((uint32_t)dd & ~z);
    rcs_norm(code, range, c1, r0, in);
    return z;
}

// s: the stream in shared memory, s[len] == 0
template <class Sink>
__device__ __forceinline__ int rc_decode_levels_sm(const uint8_t *s, uint32_t len, const uint32_t *band_start,
                                                   Sink &&sink) {
    RcSm in;
    in.s = s;
    in.len = len;
    uint32_t code = 0;
#pragma unroll
    for (uint32_t i = 0; i < 5; ++i) code = (code << 8) | s[i < len ? i : len];
    in.pos = 5;
    in.w = 0;
#pragma unroll
    for (uint32_t i = 5; i < 9; ++i) in.w = (in.w << 8) | s[i < len ? i : len];
    uint32_t range = 0xFFFFFFFFu, eob = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) eob = (eob << 1) | (rcs_bypass(code, range, in) ? 0u : 1u);
    if (eob > 32768u) eob = 32768u;   // src/vc/vc.c:549
    uint32_t mag[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) mag[k] = 2048u;
    for (int bnd = 0; bnd < 8; ++bnd) {
        uint32_t p = band_start[bnd];
        if (p >= eob) break;
        const uint32_t lim = band_start[bnd + 1] < eob ? band_start[bnd + 1] : eob;
        uint32_t sig = 2048u;
        for (;;) {
            const uint32_t z = rcs_bit(code, range, sig, in);
            if (z && p + 1u != lim) {
                ++p;
                continue;
            }
            if (!z) {
                uint32_t m = 0;   // unary magnitude, then EG0 escape (src/vc/vc.c:491-506)
#pragma unroll
                for (int k = 0; k < 12; ++k) {
                    if (rcs_bit(code, range, mag[k], in)) {
                        m = (uint32_t)k + 1u;
                        break;
                    }
                }
                if (m == 0) {
                    uint32_t ones = 0;
                    while (!rcs_bypass(code, range, in)) {
                        if (++ones > 32u) return 1;
                    }
                    uint32_t x = 1;
                    for (uint32_t i = 0; i < ones; ++i) x = (x << 1) | (rcs_bypass(code, range, in) ? 0u : 1u);
                    m = 11u + x;
                }
                const bool neg = !rcs_bypass(code, range, in);
                sink(p, (neg ? 0u - m : m) & 0xFFFFu);
            }
            if (++p == lim) break;
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
    uint32_t cap;   // bytes stored at most (the count goes on past it)

    __device__ __forceinline__ void init(uint8_t *o, uint32_t c) {
        low = 0; range = 0xFFFFFFFFu; pending = 1; nbytes = 0; cache = 0; out = o; cap = c;
    }
    __device__ __forceinline__ void shift_low() {   // src/vc/vc.c:369-380
        if (!WRITE) { ++nbytes; return; }
        if ((uint32_t)(low >> 32) != 0u || low < 0xFF000000ull) {
            uint32_t carry = (uint32_t)(low >> 32);
            uint32_t c = cache;
            do {
                if (nbytes < cap) out[nbytes] = (uint8_t)(c + carry);
                ++nbytes;
                c = 0xFFu;
            } while (--pending);
            cache = (uint32_t)(low >> 24) & 0xFFu;
        }
        ++pending;
        low = (low << 8) & 0xFFFFFFFFull;
    }
    __device__ __forceinline__ void flush() {
#pragma unroll 1
        for (int i = 0; i < 5; ++i) shift_low();
    }
    // shift_low for the lanes with ren, the others unchanged, without a branch
    // around the common case: a byte leaves (cache + carry) unless the top byte
    // is 0xFF without carry; the 0xFF bytes held back before it (pending - 1 of
    // them, rarely any) follow as 0xFF + carry.
    __device__ __forceinline__ void shift_low_if(bool ren) {
        if (!WRITE) { nbytes += ren ? 1u : 0u; return; }
        const uint32_t hi = (uint32_t)(low >> 32);
        const bool emit = ren && (hi != 0u || low < 0xFF000000ull);
        if (emit && nbytes < cap) out[nbytes] = (uint8_t)(cache + hi);
        if (emit && pending > 1u) {
            const uint8_t fill = (uint8_t)(0xFFu + hi);
            for (uint32_t j = 1; j < pending; ++j)
                if (nbytes + j < cap) out[nbytes + j] = fill;
        }
        nbytes = emit ? nbytes + pending : nbytes;
        cache = emit ? (uint32_t)(low >> 24) & 0xFFu : cache;
        pending = ren ? (emit ? 1u : pending + 1u) : pending;
        low = ren ? (low << 8) & 0xFFFFFFFFull : low;
    }
};

// ---------------------------------------------------------------- lockstep encoder
// Predicated adaptive (src/vc/vc.c:381-393) and bypass (src/vc/vc.c:394-398)
// encoder decisions; lanes with on = false keep their state.
template <bool WRITE>
__device__ __forceinline__ void enc_ctx(bool on, bool bit, RcEnc<WRITE> &e, uint32_t &prob) {
    const uint32_t r0 = rc_split(e.range, prob);
    if (WRITE && on && bit) e.low += r0;
    const uint32_t nrange = bit ? e.range - r0 : r0;
    const uint32_t nprob = rc_adapt(prob, bit);
    const bool ren = on && nrange < kTop;
    e.shift_low_if(ren);
    e.range = on ? (ren ? nrange << 8 : nrange) : e.range;
    prob = on ? nprob : prob;
}

template <bool WRITE>
__device__ __forceinline__ void enc_byp(bool on, bool bit, RcEnc<WRITE> &e) {
    const uint32_t r0 = e.range >> 1;
    if (WRITE && on && bit) e.low += r0;
    const bool ren = on && r0 < kTop;
    e.shift_low_if(ren);
    e.range = on ? (ren ? r0 << 8 : r0) : e.range;
}

// Every lane of the warp must call this together; `active` lanes encode their
// list ent[0..nnz) (scan position | level << 16, 16-byte aligned) and return
// the coder byte count (inactive lanes return 0): the reference encoder's bytes
// (src/vc/vc.c:471-490, 512-544). At most `cap` bytes are stored.
template <bool WRITE>
__device__ __forceinline__ uint32_t rc_encode_levels_warp(const uint32_t *ent, uint32_t nnz, bool active,
                                                          const uint32_t *band_start, uint8_t *out,
                                                          uint32_t cap = 0xFFFFFFFFu) {
    RcEnc<WRITE> e;
    e.init(out, cap);
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
            // every lane with a nonzero takes unary step 0, so it needs no vote;
            // the escape vote is taken with the last step
            bool go = nz, esc = false;
#pragma unroll
            for (int k = 0; k < 12; ++k) {
                if (k > 0 && !__any_sync(kFull, go)) break;
                const bool one = m > (uint32_t)k + 1u;   // unary: 1 while more remains
                enc_ctx(go, one, e, mag[k]);
                go = go && one;
                if (k == 11) esc = __any_sync(kFull, go);
            }
            if (esc) {   // escape: EG0 of m - 12 in bypass bits (rare)
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

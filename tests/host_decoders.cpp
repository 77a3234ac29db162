// Host build of the device range decoders (volume-compressor_gb300/csrc/
// rangecoder.cuh) with single-lane stand-ins for the CUDA intrinsics. Test
// infrastructure: every decoder must give the oracle's level list and status for
// the streams of the input file (tests/test_host_decoders.py writes it from the
// oracle's decode of golden archives, coded noise and crafted streams).
//
// Input (little-endian): u32 n; per stream: u32 len, u32 bad, u32 nent, then
// len stream bytes, then nent entries (scan position | level << 16, scan order).
// Output: one line per decoder, "<name> <streams that differ> <streams>".
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <vector>

#define __device__
#define __host__
#define __forceinline__ inline
#define __global__
#define __constant__

static inline uint32_t __umulhi(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * b) >> 32); }
static inline uint32_t __ldg(const uint32_t *p) { return *p; }
static inline uint8_t __ldg(const uint8_t *p) { return *p; }
static inline uint32_t __byte_perm(uint32_t x, uint32_t y, uint32_t s) {
    const uint64_t v = ((uint64_t)y << 32) | x;
    uint32_t r = 0;
    for (int i = 0; i < 4; ++i) r |= (uint32_t)((v >> (8 * ((s >> (4 * i)) & 7u))) & 0xFFu) << (8 * i);
    return r;
}
static inline uint32_t __funnelshift_l(uint32_t lo, uint32_t hi, uint32_t sh) {
    return (uint32_t)(((((uint64_t)hi << 32) | lo) << (sh & 31u)) >> 32);
}
static inline int __clz(uint32_t x) { return x ? __builtin_clz(x) : 32; }
static inline bool __any_sync(uint32_t, bool v) { return v; }   // one lane: the warp is this lane
static inline uint32_t __reduce_max_sync(uint32_t, uint32_t v) { return v; }
struct uint2 { uint32_t x, y; };
struct uint4 { uint32_t x, y, z, w; };
static inline uint4 make_uint4(uint32_t a, uint32_t b, uint32_t c, uint32_t d) { return uint4{a, b, c, d}; }
static inline uint4 __ldg(const uint4 *p) { return *p; }

#include "rangecoder.cuh"

using namespace vcg;

// first scan position of each significance band: frequency classes f = x + y + z
// (0..93) in 8 bands of 12 classes, the last one shorter
static void band_table(uint32_t *bs) {
    uint32_t cnt[94] = {0};
    for (int a = 0; a < 32; ++a)
        for (int b = 0; b < 32; ++b)
            for (int c = 0; c < 32; ++c) cnt[a + b + c]++;
    uint32_t pos = 0;
    int b = 0;
    bs[0] = 0;
    for (int f = 0; f < 94; ++f) {
        int bb = f * 8 / 96;
        if (bb > 7) bb = 7;
        while (b < bb) bs[++b] = pos;
        pos += cnt[f];
    }
    while (b < 8) bs[++b] = pos;
}

struct Result {
    int bad;
    std::vector<uint32_t> ent;
};

// The oracle's decode is a raster of 16-bit levels, so a level whose low 16
// bits are 0 (a crafted escape of 65536 k) is not in its list: compare the
// decoders' entries without those.
static bool same(const Result &r, uint32_t bad, const uint32_t *want, uint32_t nent) {
    if ((r.bad != 0) != (bad != 0)) return false;
    if (bad) return true;   // a malformed stream: the status is the result
    std::vector<uint32_t> got;
    for (uint32_t e : r.ent)
        if (e >> 16) got.push_back(e);
    return got.size() == nent && (nent == 0 || memcmp(got.data(), want, 4ull * nent) == 0);
}

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    uint32_t n = 0;
    if (fread(&n, 4, 1, f) != 1) return 2;
    uint32_t bs[10];   // the band table and a copy of its end, as the kernels hold it for RcLane
    band_table(bs);
    bs[9] = bs[8];
    const char *names[5] = {"latency", "staged", "scalar", "lockstep", "per-lane"};
    int diff[5] = {0, 0, 0, 0, 0};
    for (uint32_t k = 0; k < n; ++k) {
        uint32_t h[3];
        if (fread(h, 4, 3, f) != 3) return 2;
        const uint32_t len = h[0], bad = h[1], nent = h[2];
        // the stream at a varying misalignment between zero guard bytes
        std::vector<uint8_t> buf(len + 48, 0);
        uint8_t *src = buf.data() + 16 + (k & 3u);
        if (len && fread(src, 1, len, f) != len) return 2;
        std::vector<uint32_t> want(nent);
        if (nent && fread(want.data(), 4, nent, f) != nent) return 2;
        Result r[5];
        for (auto &x : r) x.ent.reserve(nent + 16);
        auto sink_to = [](Result &x) { return [&x](uint32_t p, uint32_t lv) { x.ent.push_back(p | (lv << 16)); }; };
        r[0].bad = rc_decode_levels_lat(src, len, bs, sink_to(r[0]));
        r[1].bad = rc_decode_levels_sm(src, len, bs, sink_to(r[1]));   // src[len] is a zero guard byte
        r[2].bad = rc_decode_levels_lane(src, len, bs, sink_to(r[2]));
        r[3].bad = rc_decode_levels_warp(src, len, true, bs, sink_to(r[3]));
        {
            const uint32_t cap = 65536;   // more than any stream's levels (at most 32768)
            std::vector<uint32_t> dst(cap);
            uint32_t S[12];
            RcLane L;
            L.init(src, len, true, bs, S, 1, dst.data(), cap);
            while (L.c != kLaneDone) L.step(bs, S, 1);
            for (int i = 0; i < 37; ++i) L.step(bs, S, 1);   // a finished lane steps on with its warp
            r[4].bad = (int)L.bad;
            r[4].ent.assign(dst.begin(), dst.begin() + (L.n < cap ? L.n : cap));
        }
        for (int d = 0; d < 5; ++d) diff[d] += !same(r[d], bad, want.data(), nent);
    }
    fclose(f);
    for (int d = 0; d < 5; ++d) printf("%s %d %u\n", names[d], diff[d], n);
    return 0;
}

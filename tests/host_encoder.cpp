// Host build of the device range encoder (volume-compressor_gb300/csrc/
// rangecoder.cuh: rc_encode_levels_warp, the warp-lockstep encoder run here as
// one lane, with single-lane stand-ins for the CUDA intrinsics). Test
// infrastructure: tests/test_host_encoder.py writes level lists with the
// oracle's bytes for them; every list must encode to those bytes (and the
// size-only pass to their count), also into a buffer too small for them.
//
// Input (little-endian): u32 n; per list: u32 nent, u32 nbytes, then nent
// entries (scan position | level << 16, scan order), then nbytes bytes.
// Output: "write <lists that differ> <lists>", "size ...", "capped ...".
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
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

static void band_table(uint32_t *bs) {   // first scan position of each significance band
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

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    uint32_t n = 0;
    if (fread(&n, 4, 1, f) != 1) return 2;
    uint32_t bs[9];
    band_table(bs);
    int dw = 0, ds = 0, dc = 0;
    for (uint32_t k = 0; k < n; ++k) {
        uint32_t h[2];
        if (fread(h, 4, 2, f) != 2) return 2;
        const uint32_t nent = h[0], nbytes = h[1];
        // entries 16-byte aligned with room for the encoder's look-ahead loads
        const size_t ebytes = (4 * ((size_t)nent + 16) + 64 + 15) & ~(size_t)15;   // a multiple of the alignment
        uint32_t *ent = (uint32_t *)aligned_alloc(16, ebytes);
        memset(ent, 0, ebytes);
        std::vector<uint8_t> want(nbytes + 1);
        if (nent && fread(ent, 4, nent, f) != nent) return 2;
        if (nbytes && fread(want.data(), 1, nbytes, f) != nbytes) return 2;
        std::vector<uint8_t> out(nbytes + 4096, 0xA5);
        const uint32_t got = rc_encode_levels_warp<true>(ent, nent, true, bs, out.data());
        dw += got != nbytes || memcmp(out.data(), want.data(), nbytes) != 0;
        ds += rc_encode_levels_warp<false>(ent, nent, true, bs, nullptr) != nbytes;
        // into a buffer of half the size: the count goes on, nothing is stored past the cap
        const uint32_t cap = nbytes / 2;
        std::vector<uint8_t> half(nbytes + 64, 0x3C);
        const uint32_t gc = rc_encode_levels_warp<true>(ent, nent, true, bs, half.data(), cap);
        bool okc = gc == nbytes && memcmp(half.data(), want.data(), cap) == 0;
        for (uint32_t i = cap; i < half.size(); ++i) okc = okc && half[i] == 0x3C;
        dc += !okc;
        free(ent);
    }
    fclose(f);
    printf("write %d %u\nsize %d %u\ncapped %d %u\n", dw, n, ds, n, dc, n);
    return 0;
}

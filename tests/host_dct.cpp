// Host build of the device's exact DCT-32 line transforms (volume-compressor_gb300/
// csrc/dct32.cuh: the recursive even/odd butterfly) applied in the transform
// kernels' pass order. Test infrastructure: tests/test_host_dct.py compares the
// results with the oracle's whole-atom transforms (orc_fdct / orc_idct).
//
//   host_dct inv <in> <out>   in: n x (i32 dc, 32768 i32 coefficients, raster z,y,x)
//                             out: n x 32768 u8 voxels (passes x, y, z; + dc; clamp)
//   host_dct fwd <in> <out>   in: n x (i32 dc, 32768 u8 voxels)
//                             out: n x 32768 i32 coefficients (vox - dc; passes x, y, z)
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#define __device__
#define __host__
#define __forceinline__ inline
#define __constant__

#include "dct32.cuh"

using namespace vcg;

static inline int idx(int z, int y, int x) { return (z * 32 + y) * 32 + x; }

// one pass over the 1024 lines along axis (0: x, 1: y, 2: z) of a 32^3 i32 field
template <bool INV>
static void pass(std::vector<int32_t> &f, int axis) {
    int32_t v[32], o[32];
    for (int a = 0; a < 32; ++a)
        for (int b = 0; b < 32; ++b) {
            for (int k = 0; k < 32; ++k)
                v[k] = f[axis == 0 ? idx(a, b, k) : axis == 1 ? idx(a, k, b) : idx(k, a, b)];
            if (INV) idct32_line(v, o);
            else fdct32_line(v, o);
            for (int k = 0; k < 32; ++k) f[axis == 0 ? idx(a, b, k) : axis == 1 ? idx(a, k, b) : idx(k, a, b)] = o[k];
        }
}

int main(int argc, char **argv) {
    if (argc != 4) return 2;
    const bool inv = strcmp(argv[1], "inv") == 0;
    FILE *fi = fopen(argv[2], "rb"), *fo = fopen(argv[3], "wb");
    if (!fi || !fo) return 2;
    std::vector<int32_t> f(32768);
    std::vector<uint8_t> vox(32768);
    int32_t dc;
    while (fread(&dc, 4, 1, fi) == 1) {
        if (inv) {
            if (fread(f.data(), 4, 32768, fi) != 32768) return 2;
            for (int axis = 0; axis < 3; ++axis) pass<true>(f, axis);
            for (int i = 0; i < 32768; ++i) {
                const int32_t x = (int32_t)((uint32_t)f[i] + (uint32_t)dc);
                vox[i] = (uint8_t)(x < 0 ? 0 : x > 255 ? 255 : x);
            }
            fwrite(vox.data(), 1, 32768, fo);
        } else {
            if (fread(vox.data(), 1, 32768, fi) != 32768) return 2;
            for (int i = 0; i < 32768; ++i) f[i] = (int32_t)vox[i] - dc;
            for (int axis = 0; axis < 3; ++axis) pass<false>(f, axis);
            fwrite(f.data(), 4, 32768, fo);
        }
    }
    fclose(fi);
    fclose(fo);
    return 0;
}

// Shared pieces of the inverse-transform kernels (device): level scatter into a
// padded shared-memory tile, dequantisation, inverse passes along x and y per
// slab, the pass along z per column, and the cropped store into a box raster.
#pragma once
#include <stdint.h>

#include "dct32.cuh"
#include "kernels.cuh"
#include "rangecoder.cuh"

namespace vcg {

// Barrier of the NT threads that work on one tile: the whole CTA (BAR = 0), or
// named barrier BAR when the tile's threads are only part of the CTA.
template <int NT, int BAR>
__device__ __forceinline__ void tile_sync() {
    if (BAR == 0) __syncthreads();
    else asm volatile("bar.sync %0, %1;" ::"r"(BAR), "r"(NT) : "memory");
}

// dequantised coefficient of raw level l at raster r (src/vc/vc.c:327-338, i32 wrap)
__device__ __forceinline__ int32_t dequant(int32_t l, uint32_t r, const int32_t *dqs, const int32_t *dqb,
                                           const uint32_t *alt) {
    uint32_t f = (r >> 10) + ((r >> 5) & 31u) + (r & 31u);
    uint32_t cls = f + 94u * ((alt[r >> 5] >> (r & 31u)) & 1u);
    uint32_t m = (uint32_t)(l < 0 ? -l : l);
    int32_t v = (int32_t)(m * (uint32_t)dqs[cls] + (uint32_t)dqb[cls] + 128u) >> 8;
    return l == 0 ? 0 : (l < 0 ? (int32_t)(0u - (uint32_t)v) : v);
}

// Scratch after the tile (kIdctTileBytes in all): the rows (kz, ky) that hold a
// level, as one 32-bit mask per slab, the prefix of their counts over the
// slabs, and the list of those rows.
constexpr int kTileExtraInts = 32 + 32 + 4 + 512;
constexpr size_t kIdctTileBytes = (size_t)(kTileInts + kTileExtraInts) * sizeof(int32_t);

// Tile of one PRESENT atom after the inverse passes along x and y: levels
// dequantised as they are scattered into T (32 slabs x padded 32x32, i32;
// only the nonzero levels are touched). Then, by default, one warp per slab
// (lane per row, then lane per column), all-zero slabs skipped. With COMPACT,
// the rows that received a level are marked, the pass along x runs only on
// those (lane per row, from a compact list: a row without a level stays zero,
// as the reference skips zero lines, src/vc/vc.c:177) and the pass along y on
// slabs with a marked row. COMPACT runs fewer multiplies but mixes slabs in a
// warp (shared-memory bank conflicts) and adds barriers: measured on GB300 it
// pays only where the transform shares the SM with the range decoder (the
// fused decode: 1024^3 t50 5.96 -> 5.63 ms), not in the transform kernel alone
// (t10 3.40 -> 3.50 ms). T needs kIdctTileBytes. Ends with a barrier.
// tid: the thread's index among the tile's NT threads. COH: the lists were
// written during this kernel (fused decode): read them through L2.
template <int NT, int BAR = 0, bool COH = false, bool COMPACT = false>
__device__ __forceinline__ void idct_tile_xy(int32_t *T, const uint8_t *arc, const vcd_atom &e, uint32_t c,
                                             const uint32_t *src, const uint16_t *scan, const uint32_t *band_start,
                                             const int32_t *dqs, const int32_t *dqb, const uint32_t *alt,
                                             int tid) {
    const int lane = tid & 31, warp = tid >> 5;
    int4 *T4 = reinterpret_cast<int4 *>(T);
    uint32_t *rowmask = reinterpret_cast<uint32_t *>(T + kTileInts);
    uint32_t *pre = rowmask + 32, *nrows = pre + 32;
    uint16_t *rows = reinterpret_cast<uint16_t *>(nrows + 4);
    for (int i = tid; i < kTileInts / 4; i += NT) T4[i] = make_int4(0, 0, 0, 0);
    if (tid < 32) rowmask[tid] = 0;
    tile_sync<NT, BAR>();
    if (c & kEntOverflow) {
        // slow path for streams whose list exceeded its capacity
        if (tid == 0)
            rc_decode_levels_lane(arc + e.off + 1, e.len - 1, band_start, [&](uint32_t p, uint32_t lv) {
                const uint32_t r = scan[p];
                T[tile_idx(r)] = dequant((int16_t)lv, r, dqs, dqb, alt);
                if (COMPACT) rowmask[r >> 10] |= 1u << ((r >> 5) & 31u);
            });
    } else {
        // batches of kB entries per thread: every list load of a batch is issued
        // before the first scan lookup, and every lookup before the first store,
        // so a batch waits for one memory latency instead of one per entry
        constexpr uint32_t kB = 16;
        const uint32_t n = c & kEntMask;
        for (uint32_t i0 = 0; i0 < n; i0 += kB * NT) {
            uint32_t w[kB], r[kB];
#pragma unroll
            for (uint32_t j = 0; j < kB; ++j) {
                const uint32_t i = i0 + j * NT + tid;
                w[j] = i < n ? (COH ? __ldcg(src + i) : __ldg(src + i)) : 0u;
            }
#pragma unroll
            for (uint32_t j = 0; j < kB; ++j) r[j] = __ldg(scan + (w[j] & 0xFFFFu));
#pragma unroll
            for (uint32_t j = 0; j < kB; ++j)
                if (i0 + j * NT + tid < n) {
                    T[tile_idx(r[j])] = dequant((int16_t)(w[j] >> 16), r[j], dqs, dqb, alt);
                    if (COMPACT) atomicOr(&rowmask[r[j] >> 10], 1u << ((r[j] >> 5) & 31u));
                }
        }
    }
    tile_sync<NT, BAR>();
    if (!COMPACT) {
        for (int kz = warp; kz < 32; kz += NT / 32) {
            int32_t *S = T + kz * kSlabPitch;
            int32_t *row = S + lane * kRowPitch, *col = S + lane;
            int32_t v[32], o[32];
            int any = 0;
#pragma unroll
            for (int kx = 0; kx < 32; ++kx) {
                v[kx] = row[kx];
                any |= v[kx];
            }
            if (__any_sync(0xFFFFFFFFu, any)) {   // an all-zero slab stays zero
                idct32_line(v, o);
#pragma unroll
                for (int x = 0; x < 32; ++x) row[x] = o[x];
                __syncwarp();
#pragma unroll
                for (int ky = 0; ky < 32; ++ky) v[ky] = col[ky * kRowPitch];
                idct32_line(v, o);
                __syncwarp();
#pragma unroll
                for (int y = 0; y < 32; ++y) col[y * kRowPitch] = o[y];
            }
            __syncwarp();
        }
        tile_sync<NT, BAR>();
        return;
    }
    if (warp == 0) {   // rows before each slab's, and their total
        const uint32_t m = __popc(rowmask[lane]);
        uint32_t incl = m;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += y;
        }
        pre[lane] = incl - m;
        if (lane == 31) *nrows = incl;
    }
    tile_sync<NT, BAR>();
    for (int i = tid; i < 1024; i += NT) {
        const uint32_t m = rowmask[i >> 5], bit = (uint32_t)i & 31u;
        if ((m >> bit) & 1u) rows[pre[i >> 5] + __popc(m & ((1u << bit) - 1u))] = (uint16_t)i;
    }
    tile_sync<NT, BAR>();
    const uint32_t nr = *nrows;
    for (uint32_t b = (uint32_t)warp * 32u; b < nr; b += NT) {   // along x, listed rows only
        const uint32_t idx = b + (uint32_t)lane;
        if (idx < nr) {
            const uint32_t ri = rows[idx];
            int32_t *row = T + (ri >> 5) * kSlabPitch + (ri & 31u) * kRowPitch;
            int32_t v[32], o[32];
#pragma unroll
            for (int kx = 0; kx < 32; ++kx) v[kx] = row[kx];
            idct32_line(v, o);
#pragma unroll
            for (int x = 0; x < 32; ++x) row[x] = o[x];
        }
    }
    tile_sync<NT, BAR>();
    for (int kz = warp; kz < 32; kz += NT / 32) {   // along y, slabs with a row
        if (!rowmask[kz]) continue;   // an all-zero slab stays zero
        int32_t *col = T + kz * kSlabPitch + lane;
        int32_t v[32], o[32];
#pragma unroll
        for (int ky = 0; ky < 32; ++ky) v[ky] = col[ky * kRowPitch];
        idct32_line(v, o);
#pragma unroll
        for (int y = 0; y < 32; ++y) col[y * kRowPitch] = o[y];
    }
    tile_sync<NT, BAR>();
}

// Pass along z for column (y, x = lane): voxel values before +dc.
__device__ __forceinline__ void idct_col_z(const int32_t *T, int y, int lane, int32_t (&o)[32]) {
    const int32_t *c = T + y * kRowPitch + lane;
    int32_t v[32];
#pragma unroll
    for (int kz = 0; kz < 32; ++kz) v[kz] = c[kz * kSlabPitch];
    idct32_line(v, o);
}

// Crop window of atom origin g (voxels) inside box [b0, b1) on one axis, atom-local.
struct Crop {
    uint32_t lx0, lx1, ly0, ly1, lz0, lz1;
    __device__ __forceinline__ void set(uint32_t gx, uint32_t gy, uint32_t gz, uint32_t x0, uint32_t y0, uint32_t z0,
                                        uint32_t x1, uint32_t y1, uint32_t z1) {
        lx0 = x0 > gx ? x0 - gx : 0; lx1 = x1 < gx + 32 ? x1 - gx : 32;
        ly0 = y0 > gy ? y0 - gy : 0; ly1 = y1 < gy + 32 ? y1 - gy : 32;
        lz0 = z0 > gz ? z0 - gz : 0; lz1 = z1 < gz + 32 ? z1 - gz : 32;
    }
};

// Store column (y, lane) of the atom (o + dc, clamped) into the crop window;
// obase points at the window's first voxel inside a box raster of pitch ox, oy.
__device__ __forceinline__ void store_col(uint8_t *obase, uint64_t ox, uint64_t oy, const Crop &k, int y, int lane,
                                          const int32_t (&o)[32], int32_t dc) {
    if ((uint32_t)lane < k.lx0 || (uint32_t)lane >= k.lx1 || (uint32_t)y < k.ly0 || (uint32_t)y >= k.ly1) return;
    uint8_t *col = obase + (uint64_t)(y - k.ly0) * ox + (lane - k.lx0);
#pragma unroll
    for (int z = 0; z < 32; ++z) {
        if ((uint32_t)z >= k.lz0 && (uint32_t)z < k.lz1) {
            int32_t x = (int32_t)((uint32_t)o[z] + (uint32_t)dc);
            col[(uint64_t)(z - k.lz0) * oy * ox] = (uint8_t)(x < 0 ? 0 : x > 255 ? 255 : x);
        }
    }
}

// The same for a window that holds all 32 planes of the atom (lz0 = 0, lz1 =
// 32): one pointer step per plane, no per-plane test.
__device__ __forceinline__ void store_col_full(uint8_t *obase, uint64_t ox, uint64_t oy, const Crop &k, int y,
                                               int lane, const int32_t (&o)[32], int32_t dc) {
    if ((uint32_t)lane < k.lx0 || (uint32_t)lane >= k.lx1 || (uint32_t)y < k.ly0 || (uint32_t)y >= k.ly1) return;
    uint8_t *p = obase + (uint64_t)(y - k.ly0) * ox + (lane - k.lx0);
    const uint64_t plane = ox * oy;
#pragma unroll
    for (int z = 0; z < 32; ++z) {
        const int32_t x = (int32_t)((uint32_t)o[z] + (uint32_t)dc);
        *p = (uint8_t)(x < 0 ? 0 : x > 255 ? 255 : x);
        p += plane;
    }
}

template <int NT>
__device__ __forceinline__ void zero_window(uint8_t *obase, uint64_t ox, uint64_t oy, const Crop &k,
                                            uint32_t tid) {
    const uint32_t cw = k.lx1 - k.lx0, ch = k.ly1 - k.ly0, cd = k.lz1 - k.lz0;
    for (uint32_t i = tid; i < cw * ch * cd; i += NT) {
        uint32_t x = i % cw, y = (i / cw) % ch, z = i / (cw * ch);
        obase[((uint64_t)z * oy + y) * ox + x] = 0;
    }
}

}  // namespace vcg

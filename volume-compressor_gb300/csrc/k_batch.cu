// Batched region decode (device): a persistent range-decode pass over the
// batch's distinct atoms, then a persistent transform pass that takes atoms from
// a device work counter and crops each decoded atom into every request box that
// overlaps it (src/vc/vc.c:1535-1555 per box). The counts are read from device
// memory, so the same launches (and a CUDA graph of them) serve any batch that
// fits the buffers.
#include <cuda_runtime.h>
#include <stdint.h>

#include "idct_tile.cuh"
#include "imma.cuh"
#include "kernels.cuh"
#include "rangecoder.cuh"

namespace vcg {

constexpr size_t kTileSmem = kIdctTileBytes;   // the butterfly's padded tile + its row lists (idct_tile.cuh)

// Persistent over the batch's distinct atoms (their number is read from device
// memory) while the policy keeps one atom per warp (rc_lanes_for gives 1):
// scalar decoder. With more atoms, k_rc_batch_lanes takes them instead (or,
// without its order buffer, the lockstep decoder here).
constexpr int kRcBatchThreads = 128;
// Stream bytes a warp stages in shared memory for the latency decoder, when the
// batch's capacity keeps it on that decoder (launched with these slices).
constexpr uint32_t kBatchStage = 40u * 1024u;
constexpr uint32_t kBatchStageSmem = (kRcBatchThreads / 32) * kBatchStage;

__device__ __forceinline__ uint32_t dynamic_smem_bytes() {
    uint32_t v;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(v));
    return v;
}

__global__ void __launch_bounds__(kRcBatchThreads) k_rc_batch(BatchJob J) {
    extern __shared__ uint8_t bstage[];
    __shared__ uint32_t bstart[9];
    if (threadIdx.x < 9) bstart[threadIdx.x] = J.band_start[threadIdx.x];
    __syncthreads();
    const uint32_t n = *J.n_ua;
    const uint32_t G = rc_lanes_for(n, J.sms, J.rc_scalar_warps);
    if (G > 1 && J.order) return;   // k_rc_batch_lanes decodes this batch
    const uint32_t lane = threadIdx.x & 31u;
    // latency decoder with the stream staged by the whole warp
    const bool staged = G == 1 && n <= 4u * J.sms && dynamic_smem_bytes() >= kBatchStageSmem;
    if (G == 1 && !staged && lane != 0) return;
    uint8_t *stage = bstage + (threadIdx.x >> 5) * kBatchStage;
    const uint32_t slot = G == 1 ? 0u : lane;
    const uint64_t nwarps = (uint64_t)gridDim.x * (kRcBatchThreads / 32);
    for (uint64_t w = ((uint64_t)blockIdx.x * kRcBatchThreads + threadIdx.x) >> 5; w * G < n; w += nwarps) {
        const uint64_t u = w * G + slot;
        bool active = false;
        vcd_atom e = {};
        if (slot < G && u < n) {
            e = J.atoms[J.ua[u].idx];
            active = e.kind == VCD_PRESENT;
            if (!active && lane == 0) J.cnt[u] = 0;
        }
        bool in_smem = false;
        if (staged) {
            __syncwarp();   // lane 0 is done with the slice (its previous atom)
            const uint32_t len = active ? e.len - 1u : 0u;
            in_smem = active && len < kBatchStage;
            if (in_smem) {   // 8 independent byte loads per lane in flight, then their stores
                const uint8_t *src = J.arc + e.off + 1;
                for (uint32_t i0 = 0; i0 < len; i0 += 8u * 32u) {
                    uint32_t b[8];
#pragma unroll
                    for (uint32_t k = 0; k < 8; ++k) {
                        const uint32_t i = i0 + k * 32u + lane;
                        b[k] = i < len ? (uint32_t)__ldg(src + i) : 0u;
                    }
#pragma unroll
                    for (uint32_t k = 0; k < 8; ++k) {
                        const uint32_t i = i0 + k * 32u + lane;
                        if (i < len) stage[i] = (uint8_t)b[k];
                    }
                }
                if (lane == 0) stage[len] = 0;
            }
            __syncwarp();
            if (lane != 0) continue;
        }
        uint32_t cap = 0, cnt = 0;
        uint32_t *dst = J.ent;
        if (active) {
            cap = 8u * (e.len - 1u) + 64u;
            if (e.len - 1u > VCD_MAX_ENTRIES / 8u || cap > VCD_MAX_ENTRIES) cap = VCD_MAX_ENTRIES;
            dst = J.ent + J.ent_off[u];
        }
        auto sink = [&](uint32_t p, uint32_t lv) {
            if (cnt < cap) dst[cnt] = p | (lv << 16);
            ++cnt;
        };
        int bad = 0;
        if (G == 1) {
            // up to one atom per SM sub-partition the latency decoder, else the compact scalar one
            if (in_smem) bad = rc_decode_levels_sm(stage, e.len - 1, bstart, sink);
            else if (active && n <= 4u * J.sms) bad = rc_decode_levels_lat(J.arc + e.off + 1, e.len - 1, bstart, sink);
            else if (active) bad = rc_decode_levels_lane(J.arc + e.off + 1, e.len - 1, bstart, sink);
        } else {
            bad = rc_decode_levels_warp(J.arc + e.off + 1, active ? e.len - 1 : 0u, active, bstart, sink);
        }
        if (!active) continue;
        J.cnt[u] = (cnt > cap ? cap : cnt) | (cnt > cap ? kEntOverflow : 0u) | (bad ? kEntBad : 0u);
        if (bad) {
            const UAtom a = J.ua[u];
            for (uint32_t d = a.dst_begin; d < a.dst_end; ++d) atomicOr(J.req_err + J.dst[d], 1u);
        }
    }
}

// ---- per-lane decoder over the distinct atoms, in payload-length order
// (the same counting sort as the plain path's), when the policy gives more
// than one atom per warp. The counts are read from device memory, so these
// run in the batch's graph; with one atom per warp they return at once.
__device__ __forceinline__ uint32_t ua_bucket(uint32_t len) {
    const uint32_t k = len >> 5;
    return kSortBuckets - 1u - (k < kSortBuckets - 1u ? k : kSortBuckets - 1u);
}

__global__ void k_ua_hist(BatchJob J) {
    const uint32_t n = *J.n_ua;
    if (rc_lanes_for(n, J.sms, J.rc_scalar_warps) == 1) return;
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
        const vcd_atom e = J.atoms[J.ua[u].idx];
        if (e.kind == VCD_PRESENT) atomicAdd(&J.sort_ctl[ua_bucket(e.len)], 1u);
        else J.cnt[u] = 0;
    }
}

__global__ void k_ua_scatter(BatchJob J) {
    const uint32_t n = *J.n_ua;
    if (rc_lanes_for(n, J.sms, J.rc_scalar_warps) == 1) return;
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
        const vcd_atom e = J.atoms[J.ua[u].idx];
        if (e.kind == VCD_PRESENT) J.order[atomicAdd(&J.sort_ctl[ua_bucket(e.len)], 1u)] = u;
    }
}

constexpr int kBatchLaneThreads = 64;

__global__ void __launch_bounds__(kBatchLaneThreads) k_rc_batch_lanes(BatchJob J) {
    __shared__ uint32_t bstart[10];   // the band table and a copy of its end (RcLane)
    __shared__ uint32_t S[12 * kBatchLaneThreads];
    if (threadIdx.x < 10) bstart[threadIdx.x] = J.band_start[threadIdx.x < 9 ? threadIdx.x : 8];
    __syncthreads();
    const uint32_t n_present = J.sort_ctl[kSortBuckets];   // 0 when the scalar kernel decodes this batch
    if ((uint64_t)blockIdx.x * kBatchLaneThreads >= n_present) return;   // whole CTA idle
    const uint32_t i = blockIdx.x * kBatchLaneThreads + threadIdx.x;
    const bool active = i < n_present;
    uint32_t u = 0, cap = 0;
    vcd_atom e = {};
    uint32_t *dst = J.ent;
    if (active) {
        u = J.order[i];
        e = J.atoms[J.ua[u].idx];
        cap = 8u * (e.len - 1u) + 64u;
        if (e.len - 1u > VCD_MAX_ENTRIES / 8u || cap > VCD_MAX_ENTRIES) cap = VCD_MAX_ENTRIES;
        dst = J.ent + J.ent_off[u];
    }
    uint32_t *Sl = S + threadIdx.x;
    RcLane L;
    L.init(J.arc + e.off + 1, e.len - 1u, active, bstart, Sl, kBatchLaneThreads, dst, cap);
    while (__any_sync(0xFFFFFFFFu, L.c != kLaneDone)) {
#pragma unroll
        for (int k = 0; k < 8; ++k) L.step(bstart, Sl, kBatchLaneThreads);
    }
    if (!active) return;
    const uint32_t cnt = L.n > cap ? cap : L.n;
    J.cnt[u] = cnt | (L.n > cap ? kEntOverflow : 0u) | (L.bad ? kEntBad : 0u);
    if (L.bad) {
        const UAtom a = J.ua[u];
        for (uint32_t d = a.dst_begin; d < a.dst_end; ++d) atomicOr(J.req_err + J.dst[d], 1u);
    }
}

// window of box request r inside atom origin (gx, gy, gz), and its first voxel
struct BoxWin {
    Crop k;
    uint64_t ox, oy;
    uint8_t *ob;
    __device__ __forceinline__ BoxWin(const BoxReq &r, uint32_t gx, uint32_t gy, uint32_t gz) {
        k.set(gx, gy, gz, r.x0, r.y0, r.z0, r.x1, r.y1, r.z1);
        ox = r.x1 - r.x0;
        oy = r.y1 - r.y0;
        ob = r.out + ((uint64_t)(gz + k.lz0 - r.z0) * oy + (gy + k.ly0 - r.y0)) * ox + (gx + k.lx0 - r.x0);
    }
};

// ABSENT / KNOWN_ZERO / malformed atom: zeros in every box it overlaps
template <int NT>
__device__ __forceinline__ void zero_all(const BatchJob &J, const UAtom &a) {
    for (uint32_t d = a.dst_begin; d < a.dst_end; ++d) {
        const BoxWin w(J.reqs[J.dst[d]], a.ax * 32, a.ay * 32, a.az * 32);
        zero_window<NT>(w.ob, w.ox, w.oy, w.k, threadIdx.x);
    }
}

// Window of one box in the atom being transformed, staged in shared memory
// once per atom: the column stores below then need no request loads, crop
// arithmetic or 64-bit multiplies per row.
struct BoxStage {
    uint8_t *ob;       // first voxel of the window
    uint64_t plane;    // box bytes per z
    uint32_t ox;       // box bytes per y
    uint8_t lx0, lx1, ly0, ly1, lz0, lz1, full, pad;   // atom-local window; full: all 32 z
};
constexpr uint32_t kBoxStage = 64;   // windows staged per atom; further boxes take BoxWin per row

// Butterfly inverse transform of distinct atom u (T: the 132 KiB padded tile),
// cropped into every box it overlaps: each row's 32 voxels are clamped once,
// then stored into every box window. Ends with a barrier.
template <int NT>
__device__ __forceinline__ void bf_atom_to_boxes(int32_t *T, const BatchJob &J, const UAtom &a, uint32_t u,
                                                 const vcd_atom &e, uint32_t c, const int32_t *dqs,
                                                 const int32_t *dqb, const uint32_t *alt) {
    __shared__ BoxStage bs[kBoxStage];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int32_t dc = J.arc[e.off];
    const uint32_t nb = a.dst_end - a.dst_begin, ns = nb < kBoxStage ? nb : kBoxStage;
    if ((uint32_t)threadIdx.x < ns) {   // read after idct_tile_xy's first barrier
        const BoxWin w(J.reqs[J.dst[a.dst_begin + threadIdx.x]], a.ax * 32, a.ay * 32, a.az * 32);
        BoxStage b;
        b.ob = w.ob;
        b.plane = w.ox * w.oy;
        b.ox = (uint32_t)w.ox;
        b.lx0 = (uint8_t)w.k.lx0; b.lx1 = (uint8_t)w.k.lx1;
        b.ly0 = (uint8_t)w.k.ly0; b.ly1 = (uint8_t)w.k.ly1;
        b.lz0 = (uint8_t)w.k.lz0; b.lz1 = (uint8_t)w.k.lz1;
        b.full = w.k.lz0 == 0 && w.k.lz1 == 32;
        b.pad = 0;
        bs[threadIdx.x] = b;
    }
    idct_tile_xy<NT>(T, J.arc, e, c, J.ent + J.ent_off[u], J.scan, J.band_start, dqs, dqb, alt, threadIdx.x);
    for (int y = warp; y < 32; y += NT / 32) {
        int32_t o[32];
        idct_col_z(T, y, lane, o);
        uint32_t v[32];
#pragma unroll
        for (int z = 0; z < 32; ++z) {
            const int32_t x = (int32_t)((uint32_t)o[z] + (uint32_t)dc);
            v[z] = (uint32_t)(x < 0 ? 0 : x > 255 ? 255 : x);
        }
        for (uint32_t i = 0; i < ns; ++i) {
            const BoxStage b = bs[i];
            if ((uint32_t)y < b.ly0 || (uint32_t)y >= b.ly1 || (uint32_t)lane < b.lx0 || (uint32_t)lane >= b.lx1)
                continue;
            uint8_t *p = b.ob + (uint64_t)((uint32_t)y - b.ly0) * b.ox + ((uint32_t)lane - b.lx0);
            if (b.full) {
#pragma unroll
                for (int z = 0; z < 32; ++z) {
                    *p = (uint8_t)v[z];
                    p += b.plane;
                }
            } else {
#pragma unroll
                for (int z = 0; z < 32; ++z) {
                    if ((uint32_t)z >= b.lz0 && (uint32_t)z < b.lz1) {
                        *p = (uint8_t)v[z];
                        p += b.plane;
                    }
                }
            }
        }
        for (uint32_t d = a.dst_begin + ns; d < a.dst_end; ++d) {
            const BoxWin w(J.reqs[J.dst[d]], a.ax * 32, a.ay * 32, a.az * 32);
            store_col(w.ob, w.ox, w.oy, w.k, y, lane, o, dc);
        }
    }
    __syncthreads();   // the tile and the staged windows are reused by the next atom
}

template <int NT>
__global__ void __launch_bounds__(NT, 1) k_idct_batch(BatchJob J) {
    extern __shared__ int32_t T[];
    __shared__ int32_t dqs[VCD_NCLASS], dqb[VCD_NCLASS];
    __shared__ uint32_t alt[1024];
    __shared__ uint32_t s_u;
    const int tid = threadIdx.x;
    for (int i = tid; i < 1024; i += NT) alt[i] = J.alt_mask[i];
    const uint32_t n = *J.n_ua;
    int cur_lod = -1;
    for (;;) {
        if (tid == 0) s_u = atomicAdd(J.work, 1u);
        __syncthreads();
        const uint32_t u = s_u;
        __syncthreads();
        if (u >= n) break;
        const UAtom a = J.ua[u];
        if ((int)a.lod != cur_lod) {   // uniform: dequantisation tables of this LOD
            for (int i = tid; i < VCD_NCLASS; i += NT) { dqs[i] = J.dq[a.lod].step[i]; dqb[i] = J.dq[a.lod].bias[i]; }
            cur_lod = (int)a.lod;
            __syncthreads();
        }
        const vcd_atom e = J.atoms[a.idx];
        const uint32_t c = e.kind == VCD_PRESENT ? J.cnt[u] : kEntBad;
        if (e.kind != VCD_PRESENT || (c & kEntBad)) {   // ABSENT / KNOWN_ZERO -> zeros in every box
            zero_all<NT>(J, a);
            continue;
        }
        bf_atom_to_boxes<NT>(T, J, a, u, e, c, dqs, dqb, alt);
    }
}

// The same on the int8 tensor cores: the nonzero levels are dequantised and
// scattered as three int8 pieces into piece planes (imma.cuh), the three
// inverse passes run as MMAs, the voxels are staged in shared memory and
// cropped into every box. Lists that overflowed their capacity and atoms whose
// values leave the three-piece range take the butterfly, so every result is
// the reference's.
constexpr size_t kImmaSmem = 2 * 3 * 32768;   // two buffers of three piece planes
static_assert(kImmaSmem >= kIdctTileBytes, "an atom redone with the butterfly reuses the planes as its tile");

template <int NT>
__global__ void __launch_bounds__(NT, 1) k_idct_batch_imma(BatchJob J) {
    extern __shared__ __align__(16) uint8_t sm[];
    __shared__ int32_t dqs[VCD_NCLASS], dqb[VCD_NCLASS];
    __shared__ uint32_t alt[1024];
    __shared__ uint32_t s_u;
    __shared__ int s_bad;
    const int tid = threadIdx.x;
    uint32_t A[2][2][4];
    imma_a_frags<true>(A);
    for (int i = tid; i < 1024; i += NT) alt[i] = J.alt_mask[i];
    const uint32_t n = *J.n_ua;
    int cur_lod = -1;
    for (;;) {
        if (tid == 0) {
            s_u = atomicAdd(J.work, 1u);
            s_bad = 0;
        }
        __syncthreads();
        const uint32_t u = s_u;
        __syncthreads();
        if (u >= n) break;
        const UAtom a = J.ua[u];
        if ((int)a.lod != cur_lod) {   // uniform: dequantisation tables of this LOD
            for (int i = tid; i < VCD_NCLASS; i += NT) { dqs[i] = J.dq[a.lod].step[i]; dqb[i] = J.dq[a.lod].bias[i]; }
            cur_lod = (int)a.lod;
            __syncthreads();
        }
        const vcd_atom e = J.atoms[a.idx];
        const uint32_t c = e.kind == VCD_PRESENT ? J.cnt[u] : kEntBad;
        if (e.kind != VCD_PRESENT || (c & kEntBad)) {
            zero_all<NT>(J, a);
            continue;
        }
        if (!(c & kEntOverflow)) {
            int4 *P4 = reinterpret_cast<int4 *>(sm);
            for (int i = tid; i < 3 * 32768 / 16; i += NT) P4[i] = make_int4(0, 0, 0, 0);
            __syncthreads();
            bool bad = false;
            const uint32_t cnt = c & kEntMask;
            const uint32_t *src = J.ent + J.ent_off[u];
            for (uint32_t i = tid; i < cnt; i += NT) {
                const uint32_t w = src[i];
                const uint32_t r = __ldg(J.scan + (w & 0xFFFFu));
                const int32_t v = dequant((int16_t)(w >> 16), r, dqs, dqb, alt);
                bad |= !fits<3>(v);
                const int off = (int)(r >> 5) * 32 + ppos((int)(r & 31u));   // line (kz, ky), element kx
#pragma unroll
                for (int j = 0; j < 3; ++j) imma_plane<3>(sm, 0, j)[off] = (uint8_t)piece<3>(v, j);
            }
            if (bad) s_bad = 1;
            __syncthreads();
            if (!s_bad) {
                const int32_t dc = J.arc[e.off];
                uint8_t *vox = imma_plane<3>(sm, 1, 0);   // free while the last pass reads buffer 0
#pragma unroll 1
                for (int pass = 0; pass < 3; ++pass) {
                    imma_pass<3, NT>(sm, A, pass, bad, [&](int k, int la, int lb, int32_t o0, int32_t o1) {
                        const int32_t v0 = o0 + dc, v1 = o1 + dc;
                        const uint32_t b0 = (uint32_t)(v0 < 0 ? 0 : (v0 > 255 ? 255 : v0));
                        const uint32_t b1 = (uint32_t)(v1 < 0 ? 0 : (v1 > 255 ? 255 : v1));
                        *reinterpret_cast<uint16_t *>(vox + k * 1024 + la * 32 + lb) = (uint16_t)(b0 | (b1 << 8));
                    });
                    if (bad) s_bad = 1;
                    __syncthreads();
                }
                if (!s_bad) {   // voxels (z, y, x) of the atom -> every box it overlaps
                    for (uint32_t d = a.dst_begin; d < a.dst_end; ++d) {
                        const BoxWin w(J.reqs[J.dst[d]], a.ax * 32, a.ay * 32, a.az * 32);
                        const uint32_t cw = w.k.lx1 - w.k.lx0, ch = w.k.ly1 - w.k.ly0, cd = w.k.lz1 - w.k.lz0;
                        for (uint32_t i = tid; i < ch * cd; i += NT) {
                            const uint32_t y = i % ch, z = i / ch;
                            const uint8_t *sr = vox + (w.k.lz0 + z) * 1024 + (w.k.ly0 + y) * 32 + w.k.lx0;
                            uint8_t *dr = w.ob + ((uint64_t)z * w.oy + y) * w.ox;
                            for (uint32_t x = 0; x < cw; ++x) dr[x] = sr[x];
                        }
                    }
                    __syncthreads();
                    continue;
                }
            }
        }
        bf_atom_to_boxes<NT>(reinterpret_cast<int32_t *>(sm), J, a, u, e, c, dqs, dqb, alt);
    }
}

static void launch_rc(const BatchJob &J, int num_sms, uint32_t max_ua, cudaStream_t s) {
    // warps for the widest case up to max_ua atoms: one per atom while the
    // policy keeps atoms one per warp, else the k warps per sub-partition of
    // rc_lanes_for (k grows with the atom count); capped at a full device (the
    // kernel loops)
    const uint64_t slots = 4ull * (uint64_t)num_sms;
    const uint64_t scalar = (uint64_t)J.rc_scalar_warps * slots;
    uint64_t warps = max_ua < scalar ? max_ua : scalar;
    const uint64_t packed = ((uint64_t)max_ua + 32 * slots - 1) / (32 * slots) * slots;
    if (max_ua > scalar && packed > warps) warps = packed;
    const uint64_t cap = (uint64_t)num_sms * (2048 / kRcBatchThreads) * (kRcBatchThreads / 32);
    if (warps > cap) warps = cap;
    if (warps < 1) warps = 1;
    const unsigned grid = (unsigned)((warps * 32 + kRcBatchThreads - 1) / kRcBatchThreads);
    if (J.order && J.sort_ctl) {   // the per-lane decoder's launches (idle when one atom per warp)
        const uint64_t sort_grid = ((uint64_t)max_ua + 255) / 256;
        const unsigned sg = (unsigned)(sort_grid < 1 ? 1 : sort_grid > 4096 ? 4096 : sort_grid);
        cudaMemsetAsync(J.sort_ctl, 0, sort_ctl_words() * 4, s);
        k_ua_hist<<<sg, 256, 0, s>>>(J);
        launch_len_scan(J.sort_ctl, s);
        k_ua_scatter<<<sg, 256, 0, s>>>(J);
        const uint64_t lg = ((uint64_t)max_ua + kBatchLaneThreads - 1) / kBatchLaneThreads;
        k_rc_batch_lanes<<<(unsigned)(lg < 1 ? 1 : lg), kBatchLaneThreads, 0, s>>>(J);
    }
    // capacity within the latency decoder's range: stage the streams (one CTA
    // per SM at most, with a warp per atom)
    const bool stage = J.rc_scalar_warps && max_ua <= slots;
    if (stage) smem_attr((const void *)k_rc_batch, (int)kBatchStageSmem);
    k_rc_batch<<<grid, kRcBatchThreads, stage ? kBatchStageSmem : 0, s>>>(J);
}

template <int NT>
static void launch_tx(const BatchJob &J, int num_sms, cudaStream_t s) {
    smem_attr((const void *)k_idct_batch<NT>, (int)kTileSmem);
    k_idct_batch<NT><<<num_sms, NT, kTileSmem, s>>>(J);
}

void launch_batch(const BatchJob &J, const BatchShape &shape, int num_sms, uint32_t max_ua, cudaStream_t s,
                  cudaEvent_t mid) {
    BatchJob Jr = J;
    Jr.rc_scalar_warps = (uint32_t)shape.rc_scalar_warps;
    Jr.sms = (uint32_t)num_sms;
    launch_rc(Jr, num_sms, max_ua, s);
    if (mid) cudaEventRecord(mid, s);
    if (shape.imma) {
        smem_attr((const void *)k_idct_batch_imma<256>, (int)kImmaSmem);
        k_idct_batch_imma<256><<<num_sms, 256, kImmaSmem, s>>>(J);
    } else if (shape.idct_threads == 512) {
        launch_tx<512>(J, num_sms, s);
    } else {
        launch_tx<256>(J, num_sms, s);
    }
}

}  // namespace vcg

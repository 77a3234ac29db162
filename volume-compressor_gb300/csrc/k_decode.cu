// Decode kernels: per-atom list capacities + scan, range-decode lanes, and the
// fused dequantise + inverse DCT-32 + crop.
//
//   k_caps       one thread per box atom: coefficient-list capacity
//   k_scan_u64   one CTA: exclusive scan of the capacities (list placement)
//   k_rc_decode  one thread per PRESENT atom: serial range decode of its
//                payload into (scan position, level) pairs (src/vc/vc.c:545-560);
//                one atom per warp for small decodes, a warp of atoms in
//                lockstep for large ones
//   k_idct       one CTA per atom (persistent over the box): scatter levels into
//                a 32x32x32 i32 tile in shared memory, dequantise while loading
//                each z-slab (src/vc/vc.c:327-338), inverse passes along x and y
//                per slab (warp per slab, lane per line), then along z (lane per
//                column), add dc, clamp to u8 and store the cropped voxels
//                (src/vc/vc.c:219-229, 1535-1555)
#include <cuda_runtime.h>
#include <stdint.h>

#include "dct32.cuh"
#include "kernels.cuh"
#include "idct_tile.cuh"
#include "rangecoder.cuh"

namespace vcg {

constexpr int kIdctThreads = 512;   // 16 warps per atom (measured faster than 8 on GB300)
constexpr size_t kIdctSmem = kIdctTileBytes;

__global__ void k_caps(DecodeJob J) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= J.n_atoms) return;
    uint32_t az, ay, ax;
    box_atom(J, t, az, ay, ax);
    vcd_atom e = J.atoms[job_atom(J, t, az, ay, ax)];
    uint64_t cap = 0;
    if (e.kind == VCD_PRESENT) {   // slots of the list, a multiple of 32 (the host's entry_cap)
        cap = 8ull * (e.len - 1) + 64ull;
        if (cap > VCD_MAX_ENTRIES) cap = VCD_MAX_ENTRIES;
        cap = (cap + 31) & ~31ull;
    }
    J.ent_off[t] = cap;
}

// Exclusive scan of v[0..n) in place (+ base), total -> *total. One CTA of 1024
// threads walks the array in tiles of 4096 carrying the running sum.
__global__ void __launch_bounds__(1024) k_scan_u64(uint64_t *v, uint64_t n, uint64_t base, uint64_t *total) {
    __shared__ uint64_t warp_sum[32];
    __shared__ uint64_t carry_s;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) carry_s = base;
    __syncthreads();
    for (uint64_t tile = 0; tile < n; tile += 4096) {
        uint64_t i0 = tile + (uint64_t)tid * 4;
        uint64_t a[4];
        uint64_t s = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            a[j] = (i0 + j < n) ? v[i0 + j] : 0;
            uint64_t x = a[j];
            a[j] = s;
            s += x;
        }
        uint64_t incl = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint64_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) warp_sum[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            uint64_t w = warp_sum[lane], wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint64_t y = __shfl_up_sync(0xFFFFFFFFu, wi, o);
                if (lane >= o) wi += y;
            }
            warp_sum[lane] = wi - w;   // exclusive prefix of warp totals
        }
        __syncthreads();
        uint64_t excl = carry_s + warp_sum[wid] + (incl - s);
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (i0 + j < n) v[i0 + j] = excl + a[j];
        __syncthreads();
        if (tid == 1023) carry_s = excl + s;
        __syncthreads();
    }
    if (tid == 0 && total) *total = carry_s;
}

// Stream bytes the latency path stages in shared memory (with the zero byte
// after them, within the 48 KiB a launch may take without opting in; four
// such CTAs per SM at most).
constexpr uint32_t kLatStage = 40u * 1024u;

// One warp per CTA, G atoms per warp (rc_lanes_for): G = 1 runs a scalar
// decoder on lane 0 (the latency decoder when `lat`), G > 1 the lockstep
// decoder on lanes 0..G-1. With J.order (G = 1 only), CTA i decodes the i-th
// atom of the payload-length order. With `lat` the whole warp first copies the
// atom's stream into shared memory (kLatStage bytes of dynamic shared memory:
// streams that do not fit are read from global memory by
// rc_decode_levels_lat).
__global__ void __launch_bounds__(32) k_rc_decode(DecodeJob J, uint32_t G, uint32_t lat) {
    extern __shared__ uint8_t stage[];
    __shared__ uint32_t bstart[9];
    if (threadIdx.x < 9) bstart[threadIdx.x] = J.band_start[threadIdx.x];
    __syncthreads();
    const uint32_t lane = threadIdx.x;
    const bool staged = G == 1 && lat;
    if (G == 1 && !staged && lane != 0) return;
    const uint32_t slot = G == 1 ? 0u : lane;   // (G = 1: every lane of a staging warp takes lane 0's atom)
    uint64_t t = (uint64_t)blockIdx.x * G + slot;
    if (J.order) {
        if (t >= J.sort_ctl[kSortBuckets]) return;
        t = J.order[t];
    }
    bool active = false;
    vcd_atom e = {};
    if (slot < G && t < J.n_atoms) {
        uint32_t az, ay, ax;
        box_atom(J, t, az, ay, ax);
        e = J.atoms[job_atom(J, t, az, ay, ax)];
        active = e.kind == VCD_PRESENT;
        if (!active && lane == 0) J.cnt[t] = 0;
    }
    bool in_smem = false;
    if (staged) {
        const uint32_t len = active ? e.len - 1u : 0u;
        in_smem = active && len < kLatStage;
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
            __syncwarp();
        }
        if (lane != 0) return;
    }
    uint32_t cap = 0, n = 0;
    uint32_t *dst = J.ent;
    if (active) {
        cap = 8u * (e.len - 1u) + 64u;
        if (e.len - 1u > VCD_MAX_ENTRIES / 8u || cap > VCD_MAX_ENTRIES) cap = VCD_MAX_ENTRIES;
        dst = J.ent + J.ent_off[t];
    }
    // entries carry the scan position; the transform kernel maps it to raster
    auto sink = [&](uint32_t p, uint32_t lv) {
        if (n < cap) dst[n] = p | (lv << 16);
        ++n;
    };
    int bad = 0;
    if (G == 1) {
        if (in_smem) bad = rc_decode_levels_sm(stage, e.len - 1, bstart, sink);
        else if (active && lat) bad = rc_decode_levels_lat(J.arc + e.off + 1, e.len - 1, bstart, sink);
        else if (active) bad = rc_decode_levels_lane(J.arc + e.off + 1, e.len - 1, bstart, sink);
    } else {
        bad = rc_decode_levels_warp(J.arc + e.off + 1, active ? e.len - 1 : 0u, active, bstart, sink);
    }
    if (!active) return;
    uint32_t flags = (n > cap ? kEntOverflow : 0u) | (bad ? kEntBad : 0u);
    J.cnt[t] = (n > cap ? cap : n) | flags;
    atomicAdd(J.nnz_total, (unsigned long long)(n > cap ? cap : n));
    if (bad) atomicMin(J.err, (uint32_t)(t < 0xFFFFFFFFull ? t : 0xFFFFFFFEull));
}

// ---- per-lane decoder (RcLane) for large decodes. The atoms are first put in
// order of payload length, longest first (a counting sort on length / 32), so
// that the 32 atoms of a warp need about the same number of steps: a warp
// runs until its slowest lane is done.
__device__ __forceinline__ uint32_t len_bucket(uint32_t len) {
    const uint32_t k = len >> 5;
    return kSortBuckets - 1u - (k < kSortBuckets - 1u ? k : kSortBuckets - 1u);
}

__global__ void k_len_hist(DecodeJob J) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= J.n_atoms) return;
    uint32_t az, ay, ax;
    box_atom(J, t, az, ay, ax);
    const vcd_atom e = J.atoms[job_atom(J, t, az, ay, ax)];
    if (e.kind == VCD_PRESENT) atomicAdd(&J.sort_ctl[len_bucket(e.len)], 1u);
}

// exclusive scan of the kSortBuckets counters in place; their sum -> ctl[kSortBuckets]
__global__ void __launch_bounds__(1024) k_len_scan(uint32_t *ctl) {
    __shared__ uint32_t warp_sum[32];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, wid = tid >> 5;
    uint32_t a[4], s = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        a[j] = s;
        s += ctl[tid * 4 + j];
    }
    uint32_t incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31) warp_sum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const uint32_t w = warp_sum[lane];
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, wi, o);
            if (lane >= (uint32_t)o) wi += y;
        }
        warp_sum[lane] = wi - w;
        if (lane == 31) ctl[kSortBuckets] = wi;
    }
    __syncthreads();
    const uint32_t base = warp_sum[wid] + incl - s;
#pragma unroll
    for (int j = 0; j < 4; ++j) ctl[tid * 4 + j] = base + a[j];
}

__global__ void k_len_scatter(DecodeJob J) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= J.n_atoms) return;
    uint32_t az, ay, ax;
    box_atom(J, t, az, ay, ax);
    const vcd_atom e = J.atoms[job_atom(J, t, az, ay, ax)];
    if (e.kind == VCD_PRESENT) J.order[atomicAdd(&J.sort_ctl[len_bucket(e.len)], 1u)] = (uint32_t)t;
    else J.order[J.sort_ctl[kSortBuckets] + atomicAdd(&J.sort_ctl[kSortBuckets + 1], 1u)] = (uint32_t)t;   // after them
}

static_assert(kSortBuckets == 4 * 1024, "k_len_scan: 1024 threads x 4 counters");

constexpr int kLaneThreads = 64;   // 2 warps per CTA
constexpr int kLaneUnroll = 8;     // steps between warp votes

__global__ void __launch_bounds__(kLaneThreads) k_rc_lanes(DecodeJob J) {
    __shared__ uint32_t bstart[10];   // the band table and a copy of its end (RcLane)
    __shared__ uint32_t S[12 * kLaneThreads];   // magnitude contexts, lane-interleaved
    if (threadIdx.x < 10) bstart[threadIdx.x] = J.band_start[threadIdx.x < 9 ? threadIdx.x : 8];
    __syncthreads();
    const uint64_t i = (uint64_t)blockIdx.x * kLaneThreads + threadIdx.x;
    const bool active = i < J.sort_ctl[kSortBuckets];
    uint64_t t = 0;
    vcd_atom e = {};
    uint32_t cap = 0;
    uint32_t *dst = J.ent;
    if (active) {
        t = J.order[i];
        uint32_t az, ay, ax;
        box_atom(J, t, az, ay, ax);
        e = J.atoms[job_atom(J, t, az, ay, ax)];
        cap = 8u * (e.len - 1u) + 64u;
        if (e.len - 1u > VCD_MAX_ENTRIES / 8u || cap > VCD_MAX_ENTRIES) cap = VCD_MAX_ENTRIES;
        dst = J.ent + J.ent_off[t];
    }
    uint32_t *Sl = S + threadIdx.x;
    RcLane L;
    L.init(J.arc + e.off + 1, e.len - 1u, active, bstart, Sl, kLaneThreads, dst, cap);
    while (__any_sync(0xFFFFFFFFu, L.c != kLaneDone)) {
#pragma unroll
        for (int k = 0; k < kLaneUnroll; ++k) L.step(bstart, Sl, kLaneThreads);
    }
    if (!active) return;
    const uint32_t n = L.n > cap ? cap : L.n;
    J.cnt[t] = n | (L.n > cap ? kEntOverflow : 0u) | (L.bad ? kEntBad : 0u);
    atomicAdd(J.nnz_total, (unsigned long long)n);
    if (L.bad) atomicMin(J.err, (uint32_t)(t < 0xFFFFFFFFull ? t : 0xFFFFFFFEull));
}

// Solo atoms: the first n atoms of the length order (the longest payloads)
// each get a warp of their own whose lane 0 runs the latency decoder, on a
// second stream beside k_rc_lanes, which takes the atoms after them. The
// longest atoms set the per-lane decoder's time (every lane steps at about the
// same pace, whatever its atom, bound by its own dependency chain), and the
// latency decoder's chain is about twice as fast per decision while its one
// lane takes about a third of a sub-partition's issue slots. Off by default
// (vcg_set_rc_solo): measured on GB300 (1024^3 at target 10, range decode
// 8.26 ms without) it gave 7.88 ms with 76 solo atoms in one process and
// 8.41 ms in another, 8.0-8.3 ms with 152-608, and once 15.4 ms when the two
// kernels ran one after the other: the gain depends on where the solo warps
// land.
__global__ void __launch_bounds__(32) k_rc_solo(DecodeJob J, uint32_t n) {
    __shared__ uint32_t bstart[9];
    if (threadIdx.x < 9) bstart[threadIdx.x] = J.band_start[threadIdx.x];
    __syncthreads();
    const uint32_t k = blockIdx.x;
    if (threadIdx.x != 0 || k >= n || k >= J.sort_ctl[kSortBuckets]) return;
    const uint64_t t = J.order[k];
    uint32_t az, ay, ax;
    box_atom(J, t, az, ay, ax);
    const vcd_atom e = J.atoms[job_atom(J, t, az, ay, ax)];   // PRESENT: the order puts those first
    uint32_t cap = 8u * (e.len - 1u) + 64u;
    if (e.len - 1u > VCD_MAX_ENTRIES / 8u || cap > VCD_MAX_ENTRIES) cap = VCD_MAX_ENTRIES;
    uint32_t *dst = J.ent + J.ent_off[t];
    uint32_t m = 0;
    auto sink = [&](uint32_t p, uint32_t lv) {
        if (m < cap) dst[m] = p | (lv << 16);
        ++m;
    };
    const int bad = rc_decode_levels_lat(J.arc + e.off + 1, e.len - 1u, bstart, sink);
    J.cnt[t] = (m > cap ? cap : m) | (m > cap ? kEntOverflow : 0u) | (bad ? kEntBad : 0u);
    atomicAdd(J.nnz_total, (unsigned long long)(m > cap ? cap : m));
    if (bad) atomicMin(J.err, (uint32_t)(t < 0xFFFFFFFFull ? t : 0xFFFFFFFEull));
}

// ctl[kSortBuckets + 2] = the PRESENT atoms left to the per-lane warps after n solo atoms
__global__ void k_solo_split(uint32_t *ctl, uint32_t n) {
    const uint32_t np = ctl[kSortBuckets];
    ctl[kSortBuckets + 2] = np - (n < np ? n : np);
}

void launch_len_scan(uint32_t *sort_ctl, cudaStream_t s) { k_len_scan<<<1, 1024, 0, s>>>(sort_ctl); }

static void launch_len_sort(const DecodeJob &J, cudaStream_t s) {
    const unsigned nb = (unsigned)((J.n_atoms + 255) / 256);
    cudaMemsetAsync(J.sort_ctl, 0, sort_ctl_words() * 4, s);
    k_len_hist<<<nb, 256, 0, s>>>(J);
    k_len_scan<<<1, 1024, 0, s>>>(J.sort_ctl);
    k_len_scatter<<<nb, 256, 0, s>>>(J);
}

// The range decode of every PRESENT box atom:
//   up to one atom per SM sub-partition: latency decoder, one atom per warp;
//   up to rc_scalar_warps() per sub-partition: scalar decoder, one atom per
//     warp, longest payload first (the tail is the shortest atoms);
//   above: the per-lane decoder over atoms sorted by payload length, the
//     rc_solo_for() longest on the latency decoder (k_rc_solo, a warp each,
//     on the second stream of ev, between its fork and join events).
// Without an order buffer (no-alloc path) the unsorted forms are used.
static void launch_rc(const DecodeJob &J, int num_sms, cudaStream_t s, const StageEvents *ev) {
    const uint32_t G = rc_lanes_for(J.n_atoms, (uint32_t)num_sms, rc_scalar_warps());
    const bool sorted = J.order && J.sort_ctl && rc_sorts(J.n_atoms, (uint32_t)num_sms);
    if (sorted) launch_len_sort(J, s);
    if (G > 1 && sorted) {
        const uint32_t ns = ev && ev->side && ev->fork && ev->join ? rc_solo_for(J.n_atoms, (uint32_t)num_sms) : 0u;
        DecodeJob Jl = J;
        if (ns) {
            // (fewer PRESENT atoms than ns: k_solo_split's count is 0 and the
            // shifted order is not read)
            k_solo_split<<<1, 1, 0, s>>>(J.sort_ctl, ns);
            cudaEventRecord(ev->fork, s);
            cudaStreamWaitEvent(ev->side, ev->fork, 0);
            k_rc_solo<<<ns, 32, 0, ev->side>>>(J, ns);
            cudaEventRecord(ev->join, ev->side);
            Jl.order = J.order + ns;
            Jl.sort_ctl = J.sort_ctl + 2;   // Jl.sort_ctl[kSortBuckets]: the per-lane count
        }
        const uint64_t lane_blocks = (J.n_atoms - ns + kLaneThreads - 1) / kLaneThreads;
        if (lane_blocks) k_rc_lanes<<<(unsigned)lane_blocks, kLaneThreads, 0, s>>>(Jl);   // (0: every atom solo)
        if (ns) cudaStreamWaitEvent(s, ev->join, 0);
        return;
    }
    DecodeJob Jr = J;
    if (!sorted) {
        Jr.order = nullptr;
        Jr.sort_ctl = nullptr;
    }
    const uint32_t lat = G == 1 && J.n_atoms <= 4ull * (uint64_t)num_sms ? 1u : 0u;
    k_rc_decode<<<(unsigned)((J.n_atoms + G - 1) / G), 32, lat ? kLatStage + 16 : 0, s>>>(Jr, G, lat);
}

// Box atom t: dequantise + inverse transform + crop into the box raster, by NT
// threads (tid = 0..NT-1) that meet at barrier BAR (tile_sync); ends with one.
template <int NT, int BAR>
__device__ __forceinline__ void idct_atom(const DecodeJob &J, uint64_t t, int32_t *T, const int32_t *dqs,
                                          const int32_t *dqb, const uint32_t *alt, int tid) {
    const int lane = tid & 31, warp = tid >> 5;
    uint32_t az, ay, ax;
    box_atom(J, t, az, ay, ax);
    const vcd_atom e = J.atoms[job_atom(J, t, az, ay, ax)];
    Crop k;
    const uint32_t gx = ax * 32, gy = ay * 32, gz = az * 32;
    k.set(gx, gy, gz, J.x0, J.y0, J.z0, J.x1, J.y1, J.z1);
    uint8_t *obase = J.out + ((uint64_t)(gz + k.lz0 - J.z0) * J.oy + (gy + k.ly0 - J.y0)) * J.ox + (gx + k.lx0 - J.x0);
    // (BAR != 0: inside the fused decode, whose lists and counts this kernel wrote)
    const uint32_t c = e.kind == VCD_PRESENT ? (BAR ? __ldcg(J.cnt + t) : J.cnt[t]) : kEntBad;
    if (e.kind != VCD_PRESENT || (c & kEntBad)) {   // ABSENT / KNOWN_ZERO -> zeros
        zero_window<NT>(obase, J.ox, J.oy, k, (uint32_t)tid);
        return;
    }
    const int32_t dc = J.arc[e.off];
    idct_tile_xy<NT, BAR, BAR != 0, BAR != 0>(T, J.arc, e, c, J.ent + J.ent_off[t], J.scan, J.band_start, dqs, dqb,
                                               alt, tid);
    const bool full = k.lz0 == 0 && k.lz1 == 32;
    for (int y = warp; y < 32; y += NT / 32) {
        int32_t o[32];
        idct_col_z(T, y, lane, o);
        if (full) store_col_full(obase, J.ox, J.oy, k, y, lane, o, dc);
        else store_col(obase, J.ox, J.oy, k, y, lane, o, dc);
    }
    tile_sync<NT, BAR>();
}

__global__ void __launch_bounds__(kIdctThreads, 1) k_idct(DecodeJob J) {
    extern __shared__ int32_t T[];   // 32 slabs x padded 32x32 (idct_tile.cuh)
    __shared__ int32_t dqs[VCD_NCLASS], dqb[VCD_NCLASS];
    __shared__ uint32_t alt[1024];
    const int tid = threadIdx.x;
    for (int i = tid; i < VCD_NCLASS; i += kIdctThreads) { dqs[i] = J.dq->step[i]; dqb[i] = J.dq->bias[i]; }
    for (int i = tid; i < 1024; i += kIdctThreads) alt[i] = J.alt_mask[i];
    __syncthreads();
    for (uint64_t t = J.t_lo + blockIdx.x; t < J.t_hi; t += gridDim.x) idct_atom<kIdctThreads, 0>(J, t, T, dqs, dqb, alt, tid);
}

// ---- fused decode: range decode and inverse transform in one persistent
// kernel, one CTA per SM. Each CTA owns the entries c, c + G, c + 2G, ... of
// the payload-length order (G CTAs), so every CTA gets the same mix of long
// and short atoms. Its first 8 warps decode them: the CTA's head (entry c, its
// longest atom) on one lane of the 8th warp with the latency decoder (a
// decision in about 50 ns against about 110 ns for a step of the per-lane
// decoder in a full warp, so the longest atoms no longer set the coder's end),
// the others with the per-lane decoder on 7 warps (lane j takes the CTA's
// entries 1 + j, 1 + j + 224, ...); whenever an atom is decoded it is published
// in the CTA's queue. The other 8 warps transform the
// queued atoms in that order (ABSENT / KNOWN_ZERO atoms are queued at the
// start), so the transforms of finished atoms run while the coder is still busy
// with the longer ones: the integer-multiply pipe of the transform and the ALU
// work of the coder share the SM instead of running one after the other. Only
// warps of the same CTA wait for one another; a wait that exceeds kFusedSpin
// polls sets *fail and the transform warps stop.
constexpr int kFusedRcThreads = 256;   // 8 decoding warps
constexpr int kFusedLaneThreads = kFusedRcThreads - 32;   // 7 of them per-lane; the 8th: the CTA's head atom
constexpr int kFusedTxThreads = 256;   // 8 transforming warps
constexpr int kFusedThreads = kFusedRcThreads + kFusedTxThreads;
constexpr uint32_t kQueueEmpty = 0xFFFFFFFFu;
constexpr uint64_t kFusedSpin = 1ull << 24;   // x 256 ns sleeps: about 4 s

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// queue: G x per slots, CTA c's at [c * per, c * per + per), preset to kQueueEmpty
__global__ void __launch_bounds__(kFusedThreads, 1) k_decode_fused(DecodeJob J, uint32_t *queue, uint32_t per,
                                                                    uint32_t *fail) {
    extern __shared__ int32_t T[];   // transform tile
    __shared__ uint32_t bstart[10];   // the band table and a copy of its end (RcLane)
    __shared__ uint32_t S[12 * kFusedRcThreads];
    __shared__ int32_t dqs[VCD_NCLASS], dqb[VCD_NCLASS];
    __shared__ uint32_t alt[1024];
    __shared__ uint32_t q_tail;   // slots of this CTA's queue handed out
    __shared__ uint32_t cur[2];   // atom of the transform's current iteration (double-buffered)
    const int tid = threadIdx.x;
    if (tid < 10) bstart[tid] = J.band_start[tid < 9 ? tid : 8];
    for (int i = tid; i < VCD_NCLASS; i += kFusedThreads) { dqs[i] = J.dq->step[i]; dqb[i] = J.dq->bias[i]; }
    for (int i = tid; i < 1024; i += kFusedThreads) alt[i] = J.alt_mask[i];
    if (tid == 0) q_tail = 0;
    __syncthreads();
    const uint32_t G = gridDim.x, cta = blockIdx.x;
    const uint32_t n = (uint32_t)J.n_atoms, n_present = J.sort_ctl[kSortBuckets];
    const uint32_t n_cta = cta < n ? (n - 1 - cta) / G + 1 : 0;
    const uint32_t np_cta = cta < n_present ? (n_present - 1 - cta) / G + 1 : 0;
    uint32_t *Q = queue + (uint64_t)cta * per;
    if (tid < kFusedRcThreads) {
        for (uint32_t k = np_cta + tid; k < n_cta; k += kFusedRcThreads)   // nothing to decode
            atomicExch(Q + atomicAdd(&q_tail, 1u), J.order[cta + k * G]);
        if (tid >= kFusedLaneThreads) {   // the head: the CTA's longest atom, alone on one lane
            if (tid == kFusedLaneThreads && np_cta) {
                const uint32_t t = J.order[cta];
                uint32_t az, ay, ax;
                box_atom(J, t, az, ay, ax);
                const vcd_atom e = J.atoms[job_atom(J, t, az, ay, ax)];
                uint32_t cap = 8u * (e.len - 1u) + 64u;
                if (e.len - 1u > VCD_MAX_ENTRIES / 8u || cap > VCD_MAX_ENTRIES) cap = VCD_MAX_ENTRIES;
                uint32_t *dst = J.ent + J.ent_off[t];
                uint32_t cnt = 0;
                auto sink = [&](uint32_t p, uint32_t lv) {
                    if (cnt < cap) dst[cnt] = p | (lv << 16);
                    ++cnt;
                };
                const int bad = rc_decode_levels_lat(J.arc + e.off + 1, e.len - 1u, bstart, sink);
                const uint32_t m = cnt > cap ? cap : cnt;
                J.cnt[t] = m | (cnt > cap ? kEntOverflow : 0u) | (bad ? kEntBad : 0u);
                atomicAdd(J.nnz_total, (unsigned long long)m);
                if (bad) atomicMin(J.err, t);
                __threadfence();
                atomicExch(Q + atomicAdd(&q_tail, 1u), t);
            }
            return;
        }
        uint32_t *Sl = S + tid;
        uint32_t k = 1u + (uint32_t)tid, t = 0, cap = 0;   // the CTA's entries after its head
        bool have = false;
        RcLane L;
        auto start = [&]() {   // the lane's next atom, if any
            have = k < np_cta;
            vcd_atom e = {};
            uint32_t *dst = J.ent;
            if (have) {
                t = J.order[cta + k * G];
                uint32_t az, ay, ax;
                box_atom(J, t, az, ay, ax);
                e = J.atoms[job_atom(J, t, az, ay, ax)];
                cap = 8u * (e.len - 1u) + 64u;
                if (e.len - 1u > VCD_MAX_ENTRIES / 8u || cap > VCD_MAX_ENTRIES) cap = VCD_MAX_ENTRIES;
                dst = J.ent + J.ent_off[t];
            }
            L.init(J.arc + e.off + 1, e.len - 1u, have, bstart, Sl, kFusedRcThreads, dst, cap);
        };
        start();
        while (__any_sync(0xFFFFFFFFu, have)) {
#pragma unroll
            for (int s = 0; s < kLaneUnroll; ++s) L.step(bstart, Sl, kFusedRcThreads);
            if (have && L.c == kLaneDone) {   // finished: counts, then publish the atom
                const uint32_t m = L.n > cap ? cap : L.n;
                J.cnt[t] = m | (L.n > cap ? kEntOverflow : 0u) | (L.bad ? kEntBad : 0u);
                atomicAdd(J.nnz_total, (unsigned long long)m);
                if (L.bad) atomicMin(J.err, t);
                __threadfence();
                atomicExch(Q + atomicAdd(&q_tail, 1u), t);
                k += kFusedLaneThreads;
                start();
            }
        }
    } else {
        const int tt = tid - kFusedRcThreads;
        for (uint32_t k = 0; k < n_cta; ++k) {
            if (tt == 0) {
                uint32_t v = ld_acquire_u32(Q + k);
                for (uint64_t spins = 0; v == kQueueEmpty; v = ld_acquire_u32(Q + k)) {
                    if (++spins > kFusedSpin) {
                        atomicExch(fail, 1u);
                        break;
                    }
                    __nanosleep(256);
                }
                cur[k & 1] = v;
            }
            tile_sync<kFusedTxThreads, 1>();
            const uint32_t t = cur[k & 1];
            if (t == kQueueEmpty) break;   // gave up waiting (every transform thread sees it)
            __threadfence();
            idct_atom<kFusedTxThreads, 1>(J, t, T, dqs, dqb, alt, tt);
        }
    }
}

// Fused range decode + transform of a whole box: above one atom per warp (the
// per-lane decoder's range) with an order buffer; queue: per-CTA slots
// (decode_fused_queue_words(n) words), fail: a zeroed word. Returns false when
// the box takes the separate kernels instead.
bool launch_decode_fused(const DecodeJob &J, int num_sms, cudaStream_t s, uint32_t *queue, uint32_t *fail,
                         const StageEvents *ev) {
    if (!J.order || !J.sort_ctl || !queue || rc_lanes_for(J.n_atoms, (uint32_t)num_sms, rc_scalar_warps()) <= 1)
        return false;
    const uint32_t G = (uint32_t)num_sms;
    const uint32_t per = (uint32_t)((J.n_atoms + G - 1) / G);
    if (ev) cudaEventRecord(ev->ev[0], s);
    const unsigned nb = (unsigned)((J.n_atoms + 127) / 128);
    k_caps<<<nb, 128, 0, s>>>(J);
    launch_scan_u64(J.ent_off, J.n_atoms, 0, nullptr, s);
    if (ev) cudaEventRecord(ev->ev[1], s);
    launch_len_sort(J, s);
    cudaMemsetAsync(queue, 0xFF, (size_t)G * per * 4, s);
    if (ev) cudaEventRecord(ev->ev[2], s);
    smem_attr((const void *)k_decode_fused, (int)kIdctSmem);
    k_decode_fused<<<G, kFusedThreads, kIdctSmem, s>>>(J, queue, per, fail);
    if (ev) cudaEventRecord(ev->ev[3], s);
    return true;
}

void launch_scan_u64(uint64_t *v, uint64_t n, uint64_t base, uint64_t *total, cudaStream_t s) {
    k_scan_u64<<<1, 1024, 0, s>>>(v, n, base, total);
}

void launch_idct(const DecodeJob &J, int num_sms, cudaStream_t s, uint64_t t_lo, uint64_t t_hi) {
    if (t_hi <= t_lo) return;
    smem_attr((const void *)k_idct, (int)kIdctSmem);
    DecodeJob Jr = J;
    Jr.t_lo = t_lo;
    Jr.t_hi = t_hi;
    const uint64_t n = t_hi - t_lo;
    const uint64_t grid = n < (uint64_t)num_sms ? n : (uint64_t)num_sms;
    k_idct<<<(unsigned)grid, kIdctThreads, kIdctSmem, s>>>(Jr);
}

void launch_decode_lists(const DecodeJob &J, int num_sms, cudaStream_t s) {
    if (!J.n_atoms) return;
    launch_rc(J, num_sms, s, nullptr);
    launch_idct(J, num_sms, s, 0, J.n_atoms);
}

void launch_decode_front(const DecodeJob &J, int num_sms, cudaStream_t s, const StageEvents *ev) {
    if (ev) cudaEventRecord(ev->ev[0], s);
    unsigned nb = (unsigned)((J.n_atoms + 127) / 128);
    if (J.n_atoms) {
        k_caps<<<nb, 128, 0, s>>>(J);
        launch_scan_u64(J.ent_off, J.n_atoms, 0, nullptr, s);
    }
    if (ev) cudaEventRecord(ev->ev[1], s);
    if (J.n_atoms) launch_rc(J, num_sms, s, ev);
    if (ev) cudaEventRecord(ev->ev[2], s);
}

void launch_decode(const DecodeJob &J, int num_sms, cudaStream_t s, const StageEvents *ev) {
    launch_decode_front(J, num_sms, s, ev);
    launch_idct(J, num_sms, s, 0, J.n_atoms);
    if (ev) cudaEventRecord(ev->ev[3], s);
}

}  // namespace vcg

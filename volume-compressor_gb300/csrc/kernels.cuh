// Kernel interfaces shared by the CUDA translation units (private).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "vc_internal.h"

namespace vcg {

constexpr uint32_t kEntOverflow = 1u << 31;   // cnt flag: list exceeded its capacity
constexpr uint32_t kEntBad = 1u << 30;        // cnt flag: malformed stream
constexpr uint32_t kEntMask = (1u << 30) - 1u;

// Region / LOD decode, box atoms in (z, y, x) order.
struct DecodeJob {
    const uint8_t *arc;          // device archive bytes
    const vcd_atom *atoms;       // device atom table of the LOD
    uint32_t acx, acy;           // LOD atom grid (x, y)
    uint32_t bax, bay, baz, bnx, bny;
    uint64_t n_atoms;
    uint32_t x0, y0, z0, x1, y1, z1;   // box
    uint8_t *out;                // box raster (x fastest)
    uint64_t ox, oy;             // box extent x, y
    uint32_t *ent;               // coefficient lists: raster index | level << 16
    uint64_t *ent_off;           // per box atom: first list slot (after the scan)
    uint32_t *cnt;               // per box atom: entries | flags
    const vcd_dq *dq;            // dequant tables of the LOD
    const uint32_t *alt_mask;    // step-class alternate bits
    const uint16_t *scan;        // scan position -> raster
    uint32_t *err;               // lowest malformed box atom (atomicMin)
    unsigned long long *nnz_total;   // coefficient-list entries written (sum over atoms)
    uint32_t band_start[9];      // first scan position of each significance band
    uint64_t t_lo, t_hi;         // box atoms the inverse transform launch covers
    uint32_t box_table;          // 1: atoms[] is indexed by box atom (staged decode), 0: by LOD raster
    // per-lane range decoder of large decodes (optional; NULL: the warp decoders):
    uint32_t *order;             // n_atoms slots: PRESENT box atoms, longest payload first
    uint32_t *sort_ctl;          // kSortBuckets counters + present-atom count
};
constexpr uint32_t kSortBuckets = 4096;   // payload length / 32, clamped
__host__ __device__ inline size_t sort_ctl_words() { return kSortBuckets + 4; }

__host__ __device__ inline uint64_t job_atom(const DecodeJob &J, uint64_t t, uint32_t az, uint32_t ay,
                                             uint32_t ax) {
    return J.box_table ? t : ((uint64_t)az * J.acy + ay) * J.acx + ax;
}

// Optional per-stage events: ev[0] before the list placement, ev[1] before the
// range decoder, ev[2] before the inverse transform, ev[3] after it.
struct StageEvents {
    cudaEvent_t ev[4];
    // optional: a second stream with two events for work beside the range
    // decode (the solo atoms of rc_solo_for); null: none
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};

__host__ __device__ inline void box_atom(const DecodeJob &J, uint64_t t, uint32_t &az, uint32_t &ay,
                                         uint32_t &ax) {
    ax = J.bax + (uint32_t)(t % J.bnx);
    ay = J.bay + (uint32_t)((t / J.bnx) % J.bny);
    az = J.baz + (uint32_t)(t / ((uint64_t)J.bnx * J.bny));
}

// ---- batched region decode: every distinct atom of a batch of boxes is decoded
// once and cropped into each box that overlaps it.
using BoxReq = vcd_boxreq;
using UAtom = vcd_uatom;
struct BatchJob {
    const uint8_t *arc;
    const vcd_atom *atoms;       // archive atom table (all LODs)
    const UAtom *ua;
    const uint32_t *dst;         // request ids, grouped per distinct atom
    const BoxReq *reqs;
    const uint32_t *n_ua;        // device: number of distinct atoms (read at run time)
    uint32_t *ent;
    const uint64_t *ent_off;     // per distinct atom
    uint32_t *cnt;
    const vcd_dq *dq;            // per LOD
    const uint32_t *alt_mask;
    const uint16_t *scan;
    uint32_t *work;              // transform work counter (reset per batch)
    uint32_t *req_err;           // per request: set when one of its atoms is malformed
    uint32_t band_start[9];
    uint32_t sms;                // SM count of the device
    uint32_t rc_scalar_warps;    // range-decoder policy (rc_lanes_for)
    uint32_t *order;             // distinct atoms in payload-length order (per-lane decoder)
    uint32_t *sort_ctl;          // kSortBuckets counters + present-atom count
};
struct BatchShape {              // tunables the autotuner chooses among
    int rc_scalar_warps;         // range-decoder policy: 1, 4 or 16 (rc_lanes_for)
    int idct_threads;            // transform CTA size (warps per atom x 32): 256 or 512
    int imma;                    // transform on the int8 tensor cores (256 threads) instead of the butterfly
};

// Atoms per warp for the range decoder. A warp that decodes one atom runs the
// scalar decoder, whose latency per atom is the lowest. One atom per warp while
// that makes at most `scalar_warps` warps per SM sub-partition (4 per SM);
// above that the plain decode path runs the per-lane decoder (k_rc_lanes: all
// 32 lanes of a warp, each its own atom; measured on GB300 it overtakes the
// scalar decoder between 2,048 and 4,096 atoms, and at 9,728 t10 atoms it
// takes 5.4 ms against 11.8 ms). The batched path still runs the lockstep
// decoder for G > 1: the fewest warps per sub-partition k that keep a warp at
// 32 atoms or fewer, the atoms spread evenly over k warps per sub-partition.
__host__ __device__ inline uint32_t rc_lanes_for(uint64_t n_atoms, uint32_t sms, uint32_t scalar_warps) {
    const uint64_t slots = 4ull * sms;
    if (n_atoms <= (uint64_t)scalar_warps * slots) return 1;
    const uint64_t k = (n_atoms + 32 * slots - 1) / (32 * slots);
    const uint64_t g = (n_atoms + k * slots - 1) / (k * slots);
    return g < 2 ? 2u : (uint32_t)g;
}
constexpr uint32_t kRcScalarWarpsDefault = 8;   // measured crossover with the per-lane decoder: 3-5k atoms
// the plain decode path puts atoms in payload-length order (and needs the order
// buffer) above one atom per SM sub-partition
__host__ __device__ inline bool rc_sorts(uint64_t n_atoms, uint32_t sms) { return n_atoms > 4ull * sms; }

// policy of the plain decode path (vcg_set_rc_scalar_warps)
uint32_t rc_scalar_warps();
// longest atoms of a per-lane decode that get a latency-decoder warp each
// (vcg_set_rc_solo); rc_solo_for: how many a decode of n box atoms gets (0 when
// it does not run the per-lane decoder)
constexpr uint32_t kRcSoloDefault = 0;
uint32_t rc_solo_atoms();
inline uint32_t rc_solo_for(uint64_t n_atoms, uint32_t sms) {
    if (rc_lanes_for(n_atoms, sms, rc_scalar_warps()) <= 1 || !rc_sorts(n_atoms, sms)) return 0;
    const uint32_t k = rc_solo_atoms();
    return (uint64_t)k < n_atoms ? k : (uint32_t)n_atoms;
}
// mid (optional): recorded between the range decode and the transform
void launch_batch(const BatchJob &J, const BatchShape &shape, int num_sms, uint32_t max_ua, cudaStream_t s,
                  cudaEvent_t mid = nullptr);

void launch_decode(const DecodeJob &J, int num_sms, cudaStream_t s, const StageEvents *ev);
// The decode in two halves: list placement + range decode (events ev[0..2]),
// then the inverse transform of box atoms [t_lo, t_hi).
void launch_decode_front(const DecodeJob &J, int num_sms, cudaStream_t s, const StageEvents *ev);
void launch_idct(const DecodeJob &J, int num_sms, cudaStream_t s, uint64_t t_lo, uint64_t t_hi);
// Range decode + inverse transform only: J.ent_off must already hold each
// atom's list offset (each list can take VCD_MAX_ENTRIES entries).
void launch_decode_lists(const DecodeJob &J, int num_sms, cudaStream_t s);
void launch_scan_u64(uint64_t *v, uint64_t n, uint64_t base, uint64_t *total, cudaStream_t s);
// exclusive scan of the kSortBuckets length counters in place, their sum after them
void launch_len_scan(uint32_t *sort_ctl, cudaStream_t s);
// Range decode and inverse transform of a whole box in one kernel (k_decode_fused)
// when the box takes the per-lane decoder and J has an order buffer: queue holds
// n_atoms + num_sms words, fail a word that starts at zero (set if the kernel
// gave up waiting). Records ev[0..3] like launch_decode. False: not applicable.
bool launch_decode_fused(const DecodeJob &J, int num_sms, cudaStream_t s, uint32_t *queue, uint32_t *fail,
                         const StageEvents *ev);

// cudaFuncAttributeMaxDynamicSharedMemorySize of kernel fn, set on the calling
// thread's current device. The attribute belongs to the device's context, not
// to the process, so it is set once per (kernel, device) pair.
cudaError_t smem_attr(const void *fn, int bytes);

}  // namespace vcg

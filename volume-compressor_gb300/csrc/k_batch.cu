// Batched region decode (device): a persistent range-decode pass over the
// batch's distinct atoms, then a persistent transform pass that takes atoms from
// a device work counter and crops each decoded atom into every request box that
// overlaps it (src/vc/vc.c:1535-1555 per box). The counts are read from device
// memory, so the same launches (and a CUDA graph of them) serve any batch that
// fits the buffers.
#include <cuda_runtime.h>
#include <stdint.h>

#include "idct_tile.cuh"
#include "kernels.cuh"
#include "rangecoder.cuh"

namespace vcg {

constexpr size_t kTileSmem = 32768 * sizeof(int32_t);

// Persistent over the batch's distinct atoms (their number is read from device
// memory): G atoms per warp by rc_lanes_for, scalar decoder for G = 1, lockstep
// decoder otherwise.
constexpr int kRcBatchThreads = 128;

__global__ void __launch_bounds__(kRcBatchThreads) k_rc_batch(BatchJob J) {
    __shared__ uint32_t bstart[9];
    if (threadIdx.x < 9) bstart[threadIdx.x] = J.band_start[threadIdx.x];
    __syncthreads();
    const uint32_t n = *J.n_ua;
    const uint32_t G = rc_lanes_for(n, J.sms, J.rc_scalar_warps);
    const uint32_t lane = threadIdx.x & 31u;
    if (G == 1 && lane != 0) return;
    const uint64_t nwarps = (uint64_t)gridDim.x * (kRcBatchThreads / 32);
    for (uint64_t w = ((uint64_t)blockIdx.x * kRcBatchThreads + threadIdx.x) >> 5; w * G < n; w += nwarps) {
        const uint64_t u = w * G + lane;
        bool active = false;
        vcd_atom e = {};
        if (lane < G && u < n) {
            e = J.atoms[J.ua[u].idx];
            active = e.kind == VCD_PRESENT;
            if (!active) J.cnt[u] = 0;
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
            if (active) bad = rc_decode_levels_lane(J.arc + e.off + 1, e.len - 1, bstart, sink);
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

template <int NT>
__global__ void __launch_bounds__(NT, 1) k_idct_batch(BatchJob J) {
    extern __shared__ int32_t T[];
    __shared__ int32_t dqs[VCD_NCLASS], dqb[VCD_NCLASS];
    __shared__ uint32_t alt[1024];
    __shared__ uint32_t s_u;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
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
        const uint32_t gx = a.ax * 32, gy = a.ay * 32, gz = a.az * 32;
        if (e.kind != VCD_PRESENT || (c & kEntBad)) {   // ABSENT / KNOWN_ZERO -> zeros in every box
            for (uint32_t d = a.dst_begin; d < a.dst_end; ++d) {
                const BoxReq r = J.reqs[J.dst[d]];
                Crop k;
                k.set(gx, gy, gz, r.x0, r.y0, r.z0, r.x1, r.y1, r.z1);
                const uint64_t ox = r.x1 - r.x0, oy = r.y1 - r.y0;
                uint8_t *ob = r.out + ((uint64_t)(gz + k.lz0 - r.z0) * oy + (gy + k.ly0 - r.y0)) * ox + (gx + k.lx0 - r.x0);
                zero_window<NT>(ob, ox, oy, k);
            }
            continue;
        }
        const int32_t dc = J.arc[e.off];
        idct_tile_xy<NT>(T, J.arc, e, c, J.ent + J.ent_off[u], J.scan, J.band_start, dqs, dqb, alt);
        for (int y = warp; y < 32; y += NT / 32) {
            int32_t o[32];
            idct_col_z(T, y, lane, o);
            for (uint32_t d = a.dst_begin; d < a.dst_end; ++d) {
                const BoxReq r = J.reqs[J.dst[d]];
                Crop k;
                k.set(gx, gy, gz, r.x0, r.y0, r.z0, r.x1, r.y1, r.z1);
                const uint64_t ox = r.x1 - r.x0, oy = r.y1 - r.y0;
                uint8_t *ob = r.out + ((uint64_t)(gz + k.lz0 - r.z0) * oy + (gy + k.ly0 - r.y0)) * ox + (gx + k.lx0 - r.x0);
                store_col(ob, ox, oy, k, y, lane, o, dc);
            }
        }
        __syncthreads();
    }
}

static void launch_rc(const BatchJob &J, int num_sms, uint32_t max_ua, cudaStream_t s) {
    // warps for the widest case up to max_ua atoms: one per atom while the
    // policy keeps atoms one per warp, else one per 32 atoms; capped at a full
    // device (the kernel loops)
    const uint64_t slots = 4ull * (uint64_t)num_sms;
    const uint64_t scalar = (uint64_t)J.rc_scalar_warps * slots;
    uint64_t warps = max_ua < scalar ? max_ua : scalar;
    const uint64_t packed = ((uint64_t)max_ua + 31) / 32;
    if (packed > warps) warps = packed;
    const uint64_t cap = (uint64_t)num_sms * (2048 / kRcBatchThreads) * (kRcBatchThreads / 32);
    if (warps > cap) warps = cap;
    if (warps < 1) warps = 1;
    const unsigned grid = (unsigned)((warps * 32 + kRcBatchThreads - 1) / kRcBatchThreads);
    k_rc_batch<<<grid, kRcBatchThreads, 0, s>>>(J);
}

template <int NT>
static void launch_tx(const BatchJob &J, int num_sms, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_idct_batch<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTileSmem);
        attr = true;
    }
    k_idct_batch<NT><<<num_sms, NT, kTileSmem, s>>>(J);
}

void launch_batch(const BatchJob &J, const BatchShape &shape, int num_sms, uint32_t max_ua, cudaStream_t s) {
    BatchJob Jr = J;
    Jr.rc_scalar_warps = (uint32_t)shape.rc_scalar_warps;
    Jr.sms = (uint32_t)num_sms;
    launch_rc(Jr, num_sms, max_ua, s);
    if (shape.idct_threads == 512) launch_tx<512>(J, num_sms, s);
    else launch_tx<256>(J, num_sms, s);
}

}  // namespace vcg

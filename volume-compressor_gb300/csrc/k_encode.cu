// Encode kernels.
//
//   k_fwd         one CTA per atom: gather (zero padding outside the volume),
//                 sum -> zero flag + dc (src/vc/vc.c:599-604), forward DCT-32
//                 passes x, y per z-slab then z per column (src/vc/vc.c:212-218),
//                 dead-zone quantiser as the release build evaluates it
//                 (src/vc/vc.c:293-306), levels scattered to scan order in
//                 shared memory and compacted to (scan position, level) lists
//   k_rc_encode   one thread per atom: range coder, size-only or writing the
//                 payload [dc][bytes] at its archive offset (src/vc/vc.c:528-544,
//                 595-622)
//   k_consume / k_slots   canonical layout: bytes consumed per atom in append
//                 order (an L2 block of 512 KiB at a region's first atom, then the
//                 payload) and the 16-byte L2 slots (src/vc/vc.c:1082-1159)
#include <cuda_runtime.h>
#include <stdint.h>

#include "dct32.cuh"
#include "k_encode.cuh"
#include "kernels.cuh"
#include "rangecoder.cuh"

namespace vcg {

constexpr int kFwdThreads = 256;
constexpr size_t kFwdSmem = kTileBytes + 32768 * sizeof(int16_t);

// 32 voxels of row (z, y) of atom (az, ay, ax), zero outside the volume, packed
// little-endian into 8 words.
__device__ __forceinline__ void load_row(const uint8_t *vol, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t gx,
                                         uint32_t gy, uint32_t gz, uint32_t (&w)[8]) {
#pragma unroll
    for (int i = 0; i < 8; ++i) w[i] = 0;
    if (gy >= ny || gz >= nz || gx >= nx) return;
    const uint8_t *p = vol + ((uint64_t)gz * ny + gy) * nx + gx;
    if (gx + 32 <= nx && ((uintptr_t)p & 15u) == 0) {
        uint4 a = __ldg(reinterpret_cast<const uint4 *>(p));
        uint4 b = __ldg(reinterpret_cast<const uint4 *>(p + 16));
        w[0] = a.x; w[1] = a.y; w[2] = a.z; w[3] = a.w; w[4] = b.x; w[5] = b.y; w[6] = b.z; w[7] = b.w;
        return;
    }
    uint32_t cnt = nx - gx < 32 ? nx - gx : 32;
    for (uint32_t i = 0; i < cnt; ++i) w[i >> 2] |= (uint32_t)__ldg(p + i) << (8 * (i & 3));
}

// Quantiser class of raster r: its frequency, + 94 where the alternate step
// applies (src/vc/vc.c:273-279, 293-306).
__device__ __forceinline__ uint32_t quant_class(uint32_t r, const uint32_t *alt) {
    const uint32_t f = (r >> 10) + ((r >> 5) & 31u) + (r & 31u);
    return f + 94u * ((alt[r >> 5] >> (r & 31u)) & 1u);
}

// A coefficient with its class, as the quantiser needs it: |cf| in bits 0-16
// (the transform of 8-bit voxels about a centre in [0, 255] reaches at most
// 46,132, the DC of a block 255 away from its centre), the class in bits 17-24,
// the sign in bit 31. Quantising it needs no scan order or class lookup.
__device__ __forceinline__ uint32_t coef_pack(int32_t cf, uint32_t r, const uint32_t *alt) {
    const uint32_t mag = cf < 0 ? 0u - (uint32_t)cf : (uint32_t)cf;
    return mag | (quant_class(r, alt) << 17) | (cf < 0 ? 0x80000000u : 0u);
}

// Dead-zone quantiser of a packed coefficient, as the release build evaluates
// it (src/vc/vc.c:293-306): level = trunc((|cf| - dz) r' + 1) for |cf| >= dz,
// clamped, with the coefficient's sign.
__device__ __forceinline__ int32_t quant_packed(uint32_t w, const float *qdz, const float *qrr) {
    const uint32_t cls = (w >> 17) & 0xFFu;
    const float fa = __int2float_rn((int32_t)(w & 0x1FFFFu));
    int32_t level = 0;
    if (fa >= qdz[cls]) {
        level = __float2int_rz(__fadd_rn(__fmul_rn(__fsub_rn(fa, qdz[cls]), qrr[cls]), 1.0f));
        if (level > 32767) level = 32767;
    }
    return (w >> 31) ? -level : level;
}

// Quantise one atom in scan order and compact its nonzero levels into the list
// dst (scan position | level << 16, in scan order); returns the count (every
// thread). Warp w owns scan positions [4096 w, 4096 w + 4096), 128 at a time,
// each lane 4 consecutive ones (pk4(p) gives the packed coefficients of scan
// positions p..p+3): pass 1 quantises, keeps the levels in lv and counts them;
// pass 2 places each lane's entries after a warp prefix sum of the per-lane
// counts, skipping groups without a nonzero level. NT must be 256.
template <int NT, class Pk4>
__device__ __forceinline__ uint32_t quant_compact(Pk4 &&pk4, const float *qdz, const float *qrr, int16_t *lv,
                                                  uint32_t *wcnt, uint32_t *dst) {
    static_assert(NT == 256, "eight warps of 4096 scan positions");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t p0 = (uint32_t)warp * 4096u + 4u * (uint32_t)lane;
    uint32_t cnt = 0;
    // groups of kG x 128 positions: every load of a group is issued before the
    // first level is stored
    constexpr uint32_t kG = 4;
#pragma unroll 1
    for (uint32_t i = 0; i < 4096; i += 128 * kG) {
        uint4 w[kG];
#pragma unroll
        for (uint32_t g = 0; g < kG; ++g) w[g] = pk4(p0 + i + 128 * g);
#pragma unroll
        for (uint32_t g = 0; g < kG; ++g) {
            const int32_t l0 = quant_packed(w[g].x, qdz, qrr), l1 = quant_packed(w[g].y, qdz, qrr);
            const int32_t l2 = quant_packed(w[g].z, qdz, qrr), l3 = quant_packed(w[g].w, qdz, qrr);
            *reinterpret_cast<uint2 *>(lv + p0 + i + 128 * g) =
                make_uint2((uint32_t)(uint16_t)l0 | ((uint32_t)l1 << 16), (uint32_t)(uint16_t)l2 | ((uint32_t)l3 << 16));
            cnt += (uint32_t)(l0 != 0) + (uint32_t)(l1 != 0) + (uint32_t)(l2 != 0) + (uint32_t)(l3 != 0);
        }
    }
    cnt = __reduce_add_sync(0xFFFFFFFFu, cnt);
    if (lane == 0) wcnt[warp] = cnt;
    __syncthreads();
    uint32_t base = 0, total = 0;
#pragma unroll
    for (int w = 0; w < NT / 32; ++w) {
        const uint32_t v = wcnt[w];
        base += w < warp ? v : 0u;
        total += v;
    }
#pragma unroll 4
    for (uint32_t i = 0; i < 4096; i += 128) {
        const uint32_t p = p0 + i;
        const uint2 pk = *reinterpret_cast<const uint2 *>(lv + p);
        if (!__any_sync(0xFFFFFFFFu, (pk.x | pk.y) != 0u)) continue;
        const uint32_t lw[4] = {pk.x & 0xFFFFu, pk.x >> 16, pk.y & 0xFFFFu, pk.y >> 16};
        const uint32_t k = (uint32_t)(lw[0] != 0) + (uint32_t)(lw[1] != 0) + (uint32_t)(lw[2] != 0) +
                           (uint32_t)(lw[3] != 0);
        uint32_t incl = k;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += y;
        }
        uint32_t *d = dst + base + (incl - k);
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (lw[j]) *d++ = (p + (uint32_t)j) | (lw[j] << 16);
        base += __shfl_sync(0xFFFFFFFFu, incl, 31);
    }
    __syncthreads();   // lv and wcnt are reused by the next atom
    return total;
}

__global__ void __launch_bounds__(kFwdThreads, 1) k_fwd(FwdJob J) {
    extern __shared__ int32_t smem[];
    int32_t *T = smem;                                          // the padded atom tile (dct32.cuh)
    int16_t *L = reinterpret_cast<int16_t *>(smem + kTileInts); // levels in scan order
    __shared__ float qdz[VCD_NCLASS], qrr[VCD_NCLASS];
    __shared__ uint32_t alt[1024];
    __shared__ uint32_t red[32];
    __shared__ uint32_t wcnt[kFwdThreads / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < 1024; i += kFwdThreads) alt[i] = J.alt_mask[i];
    int cur_lod = -1;

    for (uint64_t t = blockIdx.x; t < J.n_atoms; t += gridDim.x) {
        int lod;
        uint32_t az, ay, ax;
        const uint64_t ca = J.first + t;   // canonical index
        J.lay.coords(ca, lod, az, ay, ax);
        const int qi = J.qsel ? (int)J.qsel[t] : lod;
        if (qi != cur_lod) {   // uniform across the CTA: quantiser constants of this atom
            __syncthreads();   // every thread is done with the previous constants
            for (int i = tid; i < VCD_NCLASS; i += kFwdThreads) { qdz[i] = J.q[qi].dz[i]; qrr[i] = J.q[qi].rr[i]; }
            cur_lod = qi;
            __syncthreads();
        }
        const bool cached = J.coef && ca < J.coef_n;
        uint32_t *cptr = cached ? J.coef + ca * 32768ull : nullptr;
        uint32_t *dst = J.ent + t * (uint64_t)VCD_MAX_ENTRIES;
        int32_t dc;
        uint32_t total;
        if (cached && !J.coef_store) {
            // the transform of this atom was kept: quantise straight from it
            const uint32_t dcz = J.coef_dc[ca];
            if (dcz & kMetaZero) {
                if (tid == 0) J.meta[t] = kMetaZero;
                continue;
            }
            dc = (int32_t)(dcz & 0xFFu);
            total = quant_compact<kFwdThreads>(
                [&](uint32_t p) { return __ldcs(reinterpret_cast<const uint4 *>(cptr + p)); }, qdz, qrr, L, wcnt, dst);
        } else {
            const uint8_t *vol = J.vol[lod];
            const uint32_t nx = J.dims[lod][0], ny = J.dims[lod][1], nz = J.dims[lod][2];
            // rows r = tid + 256 j: z = r >> 5, y = r & 31 (lane)
            uint32_t w[4][8];
            uint32_t s = 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                int r = tid + kFwdThreads * j;
                load_row(vol, nx, ny, nz, ax * 32, ay * 32 + (r & 31), az * 32 + (r >> 5), w[j]);
#pragma unroll
                for (int i = 0; i < 8; ++i) s = __dp4a(w[j][i], 0x01010101u, s);
            }
#pragma unroll
            for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
            if (lane == 0) red[warp] = s;
            __syncthreads();
            uint32_t sum = 0;
#pragma unroll
            for (int i = 0; i < kFwdThreads / 32; ++i) sum += red[i];
            if (sum == 0) {   // all-zero atom: no payload (src/vc/vc.c:601)
                if (tid == 0) {
                    J.meta[t] = kMetaZero;
                    if (cached) J.coef_dc[ca] = kMetaZero;
                }
                __syncthreads();
                continue;
            }
            dc = (int32_t)((sum + 16384u) / 32768u);
            if (cached && tid == 0) J.coef_dc[ca] = (uint32_t)dc;
            // pass along x for the thread's 4 rows, straight from registers
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                int r = tid + kFwdThreads * j;
                int32_t v[32], o[32];
#pragma unroll
                for (int i = 0; i < 32; ++i) v[i] = (int32_t)((w[j][i >> 2] >> (8 * (i & 3))) & 0xFFu) - dc;
                fdct32_line(v, o);
                int32_t *S = T + (r >> 5) * kSlabPitch + (r & 31) * kRowPitch;
#pragma unroll
                for (int k = 0; k < 32; ++k) S[k] = o[k];
            }
            __syncthreads();
            // pass along y, warp per z-slab, lane per column kx
            for (int z = warp; z < 32; z += kFwdThreads / 32) {
                int32_t *S = T + z * kSlabPitch + lane;
                int32_t v[32], o[32];
#pragma unroll
                for (int y = 0; y < 32; ++y) v[y] = S[y * kRowPitch];
                fdct32_line(v, o);
#pragma unroll
                for (int k = 0; k < 32; ++k) S[k * kRowPitch] = o[k];
            }
            __syncthreads();
            // pass along z per column (ky, kx = lane), coefficients back in place
            for (int ky = warp; ky < 32; ky += kFwdThreads / 32) {
                int32_t *C = T + ky * kRowPitch + lane;
                int32_t v[32], o[32];
#pragma unroll
                for (int z = 0; z < 32; ++z) v[z] = C[z * kSlabPitch];
                fdct32_line(v, o);
#pragma unroll
                for (int kz = 0; kz < 32; ++kz) C[kz * kSlabPitch] = o[kz];
            }
            __syncthreads();
            auto tile = [&](uint32_t p) {
                const uint2 sc = __ldg(reinterpret_cast<const uint2 *>(J.scan + p));
                const uint32_t r0 = sc.x & 0xFFFFu, r1 = sc.x >> 16, r2 = sc.y & 0xFFFFu, r3 = sc.y >> 16;
                const uint4 w = make_uint4(coef_pack(T[tile_idx(r0)], r0, alt), coef_pack(T[tile_idx(r1)], r1, alt),
                                           coef_pack(T[tile_idx(r2)], r2, alt), coef_pack(T[tile_idx(r3)], r3, alt));
                if (cached) *reinterpret_cast<uint4 *>(cptr + p) = w;   // kept in scan order
                return w;
            };
            total = quant_compact<kFwdThreads>(tile, qdz, qrr, L, wcnt, dst);
        }
        if (tid == 0) J.meta[t] = total | ((uint32_t)dc << 16);
    }
}

// LOD0 atoms whose transform was kept: quantise in scan order and compact, with
// a quarter of the shared memory of k_fwd (three CTAs per SM).
constexpr size_t kQuantSmem = 32768 * sizeof(int16_t);

__global__ void __launch_bounds__(kFwdThreads) k_quant_cached(FwdJob J) {
    extern __shared__ int16_t lv[];
    __shared__ float qdz[VCD_NCLASS], qrr[VCD_NCLASS];
    __shared__ uint32_t wcnt[kFwdThreads / 32];
    const int tid = threadIdx.x;
    for (int i = tid; i < VCD_NCLASS; i += kFwdThreads) { qdz[i] = J.q[0].dz[i]; qrr[i] = J.q[0].rr[i]; }
    __syncthreads();
    for (uint64_t t = blockIdx.x; t < J.n_atoms; t += gridDim.x) {
        const uint64_t ca = J.first + t;
        const uint32_t dcz = J.coef_dc[ca];
        if (dcz & kMetaZero) {
            if (tid == 0) J.meta[t] = kMetaZero;
            continue;
        }
        const uint32_t *cptr = J.coef + ca * 32768ull;
        const uint32_t total = quant_compact<kFwdThreads>(
            [&](uint32_t p) { return __ldcs(reinterpret_cast<const uint4 *>(cptr + p)); }, qdz, qrr, lv, wcnt,
            J.ent + t * (uint64_t)VCD_MAX_ENTRIES);
        if (tid == 0) J.meta[t] = total | ((dcz & 0xFFu) << 16);
    }
}

// G atoms per warp (lanes 0..G-1; enc_lanes_for). Every lane takes part in the
// warp-lockstep coder; lanes without a present atom run along inactive.
template <bool WRITE>
__global__ void __launch_bounds__(128) k_rc_encode(RcJob J, uint32_t G) {
    __shared__ uint32_t bstart[9];
    if (threadIdx.x < 9) bstart[threadIdx.x] = J.band_start[threadIdx.x];
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t t = lane < G ? w * G + lane : ~0ull;
    const uint32_t meta = t < J.n_atoms ? J.meta[t] : kMetaZero;
    const bool active = !(meta & kMetaZero);
    if (!WRITE && t < J.n_atoms && !active) J.len[t] = 0;
    const uint32_t nnz = meta & 0xFFFFu;
    const uint32_t *ent = J.ent + (active ? t : 0) * (uint64_t)VCD_MAX_ENTRIES;
    if (!WRITE) {
        uint32_t n = rc_encode_levels_warp<false>(ent, nnz, active, bstart, nullptr);
        if (!active) return;
        J.len[t] = n + 1;
        atomicAdd(J.total_bytes, (unsigned long long)(n + 1));
        atomicAdd(J.total_present, 1ull);
        return;
    }
    uint8_t *dst = nullptr;
    if (active) {
        if (J.slot_bytes) {
            dst = J.arc + t * J.slot_bytes;
        } else if (J.dst_off) {
            dst = J.arc + J.dst_off[t];
        } else {
            const uint64_t a = J.canon_first + t;   // canonical index
            dst = J.arc + J.pos[a] + (J.lay.first_in_region(a) ? kL2Bytes : 0ull);
        }
        dst[0] = (uint8_t)((meta >> 16) & 0xFFu);
    }
    const uint32_t nb = rc_encode_levels_warp<true>(ent, nnz, active, bstart, active ? dst + 1 : nullptr,
                                                    J.slot_bytes ? (uint32_t)(J.slot_bytes - 1) : 0xFFFFFFFFu);
    if (J.len && t < J.n_atoms) J.len[t] = active ? nb + 1 : 0u;
}

// one warp per atom: bytes of its slot to its packed offset
__global__ void k_pack(const uint8_t *slots, uint64_t slot, const uint32_t *len, const uint64_t *off, uint64_t n,
                       uint8_t *dst) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x / 32);
    for (uint64_t t = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < n; t += nw) {
        const uint8_t *s = slots + t * slot;
        uint8_t *d = dst + off[t];
        const uint32_t l = len[t];
        for (uint32_t k = lane; k < l; k += 32) d[k] = s[k];
    }
}

void launch_pack(const uint8_t *slots, uint64_t slot, const uint32_t *len, const uint64_t *off, uint64_t n,
                 uint8_t *dst, cudaStream_t s) {
    if (!n) return;
    const uint64_t blocks = (n + 7) / 8 < 4096 ? (n + 7) / 8 : 4096;
    k_pack<<<(unsigned)blocks, 256, 0, s>>>(slots, slot, len, off, n, dst);
}

// consume[a] = (first atom of its region ? L2 block : 0) + payload length
__global__ void k_consume(PlaceJob J) {
    uint64_t a = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= J.n_total) return;
    J.pos[a] = (J.lay.first_in_region(a) ? kL2Bytes : 0ull) + J.len[a];
}

__global__ void k_slots(PlaceJob J) {
    uint64_t a = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= J.n_total) return;
    int lod;
    uint32_t az, ay, ax;
    J.lay.coords(a, lod, az, ay, ax);
    const uint64_t blk = J.pos[J.lay.region_first(lod, az, ay, ax)];
    uint8_t *slot = J.arc + blk + ((((uint64_t)(az & 31) * 32 + (ay & 31)) * 32 + (ax & 31)) * 16);
    const uint32_t len = J.len[a];
    uint4 v;
    if (len == 0) {   // known-zero atom (src/vc/vc.c:1133-1141)
        v = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 2u);
    } else {
        const uint64_t off = J.pos[a] + (J.lay.first_in_region(a) ? kL2Bytes : 0ull);
        v = make_uint4((uint32_t)off, (uint32_t)(off >> 32), len, 1u | ((J.dc[a] & 0xFFu) << 8));
    }
    // an L2 block starts wherever the cursor was (any byte offset): store bytewise
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int i = 0; i < 16; ++i) slot[i] = (uint8_t)(w[i >> 2] >> (8 * (i & 3)));
}

__global__ void k_gather_dc(const uint32_t *meta, uint64_t n, uint8_t *dc) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) dc[t] = (meta[t] & kMetaZero) ? 0 : (uint8_t)(meta[t] >> 16);
}

void enc_set_smem() {
    smem_attr((const void *)k_fwd, (int)kFwdSmem);
    smem_attr((const void *)k_quant_cached, (int)kQuantSmem);
}

void launch_quant_cached(const FwdJob &J, int num_sms, cudaStream_t s) {
    enc_set_smem();
    if (!J.n_atoms) return;
    const uint64_t cap = (uint64_t)num_sms * 3;
    k_quant_cached<<<(unsigned)(J.n_atoms < cap ? J.n_atoms : cap), kFwdThreads, kQuantSmem, s>>>(J);
}

void launch_fwd(const FwdJob &J, int num_sms, cudaStream_t s) {
    enc_set_smem();
    if (!J.n_atoms) return;
    uint64_t grid = J.n_atoms < (uint64_t)num_sms ? J.n_atoms : (uint64_t)num_sms;
    k_fwd<<<(unsigned)grid, kFwdThreads, kFwdSmem, s>>>(J);
}

// Atoms per warp of the lockstep encoder: the fewest warps per SM
// sub-partition k that keep a warp at 32 atoms or fewer, the atoms spread
// evenly over k warps per sub-partition (as rc_lanes_for, without its
// one-lane decoder); small batches get one atom per warp.
static uint32_t enc_lanes_for(uint64_t n, int num_sms) {
    const uint64_t slots = 4ull * (uint64_t)num_sms;
    const uint64_t k = (n + 32 * slots - 1) / (32 * slots);
    const uint64_t g = (n + k * slots - 1) / (k * slots);
    return g < 1 ? 1u : (uint32_t)g;
}

void launch_rc_encode(const RcJob &J, bool write, int num_sms, cudaStream_t s) {
    if (!J.n_atoms) return;
    const uint32_t G = enc_lanes_for(J.n_atoms, num_sms);
    const uint64_t warps = (J.n_atoms + G - 1) / G;
    const unsigned nb = (unsigned)((warps + 3) / 4);
    if (write) k_rc_encode<true><<<nb, 128, 0, s>>>(J, G);
    else k_rc_encode<false><<<nb, 128, 0, s>>>(J, G);
}

void launch_consume(const PlaceJob &J, cudaStream_t s) {
    k_consume<<<(unsigned)((J.n_total + 255) / 256), 256, 0, s>>>(J);
}

void launch_slots(const PlaceJob &J, cudaStream_t s) {
    k_slots<<<(unsigned)((J.n_total + 255) / 256), 256, 0, s>>>(J);
}

void launch_gather_dc(const uint32_t *meta, uint64_t n, uint8_t *dc, cudaStream_t s) {
    k_gather_dc<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(meta, n, dc);
}

}  // namespace vcg

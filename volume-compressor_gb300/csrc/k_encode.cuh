// Encode kernel interfaces (private).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "vc_internal.h"

namespace vcg {

constexpr uint64_t kL2Bytes = 32768ull * 16ull;   // one region's slot block
constexpr uint32_t kMetaZero = 1u << 31;           // meta: all-zero atom
// meta = nnz (bits 0-15, up to 32768) | dc << 16 | kMetaZero

// Canonical append order: LOD-major, atoms in raster (z, y, x) order.
struct Layout {
    int nlod;
    uint64_t base[9];
    uint32_t acx[8], acy[8], acz[8];

    __host__ __device__ void coords(uint64_t a, int &lod, uint32_t &az, uint32_t &ay, uint32_t &ax) const {
        lod = 0;
        while (lod + 1 < nlod && a >= base[lod + 1]) ++lod;
        uint64_t l = a - base[lod];
        ax = (uint32_t)(l % acx[lod]);
        ay = (uint32_t)((l / acx[lod]) % acy[lod]);
        az = (uint32_t)(l / ((uint64_t)acx[lod] * acy[lod]));
    }
    __host__ __device__ bool first_in_region(uint64_t a) const {
        int lod;
        uint32_t az, ay, ax;
        coords(a, lod, az, ay, ax);
        return ((az | ay | ax) & 31u) == 0;
    }
    __host__ __device__ uint64_t region_first(int lod, uint32_t az, uint32_t ay, uint32_t ax) const {
        return base[lod] + ((uint64_t)(az & ~31u) * acy[lod] + (ay & ~31u)) * acx[lod] + (ax & ~31u);
    }
};

// Forward pass over canonical atoms [first, first + n_atoms) of the pyramid
// (any mix of LODs).
struct FwdJob {
    Layout lay;
    const uint8_t *vol[8];       // LOD volumes (x fastest)
    uint32_t dims[8][3];         // nx, ny, nz per LOD
    uint64_t first;              // canonical index of this launch's first atom
    uint64_t n_atoms;
    const vcd_quant *q;          // per-LOD quantiser constants (device, [lod])
    const uint8_t *qsel;         // optional: per atom (this launch) index into q instead of its LOD
    const uint16_t *scan;        // scan position -> raster index
    const uint32_t *alt_mask;
    uint32_t *ent;               // per atom VCD_MAX_ENTRIES slots: scan position | level << 16
    uint32_t *meta;              // per atom
    // coefficient cache of canonical atoms [0, coef_n): 32768 packed words per
    // atom in scan order (coef_pack: magnitude, quantiser class, sign), and
    // dc | kMetaZero per atom; coef_store != 0 fills it, else atoms below
    // coef_n are quantised from it
    uint32_t *coef;
    uint32_t *coef_dc;
    uint64_t coef_n;
    int coef_store;
};

struct RcJob {
    uint64_t n_atoms;
    const uint32_t *meta;
    const uint32_t *ent;
    uint32_t band_start[9];
    // size pass
    uint32_t *len;                       // payload bytes per atom ([dc] + coder bytes; 0 = zero atom)
    unsigned long long *total_bytes;
    unsigned long long *total_present;
    // write pass
    uint8_t *arc;
    const uint64_t *dst_off;             // optional: per atom (this launch) payload offset in arc
    uint64_t slot_bytes;                 // optional: atom t's payload at arc + t * slot_bytes, at most that long
                                         // (len[t] receives the full length, stored or not)
    const uint64_t *pos;                 // canonical exclusive scan of consumed bytes
    uint64_t canon_first;                // canonical index of this chunk's first atom
    Layout lay;
};

struct PlaceJob {
    uint64_t n_total;
    uint64_t *pos;                       // in: consume; out after scan: cursor before each atom
    const uint32_t *len;
    const uint8_t *dc;
    uint8_t *arc;
    Layout lay;
};

void launch_fwd(const FwdJob &J, int num_sms, cudaStream_t s);
// atoms that are all LOD0 with kept coefficients: quantise and compact only
void launch_quant_cached(const FwdJob &J, int num_sms, cudaStream_t s);
void launch_rc_encode(const RcJob &J, bool write, int num_sms, cudaStream_t s);
void launch_consume(const PlaceJob &J, cudaStream_t s);
void launch_slots(const PlaceJob &J, cudaStream_t s);
void launch_gather_dc(const uint32_t *meta, uint64_t n, uint8_t *dc, cudaStream_t s);
// payloads of n atoms from fixed slots (slot bytes apart) to packed offsets
void launch_pack(const uint8_t *slots, uint64_t slot, const uint32_t *len, const uint64_t *off, uint64_t n,
                 uint8_t *dst, cudaStream_t s);

}  // namespace vcg

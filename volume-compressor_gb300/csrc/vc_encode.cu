// Whole-volume encode on the device: LOD pyramid, rate control, canonical
// placement and archive assembly (the composition vc_encode is defined as in
// include/vc.h). Host work is limited to the bisection decisions, the 128-byte
// header and the L1 hash table (a few entries per LOD).
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "k_ds.cuh"
#include "k_encode.cuh"
#include "kernels.cuh"
#include "vc_device.h"

using namespace vcg;

static const uint64_t kChunk = 32768;   // atoms per forward/coder launch (4 GiB of list scratch)

static inline float f_of(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static inline uint32_t b_of(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

#define CK(call, what)                                 \
    do {                                               \
        cudaError_t e_ = (call);                       \
        if (e_ != cudaSuccess) {                       \
            vcd_set_error(what, e_);                   \
            return vcd_status_of(e_);                  \
        }                                              \
    } while (0)

struct EncState {
    vcd_ctx *c;
    Layout lay;
    const uint8_t *lvol[8];
    uint32_t dims[8][3];
    uint32_t *ent, *meta, *len, *best;
    uint64_t *pos;
    uint8_t *dc, *arc;
    unsigned long long *red;
    vcd_quant *qtab;          // device, per LOD
    vcd_quant qh;             // host staging
    // LOD0 forward transform kept across passes, packed (null when it does not fit)
    uint32_t *coef;
    uint32_t *coef_dc;
    uint64_t coef_n;
    bool coef_valid;
};

// Quantiser constants of `lod` at q, into the device table.
static void set_q(EncState &S, int lod, float q) {
    vch_quant_consts(q, &S.qh);
    cudaMemcpyAsync(S.qtab + lod, &S.qh, sizeof(vcd_quant), cudaMemcpyHostToDevice, S.c->stream);
}

// Forward + coder passes over canonical atoms [a0, a1) (any mix of LODs, each at
// the q in the device table) on stream st with list and metadata scratch ent,
// meta (kChunk atoms): size-only (lengths into len and the totals) or writing
// payloads into the archive. One launch pair per kChunk atoms: a coder launch
// costs about one atom's serial coding time however many atoms it holds.
static int run_range(EncState &S, uint64_t a0, uint64_t a1, bool write, cudaStream_t st, uint32_t *ent,
                     uint32_t *meta) {
    for (uint64_t c0 = a0; c0 < a1; c0 += kChunk) {
        const uint64_t n = a1 - c0 < kChunk ? a1 - c0 : kChunk;
        FwdJob F;
        memset(&F, 0, sizeof F);   // fields this pass does not use stay null
        F.lay = S.lay;
        memcpy(F.vol, S.lvol, sizeof F.vol);
        memcpy(F.dims, S.dims, sizeof F.dims);
        F.first = c0;
        F.n_atoms = n;
        F.q = S.qtab;
        F.scan = g_dev.tables->scan;
        F.alt_mask = g_dev.tables->alt_mask;
        F.ent = ent;
        F.meta = meta;
        F.coef = S.coef;
        F.coef_dc = S.coef_dc;
        F.coef_n = S.coef_n;
        F.coef_store = !S.coef_valid;
        const bool from_cache = S.coef && S.coef_valid && c0 + n <= S.coef_n;
        const bool prof = vcd_prof_on();
        if (prof) cudaEventRecord(S.c->ev[4], st);
        if (from_cache) launch_quant_cached(F, g_dev.num_sms, st);
        else launch_fwd(F, g_dev.num_sms, st);
        RcJob R;
        memset(&R, 0, sizeof R);
        R.n_atoms = n;
        R.meta = meta;
        R.ent = ent;
        memcpy(R.band_start, g_dev.band_start, sizeof R.band_start);
        if (!write) {
            R.len = S.len + c0;
            R.total_bytes = S.red;
            R.total_present = S.red + 1;
        } else {
            R.arc = S.arc;
            R.pos = S.pos;
            R.canon_first = c0;
            R.lay = S.lay;
            launch_gather_dc(meta, n, S.dc + c0, st);
        }
        if (prof) cudaEventRecord(S.c->ev[5], st);
        launch_rc_encode(R, write, g_dev.num_sms, st);
        if (S.coef && c0 < S.coef_n && c0 + n >= S.coef_n) S.coef_valid = true;   // LOD0 transform kept
        if (prof) {
            cudaEventRecord(S.c->ev[1], st);
            cudaEventSynchronize(S.c->ev[1]);
            // forward: volume bytes in (the lists it writes are scratch, not counted)
            if (from_cache)   // coefficients in, lists out (scratch, not counted)
                vcd_prof_add("quant_cached", vcd_elapsed(S.c->ev[4], S.c->ev[5]), 1, n * 131072ull, 0, n);
            else
                vcd_prof_add("fwd_dct_quant", vcd_elapsed(S.c->ev[4], S.c->ev[5]), 1, n * 32768ull, 0, n);
            vcd_prof_add(write ? "rc_encode_write" : "rc_encode_size", vcd_elapsed(S.c->ev[5], S.c->ev[1]), 1, 0,
                         0, n);
        }
    }
    return 0;
}

// The same over [0, total): LOD0 on the context's stream and the coarser LODs
// beside it on the second stream, with their own list scratch. The coarser LODs
// are few atoms but the finest-quantised ones (q down to 0.05): one of them is a
// serial coder chain longer than a whole LOD0 pass, so run after LOD0 it would
// add its length. Serial under per-stage measurement (its events are per stream).
static int run_split(EncState &S, uint64_t na0, uint64_t total, bool write) {
    vcd_ctx *c = S.c;
    cudaStream_t side = (total > na0 && na0 && !vcd_prof_on()) ? vcd_side_stream(c) : NULL;
    void *pe = NULL, *pm = NULL;
    const uint64_t n1 = total - na0 < kChunk ? total - na0 : kChunk;
    if (side && (vcd_scratch(c, VCD_BUF_EENT2, n1 * VCD_MAX_ENTRIES * 4 + 16, &pe) != cudaSuccess ||
                 vcd_scratch(c, VCD_BUF_EMETA2, n1 * 4 + 16, &pm) != cudaSuccess)) {
        cudaGetLastError();
        side = NULL;
    }
    if (!side) return run_range(S, 0, total, write, c->stream, S.ent, S.meta);
    cudaEventRecord(c->chunk_ev[0], c->stream);   // the side stream starts after the work queued so far
    cudaStreamWaitEvent(side, c->chunk_ev[0], 0);
    run_range(S, na0, total, write, side, (uint32_t *)pe, (uint32_t *)pm);
    run_range(S, 0, na0, write, c->stream, S.ent, S.meta);
    cudaEventRecord(c->chunk_ev[1], side);
    cudaStreamWaitEvent(c->stream, c->chunk_ev[1], 0);
    return 0;
}

extern "C" int vcd_encode(const uint8_t *vol, int on_dev, vcd_encode_info *info, uint8_t **out, size_t *out_len) {
    vcd_ctx *c = vcd_thread_ctx();
    if (!c) return 4;
    cudaStream_t st = c->stream;
    EncState S;
    memset(&S, 0, sizeof S);
    S.c = c;
    const int nlod = info->nlod;
    S.lay.nlod = nlod;
    uint64_t nvox[8], pyr_bytes = 0, pyr_vox = 0, total_atoms = 0;
    uint32_t d[3] = {info->nx, info->ny, info->nz};
    for (int l = 0; l < nlod; ++l) {
        if (l) for (int k = 0; k < 3; ++k) d[k] = (d[k] + 1) / 2;
        memcpy(S.dims[l], d, sizeof d);
        nvox[l] = (uint64_t)d[0] * d[1] * d[2];
        if (l) pyr_bytes += (nvox[l] + 255) & ~255ull, pyr_vox += nvox[l];
        S.lay.acx[l] = (d[0] + 31) / 32; S.lay.acy[l] = (d[1] + 31) / 32; S.lay.acz[l] = (d[2] + 31) / 32;
        S.lay.base[l] = total_atoms;
        total_atoms += (uint64_t)S.lay.acx[l] * S.lay.acy[l] * S.lay.acz[l];
    }
    S.lay.base[nlod] = total_atoms;
    for (int l = nlod + 1; l <= 8; ++l) S.lay.base[l] = total_atoms;

    // ---- buffers
    void *p;
    if (on_dev) {
        S.lvol[0] = vol;
    } else {
        CK(vcd_scratch(c, VCD_BUF_VOL, nvox[0], &p), "encode volume");
        CK(vcd_copy_from_host(c, p, vol, nvox[0]), "volume upload");
        S.lvol[0] = (const uint8_t *)p;
    }
    CK(vcd_scratch(c, VCD_BUF_PYR, pyr_bytes + 16, &p), "pyramid");
    cudaEventRecord(c->ev[6], st);   // device work starts (input already on the device)
    const bool prof = vcd_prof_on();
    {
        uint8_t *q = (uint8_t *)p;
        for (int l = 1; l < nlod; ++l) {
            launch_ds2x(S.lvol[l - 1], S.dims[l - 1][0], S.dims[l - 1][1], S.dims[l - 1][2], q, info->ds_method,
                        info->ds_alpha, g_dev.num_sms, st);
            S.lvol[l] = q;
            q += (nvox[l] + 255) & ~255ull;   // 256-byte aligned levels (vector loads)
        }
    }
    if (prof && nlod > 1) {   // pyramid: every coarser voxel reads its (up to) 8 children
        cudaEventRecord(c->ev[5], st);
        cudaEventSynchronize(c->ev[5]);
        vcd_prof_add("downsample", vcd_elapsed(c->ev[6], c->ev[5]), (uint64_t)(nlod - 1), nvox[0] + pyr_vox - nvox[nlod - 1],
                     pyr_vox, pyr_vox);
    }
    const uint64_t chunk = total_atoms < kChunk ? total_atoms : kChunk;
    CK(vcd_scratch(c, VCD_BUF_EENT, chunk * VCD_MAX_ENTRIES * 4 + 16, &p), "coefficient lists");
    S.ent = (uint32_t *)p;
    const uint64_t na0 = S.lay.base[1];
    // quant table (8 LODs) | meta (chunk) | len (all atoms) | best LOD0 len | dc (all atoms)
    size_t q_b = 8 * sizeof(vcd_quant), meta_b = chunk * 4, len_b = total_atoms * 4, best_b = na0 * 4;
    size_t dc_b = total_atoms + 16;
    CK(vcd_scratch(c, VCD_BUF_EMETA, q_b + meta_b + len_b + best_b + dc_b + 64, &p), "encode metadata");
    S.qtab = (vcd_quant *)p;
    S.meta = (uint32_t *)((uint8_t *)p + q_b);
    S.len = S.meta + chunk;
    S.best = S.len + total_atoms;
    S.dc = (uint8_t *)(S.best + na0);
    CK(vcd_scratch(c, VCD_BUF_POS, (total_atoms + 1) * 8, &p), "placement");
    S.pos = (uint64_t *)p;
    CK(vcd_scratch(c, VCD_BUF_RED, 64, &p), "totals");
    S.red = (unsigned long long *)p;
    {   // keep LOD0's forward transform (128 KiB per atom) when it takes at most half the free memory
        size_t fr = 0, tot = 0;
        const size_t cb = (size_t)na0 * 131072 + (size_t)na0 * 4 + 64;
        if (cudaMemGetInfo(&fr, &tot) == cudaSuccess && (c->cap[VCD_BUF_COEF] >= cb || cb <= fr / 2) &&
            vcd_scratch(c, VCD_BUF_COEF, cb, &p) == cudaSuccess) {
            S.coef = (uint32_t *)p;
            S.coef_dc = (uint32_t *)((uint8_t *)p + (size_t)na0 * 131072);
            S.coef_n = na0;
        }
        cudaGetLastError();
    }

    // ---- rate control on LOD0 (bisection over float bit patterns of [0.05, 4096])
    uint32_t lo = b_of(0.05f), hi = b_of(4096.0f);
    float best_q = 1.0f;
    double best_err = INFINITY;
    uint64_t present = 0, best_bytes = 0;
    bool have_best = false;
    for (int it = 0; it < (info->fixed_q ? 0 : 24); ++it) {
        uint32_t mid = lo + (hi - lo) / 2;
        float q = f_of(mid);
        CK(cudaMemsetAsync(S.red, 0, 16, st), "totals reset");
        set_q(S, 0, q);
        run_range(S, 0, na0, false, st, S.ent, S.meta);
        unsigned long long h[2];
        CK(cudaMemcpyAsync(h, S.red, 16, cudaMemcpyDeviceToHost, st), "totals read");
        CK(cudaStreamSynchronize(st), "rate control pass");
        present = h[1];
        if (present == 0) break;
        double ratio = (double)(32768ull * present) / (double)h[0];
        double err = fabs(ratio - (double)info->target_ratio);
        if (err < best_err || (err == best_err && q > best_q)) {
            best_err = err;
            best_q = q;
            best_bytes = h[0];
            have_best = true;
            CK(cudaMemcpyAsync(S.best, S.len, na0 * 4, cudaMemcpyDeviceToDevice, st), "keep sizes");
        }
        if (ratio < (double)info->target_ratio) lo = mid; else hi = mid;
    }
    info->q0 = best_q;
    info->present0 = present;
    info->bytes0 = best_bytes;
    float qs[8];
    if (info->fixed_q) {
        for (int l = 0; l < nlod; ++l) qs[l] = vch_clamp_q(info->q[l]);
        info->q0 = qs[0];
    } else {
        float q = best_q;
        for (int l = 0; l < nlod; ++l) { qs[l] = vch_clamp_q(q < 0.05f ? 0.05f : q); q = q * 0.6f; }
    }

    // ---- sizes of every atom at its LOD's q (LODs 1.. together in one pass)
    for (int l = 0; l < nlod; ++l) set_q(S, l, qs[l]);
    if (have_best) {
        CK(cudaMemcpyAsync(S.len, S.best, na0 * 4, cudaMemcpyDeviceToDevice, st), "restore sizes");
        run_range(S, na0, total_atoms, false, st, S.ent, S.meta);
    } else {
        CK(cudaMemsetAsync(S.red, 0, 16, st), "totals reset");
        run_split(S, na0, total_atoms, false);
    }

    // ---- canonical placement: exclusive scan of consumed bytes
    const uint64_t head = 128 + 16 * info->l1_cap;
    PlaceJob P;
    memset(&P, 0, sizeof P);
    P.n_total = total_atoms;
    P.pos = S.pos;
    P.len = S.len;
    P.dc = S.dc;
    P.lay = S.lay;
    if (prof) cudaEventRecord(c->ev[4], st);
    launch_consume(P, st);
    launch_scan_u64(S.pos, total_atoms, head, S.pos + total_atoms, st);
    if (prof) {   // lengths in, consumed bytes out, scanned in place
        cudaEventRecord(c->ev[5], st);
        cudaEventSynchronize(c->ev[5]);
        vcd_prof_add("encode_place", vcd_elapsed(c->ev[4], c->ev[5]), 2, total_atoms * 12, total_atoms * 16, total_atoms);
    }
    uint64_t *pos_h = (uint64_t *)malloc((total_atoms + 1) * 8);
    if (!pos_h) return 3;
    cudaError_t e = cudaMemcpyAsync(pos_h, S.pos, (total_atoms + 1) * 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { free(pos_h); vcd_set_error("placement", e); return vcd_status_of(e); }
    const uint64_t total = pos_h[total_atoms];

    // ---- archive: zeroed, payloads + slots on the device, head on the host
    e = vcd_scratch(c, VCD_BUF_ARC, total + 16, &p);
    if (e != cudaSuccess) { free(pos_h); vcd_set_error("archive buffer", e); return vcd_status_of(e); }
    S.arc = (uint8_t *)p;
    P.arc = S.arc;
    cudaMemsetAsync(S.arc, 0, total, st);
    run_split(S, na0, total_atoms, true);
    if (prof) cudaEventRecord(c->ev[4], st);
    launch_slots(P, st);
    if (prof) {   // one 16-byte slot per atom
        cudaEventRecord(c->ev[5], st);
        cudaEventSynchronize(c->ev[5]);
        vcd_prof_add("encode_slots", vcd_elapsed(c->ev[4], c->ev[5]), 1, total_atoms * 21, total_atoms * 16, total_atoms);
    }
    cudaEventRecord(c->ev[7], st);   // device work ends (the archive head and copy-out follow)

    uint8_t *hd = (uint8_t *)calloc(head, 1);
    if (!hd) { free(pos_h); return 3; }
    uint32_t w32[9] = {0x00314356u, 1u, 32u, 1u, 32u, (uint32_t)nlod, info->nx, info->ny, info->nz};
    memcpy(hd, w32, sizeof w32);
    memcpy(hd + 36, &info->target_ratio, 4);
    uint64_t regions = 0;
    const uint64_t mask = info->l1_cap - 1;
    for (int l = 0; l < nlod; ++l) {   // regions in creation order (raster of regions)
        uint32_t nrx = (S.lay.acx[l] + 31) / 32, nry = (S.lay.acy[l] + 31) / 32, nrz = (S.lay.acz[l] + 31) / 32;
        for (uint32_t rz = 0; rz < nrz; ++rz)
            for (uint32_t ry = 0; ry < nry; ++ry)
                for (uint32_t rx = 0; rx < nrx; ++rx) {
                    uint64_t key = vch_region_key(l, rz, ry, rx);
                    uint64_t blk = pos_h[S.lay.region_first(l, rz * 32, ry * 32, rx * 32)];
                    uint64_t i = vch_mix64(key) & mask;
                    while (1) {
                        uint64_t bref;
                        memcpy(&bref, hd + 128 + i * 16 + 8, 8);
                        if (!bref) break;
                        i = (i + 1) & mask;
                    }
                    memcpy(hd + 128 + i * 16, &key, 8);
                    memcpy(hd + 128 + i * 16 + 8, &blk, 8);
                    ++regions;
                }
    }
    uint64_t h64[4] = {info->l1_cap, regions, 128, total};
    memcpy(hd + 40, h64, sizeof h64);
    for (int l = 0; l < nlod; ++l) memcpy(hd + 72 + 4 * l, &qs[l], 4);
    free(pos_h);
    e = cudaMemcpyAsync(S.arc, hd, head, cudaMemcpyHostToDevice, st);
    uint8_t *res = (uint8_t *)malloc(total);
    if (!res) { cudaStreamSynchronize(st); free(hd); return 3; }
    if (e == cudaSuccess) e = vcd_copy_to_host(c, res, S.arc, total);   // after the head on the same stream
    if (e == cudaSuccess) e = cudaGetLastError();
    free(hd);
    if (e != cudaSuccess) { free(res); vcd_set_error("archive assembly", e); return vcd_status_of(e); }
    c->last_ms = vcd_elapsed(c->ev[6], c->ev[7]);
    {   // a large transform cache is not kept between encodes (more than 1/8 of the device memory)
        size_t fr = 0, tot = 0;
        if (c->buf[VCD_BUF_COEF] && cudaMemGetInfo(&fr, &tot) == cudaSuccess && c->cap[VCD_BUF_COEF] > tot / 8) {
            cudaFree(c->buf[VCD_BUF_COEF]);
            c->buf[VCD_BUF_COEF] = NULL;
            c->cap[VCD_BUF_COEF] = 0;
        }
        cudaGetLastError();
    }
    *out = res;
    *out_len = total;
    return 0;
}

// ---------------------------------------------------------------- writer batches
// Independent atoms (box rasters or stacked single atoms) through the same
// forward and coder kernels as the whole-volume encoder, with one coder pass:
// per chunk of at most kWChunk atoms a forward pass and a writing coder pass
// into fixed slots of kSlot bytes (the reference encoder's largest atom:
// 1 + 4 * 32768 + 64 bytes, rounded up), the lengths back to the host for the
// packing offsets, and a packing kernel whose output is copied into the
// thread's pinned buffer. An atom longer than its slot (where the reference's
// encoder stops with "range encoder overflow") makes its chunk take a second,
// exact writing pass.
static const uint64_t kWChunk = 8192;
static const uint64_t kSlot = 131200;

extern "C" int vcd_encode_segments(const vcd_seg *segs, int nseg, const float *qs, int nq, uint8_t **pay,
                                   uint64_t *pay_bytes) {
    vcd_ctx *c = vcd_thread_ctx();
    if (!c) return 4;
    if (nq < 1 || nq > 256) return 2;
    cudaStream_t st = c->stream;
    void *p;
    const size_t q_b = ((size_t)nq * sizeof(vcd_quant) + 255) & ~(size_t)255;
    CK(vcd_scratch(c, VCD_BUF_EMETA, q_b + kWChunk * (4 + 4 + 8 + 1) + 256, &p), "writer metadata");
    vcd_quant *qtab = (vcd_quant *)p;
    uint32_t *dmeta = (uint32_t *)((uint8_t *)p + q_b);
    uint32_t *dlen = dmeta + kWChunk;
    uint64_t *doff = (uint64_t *)(dlen + kWChunk);
    uint8_t *dqsel = (uint8_t *)(doff + kWChunk);
    vcd_quant *qh = (vcd_quant *)malloc((size_t)nq * sizeof(vcd_quant));
    uint64_t *offh = (uint64_t *)malloc(kWChunk * sizeof(uint64_t));
    if (!qh || !offh) { free(qh); free(offh); return 3; }
    for (int i = 0; i < nq; ++i) vch_quant_consts(qs[i], &qh[i]);
    cudaError_t e = cudaEventRecord(c->ev[6], st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(qtab, qh, (size_t)nq * sizeof(vcd_quant), cudaMemcpyHostToDevice, st);
    uint64_t total = 0;
    for (int sg = 0; sg < nseg && e == cudaSuccess; ++sg) {
        const vcd_seg &S = segs[sg];
        const uint64_t acx = S.nx / 32, acy = S.ny / 32, acz = S.nz / 32, na = acx * acy * acz;
        if (!na) continue;
        if ((e = vcd_scratch(c, VCD_BUF_VOL, (size_t)S.nx * S.ny * S.nz + 16, &p)) != cudaSuccess) break;
        const uint8_t *dvol = (const uint8_t *)p;
        if ((e = vcd_copy_from_host(c, p, S.vox, (size_t)S.nx * S.ny * S.nz)) != cudaSuccess) break;
        Layout lay;
        memset(&lay, 0, sizeof lay);
        lay.nlod = 1;
        for (int l = 1; l <= 8; ++l) lay.base[l] = na;
        lay.acx[0] = (uint32_t)acx; lay.acy[0] = (uint32_t)acy; lay.acz[0] = (uint32_t)acz;
        for (uint64_t c0 = 0; c0 < na && e == cudaSuccess; c0 += kWChunk) {
            const uint64_t n = na - c0 < kWChunk ? na - c0 : kWChunk;
            if ((e = vcd_scratch(c, VCD_BUF_EENT, n * VCD_MAX_ENTRIES * 4 + 16, &p)) != cudaSuccess) break;
            uint32_t *ent = (uint32_t *)p;
            if ((e = cudaMemcpyAsync(dqsel, S.qsel + c0, n, cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
            FwdJob F;
            memset(&F, 0, sizeof F);
            F.lay = lay;
            F.vol[0] = dvol;
            F.dims[0][0] = S.nx; F.dims[0][1] = S.ny; F.dims[0][2] = S.nz;
            F.first = c0;
            F.n_atoms = n;
            F.q = qtab;
            F.qsel = dqsel;
            F.scan = g_dev.tables->scan;
            F.alt_mask = g_dev.tables->alt_mask;
            F.ent = ent;
            F.meta = dmeta;
            launch_fwd(F, g_dev.num_sms, st);
            if ((e = vcd_scratch(c, VCD_BUF_ARC, n * kSlot + 16, &p)) != cudaSuccess) break;
            uint8_t *dslots = (uint8_t *)p;
            RcJob W;
            memset(&W, 0, sizeof W);
            W.n_atoms = n;
            W.meta = dmeta;
            W.ent = ent;
            memcpy(W.band_start, g_dev.band_start, sizeof W.band_start);
            W.arc = dslots;
            W.slot_bytes = kSlot;
            W.len = dlen;
            launch_rc_encode(W, true, g_dev.num_sms, st);
            if ((e = cudaMemcpyAsync(S.len + c0, dlen, n * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                (e = cudaStreamSynchronize(st)) != cudaSuccess)
                break;
            uint64_t bytes = 0;
            bool over = false;
            for (uint64_t i = 0; i < n; ++i) {
                offh[i] = bytes;
                S.off[c0 + i] = total + bytes;
                bytes += S.len[c0 + i];
                over |= S.len[c0 + i] > kSlot;
            }
            if ((e = vcd_scratch(c, VCD_BUF_WPACK, bytes + 16, &p)) != cudaSuccess) break;
            uint8_t *dpack = (uint8_t *)p;
            if ((e = cudaMemcpyAsync(doff, offh, n * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
            if (!over) {
                launch_pack(dslots, kSlot, dlen, doff, n, dpack, st);
            } else {   // exact second pass for a chunk with an atom longer than its slot
                W.slot_bytes = 0;
                W.len = nullptr;
                W.arc = dpack;
                W.dst_off = doff;
                launch_rc_encode(W, true, g_dev.num_sms, st);
            }
            if (total + bytes > c->wpin_cap) {   // grow the pinned output, keeping what it holds
                if ((e = cudaStreamSynchronize(st)) != cudaSuccess) break;
                size_t want = (total + bytes) + (total + bytes) / 2 + (1 << 20);
                uint8_t *np_ = NULL;
                if ((e = vcd_malloc_host((void **)&np_, want)) != cudaSuccess) break;
                if (c->wpin) {
                    memcpy(np_, c->wpin, total);
                    cudaFreeHost(c->wpin);
                }
                c->wpin = np_;
                c->wpin_cap = want;
            }
            if (bytes && (e = cudaMemcpyAsync(c->wpin + total, dpack, bytes, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
                break;
            // offh and the staging are reused by the next chunk
            if ((e = cudaStreamSynchronize(st)) != cudaSuccess) break;
            total += bytes;
        }
    }
    if (e == cudaSuccess) e = cudaEventRecord(c->ev[7], st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    free(qh);
    free(offh);
    if (e != cudaSuccess) {
        vcd_set_error("writer batch", e);
        return vcd_status_of(e);
    }
    c->last_ms = vcd_elapsed(c->ev[6], c->ev[7]);
    *pay = c->wpin;
    *pay_bytes = total;
    return 0;
}

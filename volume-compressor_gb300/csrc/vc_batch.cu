// Batched region decode orchestration: upload the batch description (distinct
// atoms, their destination lists, the request boxes, list offsets) into
// grow-only device buffers, then replay one CUDA graph of the persistent
// range-decode + transform launches. The launch shape (range-decoder policy:
// warps per SM sub-partition that decode one atom each before atoms share warps
// in lockstep; transform on the CUDA cores with 8 or 16 warps per atom, or on
// the int8 tensor cores) is picked once per process by timing every candidate on
// the first batch (all candidates produce identical bytes); threads that start
// later take the tuned shape.
#include <cuda_runtime.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "kernels.cuh"
#include "vc_device.h"

using namespace vcg;

#define VC_API extern "C" __attribute__((visibility("default")))

static const BatchShape kShapes[] = {{1, 256, 0}, {4, 256, 0}, {16, 256, 0}, {1, 512, 0}, {4, 512, 0},
                                     {16, 512, 0}, {1, 256, 1}, {4, 256, 1}, {16, 256, 1}};

#define CKB(call, what)                                \
    do {                                               \
        cudaError_t e_ = (call);                       \
        if (e_ != cudaSuccess) {                       \
            vcd_set_error(what, e_);                   \
            return vcd_status_of(e_);                  \
        }                                              \
    } while (0)

static size_t cap_of(const vcd_ctx *c, int slot) { return c->cap[slot]; }

// tuned shape shared by all threads: rc policy << 20 | imma << 16 | transform threads (0 = not yet)
static int g_tuned_shape = 0;
// shape set by vcg_set_batch_shape, same packing (0 = autotune)
static int g_forced_shape = 0;

// Staged outputs (request i at its 16-byte-aligned offset in src) to the callers'
// buffers. From 16 MiB on, kCopyThreads threads each copy the parts of the
// requests inside one contiguous stripe of src.
namespace {
constexpr int kCopyThreads = 12;
constexpr uint64_t kCopyParallelMin = 16ull << 20;

struct CopyJob {
    const vcd_batch *b;
    uint8_t *const *out;
    const uint8_t *src;
    uint64_t lo, hi;   // stripe of src
};

static void *copy_stripe(void *p) {
    const CopyJob &j = *(const CopyJob *)p;
    uint64_t o = 0;
    for (uint32_t i = 0; i < j.b->n_req && o < j.hi; ++i) {
        const vcd_boxreq &r = j.b->reqs[i];
        const uint64_t n = (uint64_t)(r.x1 - r.x0) * (r.y1 - r.y0) * (r.z1 - r.z0);
        const uint64_t a = o > j.lo ? o : j.lo, e = o + n < j.hi ? o + n : j.hi;
        if (j.out[i] && a < e) memcpy(j.out[i] + (a - o), j.src + a, e - a);
        o += (n + 15) & ~15ull;
    }
    return NULL;
}
}  // namespace

static void copy_to_requests(const vcd_batch *b, uint8_t *const *out, const uint8_t *src, uint64_t total) {
    CopyJob jobs[kCopyThreads];
    pthread_t th[kCopyThreads];
    const int nt = total >= kCopyParallelMin ? kCopyThreads : 1;
    const uint64_t per = (total + nt - 1) / nt;
    int started = 0;
    for (int t = 0; t < nt; ++t) {
        jobs[t] = {b, out, src, (uint64_t)t * per, (uint64_t)(t + 1) * per < total ? (uint64_t)(t + 1) * per : total};
        if (t == 0 || pthread_create(&th[t], NULL, copy_stripe, &jobs[t]) != 0) {
            if (t) copy_stripe(&jobs[t]);   // no thread: this one copies the stripe itself
        } else {
            started |= 1 << t;
        }
    }
    copy_stripe(&jobs[0]);
    for (int t = 1; t < nt; ++t)
        if (started & (1 << t)) pthread_join(th[t], NULL);
}

extern "C" int vcd_decode_batch(vcd_archive *d, const vcd_batch *b, uint8_t *const *host_out, uint32_t *req_err) {
    vcd_ctx *c = vcd_thread_ctx();
    if (!c) return 4;
    cudaStream_t st = c->stream;
    if (b->n_req == 0) return 0;
    void *p_ua, *p_dst, *p_req, *p_off, *p_cnt, *p_ent, *p_ctl, *p_out = NULL;
    CKB(vcd_scratch(c, VCD_BUF_BUA, (size_t)b->n_ua * sizeof(vcd_uatom) + 64, &p_ua), "batch atoms");
    CKB(vcd_scratch(c, VCD_BUF_BDST, (size_t)b->n_dst * 4 + 64, &p_dst), "batch destinations");
    CKB(vcd_scratch(c, VCD_BUF_BREQ, (size_t)b->n_req * sizeof(vcd_boxreq) + 64, &p_req), "batch requests");
    CKB(vcd_scratch(c, VCD_BUF_BOFF, (size_t)b->n_ua * 8 + 64, &p_off), "batch list offsets");
    CKB(vcd_scratch(c, VCD_BUF_BCNT, (size_t)b->n_ua * 4 + 64, &p_cnt), "batch counts");
    CKB(vcd_scratch(c, VCD_BUF_BENT, b->cap_total * 4 + 64, &p_ent), "batch lists");
    CKB(vcd_scratch(c, VCD_BUF_BCTL, 16 + (size_t)b->n_req * 4 + 64, &p_ctl), "batch control");
    uint64_t out_total = 0;
    if (host_out) {   // outputs staged in one device arena
        for (uint32_t i = 0; i < b->n_req; ++i) {
            const vcd_boxreq &r = b->reqs[i];
            out_total += ((uint64_t)(r.x1 - r.x0) * (r.y1 - r.y0) * (r.z1 - r.z0) + 15) & ~15ull;
        }
        CKB(vcd_scratch(c, VCD_BUF_BOUT, out_total + 16, &p_out), "batch outputs");
        uint64_t o = 0;
        for (uint32_t i = 0; i < b->n_req; ++i) {
            vcd_boxreq &r = b->reqs[i];
            r.out = (uint8_t *)p_out + o;
            o += ((uint64_t)(r.x1 - r.x0) * (r.y1 - r.y0) * (r.z1 - r.z0) + 15) & ~15ull;
        }
    }
    uint32_t *ctl = (uint32_t *)p_ctl;   // [0] distinct atoms, [1] work counter, [4..] per-request errors
    CKB(cudaMemcpyAsync(p_ua, b->ua, (size_t)b->n_ua * sizeof(vcd_uatom), cudaMemcpyHostToDevice, st), "upload");
    CKB(cudaMemcpyAsync(p_dst, b->dst, (size_t)b->n_dst * 4, cudaMemcpyHostToDevice, st), "upload");
    CKB(cudaMemcpyAsync(p_req, b->reqs, (size_t)b->n_req * sizeof(vcd_boxreq), cudaMemcpyHostToDevice, st), "upload");
    CKB(cudaMemcpyAsync(p_off, b->ent_off, (size_t)b->n_ua * 8, cudaMemcpyHostToDevice, st), "upload");
    CKB(cudaMemsetAsync(p_ctl, 0, 16 + (size_t)b->n_req * 4, st), "reset");
    CKB(cudaMemcpyAsync(ctl, &b->n_ua, 4, cudaMemcpyHostToDevice, st), "upload");

    BatchJob J;
    memset(&J, 0, sizeof J);
    J.arc = d->arc;
    J.atoms = d->atoms;
    J.ua = (const UAtom *)p_ua;
    J.dst = (const uint32_t *)p_dst;
    J.reqs = (const BoxReq *)p_req;
    J.n_ua = ctl;
    J.ent = (uint32_t *)p_ent;
    J.ent_off = (const uint64_t *)p_off;
    J.cnt = (uint32_t *)p_cnt;
    J.dq = d->dq;
    J.alt_mask = g_dev.tables->alt_mask;
    J.scan = g_dev.tables->scan;
    J.work = ctl + 1;
    J.req_err = ctl + 4;
    memcpy(J.band_start, g_dev.band_start, sizeof J.band_start);
    // capacity in distinct atoms the range-decode grid must cover (the buffer's)
    const uint32_t max_ua = (uint32_t)((cap_of(c, VCD_BUF_BUA) - 64) / sizeof(vcd_uatom));
    void *p_ord;
    CKB(vcd_scratch(c, VCD_BUF_BORD, ((size_t)max_ua + sort_ctl_words()) * 4 + 64, &p_ord), "batch order");
    J.sort_ctl = (uint32_t *)p_ord;
    J.order = J.sort_ctl + sort_ctl_words();

    const int forced = __atomic_load_n(&g_forced_shape, __ATOMIC_ACQUIRE);
    if (forced) {
        c->batch_rc_scalar_warps = forced >> 20;
        c->batch_imma = (forced >> 16) & 1;
        c->batch_tx_threads = forced & 0xFFFF;
        c->batch_forced = 1;
    } else if (c->batch_forced) {   // back to the tuned shape
        c->batch_rc_scalar_warps = 0;
        c->batch_forced = 0;
    }
    if (!c->batch_rc_scalar_warps) {
        const int t = __atomic_load_n(&g_tuned_shape, __ATOMIC_ACQUIRE);
        if (t) {
            c->batch_rc_scalar_warps = t >> 20;
            c->batch_imma = (t >> 16) & 1;
            c->batch_tx_threads = t & 0xFFFF;
        }
    }
    if (!c->batch_rc_scalar_warps) {   // autotune on the process's first batch
        float best = 1e30f;
        for (const BatchShape &s : kShapes) {
            CKB(cudaMemsetAsync(ctl + 1, 0, 4, st), "reset");
            cudaEventRecord(c->ev[0], st);
            launch_batch(J, s, g_dev.num_sms, max_ua, st);
            cudaEventRecord(c->ev[1], st);
            CKB(cudaEventSynchronize(c->ev[1]), "autotune");
            CKB(cudaGetLastError(), "autotune");
            float ms = vcd_elapsed(c->ev[0], c->ev[1]);
            if (ms < best) {
                best = ms;
                c->batch_rc_scalar_warps = s.rc_scalar_warps;
                c->batch_tx_threads = s.idct_threads;
                c->batch_imma = s.imma;
            }
        }
        CKB(cudaMemsetAsync(ctl + 1, 0, 4, st), "reset");
        CKB(cudaMemsetAsync(ctl + 4, 0, (size_t)b->n_req * 4, st), "reset");
        __atomic_store_n(&g_tuned_shape, c->batch_rc_scalar_warps << 20 | c->batch_imma << 16 | c->batch_tx_threads,
                         __ATOMIC_RELEASE);
    }
    const BatchShape shape = {c->batch_rc_scalar_warps, c->batch_tx_threads, c->batch_imma};
    // the graph bakes in every kernel parameter (buffers, archive tables) and the
    // grid size: replay it only when all of them are unchanged
    unsigned char key[512];
    static_assert(sizeof(BatchJob) + sizeof(BatchShape) + sizeof(uint32_t) <= sizeof key, "graph key too small");
    memset(key, 0, sizeof key);
    memcpy(key, &J, sizeof J);
    memcpy(key + sizeof J, &shape, sizeof shape);
    memcpy(key + sizeof J + sizeof shape, &max_ua, sizeof max_ua);
    if (!c->batch_graph || memcmp(key, c->batch_key, sizeof key) != 0) {
        if (c->batch_graph) cudaGraphExecDestroy(c->batch_graph);
        c->batch_graph = NULL;
        cudaGraph_t g;
        CKB(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "graph capture");
        launch_batch(J, shape, g_dev.num_sms, max_ua, st);
        CKB(cudaStreamEndCapture(st, &g), "graph capture");
        cudaError_t e = cudaGraphInstantiate(&c->batch_graph, g, 0);
        cudaGraphDestroy(g);
        CKB(e, "graph instantiate");
        memcpy(c->batch_key, key, sizeof key);
    }
    // with per-stage measurement on, the same two kernels run without the graph
    // and an event between them splits the time
    const bool prof = vcd_prof_on();
    cudaEventRecord(c->ev[2], st);
    if (prof) {
        launch_batch(J, shape, g_dev.num_sms, max_ua, st, c->ev[5]);
        CKB(cudaGetLastError(), "batch launch");
    } else {
        CKB(cudaGraphLaunch(c->batch_graph, st), "graph launch");
    }
    cudaEventRecord(c->ev[3], st);
    CKB(cudaMemcpyAsync(req_err, ctl + 4, (size_t)b->n_req * 4, cudaMemcpyDeviceToHost, st), "errors");
    CKB(cudaStreamSynchronize(st), "batch decode");
    CKB(cudaGetLastError(), "batch decode");
    c->last_ms = vcd_elapsed(c->ev[2], c->ev[3]);
    if (prof) {
        uint64_t out_bytes = 0;
        for (uint32_t i = 0; i < b->n_req; ++i) {
            const vcd_boxreq &r = b->reqs[i];
            out_bytes += (uint64_t)(r.x1 - r.x0) * (r.y1 - r.y0) * (r.z1 - r.z0);
        }
        vcd_prof_add("batch_decode", c->last_ms, 2, 0, out_bytes, b->n_ua);
        vcd_prof_add("batch_rc_decode", vcd_elapsed(c->ev[2], c->ev[5]), 1, 0, 0, b->n_ua);
        vcd_prof_add("batch_transform", vcd_elapsed(c->ev[5], c->ev[3]), 1, 0, out_bytes, b->n_ua);
    }
    if (host_out) {
        void *pin;
        CKB(vcd_pinned(c, out_total + 16, &pin), "batch staging");
        CKB(cudaMemcpyAsync(pin, p_out, out_total, cudaMemcpyDeviceToHost, st), "batch copy-out");
        CKB(cudaStreamSynchronize(st), "batch copy-out");
        copy_to_requests(b, host_out, (const uint8_t *)pin, out_total);
    }
    return 0;
}

// Fix the launch shape of every later batch (rc_scalar_warps 1, 4 or 16;
// transform_threads 256 or 512 for the butterfly, 256 for the tensor cores);
// rc_scalar_warps = 0 returns to the autotuned shape. Results do not depend on it.
VC_API int vcg_set_batch_shape(int rc_scalar_warps, int transform_threads, int transform_imma) {
    if (rc_scalar_warps == 0) {
        __atomic_store_n(&g_forced_shape, 0, __ATOMIC_RELEASE);
        return 0;
    }
    for (const BatchShape &s : kShapes) {
        if (s.rc_scalar_warps == rc_scalar_warps && s.idct_threads == transform_threads &&
            s.imma == (transform_imma ? 1 : 0)) {
            __atomic_store_n(&g_forced_shape, rc_scalar_warps << 20 | s.imma << 16 | transform_threads,
                             __ATOMIC_RELEASE);
            return 0;
        }
    }
    return 2;   // VC_ERR_RANGE
}

// Launch shape the calling thread uses (0 before its first batch).
VC_API void vcg_batch_shape(int *rc_scalar_warps, int *transform_threads, int *transform_imma) {
    vcd_ctx *c = vcd_thread_ctx();
    if (rc_scalar_warps) *rc_scalar_warps = c ? c->batch_rc_scalar_warps : 0;
    if (transform_threads) *transform_threads = c ? c->batch_tx_threads : 0;
    if (transform_imma) *transform_imma = c ? c->batch_imma : 0;
}

// Device runtime: one CUDA context per process, one stream + grow-only scratch
// per host thread, archive residency, and the decode orchestration.
#include <cuda_runtime.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "kernels.cuh"
#include "vc_device.h"

using namespace vcg;

// ---------------------------------------------------------------- errors
static __thread char g_err[256];
extern "C" const char *vcd_last_error(void) { return g_err; }
void vcd_set_error(const char *what, cudaError_t e) {
    snprintf(g_err, sizeof g_err, "%s: %s", what, e == cudaSuccess ? "failed" : cudaGetErrorString(e));
}
int vcd_status_of(cudaError_t e) { return e == cudaErrorMemoryAllocation ? 3 /*VC_ERR_OOM*/ : 4 /*VC_ERR_IO*/; }

// ---------------------------------------------------------------- process context
static pthread_once_t g_once = PTHREAD_ONCE_INIT;
static int g_init_rc = -1;
vcd_device g_dev;

static void init_once(void) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n <= 0) { vcd_set_error("cudaGetDeviceCount", e); return; }
    int dev = 0;
    const char *env = getenv("VC_DEVICE");
    if (env) dev = atoi(env);
    if ((e = cudaSetDevice(dev)) != cudaSuccess) { vcd_set_error("cudaSetDevice", e); return; }
    cudaDeviceProp prop;
    if ((e = cudaGetDeviceProperties(&prop, dev)) != cudaSuccess) { vcd_set_error("cudaGetDeviceProperties", e); return; }
    if (prop.major < 10) {
        snprintf(g_err, sizeof g_err, "device %d (sm_%d%d) cannot run sm_103a code", dev, prop.major, prop.minor);
        return;
    }
    g_dev.device = dev;
    g_dev.num_sms = prop.multiProcessorCount;
    vcd_tables *t = (vcd_tables *)malloc(sizeof(vcd_tables));
    vch_tables(t);
    memcpy(g_dev.band_start, t->band_start, sizeof g_dev.band_start);
    if ((e = cudaMalloc(&g_dev.tables, sizeof(vcd_tables))) != cudaSuccess ||   // process set-up: not injected
        (e = cudaMemcpy(g_dev.tables, t, sizeof(vcd_tables), cudaMemcpyHostToDevice)) != cudaSuccess) {
        vcd_set_error("table upload", e);
        free(t);
        return;
    }
    free(t);
    __atomic_store_n(&g_init_rc, 0, __ATOMIC_RELEASE);
}

static void make_current(void) {
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cur != g_dev.device) cudaSetDevice(g_dev.device);
}

extern "C" int vcd_init(void) {
    pthread_once(&g_once, init_once);
    if (g_init_rc == 0) make_current();
    return g_init_rc;
}

extern "C" int vcd_enter(void) {
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    if (__atomic_load_n(&g_init_rc, __ATOMIC_ACQUIRE) == 0 && prev != g_dev.device) cudaSetDevice(g_dev.device);
    return prev;
}

extern "C" void vcd_leave(int *prev) {
    int cur = -1;
    if (*prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != *prev) cudaSetDevice(*prev);
}

// ---------------------------------------------------------------- per-thread context
static pthread_key_t g_ctx_key;
static pthread_once_t g_key_once = PTHREAD_ONCE_INIT;

static void ctx_free(void *p) {
    vcd_ctx *c = (vcd_ctx *)p;
    if (!c) return;
    for (int i = 0; i < VCD_NBUF; ++i)
        if (c->buf[i]) cudaFree(c->buf[i]);
    if (c->pinned) cudaFreeHost(c->pinned);
    if (c->stage_host) cudaFreeHost(c->stage_host);
    if (c->wpin) cudaFreeHost(c->wpin);
    if (c->batch_graph) cudaGraphExecDestroy(c->batch_graph);
    if (c->copy_stream) {
        for (int i = 0; i < VCD_SLABS; ++i) cudaEventDestroy(c->chunk_ev[i]);
        for (int i = 0; i < 4; ++i) cudaEventDestroy(c->ring_ev[i]);
        cudaStreamDestroy(c->copy_stream);
    }
    if (c->stream) cudaStreamDestroy(c->stream);
    free(c);
}
static void key_once(void) { pthread_key_create(&g_ctx_key, ctx_free); }

vcd_ctx *vcd_thread_ctx(void) {
    pthread_once(&g_key_once, key_once);
    vcd_ctx *c = (vcd_ctx *)pthread_getspecific(g_ctx_key);
    if (c) return c;
    c = (vcd_ctx *)calloc(1, sizeof(vcd_ctx));
    cudaSetDevice(g_dev.device);
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { vcd_set_error("cudaStreamCreate", e); free(c); return NULL; }
    for (int i = 0; i < 8; ++i) cudaEventCreate(&c->ev[i]);
    pthread_setspecific(g_ctx_key, c);
    return c;
}

// ---------------------------------------------------------------- profiling
struct vcd_stat {
    char name[32];
    double ms;
    uint64_t launches, bytes_read, bytes_written, units;
};
static vcd_stat g_stats[32];
static int g_nstats, g_prof;
static pthread_mutex_t g_stat_mu = PTHREAD_MUTEX_INITIALIZER;

int vcd_prof_on(void) { return g_prof; }

float vcd_elapsed(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
        cudaGetLastError();   // a timing that cannot be read is not an error of the next call
        ms = 0.f;
    }
    return ms;
}

void vcd_prof_add(const char *name, double ms, uint64_t launches, uint64_t br, uint64_t bw, uint64_t units) {
    pthread_mutex_lock(&g_stat_mu);
    int i = 0;
    while (i < g_nstats && strcmp(g_stats[i].name, name)) ++i;
    if (i == g_nstats && g_nstats < 32) {
        memset(&g_stats[i], 0, sizeof g_stats[i]);
        snprintf(g_stats[i].name, sizeof g_stats[i].name, "%s", name);
        ++g_nstats;
    }
    if (i < 32) {
        g_stats[i].ms += ms;
        g_stats[i].launches += launches;
        g_stats[i].bytes_read += br;
        g_stats[i].bytes_written += bw;
        g_stats[i].units += units;
    }
    pthread_mutex_unlock(&g_stat_mu);
}

extern "C" __attribute__((visibility("default"))) void vcg_profile_enable(int on) { g_prof = on; }

// Copies up to max accumulated kernel statistics into out (layout of
// vcg_kernel_stat in vcg.h); returns how many exist; reset clears them.
extern "C" __attribute__((visibility("default"))) int vcg_profile_read(void *out, int max, int reset) {
    pthread_mutex_lock(&g_stat_mu);
    int n = g_nstats;
    if (out) memcpy(out, g_stats, sizeof(vcd_stat) * (size_t)(n < max ? n : max));
    if (reset) g_nstats = 0;
    pthread_mutex_unlock(&g_stat_mu);
    return n;
}

extern "C" __attribute__((visibility("default"))) double vcg_last_call_ms(void) {
    vcd_ctx *c = vcd_thread_ctx();
    return c ? c->last_ms : -1.0;
}

// Dynamic shared-memory limits already raised, per kernel: bit d of devs is
// device d (devices from 64 up are set on every call).
namespace {
struct SmemAttr {
    const void *fn;
    int bytes;
    uint64_t devs;
};
SmemAttr g_smem_attr[32];
int g_n_smem_attr;
pthread_mutex_t g_smem_mu = PTHREAD_MUTEX_INITIALIZER;
}  // namespace

cudaError_t vcg::smem_attr(const void *fn, int bytes) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint64_t bit = dev < 64 ? 1ull << dev : 0;
    pthread_mutex_lock(&g_smem_mu);
    int i = 0;
    while (i < g_n_smem_attr && (g_smem_attr[i].fn != fn || g_smem_attr[i].bytes != bytes)) ++i;
    if (i < g_n_smem_attr && bit && (g_smem_attr[i].devs & bit)) {
        pthread_mutex_unlock(&g_smem_mu);
        return cudaSuccess;
    }
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess && bit) {
        if (i == g_n_smem_attr && g_n_smem_attr < 32) g_smem_attr[g_n_smem_attr++] = SmemAttr{fn, bytes, 0};
        if (i < g_n_smem_attr) g_smem_attr[i].devs |= bit;
    }
    pthread_mutex_unlock(&g_smem_mu);
    return e;
}

// Range-decoder policy of the plain decode path (rc_lanes_for).
static uint32_t g_rc_scalar_warps = vcg::kRcScalarWarpsDefault;
uint32_t vcg::rc_scalar_warps() { return __atomic_load_n(&g_rc_scalar_warps, __ATOMIC_RELAXED); }
extern "C" __attribute__((visibility("default"))) void vcg_set_rc_scalar_warps(int w) {
    const uint32_t v = w < 0 ? vcg::kRcScalarWarpsDefault : (uint32_t)(w > 64 ? 64 : w);
    __atomic_store_n(&g_rc_scalar_warps, v, __ATOMIC_RELAXED);
}
static uint32_t g_rc_solo = vcg::kRcSoloDefault;
uint32_t vcg::rc_solo_atoms() { return __atomic_load_n(&g_rc_solo, __ATOMIC_RELAXED); }
extern "C" __attribute__((visibility("default"))) void vcg_set_rc_solo(int n) {
    __atomic_store_n(&g_rc_solo, n < 0 ? vcg::kRcSoloDefault : (uint32_t)n, __ATOMIC_RELAXED);
}

// ---------------------------------------------------------------- allocation-failure injection
// g_fail_alloc > 0: allocations left before one fails; -1: that failure
// happened; 0: off. Tests use it to show that every allocation failure comes
// back as a status and leaves the library usable.
static int64_t g_fail_alloc;

static bool injected_failure(void) {
    int64_t v = __atomic_load_n(&g_fail_alloc, __ATOMIC_ACQUIRE);
    while (v > 0) {
        const int64_t nv = v == 1 ? -1 : v - 1;
        if (__atomic_compare_exchange_n(&g_fail_alloc, &v, nv, false, __ATOMIC_ACQ_REL, __ATOMIC_ACQUIRE))
            return nv == -1;
    }
    return false;
}

namespace {
bool block_trim(void);
}

// cudaMalloc that, when the device is out of memory, first gives back the
// cached blocks of closed archives and tries once more
cudaError_t vcd_malloc(void **p, size_t bytes) {
    if (injected_failure()) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaErrorMemoryAllocation && block_trim()) {
        cudaGetLastError();
        e = cudaMalloc(p, bytes);
    }
    if (e != cudaSuccess) cudaGetLastError();   // not sticky: clear it for the next call
    return e;
}

cudaError_t vcd_malloc_host(void **p, size_t bytes) {
    if (injected_failure()) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMallocHost(p, bytes);
    if (e != cudaSuccess) cudaGetLastError();
    return e;
}

// Arming also empties the cache of archive blocks, so that the allocations a
// call makes do not depend on the archives closed before it.
extern "C" __attribute__((visibility("default"))) int64_t vcg_debug_fail_alloc(int64_t n) {
    if (n > 0) block_trim();
    return __atomic_exchange_n(&g_fail_alloc, n > 0 ? n : 0, __ATOMIC_ACQ_REL);
}

// grow-only scratch buffer `slot` of the calling thread
cudaError_t vcd_scratch(vcd_ctx *c, int slot, size_t bytes, void **out) {
    if (bytes == 0) bytes = 16;
    if (c->cap[slot] < bytes) {
        if (c->buf[slot]) {
            cudaStreamSynchronize(c->stream);
            cudaFree(c->buf[slot]);
            c->buf[slot] = NULL;
            c->cap[slot] = 0;
        }
        size_t want = bytes + bytes / 8;
        cudaError_t e = vcd_malloc((void **)&c->buf[slot], want);
        if (e != cudaSuccess) return e;
        c->cap[slot] = want;
    }
    *out = c->buf[slot];
    return cudaSuccess;
}

cudaError_t vcd_pinned(vcd_ctx *c, size_t bytes, void **out) {
    if (c->pinned_cap < bytes) {
        if (c->pinned) cudaFreeHost(c->pinned);
        c->pinned = NULL;
        c->pinned_cap = 0;
        cudaError_t e = vcd_malloc_host((void **)&c->pinned, bytes);
        if (e != cudaSuccess) return e;
        c->pinned_cap = bytes;
    }
    *out = c->pinned;
    return cudaSuccess;
}

// ---------------------------------------------------------------- archive residency
// Device blocks of closed archives are kept for the next archive that fits
// (at most kBlockCache blocks, each reused only for a request of at least half
// its size), so a caller that opens and closes archives of similar size does
// not pay cudaMalloc / cudaFree (and the synchronisation cudaFree implies) per
// archive.
namespace {
constexpr int kBlockCache = 6;
struct CachedBlock {
    void *p;
    size_t cap;
};
CachedBlock g_blocks[kBlockCache];
pthread_mutex_t g_block_mu = PTHREAD_MUTEX_INITIALIZER;

cudaError_t block_alloc(size_t bytes, void **out, size_t *cap) {
    pthread_mutex_lock(&g_block_mu);
    int best = -1;
    for (int i = 0; i < kBlockCache; ++i)
        if (g_blocks[i].p && g_blocks[i].cap >= bytes && g_blocks[i].cap / 2 <= bytes &&
            (best < 0 || g_blocks[i].cap < g_blocks[best].cap))
            best = i;
    if (best >= 0) {
        *out = g_blocks[best].p;
        *cap = g_blocks[best].cap;
        g_blocks[best].p = NULL;
        pthread_mutex_unlock(&g_block_mu);
        return cudaSuccess;
    }
    pthread_mutex_unlock(&g_block_mu);
    *cap = bytes;
    return vcd_malloc((void **)out, bytes);
}

// p must be idle (no work of any stream still using it)
void block_release(void *p, size_t cap) {
    if (!p) return;
    pthread_mutex_lock(&g_block_mu);
    int slot = -1;
    for (int i = 0; i < kBlockCache; ++i)
        if (!g_blocks[i].p) { slot = i; break; }
    if (slot < 0) {   // full: evict the smallest cached block if this one is larger
        int small = 0;
        for (int i = 1; i < kBlockCache; ++i)
            if (g_blocks[i].cap < g_blocks[small].cap) small = i;
        if (g_blocks[small].cap < cap) {
            cudaFree(g_blocks[small].p);
            slot = small;
        }
    }
    if (slot >= 0) g_blocks[slot] = CachedBlock{p, cap};
    else cudaFree(p);
    pthread_mutex_unlock(&g_block_mu);
}

// frees every cached block; true if there was one
bool block_trim(void) {
    bool any = false;
    pthread_mutex_lock(&g_block_mu);
    for (int i = 0; i < kBlockCache; ++i)
        if (g_blocks[i].p) {
            cudaFree(g_blocks[i].p);
            g_blocks[i] = CachedBlock{NULL, 0};
            any = true;
        }
    pthread_mutex_unlock(&g_block_mu);
    return any;
}
}  // namespace

// Residency in two steps, so that the copy of the archive bytes runs while the
// host resolves the atom table: begin allocates and starts the copy on the
// calling thread's stream, finish uploads the table and waits for both.
extern "C" int vcd_upload_begin(vcd_archive **out, const uint8_t *buf, size_t len) {
    vcd_ctx *c = vcd_thread_ctx();
    if (!c) return 4;
    vcd_archive *d = (vcd_archive *)calloc(1, sizeof(vcd_archive));
    if (!d) return 3;
    cudaError_t e;
    void *blk = NULL;
    if ((e = block_alloc(len + 16, &blk, &d->arc_cap)) != cudaSuccess ||
        (d->arc = (uint8_t *)blk, (e = cudaMemcpyAsync(d->arc, buf, len, cudaMemcpyHostToDevice, c->stream))) !=
            cudaSuccess ||
        (e = cudaMemsetAsync(d->arc + len, 0, 16, c->stream)) != cudaSuccess) {
        vcd_set_error("archive upload", e);
        cudaStreamSynchronize(c->stream);
        vcd_free_archive(d);
        return vcd_status_of(e);
    }
    d->len = len;
    *out = d;
    return 0;
}

extern "C" int vcd_upload_finish(vcd_archive *d, const vcd_atom *atoms, uint64_t n_atoms, const vcd_dq *dq, int nlod) {
    vcd_ctx *c = vcd_thread_ctx();
    if (!c) return 4;
    cudaError_t e;
    void *blk = NULL;
    if ((e = block_alloc((n_atoms ? n_atoms : 1) * sizeof(vcd_atom), &blk, &d->atoms_cap)) != cudaSuccess ||
        (d->atoms = (vcd_atom *)blk,
         (e = cudaMemcpyAsync(d->atoms, atoms, n_atoms * sizeof(vcd_atom), cudaMemcpyHostToDevice, c->stream))) !=
            cudaSuccess ||
        (e = block_alloc(nlod * sizeof(vcd_dq), &blk, &d->dq_cap)) != cudaSuccess ||
        (d->dq = (vcd_dq *)blk,
         (e = cudaMemcpyAsync(d->dq, dq, nlod * sizeof(vcd_dq), cudaMemcpyHostToDevice, c->stream))) != cudaSuccess ||
        (e = cudaStreamSynchronize(c->stream)) != cudaSuccess) {
        vcd_set_error("archive upload", e);
        cudaStreamSynchronize(c->stream);
        return vcd_status_of(e);
    }
    d->nlod = nlod;
    return 0;
}

extern "C" void vcd_free_archive(vcd_archive *d) {
    if (!d) return;
    // work on this thread's stream (a failed upload's copy) ends before its
    // blocks may serve another archive; decodes of the archive have returned
    vcd_ctx *c = vcd_thread_ctx();
    if (c) cudaStreamSynchronize(c->stream);
    if (d->arc_cap) block_release(d->arc, d->arc_cap);
    else cudaFree(d->arc);
    if (d->atoms_cap) block_release(d->atoms, d->atoms_cap);
    else cudaFree(d->atoms);
    if (d->dq_cap) block_release(d->dq, d->dq_cap);
    else cudaFree(d->dq);
    free(d);
}

cudaStream_t vcd_side_stream(vcd_ctx *c) {
    if (!c->copy_stream) {
        if (cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            c->copy_stream = NULL;
            return NULL;
        }
        for (int i = 0; i < VCD_SLABS; ++i) cudaEventCreateWithFlags(&c->chunk_ev[i], cudaEventDisableTiming);
        for (int i = 0; i < 4; ++i) cudaEventCreateWithFlags(&c->ring_ev[i], cudaEventDisableTiming);
    }
    return c->copy_stream;
}

// ---------------------------------------------------------------- pageable copy-out
// Device -> pageable host memory for large outputs. A plain cudaMemcpy into
// pageable memory goes through the CUDA runtime's own staging at about 20 GB/s
// (measured on a GB300 with a Grace host); here the
// device copies 32 MiB chunks into a ring of 4 pinned slots on stream cs while
// kBounceThreads host threads copy each finished chunk into the destination
// (each thread a stripe of it). A slot is refilled once every thread has
// finished the chunk in it. With slabs, the copy of a chunk first waits for the
// event of the slab whose end covers it, so the copy-out follows a transform
// that is still running.
namespace {
constexpr size_t kBounceChunk = 32ull << 20;
constexpr size_t kBounceMin = 16ull << 20;   // smaller outputs: one plain copy
constexpr int kBounceRing = 4;
constexpr int kBounceThreads = 12;   // 1 GiB LOD0 decode into pageable memory, end to end with 4 / 8 / 12 / 16: 28.5 / 36 / 38.6 / 38.6 GB/s

struct Bounce {
    vcd_ctx *c;
    cudaStream_t cs;
    const uint64_t *slab_end;    // optional: byte end of each slab of the source, ascending
    const cudaEvent_t *slab_ev;  // and the event recorded when that slab is written
    int nslab;
    uint8_t *dst;
    const uint8_t *src;
    uint8_t *ring;
    size_t bytes;
    uint32_t n_chunks;
    pthread_mutex_t mu;
    pthread_cond_t cv;
    uint32_t issued;             // chunks whose device copy has been queued
    uint32_t done[kBounceRing];  // threads finished with the chunk in each slot
    cudaError_t err;
};

static size_t chunk_len(const Bounce &b, uint32_t k) {
    const size_t off = (size_t)k * kBounceChunk;
    return b.bytes - off < kBounceChunk ? b.bytes - off : kBounceChunk;
}

static cudaError_t bounce_issue(Bounce &b, uint32_t k) {   // device chunk k into its slot (mu held)
    const int slot = (int)(k % kBounceRing);
    cudaError_t e = cudaSuccess;
    if (b.nslab) {   // the slab that completes this chunk
        const uint64_t end = (uint64_t)k * kBounceChunk + chunk_len(b, k);
        int j = 0;
        while (j + 1 < b.nslab && b.slab_end[j] < end) ++j;
        e = cudaStreamWaitEvent(b.cs, b.slab_ev[j], 0);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b.ring + (size_t)slot * kBounceChunk, b.src + (size_t)k * kBounceChunk, chunk_len(b, k),
                            cudaMemcpyDeviceToHost, b.cs);
    if (e == cudaSuccess) e = cudaEventRecord(b.c->ring_ev[slot], b.cs);
    b.done[slot] = 0;
    return e;
}

struct BounceWorker {
    Bounce *b;
    int id;
};

static void *bounce_worker(void *p) {
    BounceWorker *w = (BounceWorker *)p;
    Bounce &b = *w->b;
    cudaSetDevice(g_dev.device);
    for (uint32_t k = 0; k < b.n_chunks; ++k) {
        pthread_mutex_lock(&b.mu);
        while (b.issued <= k && b.err == cudaSuccess) pthread_cond_wait(&b.cv, &b.mu);
        const bool stop = b.err != cudaSuccess;
        pthread_mutex_unlock(&b.mu);
        if (stop) break;
        const int slot = (int)(k % kBounceRing);
        const cudaError_t e = cudaEventSynchronize(b.c->ring_ev[slot]);
        const size_t len = chunk_len(b, k), per = (len + kBounceThreads - 1) / kBounceThreads;
        const size_t lo = (size_t)w->id * per < len ? (size_t)w->id * per : len;
        const size_t hi = lo + per < len ? lo + per : len;
        if (e == cudaSuccess && hi > lo)
            memcpy(b.dst + (size_t)k * kBounceChunk + lo, b.ring + (size_t)slot * kBounceChunk + lo, hi - lo);
        pthread_mutex_lock(&b.mu);
        if (e != cudaSuccess && b.err == cudaSuccess) b.err = e;
        ++b.done[slot];
        pthread_cond_broadcast(&b.cv);
        pthread_mutex_unlock(&b.mu);
    }
    return NULL;
}
}  // namespace

// Returns cudaSuccess, or the first error (the destination is then incomplete).
// cs: the stream of the device copies; slab_end / slab_ev / nslab: see Bounce.
static cudaError_t copy_out_pageable(vcd_ctx *c, uint8_t *dst, const uint8_t *src_dev, size_t bytes, cudaStream_t cs,
                                     const uint64_t *slab_end, const cudaEvent_t *slab_ev, int nslab) {
    void *pin = NULL;
    cudaError_t e = vcd_pinned(c, kBounceChunk * kBounceRing, &pin);
    if (e != cudaSuccess || !vcd_side_stream(c)) {   // the slot events live with the second stream
        // no pinned ring (or no second stream): one plain copy after the work that writes the source
        cudaGetLastError();
        e = cudaStreamSynchronize(c->stream);
        if (e == cudaSuccess && cs != c->stream) e = cudaStreamSynchronize(cs);
        if (e == cudaSuccess) e = cudaMemcpy(dst, src_dev, bytes, cudaMemcpyDeviceToHost);
        return e;
    }
    Bounce b;
    memset(&b, 0, sizeof b);
    b.c = c; b.cs = cs; b.slab_end = slab_end; b.slab_ev = slab_ev; b.nslab = nslab;
    b.dst = dst; b.src = src_dev; b.ring = (uint8_t *)pin; b.bytes = bytes;
    b.n_chunks = (uint32_t)((bytes + kBounceChunk - 1) / kBounceChunk);
    b.err = cudaSuccess;
    pthread_mutex_init(&b.mu, NULL);
    pthread_cond_init(&b.cv, NULL);
    pthread_mutex_lock(&b.mu);
    for (uint32_t k = 0; k < b.n_chunks && k < (uint32_t)kBounceRing && b.err == cudaSuccess; ++k) {
        b.err = bounce_issue(b, k);
        b.issued = k + 1;
    }
    pthread_mutex_unlock(&b.mu);
    pthread_t th[kBounceThreads];
    BounceWorker wk[kBounceThreads];
    int started = 0;
    for (; started < kBounceThreads; ++started) {
        wk[started].b = &b;
        wk[started].id = started;
        if (pthread_create(&th[started], NULL, bounce_worker, &wk[started]) != 0) break;
    }
    pthread_mutex_lock(&b.mu);
    if (started < kBounceThreads && b.err == cudaSuccess) b.err = cudaErrorLaunchOutOfResources;
    // refill each slot once every thread is done with it
    for (uint32_t k = 0; k + kBounceRing < b.n_chunks && b.err == cudaSuccess; ++k) {
        const int slot = (int)(k % kBounceRing);
        while (b.done[slot] < (uint32_t)kBounceThreads && b.err == cudaSuccess) pthread_cond_wait(&b.cv, &b.mu);
        if (b.err != cudaSuccess) break;
        b.err = bounce_issue(b, k + kBounceRing);
        b.issued = k + kBounceRing + 1;
        pthread_cond_broadcast(&b.cv);
    }
    pthread_cond_broadcast(&b.cv);
    pthread_mutex_unlock(&b.mu);
    for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
    pthread_cond_destroy(&b.cv);
    pthread_mutex_destroy(&b.mu);
    const cudaError_t se = cudaStreamSynchronize(cs);   // no copy into the ring still in flight
    if (b.err == cudaSuccess) b.err = se;
    return b.err;
}

// Pageable host -> device for large inputs, the same ring the other way: the
// kBounceThreads threads copy each 32 MiB chunk of the source into a pinned
// slot (each a stripe of it), then the chunk is copied to the device on the
// context's stream; a slot is refilled once its previous copy to the device has
// completed.
namespace {
struct BounceIn {
    vcd_ctx *c;
    uint8_t *dst;
    const uint8_t *src;
    uint8_t *ring;
    size_t bytes;
    uint32_t n_chunks;
    pthread_mutex_t mu;
    pthread_cond_t cv;
    uint32_t issued;               // chunks whose device copy has been queued
    uint32_t filled[kBounceRing];  // threads done filling the chunk in each slot
    cudaError_t err;
};

static size_t in_len(const BounceIn &b, uint32_t k) {
    const size_t off = (size_t)k * kBounceChunk;
    return b.bytes - off < kBounceChunk ? b.bytes - off : kBounceChunk;
}

struct BounceInWorker {
    BounceIn *b;
    int id;
};

static void *bounce_in_worker(void *p) {
    BounceInWorker *w = (BounceInWorker *)p;
    BounceIn &b = *w->b;
    cudaSetDevice(g_dev.device);
    for (uint32_t k = 0; k < b.n_chunks; ++k) {
        const int slot = (int)(k % kBounceRing);
        if (k >= (uint32_t)kBounceRing) {   // the slot's previous chunk must have reached the device
            pthread_mutex_lock(&b.mu);
            while (b.issued <= k - kBounceRing && b.err == cudaSuccess) pthread_cond_wait(&b.cv, &b.mu);
            const bool stop = b.err != cudaSuccess;
            pthread_mutex_unlock(&b.mu);
            if (stop) break;
            const cudaError_t e = cudaEventSynchronize(b.c->ring_ev[slot]);
            if (e != cudaSuccess) {
                pthread_mutex_lock(&b.mu);
                if (b.err == cudaSuccess) b.err = e;
                pthread_cond_broadcast(&b.cv);
                pthread_mutex_unlock(&b.mu);
                break;
            }
        }
        const size_t len = in_len(b, k), per = (len + kBounceThreads - 1) / kBounceThreads;
        const size_t lo = (size_t)w->id * per < len ? (size_t)w->id * per : len;
        const size_t hi = lo + per < len ? lo + per : len;
        if (hi > lo) memcpy(b.ring + (size_t)slot * kBounceChunk + lo, b.src + (size_t)k * kBounceChunk + lo, hi - lo);
        pthread_mutex_lock(&b.mu);
        ++b.filled[slot];
        pthread_cond_broadcast(&b.cv);
        pthread_mutex_unlock(&b.mu);
    }
    return NULL;
}
}  // namespace

static cudaError_t copy_in_pageable(vcd_ctx *c, uint8_t *dst_dev, const uint8_t *src, size_t bytes) {
    void *pin = NULL;
    cudaError_t e = vcd_pinned(c, kBounceChunk * kBounceRing, &pin);
    if (e != cudaSuccess || !vcd_side_stream(c)) {   // the slot events live with the second stream
        // no pinned ring (or no second stream): one staged copy in stream order
        cudaGetLastError();
        e = cudaMemcpyAsync(dst_dev, src, bytes, cudaMemcpyHostToDevice, c->stream);
        return e != cudaSuccess ? e : cudaStreamSynchronize(c->stream);
    }
    BounceIn b;
    memset(&b, 0, sizeof b);
    b.c = c; b.dst = dst_dev; b.src = src; b.ring = (uint8_t *)pin; b.bytes = bytes;
    b.n_chunks = (uint32_t)((bytes + kBounceChunk - 1) / kBounceChunk);
    b.err = cudaSuccess;
    pthread_mutex_init(&b.mu, NULL);
    pthread_cond_init(&b.cv, NULL);
    pthread_t th[kBounceThreads];
    BounceInWorker wk[kBounceThreads];
    int started = 0;
    for (; started < kBounceThreads; ++started) {
        wk[started].b = &b;
        wk[started].id = started;
        if (pthread_create(&th[started], NULL, bounce_in_worker, &wk[started]) != 0) break;
    }
    pthread_mutex_lock(&b.mu);
    if (started < kBounceThreads) b.err = cudaErrorLaunchOutOfResources;
    for (uint32_t k = 0; k < b.n_chunks && b.err == cudaSuccess; ++k) {
        const int slot = (int)(k % kBounceRing);
        while (b.filled[slot] < (uint32_t)kBounceThreads && b.err == cudaSuccess) pthread_cond_wait(&b.cv, &b.mu);
        if (b.err != cudaSuccess) break;
        cudaError_t ie = cudaMemcpyAsync(b.dst + (size_t)k * kBounceChunk, b.ring + (size_t)slot * kBounceChunk,
                                         in_len(b, k), cudaMemcpyHostToDevice, c->stream);
        if (ie == cudaSuccess) ie = cudaEventRecord(c->ring_ev[slot], c->stream);
        b.filled[slot] = 0;
        b.issued = k + 1;
        if (ie != cudaSuccess) b.err = ie;
        pthread_cond_broadcast(&b.cv);
    }
    pthread_cond_broadcast(&b.cv);
    pthread_mutex_unlock(&b.mu);
    for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
    pthread_cond_destroy(&b.cv);
    pthread_mutex_destroy(&b.mu);
    const cudaError_t se = cudaStreamSynchronize(c->stream);   // the ring is free again
    return b.err != cudaSuccess ? b.err : se;
}

static bool host_pageable(const void *p, size_t bytes) {
    if (bytes < kBounceMin) return false;
    cudaPointerAttributes pa;
    const bool pinned = cudaPointerGetAttributes(&pa, p) == cudaSuccess && pa.type == cudaMemoryTypeHost;
    cudaGetLastError();
    return !pinned;
}

cudaError_t vcd_copy_to_host(vcd_ctx *c, void *dst, const void *src_dev, size_t bytes) {
    if (host_pageable(dst, bytes))
        return copy_out_pageable(c, (uint8_t *)dst, (const uint8_t *)src_dev, bytes, c->stream, NULL, NULL, 0);
    cudaError_t e = cudaMemcpyAsync(dst, src_dev, bytes, cudaMemcpyDeviceToHost, c->stream);
    return e != cudaSuccess ? e : cudaStreamSynchronize(c->stream);
}

cudaError_t vcd_copy_from_host(vcd_ctx *c, void *dst_dev, const void *src, size_t bytes) {
    if (host_pageable(src, bytes)) return copy_in_pageable(c, (uint8_t *)dst_dev, (const uint8_t *)src, bytes);
    cudaError_t e = cudaMemcpyAsync(dst_dev, src, bytes, cudaMemcpyHostToDevice, c->stream);
    return e != cudaSuccess ? e : cudaStreamSynchronize(c->stream);
}

// ---------------------------------------------------------------- decode
constexpr uint64_t kFusedMaxPayload = 3072;   // mean payload bytes per PRESENT atom of a fused decode

// One box decode from device bytes `arc` and atom table `atoms` (LOD raster, or
// box order when box_table). last_ms spans from `t0` (or the first stage event).
static int decode_job(vcd_ctx *c, const uint8_t *arc, const vcd_atom *atoms, uint32_t box_table, const vcd_dq *dq,
                      const vcd_region *r, uint8_t *out_dev, uint8_t *out_host, size_t out_bytes, cudaEvent_t t0) {
    cudaError_t e;
    const uint64_t n = r->n_atoms;
    const uint64_t box_atoms = (uint64_t)r->bnx * r->bny * r->bnz;
    DecodeJob J;
    memset(&J, 0, sizeof J);
    void *p_cnt, *p_off, *p_ent, *p_out, *p_err;
    if ((e = vcd_scratch(c, VCD_BUF_CNT, (n + 1) * 4 + 16, &p_cnt)) != cudaSuccess ||
        (e = vcd_scratch(c, VCD_BUF_OFF, (n + 1) * 8, &p_off)) != cudaSuccess ||
        (e = vcd_scratch(c, VCD_BUF_ENT, r->cap_total * 4 + 16, &p_ent)) != cudaSuccess) {
        vcd_set_error("decode scratch", e);
        return vcd_status_of(e);
    }
    void *p_ctl;   // [u32 first malformed atom][u32 pad][u64 entries written]
    if ((e = vcd_scratch(c, VCD_BUF_RED, 64, &p_ctl)) != cudaSuccess) {
        vcd_set_error("decode scratch", e);
        return vcd_status_of(e);
    }
    p_err = p_ctl;
    void *p_ord = NULL;   // only large decodes use the per-lane range decoder (launch_rc)
    // [sort counters][order: n][fused-decode queue: n + SMs]
    if (rc_sorts(n, (uint32_t)g_dev.num_sms) &&
        (e = vcd_scratch(c, VCD_BUF_ORD, (2 * n + g_dev.num_sms + sort_ctl_words()) * 4 + 16, &p_ord)) !=
            cudaSuccess) {
        vcd_set_error("decode scratch", e);
        return vcd_status_of(e);
    }
    if (out_dev) {
        p_out = out_dev;
    } else if ((e = vcd_scratch(c, VCD_BUF_OUT, out_bytes, &p_out)) != cudaSuccess) {
        vcd_set_error("decode output", e);
        return vcd_status_of(e);
    }
    J.arc = arc;
    J.atoms = atoms;
    J.box_table = box_table;
    J.acx = r->acx; J.acy = r->acy;
    J.bax = r->bax; J.bay = r->bay; J.baz = r->baz; J.bnx = r->bnx; J.bny = r->bny;
    J.n_atoms = n;
    J.x0 = r->x0; J.y0 = r->y0; J.z0 = r->z0; J.x1 = r->x1; J.y1 = r->y1; J.z1 = r->z1;
    J.out = (uint8_t *)p_out;
    J.ox = r->x1 - r->x0; J.oy = r->y1 - r->y0;
    J.ent = (uint32_t *)p_ent;
    J.ent_off = (uint64_t *)p_off;
    J.cnt = (uint32_t *)p_cnt;
    J.dq = dq;
    J.alt_mask = g_dev.tables->alt_mask;
    J.scan = g_dev.tables->scan;
    J.err = (uint32_t *)p_err;
    J.nnz_total = (unsigned long long *)((uint8_t *)p_ctl + 8);
    memcpy(J.band_start, g_dev.band_start, sizeof J.band_start);
    if (p_ord) {
        J.sort_ctl = (uint32_t *)p_ord;
        J.order = J.sort_ctl + sort_ctl_words();
    }

    if ((e = cudaMemsetAsync(p_ctl, 0, 16, c->stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(p_err, 0xFF, 4, c->stream)) != cudaSuccess) {
        vcd_set_error("decode control words", e);
        return vcd_status_of(e);
    }
    StageEvents ev;
    memcpy(ev.ev, c->ev, sizeof ev.ev);
    // the per-lane decoder's solo atoms run on the second stream; the slab
    // events serve as its fork and join (the copy-out slabs record them again
    // only after the range decode)
    const bool solo = p_ord && rc_solo_for(n, (uint32_t)g_dev.num_sms) && vcd_side_stream(c);
    if (solo) {
        ev.side = c->copy_stream;
        ev.fork = c->chunk_ev[0];
        ev.join = c->chunk_ev[1];
    }
    uint64_t ctl_h[2] = {0xFFFFFFFFull, 0};
    // Large outputs to pinned host memory: the inverse transform runs in up to 32
    // slabs of atom layers and each finished slab is copied out on a second stream while
    // the next one is transformed. The range decode finishes first, so a stream
    // with a malformed atom is known before any byte reaches the caller.
    // (only when every atom of the box is decoded: a box cut short by a bad
    // payload range keeps the exact per-atom copy below)
    // (pageable destinations take the same slabs, copied out through pinned
    // bounce chunks by host threads)
    bool piped = false, bounce = false, fused = false;
    const uint64_t layer = (uint64_t)r->bnx * r->bny, layers = layer ? n / layer : 0;
    if (out_host && out_bytes >= (64ull << 20) && n == box_atoms && layers * layer == n && layers >= 2) {
        cudaPointerAttributes pa;
        const bool pinned = cudaPointerGetAttributes(&pa, out_host) == cudaSuccess && pa.type == cudaMemoryTypeHost;
        cudaGetLastError();
        piped = vcd_side_stream(c) != NULL;
        bounce = piped && !pinned;
    }
    if (piped) {
        launch_decode_front(J, g_dev.num_sms, c->stream, &ev);
        cudaMemcpyAsync(ctl_h, p_ctl, 16, cudaMemcpyDeviceToHost, c->stream);
        if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) {
            vcd_set_error("decode kernels", e);
            return vcd_status_of(e);
        }
        if ((uint32_t)ctl_h[0] < n) {   // malformed: whole transform, then the partial copy below
            launch_idct(J, g_dev.num_sms, c->stream, 0, n);
            cudaEventRecord(ev.ev[3], c->stream);
            piped = false;
        } else {
            const uint64_t plane = (uint64_t)J.ox * J.oy;
            const uint64_t per = (layers + VCD_SLABS - 1) / VCD_SLABS;
            uint64_t slab_end[VCD_SLABS];
            int k = 0;
            for (uint64_t l0 = 0; l0 < layers; l0 += per, ++k) {
                const uint64_t l1 = l0 + per < layers ? l0 + per : layers;
                launch_idct(J, g_dev.num_sms, c->stream, l0 * layer, l1 * layer);
                cudaEventRecord(c->chunk_ev[k], c->stream);
                const uint64_t zlo = (r->baz + l0) * 32 > r->z0 ? (r->baz + l0) * 32 : r->z0;
                const uint64_t zhi = (r->baz + l1) * 32 < r->z1 ? (r->baz + l1) * 32 : r->z1;
                slab_end[k] = (zhi - r->z0) * plane;
                if (!bounce) {
                    cudaStreamWaitEvent(c->copy_stream, c->chunk_ev[k], 0);
                    cudaMemcpyAsync(out_host + (zlo - r->z0) * plane, (uint8_t *)p_out + (zlo - r->z0) * plane,
                                    (zhi - zlo) * plane, cudaMemcpyDeviceToHost, c->copy_stream);
                }
            }
            cudaEventRecord(ev.ev[3], c->stream);
            if (bounce &&
                (e = copy_out_pageable(c, out_host, (const uint8_t *)p_out, out_bytes, c->copy_stream, slab_end,
                                       c->chunk_ev, k)) != cudaSuccess) {
                vcd_set_error("decode copy-out", e);
                return vcd_status_of(e);
            }
        }
    } else {
        // fused only for light payloads: on GB300 a 1024^3 decode at ~4.4 KB per atom
        // (target 10) took 12.9 ms fused against 11.6 ms for the two kernels (the
        // transform warps take issue slots from the latency-bound coder), at ~1 KB
        // (target 50) 5.9 against ~7 ms and at ~0.5 KB (target 100) 4.0 against 4.5
        const bool light = r->present && r->payload_bytes <= kFusedMaxPayload * r->present;
        fused = p_ord && light &&
                launch_decode_fused(J, g_dev.num_sms, c->stream, J.order + n, (uint32_t *)p_ctl + 1, &ev);
        if (!fused) {
            launch_decode_front(J, g_dev.num_sms, c->stream, &ev);
            if ((e = cudaPeekAtLastError()) != cudaSuccess) {
                vcd_set_error("decode launch (lists, range decoder)", e);
                cudaGetLastError();
                return vcd_status_of(e);
            }
            launch_idct(J, g_dev.num_sms, c->stream, 0, n);
            cudaEventRecord(ev.ev[3], c->stream);
        }
        if ((e = cudaPeekAtLastError()) != cudaSuccess) {
            vcd_set_error("decode launch (inverse transform)", e);
            cudaGetLastError();
            return vcd_status_of(e);
        }
        if ((e = cudaMemcpyAsync(ctl_h, p_ctl, 16, cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess) {
            vcd_set_error("decode status copy", e);
            return vcd_status_of(e);
        }
    }
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess || (piped && (e = cudaStreamSynchronize(c->copy_stream)) != cudaSuccess) ||
        (e = cudaGetLastError()) != cudaSuccess) {
        vcd_set_error("decode kernels", e);
        return vcd_status_of(e);
    }
    c->last_ms = vcd_elapsed(t0 ? t0 : ev.ev[0], ev.ev[3]);
    if (fused && (ctl_h[0] >> 32) != 0) {   // the fused kernel's transform warps gave up waiting
        vcd_set_error("fused decode: an atom never reached the transform", cudaSuccess);
        return 4;
    }
    if (vcd_prof_on()) {
        const uint64_t nnz = ctl_h[1];
        vcd_prof_add("decode_place", vcd_elapsed(ev.ev[0], ev.ev[1]), n ? 2 : 0, 24 * n, 8 * n, n);
        if (fused) {   // length sort (three kernels); range decode + transform in one kernel
            vcd_prof_add("length_sort", vcd_elapsed(ev.ev[1], ev.ev[2]), 3, 16 * n, 8 * n, n);
            vcd_prof_add("decode_fused", vcd_elapsed(ev.ev[2], ev.ev[3]), 1, r->payload_bytes + 16 * n, out_bytes,
                         n);
        } else {
            // (the per-lane decoder: length sort in three kernels, then the decoder)
            vcd_prof_add("rc_decode", vcd_elapsed(ev.ev[1], ev.ev[2]), n ? (p_ord ? (solo ? 6 : 4) : 1) : 0,
                         r->payload_bytes + 16 * n, 4 * nnz, r->present);
            vcd_prof_add("idct", vcd_elapsed(ev.ev[2], ev.ev[3]), n ? 1 : 0, 4 * nnz + 16 * n, out_bytes, n);
        }
    }
    const uint32_t err_h = (uint32_t)ctl_h[0];
    const uint64_t good = err_h < n ? err_h : n;   // atoms written before the first bad one
    const int status = (good < box_atoms) ? 1 /*VC_ERR_FORMAT*/ : 0;
    if (!out_host || piped) return status;   // piped: already copied out
    if (!status) {
        cudaPointerAttributes pa;
        const bool pageable = out_bytes >= kBounceMin &&
                              (cudaPointerGetAttributes(&pa, out_host) != cudaSuccess || pa.type != cudaMemoryTypeHost);
        cudaGetLastError();
        if (pageable) {
            e = copy_out_pageable(c, out_host, (const uint8_t *)p_out, out_bytes, c->stream, NULL, NULL, 0);
        } else if ((e = cudaMemcpyAsync(out_host, p_out, out_bytes, cudaMemcpyDeviceToHost, c->stream)) == cudaSuccess) {
            e = cudaStreamSynchronize(c->stream);
        }
        if (e != cudaSuccess) {
            vcd_set_error("decode copy-out", e);
            return vcd_status_of(e);
        }
        return 0;
    }
    // error path: only the atoms before the first bad one reach the caller
    uint8_t *tmp = (uint8_t *)malloc(out_bytes ? out_bytes : 1);
    if (!tmp) return 3;
    if ((e = cudaMemcpy(tmp, p_out, out_bytes, cudaMemcpyDeviceToHost)) != cudaSuccess) {
        free(tmp);
        vcd_set_error("decode copy-out", e);
        return vcd_status_of(e);
    }
    for (uint64_t t = 0; t < good; ++t) {
        uint32_t az, ay, ax;
        box_atom(J, t, az, ay, ax);
        uint32_t x0 = ax * 32 > r->x0 ? ax * 32 : r->x0, x1 = ax * 32 + 32 < r->x1 ? ax * 32 + 32 : r->x1;
        uint32_t y0 = ay * 32 > r->y0 ? ay * 32 : r->y0, y1 = ay * 32 + 32 < r->y1 ? ay * 32 + 32 : r->y1;
        uint32_t z0 = az * 32 > r->z0 ? az * 32 : r->z0, z1 = az * 32 + 32 < r->z1 ? az * 32 + 32 : r->z1;
        for (uint32_t z = z0; z < z1; ++z)
            for (uint32_t y = y0; y < y1; ++y) {
                size_t o = ((size_t)(z - r->z0) * J.oy + (y - r->y0)) * J.ox + (x0 - r->x0);
                memcpy(out_host + o, tmp + o, x1 - x0);
            }
    }
    free(tmp);
    return status;
}

extern "C" int vcd_decode_region(vcd_archive *d, const vcd_region *r, uint8_t *out_dev, uint8_t *out_host,
                                 size_t out_bytes) {
    vcd_ctx *c = vcd_thread_ctx();
    if (!c) return 4;
    return decode_job(c, d->arc, d->atoms + r->atom_base, 0, d->dq + r->lod, r, out_dev, out_host, out_bytes, NULL);
}

// ---------------------------------------------------------------- streamed decode

extern "C" int vcd_upload_dq(vcd_archive **out, const vcd_dq *dq, int nlod) {
    vcd_archive *d = (vcd_archive *)calloc(1, sizeof(vcd_archive));
    if (!d) return 3;
    cudaError_t e;
    if ((e = vcd_malloc((void **)&d->dq, nlod * sizeof(vcd_dq))) != cudaSuccess ||
        (e = cudaMemcpy(d->dq, dq, nlod * sizeof(vcd_dq), cudaMemcpyHostToDevice)) != cudaSuccess) {
        vcd_set_error("dequantisation tables", e);
        vcd_free_archive(d);
        return vcd_status_of(e);
    }
    d->nlod = nlod;
    *out = d;
    return 0;
}

extern "C" int vcd_stage_reserve(size_t bytes, uint8_t **host) {
    vcd_ctx *c = vcd_thread_ctx();
    if (!c) return 4;
    c->stage_started = 0;
    cudaError_t e;
    // uploads of an earlier call that ended early may still read the staging
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) {
        vcd_set_error("staging", e);
        return vcd_status_of(e);
    }
    if (c->stage_cap < bytes) {
        if (c->stage_host) cudaFreeHost(c->stage_host);
        c->stage_host = NULL;
        c->stage_cap = 0;
        const size_t want = bytes + bytes / 4;
        if ((e = vcd_malloc_host((void **)&c->stage_host, want)) != cudaSuccess) {
            c->stage_host = NULL;
            vcd_set_error("staging", e);
            return vcd_status_of(e);
        }
        c->stage_cap = want;
    }
    void *dev;
    if ((e = vcd_scratch(c, VCD_BUF_STG, bytes + 16, &dev)) != cudaSuccess) {
        vcd_set_error("staging", e);
        return vcd_status_of(e);
    }
    *host = c->stage_host;
    return 0;
}

extern "C" int vcd_stage_push(size_t off, size_t bytes) {
    vcd_ctx *c = vcd_thread_ctx();
    if (!c || !c->stage_host || off + bytes > c->stage_cap || off + bytes + 16 > c->cap[VCD_BUF_STG]) return 4;
    if (!c->stage_started) {
        cudaEventRecord(c->ev[4], c->stream);
        c->stage_started = 1;
    }
    if (!bytes) return 0;
    cudaError_t e = cudaMemcpyAsync((uint8_t *)c->buf[VCD_BUF_STG] + off, c->stage_host + off, bytes,
                                    cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) {
        vcd_set_error("staging upload", e);
        return vcd_status_of(e);
    }
    return 0;
}

extern "C" int vcd_decode_staged(vcd_archive *d, const vcd_region *r, size_t table_off, size_t arena_off,
                                 size_t arena_bytes, uint8_t *out_dev, uint8_t *out_host, size_t out_bytes) {
    vcd_ctx *c = vcd_thread_ctx();
    if (!c) return 4;
    if (arena_off + arena_bytes + 16 > c->cap[VCD_BUF_STG] || table_off + r->n_atoms * sizeof(vcd_atom) > arena_off)
        return 4;
    uint8_t *stg = (uint8_t *)c->buf[VCD_BUF_STG];
    // 16 zero bytes after the last payload, as after a resident archive
    cudaError_t e = cudaMemsetAsync(stg + arena_off + arena_bytes, 0, 16, c->stream);
    if (e != cudaSuccess) {
        vcd_set_error("staging slack", e);
        return vcd_status_of(e);
    }
    const int rc = decode_job(c, stg + arena_off, (const vcd_atom *)(stg + table_off), 1, d->dq + r->lod, r, out_dev,
                              out_host, out_bytes, c->stage_started ? c->ev[4] : NULL);
    c->stage_started = 0;
    return rc;
}

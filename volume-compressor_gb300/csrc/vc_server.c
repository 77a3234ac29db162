// Decode server: continuous batching of vc_decode_region requests against one
// archive kept resident in device memory.
//
// Requests are queued by vcg_server_submit and decoded by a small pool of
// worker threads, each with its own CUDA stream. Requests fall in two classes
// by box size. A worker takes, in arrival order, as many waiting small
// requests as the shared device-memory budget and its batch limit allow,
// decodes them in one batched pass (each distinct atom once, cropped into
// every box; vcg_decode_regions) and releases their budget; a batch of one
// request takes the plain decode path (vc_decode_region), which has the lower
// latency. Large requests (kBigVoxels or more) run, when the oldest waiting
// request is a large one, on at most workers - 1 workers at a time while small
// requests wait, so that one worker is left for them (on every worker while
// none waits); the waiting large requests are shared out over the free
// large-request workers, each batch taking its share (one each while there are
// as many workers as requests).
// Requests that arrive while batches are on the GPU join the next batch of
// whichever worker frees up first, so batches from different workers overlap
// on the device. Each result is exactly what vc_decode_region returns for that
// request alone.
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "../../include/vcg.h"

#define VC_API __attribute__((visibility("default")))


#define kBigVoxels (32ull << 20)   // a box of 32 Mi voxels or more is a large request

typedef struct {
    vcg_region_request req;
    uint64_t cost;          // device bytes the request holds while decoding
    int big;                // box of kBigVoxels or more
    double t_submit, t_done;
    vc_status status;
    int state;              // 0 queued, 1 running, 2 done, 3 done and waited for
} srv_req;

typedef struct vcg_server {
    vc_archive *a;
    uint64_t budget, in_use;
    uint32_t max_batch;
    int nworkers, stop;
    pthread_t th[8];
    struct srv_worker {     // a worker's batch arrays (max_batch entries each)
        struct vcg_server *s;
        vcg_region_request *batch;
        vc_status *st;
        uint64_t *tix;
    } w[8];
    pthread_mutex_t mu;
    pthread_cond_t work_cv, done_cv;
    srv_req *reqs;          // ticket t is reqs[t - base]
    uint64_t cap, base, n;  // slots, ticket of reqs[0], tickets issued
    uint64_t head;          // first ticket not yet taken by a worker
    uint64_t lo;            // every ticket below lo has been waited for
    uint64_t q_small, q_big;   // queued (not yet taken) requests of each class
    int big_running;        // workers decoding a large request
    uint64_t batches, batched_reqs;
} vcg_server;

static srv_req *slot(vcg_server *s, uint64_t ticket) { return &s->reqs[ticket - s->base]; }

static double now_us(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec * 1e6 + ts.tv_nsec * 1e-3;
}

// Device bytes a request holds while in a batch: its staged output plus list
// scratch for the atoms it touches (bounded by 32 KiB per atom on average).
static uint64_t cost_of(const vc_box *b) {
    uint64_t vox = (uint64_t)(b->x1 - b->x0) * (b->y1 - b->y0) * (b->z1 - b->z0);
    uint64_t atoms = (uint64_t)((b->x1 - 1) / 32 - b->x0 / 32 + 1) * ((b->y1 - 1) / 32 - b->y0 / 32 + 1) *
                     ((b->z1 - 1) / 32 - b->z0 / 32 + 1);
    return vox + atoms * 32768ull;
}

static void *worker(void *arg) {
    struct srv_worker *w = (struct srv_worker *)arg;
    vcg_server *s = w->s;
    vcg_region_request *batch = w->batch;
    vc_status *st = w->st;
    uint64_t *tix = w->tix;
    pthread_mutex_lock(&s->mu);   // (held by vcg_server_create until every worker exists)
    const int big_slots = s->nworkers > 1 ? s->nworkers - 1 : 1;
    for (;;) {
        while (!s->stop && s->q_small + s->q_big == 0) pthread_cond_wait(&s->work_cv, &s->mu);
        if (s->stop && s->q_small + s->q_big == 0) break;
        // the oldest waiting request decides: a large one runs alone if a
        // large-request slot is free; else the small requests in arrival order,
        // while memory and the batch limit allow. A request larger than the
        // whole budget runs alone.
        uint32_t k = 0;
        uint64_t take = 0;
        int big = 0;
        while (s->head < s->n && slot(s, s->head)->state != 0) ++s->head;
        const int oldest_big = s->head < s->n && slot(s, s->head)->big;
        // (every worker may take a large request while no small one waits)
        const int slots_now = s->q_small ? big_slots : s->nworkers;
        if (s->q_small && !(oldest_big && s->big_running < slots_now)) {
            for (uint64_t t = s->head; t < s->n && k < s->max_batch; ++t) {
                srv_req *r = slot(s, t);
                if (r->state != 0 || r->big) continue;
                if (s->in_use + take + r->cost > s->budget && (k > 0 || s->in_use > 0)) break;
                r->state = 1;
                batch[k] = r->req;
                tix[k] = t;
                take += r->cost;
                ++k;
            }
            s->q_small -= k;
        } else if (s->q_big && s->big_running < slots_now) {
            // the waiting large requests are shared out over the free
            // large-request slots: this worker takes the oldest and, while
            // memory and the batch limit allow, its share of the others (large
            // boxes of one LOD often share atoms, which a batch decodes once;
            // one large request per worker while there are as many workers)
            const uint64_t free_slots = (uint64_t)(slots_now - s->big_running);
            const uint64_t share = (s->q_big + free_slots - 1) / free_slots;
            const uint32_t kmax = share < s->max_batch ? (uint32_t)share : s->max_batch;
            for (uint64_t t = s->head; t < s->n && k < kmax; ++t) {
                srv_req *r = slot(s, t);
                if (r->state != 0 || !r->big) continue;
                if (s->in_use + take + r->cost > s->budget && (k > 0 || s->in_use > 0)) break;
                r->state = 1;
                batch[k] = r->req;
                tix[k] = t;
                take += r->cost;
                ++k;
            }
            if (k) {
                big = 1;
                s->q_big -= k;
                s->big_running += 1;
            }
        }
        while (s->head < s->n && slot(s, s->head)->state != 0) ++s->head;
        if (k == 0) {   // waiting for memory or a large-request slot held by other workers
            pthread_cond_wait(&s->work_cv, &s->mu);
            continue;
        }
        s->in_use += take;
        pthread_mutex_unlock(&s->mu);
        vc_status rc;
        if (k == 1) {   // alone: the plain path
            rc = vc_decode_region(s->a, batch[0].lod, batch[0].box, batch[0].out);
            st[0] = rc;
            rc = rc == VC_ERR_RANGE || rc == VC_ERR_FORMAT ? VC_OK : rc;   // per-request statuses
        } else {
            rc = vcg_decode_regions(s->a, k, batch, 0, st);
        }
        double t = now_us();
        pthread_mutex_lock(&s->mu);
        for (uint32_t i = 0; i < k; ++i) {
            srv_req *r = slot(s, tix[i]);
            r->status = rc != VC_OK ? rc : st[i];
            r->t_done = t;
            r->state = 2;
        }
        s->in_use -= take;
        s->big_running -= big;
        s->batches++;
        s->batched_reqs += k;
        pthread_cond_broadcast(&s->done_cv);
        pthread_cond_broadcast(&s->work_cv);
    }
    pthread_mutex_unlock(&s->mu);
    return NULL;
}

static void free_workers(vcg_server *s) {
    for (int i = 0; i < 8; ++i) {
        free(s->w[i].batch);
        free(s->w[i].st);
        free(s->w[i].tix);
    }
}

// device_budget: device bytes that requests in flight may hold (outputs plus
// list scratch); max_batch: requests per batch; workers: 1..8 batches in flight.
VC_API vcg_server *vcg_server_create(vc_archive *a, uint64_t device_budget, uint32_t max_batch, int workers) {
    if (!a || !device_budget || !max_batch || workers < 1 || workers > 8) return NULL;
    vcg_server *s = (vcg_server *)calloc(1, sizeof *s);
    if (!s) return NULL;
    s->a = a;
    s->budget = device_budget;
    s->max_batch = max_batch;
    s->cap = 1024;
    s->reqs = (srv_req *)calloc(s->cap, sizeof(srv_req));
    if (!s->reqs) { free(s); return NULL; }
    for (int i = 0; i < workers; ++i) {
        struct srv_worker *w = &s->w[i];
        w->s = s;
        w->batch = (vcg_region_request *)malloc(max_batch * sizeof(vcg_region_request));
        w->st = (vc_status *)malloc(max_batch * sizeof(vc_status));
        w->tix = (uint64_t *)malloc(max_batch * sizeof(uint64_t));
        if (!w->batch || !w->st || !w->tix) {
            free_workers(s);
            free(s->reqs);
            free(s);
            return NULL;
        }
    }
    pthread_mutex_init(&s->mu, NULL);
    pthread_cond_init(&s->work_cv, NULL);
    pthread_cond_init(&s->done_cv, NULL);
    // the workers start once they are all created (they read nworkers under mu)
    pthread_mutex_lock(&s->mu);
    for (int i = 0; i < workers; ++i) {
        if (pthread_create(&s->th[i], NULL, worker, &s->w[i]) != 0) break;
        s->nworkers++;
    }
    pthread_mutex_unlock(&s->mu);
    if (!s->nworkers) {
        pthread_mutex_destroy(&s->mu);
        pthread_cond_destroy(&s->work_cv);
        pthread_cond_destroy(&s->done_cv);
        free_workers(s);
        free(s->reqs);
        free(s);
        return NULL;
    }
    return s;
}

// Queue one request; returns its ticket (>= 0) or -1. out is host memory of the
// box's size and must stay valid until the ticket completes.
VC_API int64_t vcg_server_submit(vcg_server *s, int lod, vc_box box, uint8_t *out) {
    if (!s) return -1;
    pthread_mutex_lock(&s->mu);
    if (s->n - s->base == s->cap) {
        if (s->lo - s->base >= s->cap / 2) {   // recycle the slots of waited tickets
            const uint64_t drop = s->lo - s->base;
            memmove(s->reqs, s->reqs + drop, (size_t)(s->cap - drop) * sizeof(srv_req));
            s->base = s->lo;
        } else {
            srv_req *t = (srv_req *)realloc(s->reqs, 2 * s->cap * sizeof(srv_req));
            if (!t) { pthread_mutex_unlock(&s->mu); return -1; }
            s->reqs = t;
            s->cap *= 2;
        }
    }
    srv_req *r = slot(s, s->n);
    memset(r, 0, sizeof *r);
    r->req.lod = lod;
    r->req.box = box;
    r->req.out = out;
    const int nonempty = box.x1 > box.x0 && box.y1 > box.y0 && box.z1 > box.z0;
    r->cost = nonempty ? cost_of(&box) : 0;
    r->big = nonempty && (uint64_t)(box.x1 - box.x0) * (box.y1 - box.y0) * (box.z1 - box.z0) >= kBigVoxels;
    if (r->big) s->q_big++;
    else s->q_small++;
    r->t_submit = now_us();
    int64_t ticket = (int64_t)s->n++;
    pthread_cond_broadcast(&s->work_cv);
    pthread_mutex_unlock(&s->mu);
    return ticket;
}

// Block until the ticket is decoded; returns its status (vc_decode_region's),
// and the submit-to-completion latency in microseconds. A ticket can be waited
// for once: its slot is recycled afterwards (VC_ERR_RANGE on a second wait).
VC_API vc_status vcg_server_wait(vcg_server *s, int64_t ticket, double *latency_us) {
    if (!s || ticket < 0) return VC_ERR_RANGE;
    pthread_mutex_lock(&s->mu);
    if ((uint64_t)ticket >= s->n || (uint64_t)ticket < s->base || slot(s, (uint64_t)ticket)->state == 3) {
        pthread_mutex_unlock(&s->mu);
        return VC_ERR_RANGE;
    }
    while (slot(s, (uint64_t)ticket)->state != 2) pthread_cond_wait(&s->done_cv, &s->mu);
    srv_req *r = slot(s, (uint64_t)ticket);
    vc_status st = r->status;
    if (latency_us) *latency_us = r->t_done - r->t_submit;
    r->state = 3;
    while (s->lo < s->n && slot(s, s->lo)->state == 3) ++s->lo;
    pthread_mutex_unlock(&s->mu);
    return st;
}

// Batches run and requests they carried so far.
VC_API void vcg_server_stats(vcg_server *s, uint64_t *batches, uint64_t *requests) {
    if (!s) return;
    pthread_mutex_lock(&s->mu);
    if (batches) *batches = s->batches;
    if (requests) *requests = s->batched_reqs;
    pthread_mutex_unlock(&s->mu);
}

// Finishes every queued request, then stops the workers.
VC_API void vcg_server_destroy(vcg_server *s) {
    if (!s) return;
    pthread_mutex_lock(&s->mu);
    s->stop = 1;
    pthread_cond_broadcast(&s->work_cv);
    pthread_mutex_unlock(&s->mu);
    for (int i = 0; i < s->nworkers; ++i) pthread_join(s->th[i], NULL);
    pthread_mutex_destroy(&s->mu);
    pthread_cond_destroy(&s->work_cv);
    pthread_cond_destroy(&s->done_cv);
    free_workers(s);
    free(s->reqs);
    free(s);
}

// The vc.h writer (src/vc/vc.c:995-1245) with the encoding on the GPU.
//
// The archive image lives in the file, mapped once over a large reservation
// (MAP_NORESERVE) so its base never moves; the file grows by ftruncate and is
// trimmed to the append cursor on close. Appends use group commit: a call
// queues its atoms (with the LOD's base_q as read at the call) and waits; one
// caller at a time takes everything queued, encodes it on the device in one
// batch (vcd_encode_segments) and lays it out on the host in queue order with
// the reference's rules: the first touch of an index region reserves its
// 512 KiB slot block at the cursor, a payload goes to the cursor, the slot
// records it. A single thread therefore produces the reference's bytes. The
// readers decode on the device through a live view of the image (vc_host.c).
#include <fcntl.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <unistd.h>

#include "../../include/vcg.h"
#include "vc_internal.h"
#include "vc_view.h"

#define VC_API __attribute__((visibility("default")))

// src/vc/vc.c:567-575, 660-718, 774
#define FILE_HDR 128u
#define MAGIC 0x00314356u
#define R_ATOMS 32u
#define L2_BYTES (32768ull * 16ull)
#define NO_OFFSET 0xFFFFFFFFFFFFFFFFull
#define ZERO_REGION 1ull
#define L1_INIT_CAP 1024ull
#define RESERVE (10ull << 40)
#define GROW_STEP (64ull << 20)
#define MAX_Q 256   // distinct base_q values in one device batch
#define ASYNC_BATCH 8192   // queued asynchronous atoms that make their caller commit

static inline uint64_t rd64(const uint8_t *p) { uint64_t v; memcpy(&v, p, 8); return v; }
static inline void wr64(uint8_t *p, uint64_t v) { memcpy(p, &v, 8); }
static inline void wr32(uint8_t *p, uint32_t v) { memcpy(p, &v, 4); }

typedef struct wreq {   // one append call waiting for its batch
    int lod, box;
    int async;              // 1: queued by vcg_append_atom_async (vox owned, nobody waits); 2: flush barrier
    uint32_t az, ay, ax;    // atom (box == 0)
    vc_box b;               // box (box == 1)
    const uint8_t *vox;
    float q;                // base_q of the LOD when the call was made (0: none)
    vc_status status;
    int done;
    struct wreq *next;
} wreq;

struct vc_writer {
    int fd;
    uint8_t *map;
    uint64_t map_len, file_len, cursor, l1_cap;
    vc_dims d0;
    int nlod;
    uint32_t qbits[VC_NLOD];      // base_q per LOD (float bits)
    pthread_mutex_t mu;           // every change of the image
    pthread_rwlock_t rw;          // readers (shared) / writes into the image (exclusive)
    pthread_mutex_t qmu;          // the queue
    pthread_cond_t qcv;
    wreq *head, *tail;
    int leader;
    uint64_t queued_async;        // asynchronous atoms in the queue
    uint64_t async_failed;        // since the last flush
    vc_status async_first;
    vc_archive *view;
    uint8_t *stack;               // single atoms of a batch, stacked
    size_t stack_cap;
};

static vc_dims lod_dims(vc_dims d, int lod) {   // src/vc/vc.c:733-739
    for (int i = 0; i < lod; ++i) { d.nx = (d.nx + 1) / 2; d.ny = (d.ny + 1) / 2; d.nz = (d.nz + 1) / 2; }
    return d;
}

static int dims_ok(vc_dims d) {
    return d.nx && d.ny && d.nz && d.nx <= VC_MAX_DIM && d.ny <= VC_MAX_DIM && d.nz <= VC_MAX_DIM;
}

static float q_of(const vc_writer *w, int lod) {
    uint32_t b = __atomic_load_n(&w->qbits[lod], __ATOMIC_ACQUIRE);
    float f;
    memcpy(&f, &b, 4);
    return f;
}

static void view_sync(vc_writer *w) {   // caller holds rw exclusively
    float q[VC_NLOD];
    for (int l = 0; l < VC_NLOD; ++l) q[l] = l < w->nlod ? q_of(w, l) : 0.0f;
    vch_view_set(w->view, w->cursor, q);
}

static vc_status view_read(void *ud, uint64_t off, uint32_t len, uint8_t *dst) {
    vc_writer *w = (vc_writer *)ud;   // called with rw held shared
    if (off > w->cursor || len > w->cursor - off) return VC_ERR_FORMAT;
    memcpy(dst, w->map + off, len);
    return VC_OK;
}

// ---------------------------------------------------------------- image (mu held)

static int grow(vc_writer *w, uint64_t need) {   // src/vc/vc.c:806-831
    if (need <= w->file_len) return 0;
    if (need > w->map_len) return -1;
    uint64_t nl = w->file_len;
    while (nl < need) nl += GROW_STEP;
    if (nl > w->map_len) nl = w->map_len;
    if (ftruncate(w->fd, (off_t)nl) != 0) return -1;
    w->file_len = nl;
    return 0;
}

static uint64_t take(vc_writer *w, uint64_t n) {   // bytes at the cursor; 0 on failure (src/vc/vc.c:835-841)
    const uint64_t off = w->cursor;
    if (grow(w, off + n) != 0) return 0;
    w->cursor = off + n;
    return off;
}

// the L1 bucket holding key, else the first empty one on its probe path; NULL
// when the table is full without it (the reference probes forever)
static uint8_t *bucket(vc_writer *w, uint64_t key) {
    const uint64_t mask = w->l1_cap - 1;
    uint64_t i = vch_mix64(key) & mask;
    for (uint64_t s = 0; s < w->l1_cap; ++s, i = (i + 1) & mask) {
        uint8_t *e = w->map + FILE_HDR + i * 16;
        if (!rd64(e + 8) || rd64(e) == key) return e;
    }
    return NULL;
}

// A region's block, created on first touch, a known-zero region promoted to
// a real block when `promote` (src/vc/vc.c:897-955, 1111-1126); ZERO_REGION,
// or 0 on failure.
static uint64_t region(vc_writer *w, uint64_t key, int promote) {
    uint8_t *e = bucket(w, key);
    if (!e) return 0;
    const uint64_t bref = rd64(e + 8);
    if (bref && bref != ZERO_REGION) return bref;
    if (bref == ZERO_REGION && !promote) return ZERO_REGION;
    const uint64_t nb = take(w, L2_BYTES);
    if (!nb) return 0;
    memset(w->map + nb, 0, L2_BYTES);
    if (!bref) {
        wr64(e, key);
        wr64(w->map + 48, rd64(w->map + 48) + 1);   // regions in the table
    }
    wr64(e + 8, nb);
    return nb;
}

static uint8_t *slot(vc_writer *w, uint64_t blk, uint32_t az, uint32_t ay, uint32_t ax) {
    return w->map + blk + ((((uint64_t)(az & 31) * 32 + (ay & 31)) * 32 + (ax & 31)) * 16);
}

static void slot_zero(uint8_t *s) {   // src/vc/vc.c:1133-1141
    wr64(s, NO_OFFSET);
    wr32(s + 8, 0);
    s[13] = 0;
    s[12] = 2;
}

// one atom laid out in call order (src/vc/vc.c:1082-1159); len 0 = all-zero
static vc_status lay_atom(vc_writer *w, int lod, uint32_t az, uint32_t ay, uint32_t ax, uint32_t len,
                          const uint8_t *pay, float q) {
    if (len && !(q > 0.0f)) return VC_ERR_RANGE;   // a nonzero atom needs base_q (src/vc/vc.c:1100)
    const uint64_t blk = region(w, vch_region_key(lod, az / R_ATOMS, ay / R_ATOMS, ax / R_ATOMS), 1);
    if (!blk) return VC_ERR_OOM;
    uint8_t *s = slot(w, blk, az, ay, ax);
    if (!len) {
        slot_zero(s);
        return VC_OK;
    }
    const uint64_t poff = take(w, len);
    if (!poff) return VC_ERR_OOM;
    memcpy(w->map + poff, pay, len);
    wr32(s + 8, len);
    s[12] = 1;
    s[13] = pay[0];   // dc
    wr64(s, poff);
    return VC_OK;
}

// ---------------------------------------------------------------- batches

static uint32_t box_atoms(const vc_box *b) {
    return ((b->x1 - b->x0) / 32) * ((b->y1 - b->y0) / 32) * ((b->z1 - b->z0) / 32);
}

// Encode and lay out the requests of `batch` in order; returns the requests
// left for the next batch (more distinct base_q values than one batch takes).
static wreq *commit(vc_writer *w, wreq *batch) {
    float qs[MAX_Q];
    uint32_t qb[MAX_Q];
    int nq = 0;
    uint64_t n1 = 0, nbox = 0;
    wreq *r = batch, *last = NULL;
    for (; r; last = r, r = r->next) {   // take requests while their q fits the table
        if (r->async == 2) continue;
        const float q = r->q > 0.0f ? r->q : 1.0f;   // without base_q: encoded only to see whether it is all-zero
        uint32_t b;
        memcpy(&b, &q, 4);
        int k = 0;
        while (k < nq && qb[k] != b) ++k;
        if (k == nq) {
            if (nq == MAX_Q) break;
            qb[nq] = b;
            qs[nq++] = q;
        }
        if (r->async == 2) continue;
        if (r->box) ++nbox;
        else ++n1;
    }
    wreq *rest = r;
    if (last) last->next = NULL;
    const int nseg = (n1 ? 1 : 0) + (int)nbox;   // flush barriers carry no atoms
    vcd_seg *segs = (vcd_seg *)calloc(nseg ? nseg : 1, sizeof(vcd_seg));
    vc_status fail = segs ? VC_OK : VC_ERR_OOM;
    if (fail == VC_OK && n1 > w->stack_cap) {
        uint8_t *ns = (uint8_t *)realloc(w->stack, n1 * VC_ATOM3);
        if (ns) { w->stack = ns; w->stack_cap = n1; }
        else fail = VC_ERR_OOM;
    }
    int sg = 0;
    if (fail == VC_OK && n1) {
        vcd_seg *S = &segs[sg++];
        S->vox = w->stack;
        S->nx = 32; S->ny = 32; S->nz = (uint32_t)(32 * n1);
        uint8_t *qsel = (uint8_t *)malloc(n1);
        S->qsel = qsel;
        S->len = (uint32_t *)malloc(n1 * 4);
        S->off = (uint64_t *)malloc(n1 * 8);
        if (!qsel || !S->len || !S->off) fail = VC_ERR_OOM;
        uint64_t i = 0;
        for (wreq *x = batch; x && fail == VC_OK; x = x->next) {
            if (x->box || x->async == 2) continue;
            memcpy(w->stack + i * VC_ATOM3, x->vox, VC_ATOM3);
            const float q = x->q > 0.0f ? x->q : 1.0f;
            uint32_t b;
            memcpy(&b, &q, 4);
            int k = 0;
            while (qb[k] != b) ++k;
            qsel[i++] = (uint8_t)k;
        }
    }
    for (wreq *x = batch; x && fail == VC_OK; x = x->next) {
        if (!x->box || x->async == 2) continue;
        vcd_seg *S = &segs[sg++];
        const uint64_t na = box_atoms(&x->b);
        S->vox = x->vox;
        S->nx = x->b.x1 - x->b.x0; S->ny = x->b.y1 - x->b.y0; S->nz = x->b.z1 - x->b.z0;
        uint8_t *qsel = (uint8_t *)malloc(na);
        S->qsel = qsel;
        S->len = (uint32_t *)malloc(na * 4);
        S->off = (uint64_t *)malloc(na * 8);
        if (!qsel || !S->len || !S->off) { fail = VC_ERR_OOM; break; }
        const float q = x->q > 0.0f ? x->q : 1.0f;
        uint32_t b;
        memcpy(&b, &q, 4);
        int k = 0;
        while (qb[k] != b) ++k;
        memset(qsel, k, na);
    }
    uint8_t *pay = NULL;
    uint64_t pay_bytes = 0;
    if (fail == VC_OK && nseg) {
        if (vcd_init() != 0) fail = VC_ERR_IO;
        else {
            const int e = vcd_encode_segments(segs, nseg, qs, nq, &pay, &pay_bytes);
            if (e) fail = (vc_status)e;
        }
    }
    pthread_rwlock_wrlock(&w->rw);
    sg = n1 ? 1 : 0;
    uint64_t i1 = 0;
    for (wreq *x = batch; x; x = x->next) {
        if (x->async == 2) { x->status = VC_OK; continue; }
        if (fail != VC_OK) { x->status = fail; continue; }
        if (!x->box) {
            const vcd_seg *S = &segs[0];
            x->status = lay_atom(w, x->lod, x->az, x->ay, x->ax, S->len[i1], pay + S->off[i1], x->q);
            ++i1;
            continue;
        }
        const vcd_seg *S = &segs[sg++];
        const uint32_t ax0 = x->b.x0 / 32, ay0 = x->b.y0 / 32, az0 = x->b.z0 / 32;
        const uint32_t nx = S->nx / 32, ny = S->ny / 32, nz = S->nz / 32;
        x->status = VC_OK;
        for (uint32_t z = 0; z < nz && x->status == VC_OK; ++z)   // src/vc/vc.c:1170-1189: (z, y, x) order
            for (uint32_t y = 0; y < ny && x->status == VC_OK; ++y)
                for (uint32_t xx = 0; xx < nx && x->status == VC_OK; ++xx) {
                    const uint64_t t = ((uint64_t)z * ny + y) * nx + xx;
                    x->status = lay_atom(w, x->lod, az0 + z, ay0 + y, ax0 + xx, S->len[t], pay + S->off[t], x->q);
                }
    }
    view_sync(w);
    pthread_rwlock_unlock(&w->rw);
    for (int k = 0; k < nseg && segs; ++k) {
        free((void *)segs[k].qsel);
        free(segs[k].len);
        free(segs[k].off);
    }
    free(segs);
    return rest;
}

// Take the queue and commit it; called with qmu held and no leader, returns
// with qmu held. Asynchronous requests are accounted and freed here.
static void lead(vc_writer *w) {
    w->leader = 1;
    wreq *batch = w->head;
    w->head = w->tail = NULL;
    pthread_mutex_unlock(&w->qmu);
    pthread_mutex_lock(&w->mu);
    wreq *rest = commit(w, batch);
    pthread_mutex_unlock(&w->mu);
    pthread_mutex_lock(&w->qmu);
    for (wreq *x = batch, *nx; x && x != rest; x = nx) {
        nx = x->next;
        if (x->async == 1) {
            if (x->status != VC_OK) {
                if (!w->async_failed) w->async_first = x->status;
                ++w->async_failed;
            }
            --w->queued_async;
            free(x);   // the atom copy lives in the same allocation
        } else {
            x->done = 1;
        }
    }
    if (rest) {   // back to the front of the queue, in order
        wreq *t = rest;
        while (t->next) t = t->next;
        t->next = w->head;
        if (!w->head) w->tail = t;
        w->head = rest;
    }
    w->leader = 0;
    pthread_cond_broadcast(&w->qcv);
}

static void enqueue(vc_writer *w, wreq *r) {   // qmu held
    r->next = NULL;
    r->done = 0;
    if (w->tail) w->tail->next = r;
    else w->head = r;
    w->tail = r;
}

static vc_status submit(vc_writer *w, wreq *r) {
    pthread_mutex_lock(&w->qmu);
    enqueue(w, r);
    while (!r->done) {
        if (w->leader) pthread_cond_wait(&w->qcv, &w->qmu);
        else lead(w);
    }
    pthread_mutex_unlock(&w->qmu);
    return r->status;
}

// ---------------------------------------------------------------- API

VC_API vc_writer *vc_create(const char *path, vc_dims lod0_dims, float target_ratio) {   // src/vc/vc.c:995-1073
    VCD_SCOPE();
    if (!path || !dims_ok(lod0_dims) || target_ratio < 1.0f) return NULL;
    int nlod = 1;
    for (int l = 1; l < VC_NLOD; ++l) {
        const vc_dims d = lod_dims(lod0_dims, l);
        nlod = l + 1;
        if (d.nx <= 1 && d.ny <= 1 && d.nz <= 1) break;
    }
    uint64_t regions = 0;
    for (int l = 0; l < nlod; ++l) {
        const vc_dims d = lod_dims(lod0_dims, l);
        regions += (uint64_t)(((d.nx + 31) / 32 + 31) / 32) * (((d.ny + 31) / 32 + 31) / 32) *
                   (((d.nz + 31) / 32 + 31) / 32);
    }
    uint64_t cap = L1_INIT_CAP;
    while (cap < regions * 2) cap <<= 1;   // never rehashed
    const uint64_t init_len = FILE_HDR + cap * 16;
    const int fd = open(path, O_RDWR | O_CREAT | O_TRUNC, 0644);
    if (fd < 0) return NULL;
    if (ftruncate(fd, (off_t)init_len) != 0) { close(fd); return NULL; }
    uint8_t *map = MAP_FAILED;
    uint64_t map_len = RESERVE;
    for (; map_len >= init_len && map_len >= (1ull << 30); map_len >>= 1) {
        map = (uint8_t *)mmap(NULL, map_len, PROT_READ | PROT_WRITE, MAP_SHARED | MAP_NORESERVE, fd, 0);
        if (map != MAP_FAILED) break;
    }
    if (map == MAP_FAILED) { close(fd); return NULL; }
    vc_writer *w = (vc_writer *)calloc(1, sizeof *w);
    if (!w) { munmap(map, map_len); close(fd); return NULL; }
    const uint32_t h32[6] = {MAGIC, 1u, 32u, 1u, R_ATOMS, (uint32_t)nlod};
    memcpy(map, h32, sizeof h32);
    const uint32_t dims[3] = {lod0_dims.nx, lod0_dims.ny, lod0_dims.nz};
    memcpy(map + 24, dims, sizeof dims);
    memcpy(map + 36, &target_ratio, 4);
    const uint64_t h64[4] = {cap, 0, FILE_HDR, init_len};   // L1 capacity, regions, L1 offset, cursor
    memcpy(map + 40, h64, sizeof h64);
    w->fd = fd;
    w->map = map;
    w->map_len = map_len;
    w->file_len = init_len;
    w->cursor = init_len;
    w->l1_cap = cap;
    w->d0 = lod0_dims;
    w->nlod = nlod;
    pthread_mutex_init(&w->mu, NULL);
    pthread_rwlock_init(&w->rw, NULL);
    pthread_mutex_init(&w->qmu, NULL);
    pthread_cond_init(&w->qcv, NULL);
    w->view = vch_view_new(view_read, w, lod0_dims, nlod, FILE_HDR, cap);
    if (!w->view) { vc_writer_close(w); return NULL; }
    view_sync(w);
    return w;
}

VC_API vc_status vc_set_base_q(vc_writer *w, int lod, float q) {   // src/vc/vc.c:1075-1080
    VCD_SCOPE();
    if (!w || lod < 0 || lod >= w->nlod || isnan(q)) return VC_ERR_RANGE;
    if (q < 0.05f) q = 0.05f;
    if (q > 4096.0f) q = 4096.0f;
    pthread_mutex_lock(&w->mu);
    pthread_rwlock_wrlock(&w->rw);
    memcpy(w->map + 72 + 4 * lod, &q, 4);
    uint32_t b;
    memcpy(&b, &q, 4);
    __atomic_store_n(&w->qbits[lod], b, __ATOMIC_RELEASE);
    view_sync(w);
    pthread_rwlock_unlock(&w->rw);
    pthread_mutex_unlock(&w->mu);
    return VC_OK;
}

VC_API vc_status vc_append_atom(vc_writer *w, int lod, uint32_t az, uint32_t ay, uint32_t ax,
                                const uint8_t vox[VC_ATOM3]) {   // src/vc/vc.c:1161-1168
    VCD_SCOPE();
    if (!w || lod < 0 || lod >= w->nlod || !vox) return VC_ERR_RANGE;
    const vc_dims d = lod_dims(w->d0, lod);
    if (ax >= (d.nx + 31) / 32 || ay >= (d.ny + 31) / 32 || az >= (d.nz + 31) / 32) return VC_ERR_RANGE;
    wreq r;
    memset(&r, 0, sizeof r);
    r.lod = lod; r.az = az; r.ay = ay; r.ax = ax;
    r.vox = vox;
    r.q = q_of(w, lod);
    return submit(w, &r);
}

VC_API vc_status vc_append_box(vc_writer *w, int lod, vc_box b, const uint8_t *voxels) {   // src/vc/vc.c:1170-1189
    VCD_SCOPE();
    if (!w || lod < 0 || lod >= w->nlod || !voxels) return VC_ERR_RANGE;
    if (b.x0 % 32 || b.y0 % 32 || b.z0 % 32) return VC_ERR_RANGE;
    if ((b.x1 - b.x0) % 32 || (b.y1 - b.y0) % 32 || (b.z1 - b.z0) % 32) return VC_ERR_RANGE;
    if (b.x1 <= b.x0 || b.y1 <= b.y0 || b.z1 <= b.z0) return VC_ERR_RANGE;
    // as in the reference, the box is not checked against the LOD: its atoms go
    // in (z, y, x) order straight to the layout (src/vc/vc.c:1180-1187)
    wreq r;
    memset(&r, 0, sizeof r);
    r.lod = lod; r.box = 1; r.b = b; r.vox = voxels; r.q = q_of(w, lod);
    return submit(w, &r);
}

VC_API vc_status vcg_append_atom_async(vc_writer *w, int lod, uint32_t az, uint32_t ay, uint32_t ax,
                                       const uint8_t vox[VC_ATOM3]) {
    VCD_SCOPE();
    if (!w || lod < 0 || lod >= w->nlod || !vox) return VC_ERR_RANGE;
    const vc_dims d = lod_dims(w->d0, lod);
    if (ax >= (d.nx + 31) / 32 || ay >= (d.ny + 31) / 32 || az >= (d.nz + 31) / 32) return VC_ERR_RANGE;
    wreq *r = (wreq *)malloc(sizeof(wreq) + VC_ATOM3);
    if (!r) return VC_ERR_OOM;
    memset(r, 0, sizeof *r);
    uint8_t *own = (uint8_t *)(r + 1);
    memcpy(own, vox, VC_ATOM3);
    r->lod = lod; r->az = az; r->ay = ay; r->ax = ax;
    r->vox = own;
    r->q = q_of(w, lod);
    r->async = 1;
    pthread_mutex_lock(&w->qmu);
    enqueue(w, r);
    if (++w->queued_async >= ASYNC_BATCH && !w->leader) lead(w);
    pthread_mutex_unlock(&w->qmu);
    return VC_OK;
}

VC_API vc_status vcg_writer_flush(vc_writer *w, uint64_t *failed) {
    VCD_SCOPE();
    if (failed) *failed = 0;
    if (!w) return VC_ERR_RANGE;
    wreq r;
    memset(&r, 0, sizeof r);
    r.async = 2;
    submit(w, &r);
    pthread_mutex_lock(&w->qmu);
    const vc_status s = w->async_failed ? w->async_first : VC_OK;
    if (failed) *failed = w->async_failed;
    w->async_failed = 0;
    pthread_mutex_unlock(&w->qmu);
    return s;
}

VC_API vc_status vc_mark_zero_atom(vc_writer *w, int lod, uint32_t az, uint32_t ay, uint32_t ax) {   // :1191-1205
    VCD_SCOPE();
    if (!w || lod < 0 || lod >= w->nlod) return VC_ERR_RANGE;
    pthread_mutex_lock(&w->mu);
    pthread_rwlock_wrlock(&w->rw);
    vc_status s = VC_OK;
    const uint64_t blk = region(w, vch_region_key(lod, az / R_ATOMS, ay / R_ATOMS, ax / R_ATOMS), 0);
    if (!blk) s = VC_ERR_OOM;
    else if (blk != ZERO_REGION) slot_zero(slot(w, blk, az, ay, ax));
    view_sync(w);
    pthread_rwlock_unlock(&w->rw);
    pthread_mutex_unlock(&w->mu);
    return s;
}

VC_API vc_status vc_mark_zero_region(vc_writer *w, int lod, uint32_t rz, uint32_t ry, uint32_t rx) {   // :1207-1229
    VCD_SCOPE();
    if (!w || lod < 0 || lod >= w->nlod) return VC_ERR_RANGE;
    pthread_mutex_lock(&w->mu);
    pthread_rwlock_wrlock(&w->rw);
    const uint64_t key = vch_region_key(lod, rz, ry, rx);
    uint8_t *e = bucket(w, key);
    vc_status s = VC_OK;
    if (!e) s = VC_ERR_OOM;
    else if (!rd64(e + 8)) {   // a region that has a block (or is zero already) keeps it
        wr64(e, key);
        wr64(e + 8, ZERO_REGION);
        wr64(w->map + 48, rd64(w->map + 48) + 1);
    }
    pthread_rwlock_unlock(&w->rw);
    pthread_mutex_unlock(&w->mu);
    return s;
}

VC_API vc_status vc_writer_decode_atom(vc_writer *w, int lod, uint32_t az, uint32_t ay, uint32_t ax,
                                       uint8_t out[VC_ATOM3]) {   // src/vc/vc.c:1484-1493
    VCD_SCOPE();
    if (!w || lod < 0 || lod >= w->nlod || !out) return VC_ERR_RANGE;
    pthread_rwlock_rdlock(&w->rw);
    const vc_status s = vc_decode_atom(w->view, lod, (int)ax, (int)ay, (int)az, out);
    pthread_rwlock_unlock(&w->rw);
    return s;
}

VC_API vc_cover vc_writer_coverage(vc_writer *w, int lod, uint32_t az, uint32_t ay, uint32_t ax) {   // :1496-1503
    if (!w || lod < 0 || lod >= w->nlod) return VC_ABSENT;
    pthread_rwlock_rdlock(&w->rw);
    const vc_cover c = vc_atom_coverage(w->view, lod, az, ay, ax);
    pthread_rwlock_unlock(&w->rw);
    return c;
}

VC_API vc_status vc_writer_decode_2x2x2(vc_writer *w, int lod, uint32_t az0, uint32_t ay0, uint32_t ax0,
                                        uint8_t out8[8][VC_ATOM3], int *any) {   // src/vc/vc.c:1507-1530
    VCD_SCOPE();
    if (!w || lod < 0 || lod >= w->nlod || !out8) return VC_ERR_RANGE;
    pthread_rwlock_rdlock(&w->rw);
    const vc_status s = vch_view_decode_2x2x2(w->view, lod, az0, ay0, ax0, out8, any);
    pthread_rwlock_unlock(&w->rw);
    return s;
}

VC_API void vc_writer_close(vc_writer *w) {   // src/vc/vc.c:1231-1245
    VCD_SCOPE();
    if (!w) return;
    vcg_writer_flush(w, NULL);   // asynchronous appends still queued
    pthread_mutex_lock(&w->mu);
    wr64(w->map + 64, w->cursor);
    msync(w->map, w->file_len, MS_SYNC);
    munmap(w->map, w->map_len);
    if (w->cursor < w->file_len && ftruncate(w->fd, (off_t)w->cursor) != 0) { /* the reference ignores it too */ }
    close(w->fd);
    pthread_mutex_unlock(&w->mu);
    if (w->view) vc_close(w->view);
    free(w->stack);
    pthread_mutex_destroy(&w->mu);
    pthread_rwlock_destroy(&w->rw);
    pthread_mutex_destroy(&w->qmu);
    pthread_cond_destroy(&w->qcv);
    free(w);
}

// Host half of the GB300 volume codec: the vc.h API, archive header parsing and
// validation, atom resolution through the v1 hash index / v2 directory, and the
// small per-q tables the kernels consume. All voxel work (encode and decode)
// is delegated to the CUDA device layer through vc_internal.h; nothing here
// decodes or encodes an atom.
#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/vcg.h"
#include "vc_internal.h"
#include "vc_release_tables.h"

#define VC_API __attribute__((visibility("default")))

// ---------------------------------------------------------------------------
// Archive format constants (src/vc/vc.c:567-575, 660-718)
// ---------------------------------------------------------------------------
#define FILE_HDR 128u
#define MAGIC 0x00314356u
#define R_ATOMS 32u
#define L2_BYTES (32768ull * 16ull)
#define NO_OFFSET 0xFFFFFFFFFFFFFFFFull
#define ZERO_REGION 1ull

static void (*g_hook)(const char *) = NULL;
VC_API void vc_set_panic_hook(void (*hook)(const char *)) { g_hook = hook; }
VC_API uint32_t vc_region_atoms(void) { return R_ATOMS; }

static void report(const char *fmt, ...) {
    char msg[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    if (g_hook) g_hook(msg);
    fprintf(stderr, "vc: %s\n", msg);
}

static inline uint32_t rd32(const uint8_t *p) { uint32_t v; memcpy(&v, p, 4); return v; }
static inline uint64_t rd64(const uint8_t *p) { uint64_t v; memcpy(&v, p, 8); return v; }
static inline float f_of(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static inline uint32_t b_of(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

// src/vc/vc.c:721-730
uint64_t vch_mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
uint64_t vch_region_key(int lod, uint32_t rz, uint32_t ry, uint32_t rx) {
    return ((uint64_t)(lod & 7) << 45) | ((uint64_t)(rz & 0x7FFF) << 30) |
           ((uint64_t)(ry & 0x7FFF) << 15) | (uint64_t)(rx & 0x7FFF);
}

static vc_dims lod_dims_of(vc_dims d, int lod) {   // src/vc/vc.c:733-739
    for (int i = 0; i < lod; ++i) { d.nx = (d.nx + 1) / 2; d.ny = (d.ny + 1) / 2; d.nz = (d.nz + 1) / 2; }
    return d;
}
static void region_grid(vc_dims d0, int lod, uint32_t *nrz, uint32_t *nry, uint32_t *nrx) {
    vc_dims d = lod_dims_of(d0, lod);
    *nrx = ((d.nx + 31) / 32 + R_ATOMS - 1) / R_ATOMS;
    *nry = ((d.ny + 31) / 32 + R_ATOMS - 1) / R_ATOMS;
    *nrz = ((d.nz + 31) / 32 + R_ATOMS - 1) / R_ATOMS;
}
static int dims_valid(vc_dims d) {
    return d.nx && d.ny && d.nz && d.nx <= VC_MAX_DIM && d.ny <= VC_MAX_DIM && d.nz <= VC_MAX_DIM;
}

// ---------------------------------------------------------------------------
// Per-q tables. The quantiser step of raster index i is base_q * g_step[i]; the
// release build's g_step holds one of two floats per frequency (step class =
// f + 94*alt). These helpers evaluate exactly the float operations of the
// reference's release build (compiled with -ffp-contract=off).
// ---------------------------------------------------------------------------
static float class_g(int cls) {
    int f = cls % 94, alt = cls / 94;
    return f_of(alt ? vc_step_alt_bits[f] : vc_step_base_bits[f]);
}

// RCPPS estimate: a function of the top 11 mantissa bits, scaled by the exponent.
static float rcp_est(float x) {
    uint32_t b = b_of(x), e = (b >> 23) & 0xFFu, r = vc_rcp_est_bits[(b >> 12) & 0x7FFu];
    uint32_t re = ((r >> 23) & 0xFFu) - (e - 127u);
    return f_of((b & 0x80000000u) | (re << 23) | (r & 0x7FFFFFu));
}

void vch_quant_consts(float base_q, vcd_quant *q) {
    for (int c = 0; c < VCD_NCLASS; ++c) {
        float step = base_q * class_g(c);
        float r = rcp_est(step);
        q->step[c] = step;
        q->dz[c] = 0.8f * step;
        q->rr[c] = (r + r) - r * (r * step);
    }
}

void vch_dq_consts(float base_q, vcd_dq *dq) {   // src/vc/vc.c:318-326
    const float c = (0.4f - 1.0f) + 0.8f;
    for (int k = 0; k < VCD_NCLASS; ++k) {
        float step = base_q * class_g(k);
        dq->step[k] = (int32_t)lrintf(step * 256.0f);
        dq->bias[k] = (int32_t)lrintf(c * step * 256.0f);
    }
}

float vch_clamp_q(float q) {   // src/vc/vc.c:1072-1073
    if (q < 0.05f) q = 0.05f;
    if (q > 4096.0f) q = 4096.0f;
    return q;
}

static uint32_t n2(int s) { return (s < 0 || s > 62) ? 0u : (uint32_t)((s < 62 - s ? s : 62 - s) + 1); }

void vch_tables(vcd_tables *t) {
    memcpy(t->alt_mask, vc_step_alt_mask, sizeof t->alt_mask);
    // scan order: ascending L1 frequency, ties by raster index (src/vc/vc.c:258-288)
    uint32_t first[95] = {0};
    for (uint32_t r = 0; r < 32768; ++r) first[(r >> 10) + ((r >> 5) & 31) + (r & 31) + 1]++;
    for (int f = 1; f <= 94; ++f) first[f] += first[f - 1];
    uint32_t fill[94];
    memcpy(fill, first, sizeof fill);
    for (uint32_t r = 0; r < 32768; ++r) t->scan[fill[(r >> 10) + ((r >> 5) & 31) + (r & 31)]++] = (uint16_t)r;
    // rank_base[f][kz]: scan position of the first index with frequency f and
    // plane kz (the one with the smallest valid ky)
    for (int f = 0; f < 94; ++f) {
        uint32_t acc = first[f];
        for (int kz = 0; kz < 32; ++kz) {
            t->rank_base[f * 32 + kz] = (uint16_t)(acc > 65535 ? 65535 : acc);
            acc += n2(f - kz);
        }
    }
    // significance band b holds frequencies [12b, 12b+11] (b = 7: >= 84) (src/vc/vc.c:462-468)
    for (int b = 0; b < 8; ++b) t->band_start[b] = first[12 * b];
    t->band_start[8] = 32768;
}

// ---------------------------------------------------------------------------
// Reader (src/vc/vc.c:1250-1555)
// ---------------------------------------------------------------------------
struct vc_archive {
    const uint8_t *buf;     // flat archive (vc_open), or the pulled copy of a resident streaming one
    size_t len;
    vc_read_fn read;        // streaming byte source (vc_open_streaming), else NULL
    void *ud;
    uint8_t *own;           // buf when pulled through read
    uint8_t hdr[FILE_HDR];
    vc_dims d0;
    int nlod, version;
    uint64_t l1_off, l1_cap, dir_off, region_prefix[VC_NLOD + 1];
    float base_q[VC_NLOD];
    // device residency, built on first decode
    pthread_mutex_t mu;
    int resident;           // 0 not (yet), 1 ok
    vcd_atom *atoms;        // all LODs, LOD-major, raster (az, ay, ax) within a LOD
    uint64_t lod_base[VC_NLOD + 1];
    vcd_archive *dev;
    vcd_archive *sdev;      // streamed decode: dequantisation tables only
    int view;               // a writer's live view: no streaming payload limit, bad slots of a 2x2x2 read as empty
};

// Bytes [off, off + len) of the archive: a pointer into a flat archive's
// buffer, or tmp filled by the read callback; NULL when the range lies outside
// a flat archive or the read fails (src/vc/vc.c:1262-1267).
static const uint8_t *at(const vc_archive *a, uint64_t off, uint32_t len, uint8_t *tmp) {
    const uint8_t *buf = __atomic_load_n(&a->buf, __ATOMIC_ACQUIRE);
    if (buf) return (off > a->len || len > a->len - off) ? NULL : buf + off;
    return a->read(a->ud, off, len, tmp) == VC_OK ? tmp : NULL;
}

static int parse_header(vc_archive *a, const uint8_t *h, uint64_t len) {   // src/vc/vc.c:1285-1314
    if (rd32(h + 0) != MAGIC || rd32(h + 8) != 32 || rd32(h + 16) != R_ATOMS) return -1;
    uint32_t ver = rd32(h + 4), nlod = rd32(h + 20);
    if (nlod == 0 || nlod > VC_NLOD) return -1;
    a->len = len;
    a->nlod = (int)nlod;
    a->d0.nx = rd32(h + 24); a->d0.ny = rd32(h + 28); a->d0.nz = rd32(h + 32);
    for (int l = 0; l < VC_NLOD; ++l) a->base_q[l] = f_of(rd32(h + 72 + 4 * l));
    if (ver == 2) {
        a->version = 2;
        a->dir_off = rd64(h + 40);
        uint64_t cnt = rd64(h + 48), acc = 0;
        if (a->dir_off > len || cnt > (len - a->dir_off) / 16) return -1;
        for (int l = 0; l < a->nlod; ++l) {
            a->region_prefix[l] = acc;
            uint32_t z, y, x;
            region_grid(a->d0, l, &z, &y, &x);
            acc += (uint64_t)z * y * x;
        }
        a->region_prefix[a->nlod] = acc;
        return acc == cnt ? 0 : -1;
    }
    if (ver != 1 || rd32(h + 12) != 1) return -1;
    a->version = 1;
    a->l1_off = rd64(h + 56);
    a->l1_cap = rd64(h + 40);
    if (!a->l1_cap || (a->l1_cap & (a->l1_cap - 1))) return -1;
    if (a->l1_off > len || a->l1_cap > (len - a->l1_off) / 16) return -1;
    return 0;
}

VC_API vc_archive *vc_open(const uint8_t *archive, size_t len) {
    if (!archive || len < FILE_HDR) return NULL;
    vc_archive *a = (vc_archive *)calloc(1, sizeof *a);
    if (!a) return NULL;
    a->buf = archive;
    if (parse_header(a, archive, len) != 0) { free(a); return NULL; }
    memcpy(a->hdr, archive, FILE_HDR);
    pthread_mutex_init(&a->mu, NULL);
    return a;
}

VC_API vc_archive *vc_open_streaming(vc_read_fn read, void *ud, uint64_t total_len) {   // src/vc/vc.c:1329-1338
    if (!read || total_len < FILE_HDR) return NULL;
    vc_archive *a = (vc_archive *)calloc(1, sizeof *a);
    if (!a) return NULL;
    if (read(ud, 0, FILE_HDR, a->hdr) != VC_OK || parse_header(a, a->hdr, total_len) != 0) { free(a); return NULL; }
    a->read = read;
    a->ud = ud;
    pthread_mutex_init(&a->mu, NULL);
    return a;
}

VC_API vc_status vcg_memory_read(void *ud, uint64_t off, uint32_t len, uint8_t *dst) {
    vcg_memory_source *m = (vcg_memory_source *)ud;
    if (!m || !dst || off > m->len || len > m->len - off) return VC_ERR_FORMAT;
    memcpy(dst, m->buf + off, len);
    __atomic_fetch_add(&m->reads, 1, __ATOMIC_RELAXED);
    __atomic_fetch_add(&m->bytes, len, __ATOMIC_RELAXED);
    return VC_OK;
}

VC_API void vc_close(vc_archive *a) {
    VCD_SCOPE();
    if (!a) return;
    if (a->dev) vcd_free_archive(a->dev);
    if (a->sdev) vcd_free_archive(a->sdev);
    free(a->own);
    free(a->atoms);
    pthread_mutex_destroy(&a->mu);
    free(a);
}

VC_API int vc_archive_version(const vc_archive *a) { return a ? a->version : 0; }

VC_API vc_status vc_lod_dims(const vc_archive *a, int lod, vc_dims *out) {
    if (!a || lod < 0 || lod >= a->nlod || !out) return VC_ERR_RANGE;
    *out = lod_dims_of(a->d0, lod);
    return VC_OK;
}

// L2 block of a region: 0 absent, ZERO_REGION, or a block offset that lies in
// the file. The v1 probe is bounded by the table size (the reference loops
// forever on a full table without the key; src/vc/vc.c:1349-1360).
static uint64_t region_block(const vc_archive *a, int lod, uint32_t rz, uint32_t ry, uint32_t rx) {
    uint64_t blk;
    uint8_t tmp[16];
    if (a->version == 2) {
        uint32_t nrz, nry, nrx;
        region_grid(a->d0, lod, &nrz, &nry, &nrx);
        if (rz >= nrz || ry >= nry || rx >= nrx) return 0;
        uint64_t ri = a->region_prefix[lod] + ((uint64_t)rz * nry + ry) * nrx + rx;
        if (ri >= a->region_prefix[a->nlod]) return 0;
        const uint8_t *e = at(a, a->dir_off + ri * 16, 16, tmp);
        if (!e) return 0;
        uint32_t fl = rd32(e + 12);
        if (fl == 0) return 0;
        if (fl == 1) return ZERO_REGION;
        blk = rd64(e);
    } else {
        uint64_t key = vch_region_key(lod, rz, ry, rx), mask = a->l1_cap - 1, i = vch_mix64(key) & mask;
        for (uint64_t step = 0;; ++step) {
            if (step >= a->l1_cap) return 0;
            const uint8_t *e = at(a, a->l1_off + i * 16, 16, tmp);
            if (!e) return 0;
            uint64_t bref = rd64(e + 8);
            if (!bref) return 0;
            if (rd64(e) == key) { blk = bref; break; }
            i = (i + 1) & mask;
        }
        if (blk == ZERO_REGION) return ZERO_REGION;
    }
    if (blk > a->len || L2_BYTES > a->len - blk) return 0;   // corrupt guard (src/vc/vc.c:1389,1400)
    return blk;
}

// slot flags of an atom given its region's block (src/vc/vc.c:1365-1373)
static int slot_of(const vc_archive *a, uint64_t blk, uint32_t az, uint32_t ay, uint32_t ax,
                   uint64_t *off, uint32_t *len, uint8_t *dc) {
    if (blk == 0) return 0;
    if (blk == ZERO_REGION) return 2;
    uint8_t tmp[16];
    const uint8_t *s = at(a, blk + ((((uint64_t)(az & 31) * 32 + (ay & 31)) * 32 + (ax & 31)) * 16), 16, tmp);
    if (!s) return 0;
    uint8_t fl = s[12];
    if (fl == 1) { *off = rd64(s); *len = rd32(s + 8); *dc = s[13]; }
    return fl;
}

static int resolve(const vc_archive *a, int lod, uint32_t az, uint32_t ay, uint32_t ax,
                   uint64_t *off, uint32_t *len, uint8_t *dc) {
    return slot_of(a, region_block(a, lod, az / 32, ay / 32, ax / 32), az, ay, ax, off, len, dc);
}

VC_API vc_cover vc_atom_coverage(const vc_archive *a, int lod, uint32_t az, uint32_t ay, uint32_t ax) {
    if (!a || lod < 0 || lod >= a->nlod) return VC_ABSENT;
    uint64_t off; uint32_t len; uint8_t dc;
    int fl = resolve(a, lod, az, ay, ax, &off, &len, &dc);
    return fl == 1 ? VC_PRESENT : fl == 2 ? VC_KNOWN_ZERO : VC_ABSENT;
}

VC_API vc_cover vc_atom_payload_range(const vc_archive *a, int lod, uint32_t az, uint32_t ay, uint32_t ax,
                                      uint64_t *off, uint32_t *len) {
    if (off) *off = 0;
    if (len) *len = 0;
    if (!a || lod < 0 || lod >= a->nlod) return VC_ABSENT;
    uint64_t o = 0; uint32_t l = 0; uint8_t dc = 0;
    int fl = resolve(a, lod, az, ay, ax, &o, &l, &dc);
    if (fl == 1) { if (off) *off = o; if (len) *len = l; return VC_PRESENT; }
    return fl == 2 ? VC_KNOWN_ZERO : VC_ABSENT;
}

VC_API vc_cover vc_region_blob_range(const vc_archive *a, int lod, uint32_t rz, uint32_t ry, uint32_t rx,
                                     uint64_t *off, uint64_t *len) {   // src/vc/vc.c:1455-1471
    if (off) *off = 0;
    if (len) *len = 0;
    if (!a || a->version != 2 || lod < 0 || lod >= a->nlod) return VC_ABSENT;
    uint32_t nrz, nry, nrx;
    region_grid(a->d0, lod, &nrz, &nry, &nrx);
    if (rz >= nrz || ry >= nry || rx >= nrx) return VC_ABSENT;
    uint64_t ri = a->region_prefix[lod] + ((uint64_t)rz * nry + ry) * nrx + rx;
    if (ri >= a->region_prefix[a->nlod]) return VC_ABSENT;
    uint8_t tmp[16];
    const uint8_t *e = at(a, a->dir_off + ri * 16, 16, tmp);
    if (!e) return VC_ABSENT;
    uint32_t fl = rd32(e + 12);
    if (fl == 1) return VC_KNOWN_ZERO;
    if (fl != 2) return VC_ABSENT;
    if (off) *off = rd64(e);
    if (len) *len = rd32(e + 8);
    return VC_PRESENT;
}

// A streaming archive pulled whole through its read callback into a host copy
// (64 MiB per call); on a failed read it stays streaming.
static int pull_whole(vc_archive *a) {
    uint8_t *b = (uint8_t *)malloc(a->len ? a->len : 1);
    if (!b) return -1;
    for (uint64_t off = 0; off < a->len;) {
        const uint32_t n = a->len - off > (64u << 20) ? (64u << 20) : (uint32_t)(a->len - off);
        if (a->read(a->ud, off, n, b + off) != VC_OK) {
            report("streaming archive: read of %u bytes at %llu failed", n, (unsigned long long)off);
            free(b);
            return -1;
        }
        off += n;
    }
    a->own = b;
    __atomic_store_n(&a->buf, (const uint8_t *)b, __ATOMIC_RELEASE);
    return 0;
}

// Resolve every atom of every LOD once, validate payload ranges, and move the
// archive bytes plus the table into device memory.
// A failed attempt (no device memory, a read that failed) leaves the archive
// not resident, so a later call tries again; the status says why it failed.
static vc_status make_resident(vc_archive *a) {
    pthread_mutex_lock(&a->mu);
    if (a->resident) { pthread_mutex_unlock(&a->mu); return VC_OK; }
    vc_status rc = VC_ERR_IO;
    int e;
    if (vcd_init() != 0) { report("no usable CUDA device: %s", vcd_last_error()); goto done; }
    if (!a->buf && pull_whole(a) != 0) goto done;
    if ((e = vcd_upload_begin(&a->dev, a->buf, a->len)) != 0) {   // the copy runs during the walk below
        report("archive upload failed: %s", vcd_last_error());
        rc = (vc_status)e;
        goto done;
    }
    uint64_t total = 0;
    for (int l = 0; l < a->nlod; ++l) {
        vc_dims d = lod_dims_of(a->d0, l);
        a->lod_base[l] = total;
        total += (uint64_t)((d.nx + 31) / 32) * ((d.ny + 31) / 32) * ((d.nz + 31) / 32);
    }
    a->lod_base[a->nlod] = total;
    a->atoms = (vcd_atom *)calloc(total ? total : 1, sizeof(vcd_atom));
    if (!a->atoms) { rc = VC_ERR_OOM; goto done; }
    vcd_dq dq[VC_NLOD];
    for (int l = 0; l < a->nlod; ++l) {
        vc_dims d = lod_dims_of(a->d0, l);
        uint32_t acx = (d.nx + 31) / 32, acy = (d.ny + 31) / 32, acz = (d.nz + 31) / 32;
        vch_dq_consts(a->base_q[l], &dq[l]);
        for (uint32_t rz = 0; rz * 32 < acz; ++rz)
            for (uint32_t ry = 0; ry * 32 < acy; ++ry)
                for (uint32_t rx = 0; rx * 32 < acx; ++rx) {
                    uint64_t blk = region_block(a, l, rz, ry, rx);
                    for (uint32_t az = rz * 32; az < acz && az < rz * 32 + 32; ++az)
                        for (uint32_t ay = ry * 32; ay < acy && ay < ry * 32 + 32; ++ay)
                            for (uint32_t ax = rx * 32; ax < acx && ax < rx * 32 + 32; ++ax) {
                                uint64_t off = 0; uint32_t len = 0; uint8_t dc = 0;
                                vcd_atom *t = &a->atoms[a->lod_base[l] + ((uint64_t)az * acy + ay) * acx + ax];
                                int fl = slot_of(a, blk, az, ay, ax, &off, &len, &dc);
                                if (fl != 1) { t->kind = VCD_EMPTY; continue; }
                                // src/vc/vc.c:1413, without the wrap-around of off + len
                                if (off == NO_OFFSET || len < 1 || off > a->len || len > a->len - off) {
                                    t->kind = VCD_BAD;
                                    continue;
                                }
                                t->kind = VCD_PRESENT; t->off = off; t->len = len; t->dc = dc;
                            }
                }
    }
    if ((e = vcd_upload_finish(a->dev, a->atoms, total, dq, a->nlod)) != 0) {
        report("archive upload failed: %s", vcd_last_error());
        rc = (vc_status)e;
        goto done;
    }
    rc = VC_OK;
done:
    if (rc != VC_OK) {
        if (a->dev) vcd_free_archive(a->dev);   // also waits for a copy still in flight
        a->dev = NULL;
        free(a->atoms);
        a->atoms = NULL;
    }
    __atomic_store_n(&a->resident, rc == VC_OK ? 1 : 0, __ATOMIC_RELEASE);
    pthread_mutex_unlock(&a->mu);
    return rc;
}

// Entry capacity of one atom's coefficient list: every nonzero level spends a
// whole bypass (sign) bit, so a stream of n range-coder bytes cannot carry more
// than 8n of them; hostile streams that would exceed it are decoded on a slow
// path inside the kernel.
// list slots of a PRESENT atom, a multiple of 32 (128 bytes): no two atoms'
// lists share a cache line (k_caps places them the same way)
static inline uint64_t entry_cap(const vcd_atom *t) {
    uint64_t c = 8ull * (t->len - 1) + 64;
    c = c > VCD_MAX_ENTRIES ? VCD_MAX_ENTRIES : c;
    return (c + 31) & ~31ull;
}

// ---------------------------------------------------------------------------
// Streamed decode (vc_open_streaming, src/vc/vc.c:1262-1280, 1329-1338): the
// box's index entries, slots and payloads come from the read callback. The
// slots of one box row inside one region are read in one call, and payloads
// that lie back to back in the file in one call per run of at most RUN_MAX
// bytes; a call that fails is repeated slot by slot / payload by payload, so
// every slot and payload gets the outcome its own read would give. Payloads
// are packed into pinned staging behind a box-local atom table, uploaded piece
// by piece while the next pieces are read, and decoded on the device.
// ---------------------------------------------------------------------------
#define STREAM_PAYLOAD_MAX (32768u * 4u + 64u)   // the reference's streaming payload scratch (src/vc/vc.c:1277)
#define RUN_MAX (4u << 20)
#define PIECE_MIN (16ull << 10)   // uploads: 1/16 of the payload, within [PIECE_MIN, PIECE_MAX]
#define PIECE_MAX (16ull << 20)

static int g_stream_threads = 1;
VC_API int vcg_set_stream_threads(int n) {
    if (n < 1) n = 1;
    if (n > 64) n = 64;
    return __atomic_exchange_n(&g_stream_threads, n, __ATOMIC_RELAXED);
}

typedef struct {
    uint64_t src, dst;      // archive offset, staging offset (relative to the payload area)
    uint32_t len, p0, p1;   // bytes; present atoms pidx[p0 .. p1)
} stream_run;

typedef struct {
    const vc_archive *a;
    const stream_run *runs;
    const uint64_t *pidx, *psrc;   // per present atom: box index, archive offset
    const vcd_atom *tab;
    uint8_t *arena;
    const uint32_t *piece_run;     // piece k = runs[piece_run[k] .. piece_run[k+1])
    uint32_t n_pieces;
    uint32_t next;                 // next piece to take (workers)
    uint8_t *done;                 // per piece
    uint64_t fail;                 // lowest box index whose payload read failed
    pthread_mutex_t mu;
    pthread_cond_t cv;
} stream_fetch;

static void fetch_piece(stream_fetch *f, uint32_t k) {
    uint64_t fail = UINT64_MAX;
    for (uint32_t r = f->piece_run[k]; r < f->piece_run[k + 1] && fail == UINT64_MAX; ++r) {
        const stream_run *R = &f->runs[r];
        if (f->a->read(f->a->ud, R->src, R->len, f->arena + R->dst) == VC_OK) continue;
        for (uint32_t p = R->p0; p < R->p1; ++p) {
            const vcd_atom *t = &f->tab[f->pidx[p]];
            if (f->a->read(f->a->ud, f->psrc[p], t->len, f->arena + t->off) != VC_OK) { fail = f->pidx[p]; break; }
        }
    }
    pthread_mutex_lock(&f->mu);
    if (fail < f->fail) f->fail = fail;
    f->done[k] = 1;
    pthread_cond_broadcast(&f->cv);
    pthread_mutex_unlock(&f->mu);
}

static void *fetch_worker(void *p) {
    stream_fetch *f = (stream_fetch *)p;
    for (;;) {
        const uint32_t k = __atomic_fetch_add(&f->next, 1, __ATOMIC_RELAXED);
        if (k >= f->n_pieces) return NULL;
        fetch_piece(f, k);
    }
}

static vc_status stream_device(vc_archive *a) {   // dequantisation tables on the device, once
    pthread_mutex_lock(&a->mu);
    vc_status rc = VC_OK;
    int e;
    if (!a->sdev) {
        vcd_dq dq[VC_NLOD];
        for (int l = 0; l < a->nlod; ++l) vch_dq_consts(a->base_q[l], &dq[l]);
        if (vcd_init() != 0) { report("no usable CUDA device: %s", vcd_last_error()); rc = VC_ERR_IO; }
        else if ((e = vcd_upload_dq(&a->sdev, dq, a->nlod)) != 0) { report("%s", vcd_last_error()); rc = (vc_status)e; }
    }
    pthread_mutex_unlock(&a->mu);
    return rc;
}

static vc_status decode_box_streamed(vc_archive *a, int lod, vc_box b, uint8_t *out, uint8_t *out_dev,
                                     int bad_as_empty, uint64_t *n_present) {
    vc_status sd = stream_device(a);
    if (sd != VC_OK) return sd;
    const vc_dims d = lod_dims_of(a->d0, lod);
    vcd_region r;
    memset(&r, 0, sizeof r);
    r.lod = lod;
    r.acx = (d.nx + 31) / 32; r.acy = (d.ny + 31) / 32; r.acz = (d.nz + 31) / 32;
    r.x0 = b.x0; r.y0 = b.y0; r.z0 = b.z0; r.x1 = b.x1; r.y1 = b.y1; r.z1 = b.z1;
    r.bax = b.x0 / 32; r.bay = b.y0 / 32; r.baz = b.z0 / 32;
    r.bnx = (b.x1 - 1) / 32 - r.bax + 1; r.bny = (b.y1 - 1) / 32 - r.bay + 1; r.bnz = (b.z1 - 1) / 32 - r.baz + 1;
    const uint64_t n = (uint64_t)r.bnx * r.bny * r.bnz;
    const size_t out_bytes = (size_t)(b.x1 - b.x0) * (b.y1 - b.y0) * (b.z1 - b.z0);
    // regions the box touches: their blocks, resolved once
    const uint32_t rx0 = r.bax / 32, ry0 = r.bay / 32, rz0 = r.baz / 32;
    const uint32_t nrx = (r.bax + r.bnx - 1) / 32 - rx0 + 1, nry = (r.bay + r.bny - 1) / 32 - ry0 + 1,
                   nrz = (r.baz + r.bnz - 1) / 32 - rz0 + 1;
    uint64_t *blk = (uint64_t *)malloc((size_t)nrx * nry * nrz * sizeof(uint64_t));
    vcd_atom *tab = (vcd_atom *)malloc(n * sizeof(vcd_atom));
    uint64_t *psrc = (uint64_t *)malloc(n * sizeof(uint64_t)), *pidx = (uint64_t *)malloc(n * sizeof(uint64_t));
    stream_run *runs = (stream_run *)malloc((n + 1) * sizeof(stream_run));
    uint32_t *piece_run = NULL;
    uint8_t *done = NULL;
    vc_status st = VC_OK;
    if (!blk || !tab || !psrc || !pidx || !runs) { st = VC_ERR_OOM; goto out; }
    for (uint32_t z = 0; z < nrz; ++z)
        for (uint32_t y = 0; y < nry; ++y)
            for (uint32_t x = 0; x < nrx; ++x)
                blk[((uint64_t)z * nry + y) * nrx + x] = region_block(a, lod, rz0 + z, ry0 + y, rx0 + x);
    // slots, box order; the first bad atom ends the box (src/vc/vc.c:1413-1416)
    uint64_t nb = n, np = 0, pay = 0;
    for (uint32_t z = 0; z < r.bnz && nb == n; ++z)
        for (uint32_t y = 0; y < r.bny && nb == n; ++y) {
            const uint32_t az = r.baz + z, ay = r.bay + y;
            for (uint32_t x = 0; x < r.bnx && nb == n;) {
                const uint32_t ax = r.bax + x, seg = (32 - (ax & 31)) < (r.bnx - x) ? 32 - (ax & 31) : r.bnx - x;
                const uint64_t t0 = ((uint64_t)z * r.bny + y) * r.bnx + x;
                const uint64_t bk = blk[((uint64_t)(az / 32 - rz0) * nry + (ay / 32 - ry0)) * nrx + (ax / 32 - rx0)];
                uint8_t row[32 * 16];
                const uint8_t *sl = NULL;
                if (bk != 0 && bk != ZERO_REGION)
                    sl = at(a, bk + ((((uint64_t)(az & 31) * 32 + (ay & 31)) * 32 + (ax & 31)) * 16), seg * 16, row);
                for (uint32_t i = 0; i < seg; ++i) {
                    vcd_atom *t = &tab[t0 + i];
                    memset(t, 0, sizeof *t);
                    uint64_t off = 0;
                    uint32_t len = 0;
                    uint8_t dc = 0;
                    int fl;
                    if (sl) {
                        const uint8_t *s8 = sl + i * 16;
                        fl = s8[12];
                        if (fl == 1) { off = rd64(s8); len = rd32(s8 + 8); dc = s8[13]; }
                    } else {
                        fl = slot_of(a, bk, az, ay, ax + i, &off, &len, &dc);
                    }
                    if (fl != 1) { t->kind = VCD_EMPTY; continue; }
                    if (off == NO_OFFSET || len < 1 || off > a->len || len > a->len - off ||
                        (len > STREAM_PAYLOAD_MAX && !a->view)) {
                        if (bad_as_empty) { t->kind = VCD_EMPTY; continue; }
                        nb = t0 + i;
                        break;
                    }
                    t->kind = VCD_PRESENT; t->off = pay; t->len = len; t->dc = dc;
                    pidx[np] = t0 + i;
                    psrc[np++] = off;
                    pay += len;
                }
                x += seg;
            }
        }
    // runs of payloads that follow one another in the file, grouped into pieces
    uint32_t nr = 0;
    for (uint64_t p = 0; p < np;) {
        stream_run *R = &runs[nr++];
        R->src = psrc[p]; R->dst = tab[pidx[p]].off; R->len = tab[pidx[p]].len; R->p0 = (uint32_t)p;
        for (++p; p < np && psrc[p] == R->src + R->len && R->len + tab[pidx[p]].len <= RUN_MAX; ++p)
            R->len += tab[pidx[p]].len;
        R->p1 = (uint32_t)p;
    }
    const uint64_t piece = pay / 16 < PIECE_MIN ? PIECE_MIN : pay / 16 > PIECE_MAX ? PIECE_MAX : pay / 16;
    const uint32_t max_pieces = (uint32_t)(pay / piece) + 2;
    piece_run = (uint32_t *)malloc((max_pieces + 1) * sizeof(uint32_t));
    done = (uint8_t *)calloc(max_pieces, 1);
    if (!piece_run || !done) { st = VC_ERR_OOM; goto out; }
    uint32_t npc = 0;
    piece_run[0] = 0;
    for (uint32_t i = 0; i < nr;) {
        const uint64_t base = runs[i].dst;
        while (i < nr && (runs[i].dst - base < piece || runs[i].dst == base)) ++i;
        piece_run[++npc] = i;
    }
    // staging: [table (nb atoms)][pad to 256][payloads]
    const size_t table_bytes = (size_t)nb * sizeof(vcd_atom), arena_off = (table_bytes + 255) & ~(size_t)255;
    uint8_t *stage = NULL;
    int e = vcd_stage_reserve(arena_off + pay, &stage);
    if (e) { st = (vc_status)e; report("streamed decode: %s", vcd_last_error()); goto out; }
    memcpy(stage, tab, table_bytes);
    if ((e = vcd_stage_push(0, table_bytes)) != 0) { st = (vc_status)e; goto out; }
    stream_fetch f;
    memset(&f, 0, sizeof f);
    f.a = a; f.runs = runs; f.pidx = pidx; f.psrc = psrc; f.tab = tab; f.arena = stage + arena_off;
    f.piece_run = piece_run; f.n_pieces = npc; f.done = done; f.fail = UINT64_MAX;
    pthread_mutex_init(&f.mu, NULL);
    pthread_cond_init(&f.cv, NULL);
    const int want = __atomic_load_n(&g_stream_threads, __ATOMIC_RELAXED);
    const int nthr = npc > 1 && want > 1 ? (want < (int)npc ? want : (int)npc) : 0;
    pthread_t th[64];
    int started = 0;
    for (; started < nthr; ++started)
        if (pthread_create(&th[started], NULL, fetch_worker, &f) != 0) break;
    for (uint32_t k = 0; k < npc && !e; ++k) {
        if (!started) {
            fetch_piece(&f, k);
        } else {
            pthread_mutex_lock(&f.mu);
            while (!done[k]) pthread_cond_wait(&f.cv, &f.mu);
            pthread_mutex_unlock(&f.mu);
        }
        const uint64_t lo = runs[piece_run[k]].dst;
        const uint64_t hi = runs[piece_run[k + 1] - 1].dst + runs[piece_run[k + 1] - 1].len;
        e = vcd_stage_push(arena_off + lo, hi - lo);
    }
    if (started) {
        __atomic_store_n(&f.next, npc, __ATOMIC_RELAXED);   // no new pieces after an upload error
        for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
    }
    pthread_cond_destroy(&f.cv);
    pthread_mutex_destroy(&f.mu);
    if (e) { st = (vc_status)e; report("streamed decode: %s", vcd_last_error()); goto out; }
    if (f.fail < nb) nb = f.fail;
    uint64_t cap = 0, bytes = 0, present = 0;
    for (uint64_t p = 0; p < np && pidx[p] < nb; ++p) {
        cap += entry_cap(&tab[pidx[p]]);
        bytes += tab[pidx[p]].len;
        ++present;
    }
    r.n_atoms = nb;
    r.cap_total = cap;
    r.payload_bytes = bytes;
    r.present = present;
    if (n_present) *n_present = present;
    e = vcd_decode_staged(a->sdev, &r, 0, arena_off, pay, out_dev, out, out_bytes);
    if (e && e != VC_ERR_FORMAT) report("streamed decode: %s", vcd_last_error());
    st = (vc_status)e;
    if (!e && nb < n) st = VC_ERR_FORMAT;
out:
    free(blk); free(tab); free(psrc); free(pidx); free(runs); free(piece_run); free(done);
    return st;
}

// Shared by decode_region / decode_atom / decode_lod: out_dev (device) or out
// (host) receives the box raster.
static vc_status decode_box(vc_archive *a, int lod, vc_box b, uint8_t *out, uint8_t *out_dev) {
    if (a->read && __atomic_load_n(&a->resident, __ATOMIC_ACQUIRE) != 1)
        return decode_box_streamed(a, lod, b, out, out_dev, 0, NULL);
    vc_status rs = make_resident(a);
    if (rs != VC_OK) return rs;
    vc_dims d = lod_dims_of(a->d0, lod);
    vcd_region r;
    memset(&r, 0, sizeof r);
    r.lod = lod;
    r.atoms = a->atoms + a->lod_base[lod];
    r.atom_base = a->lod_base[lod];
    r.acx = (d.nx + 31) / 32; r.acy = (d.ny + 31) / 32; r.acz = (d.nz + 31) / 32;
    r.x0 = b.x0; r.y0 = b.y0; r.z0 = b.z0; r.x1 = b.x1; r.y1 = b.y1; r.z1 = b.z1;
    r.bax = b.x0 / 32; r.bay = b.y0 / 32; r.baz = b.z0 / 32;
    r.bnx = (b.x1 - 1) / 32 - r.bax + 1; r.bny = (b.y1 - 1) / 32 - r.bay + 1; r.bnz = (b.z1 - 1) / 32 - r.baz + 1;
    uint64_t n = (uint64_t)r.bnx * r.bny * r.bnz, cap = 0, i = 0, pay = 0, present = 0;
    vc_status st = VC_OK;
    for (uint32_t z = 0; z < r.bnz && st == VC_OK; ++z)
        for (uint32_t y = 0; y < r.bny && st == VC_OK; ++y)
            for (uint32_t x = 0; x < r.bnx; ++x, ++i) {
                const vcd_atom *t = &r.atoms[((uint64_t)(r.baz + z) * r.acy + (r.bay + y)) * r.acx + r.bax + x];
                if (t->kind == VCD_BAD) { st = VC_ERR_FORMAT; break; }
                if (t->kind == VCD_PRESENT) { cap += entry_cap(t); pay += t->len; ++present; }
            }
    r.n_atoms = st == VC_OK ? n : i;
    r.cap_total = cap;
    r.payload_bytes = pay;
    r.present = present;
    size_t bytes = (size_t)(b.x1 - b.x0) * (b.y1 - b.y0) * (b.z1 - b.z0);
    int rc = vcd_decode_region(a->dev, &r, out_dev, out, bytes);
    if (rc == VC_ERR_FORMAT || st == VC_ERR_FORMAT) return VC_ERR_FORMAT;
    if (rc) report("decode failed: %s", vcd_last_error());
    return (vc_status)rc;
}

VC_API vc_status vc_decode_region(vc_archive *a, int lod, vc_box b, uint8_t *out) {
    VCD_SCOPE();
    if (!a || lod < 0 || lod >= a->nlod || !out) return VC_ERR_RANGE;
    vc_dims d = lod_dims_of(a->d0, lod);
    if (b.x1 > d.nx || b.y1 > d.ny || b.z1 > d.nz) return VC_ERR_RANGE;
    if (b.x0 >= b.x1 || b.y0 >= b.y1 || b.z0 >= b.z1) return VC_ERR_RANGE;
    return decode_box(a, lod, b, out, NULL);
}

VC_API vc_status vc_decode_atom(vc_archive *a, int lod, int ax, int ay, int az, uint8_t out[VC_ATOM3]) {
    VCD_SCOPE();
    if (!a || lod < 0 || lod >= a->nlod || !out) return VC_ERR_RANGE;
    vc_dims d = lod_dims_of(a->d0, lod);
    if ((uint32_t)ax >= (d.nx + 31) / 32 || (uint32_t)ay >= (d.ny + 31) / 32 || (uint32_t)az >= (d.nz + 31) / 32)
        return VC_ERR_RANGE;
    vc_box b = {(uint32_t)ax * 32, (uint32_t)ay * 32, (uint32_t)az * 32,
                (uint32_t)ax * 32 + 32, (uint32_t)ay * 32 + 32, (uint32_t)az * 32 + 32};
    vc_status s = decode_box(a, lod, b, out, NULL);
    if (s == VC_ERR_FORMAT) memset(out, 0, VC_ATOM3);
    return s;
}

VC_API vc_status vc_decode_lod(vc_archive *a, int lod, uint8_t *out_vol, vc_dims *out_dims) {
    VCD_SCOPE();
    vc_dims d;
    vc_status s = vc_lod_dims(a, lod, &d);
    if (s != VC_OK) return s;
    if (out_dims) *out_dims = d;
    vc_box b = {0, 0, 0, d.nx, d.ny, d.nz};
    return vc_decode_region(a, lod, b, out_vol);
}

// Device-output variants (include/vcg.h).
VC_API vc_status vcg_decode_region_device(vc_archive *a, int lod, vc_box b, uint8_t *out_dev) {
    VCD_SCOPE();
    if (!a || lod < 0 || lod >= a->nlod || !out_dev) return VC_ERR_RANGE;
    vc_dims d = lod_dims_of(a->d0, lod);
    if (b.x1 > d.nx || b.y1 > d.ny || b.z1 > d.nz) return VC_ERR_RANGE;
    if (b.x0 >= b.x1 || b.y0 >= b.y1 || b.z0 >= b.z1) return VC_ERR_RANGE;
    return decode_box(a, lod, b, NULL, out_dev);
}

VC_API vc_status vcg_decode_lod_device(vc_archive *a, int lod, uint8_t *out_dev, vc_dims *out_dims) {
    VCD_SCOPE();
    vc_dims d;
    vc_status s = vc_lod_dims(a, lod, &d);
    if (s != VC_OK) return s;
    if (out_dims) *out_dims = d;
    vc_box b = {0, 0, 0, d.nx, d.ny, d.nz};
    return vcg_decode_region_device(a, lod, b, out_dev);
}

// ---------------------------------------------------------------------------
// Batched region decode (include/vcg.h). Each request follows vc_decode_region
// (src/vc/vc.c:1535-1555): its status is what that call would return, and a
// request that meets a bad atom gets only the atoms before it (z, y, x order).
// Across requests every distinct atom is decoded once.
// ---------------------------------------------------------------------------

VC_API vc_status vcg_decode_regions(vc_archive *a, uint32_t n, const vcg_region_request *reqs, int out_on_device,
                                    vc_status *status) {
    VCD_SCOPE();
    if (!a || (n && (!reqs || !status))) return VC_ERR_RANGE;
    if (n == 0) return VC_OK;
    vc_status rs = make_resident(a);
    if (rs != VC_OK) return rs;
    const uint64_t total_atoms = a->lod_base[a->nlod];
    int32_t *uid = (int32_t *)malloc((total_atoms ? total_atoms : 1) * sizeof(int32_t));
    vcd_boxreq *br = (vcd_boxreq *)calloc(n, sizeof(vcd_boxreq));
    uint32_t *rmap = (uint32_t *)malloc(n * sizeof(uint32_t));   // device request slot -> request
    size_t ref_cap = 1 << 16, nref = 0, ua_cap = 1 << 12, nua = 0;
    uint32_t *ref_u = (uint32_t *)malloc(ref_cap * 4), *ref_r = (uint32_t *)malloc(ref_cap * 4);
    vcd_uatom *ua = (vcd_uatom *)malloc(ua_cap * sizeof(vcd_uatom));
    vc_status rc = VC_OK;
    if (!uid || !br || !rmap || !ref_u || !ref_r || !ua) { rc = VC_ERR_OOM; goto done; }
    memset(uid, 0xFF, total_atoms * sizeof(int32_t));
    uint32_t nreq = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const vcg_region_request *q = &reqs[i];
        vc_box b = q->box;
        status[i] = VC_OK;
        if (q->lod < 0 || q->lod >= a->nlod || !q->out) { status[i] = VC_ERR_RANGE; continue; }
        vc_dims d = lod_dims_of(a->d0, q->lod);
        if (b.x1 > d.nx || b.y1 > d.ny || b.z1 > d.nz || b.x0 >= b.x1 || b.y0 >= b.y1 || b.z0 >= b.z1) {
            status[i] = VC_ERR_RANGE;
            continue;
        }
        const uint32_t acx = (d.nx + 31) / 32, acy = (d.ny + 31) / 32;
        if (!out_on_device) {
            // a bad atom: only the atoms before it may reach the caller's buffer,
            // which the plain path does exactly (rare: corrupt archives only)
            int has_bad = 0;
            for (uint32_t az = b.z0 / 32; az <= (b.z1 - 1) / 32 && !has_bad; ++az)
                for (uint32_t ay = b.y0 / 32; ay <= (b.y1 - 1) / 32 && !has_bad; ++ay)
                    for (uint32_t ax = b.x0 / 32; ax <= (b.x1 - 1) / 32; ++ax)
                        if (a->atoms[a->lod_base[q->lod] + ((uint64_t)az * acy + ay) * acx + ax].kind == VCD_BAD) {
                            has_bad = 1;
                            break;
                        }
            if (has_bad) {
                status[i] = decode_box(a, q->lod, b, q->out, NULL);
                continue;
            }
        }
        const uint32_t slot = nreq++;
        rmap[slot] = i;
        vcd_boxreq *r = &br[slot];
        r->out = out_on_device ? q->out : NULL;
        r->x0 = b.x0; r->y0 = b.y0; r->z0 = b.z0; r->x1 = b.x1; r->y1 = b.y1; r->z1 = b.z1;
        r->lod = (uint32_t)q->lod;
        int stop = 0;
        for (uint32_t az = b.z0 / 32; az <= (b.z1 - 1) / 32 && !stop; ++az)
            for (uint32_t ay = b.y0 / 32; ay <= (b.y1 - 1) / 32 && !stop; ++ay)
                for (uint32_t ax = b.x0 / 32; ax <= (b.x1 - 1) / 32; ++ax) {
                    const uint64_t g = a->lod_base[q->lod] + ((uint64_t)az * acy + ay) * acx + ax;
                    if (a->atoms[g].kind == VCD_BAD) { status[i] = VC_ERR_FORMAT; stop = 1; break; }
                    if (uid[g] < 0) {
                        if (nua == ua_cap) {
                            ua_cap *= 2;
                            vcd_uatom *t = (vcd_uatom *)realloc(ua, ua_cap * sizeof(vcd_uatom));
                            if (!t) { rc = VC_ERR_OOM; goto done; }
                            ua = t;
                        }
                        uid[g] = (int32_t)nua;
                        vcd_uatom *u = &ua[nua++];
                        memset(u, 0, sizeof *u);
                        u->idx = g; u->lod = (uint32_t)q->lod; u->az = az; u->ay = ay; u->ax = ax;
                    }
                    if (nref == ref_cap) {
                        ref_cap *= 2;
                        uint32_t *t1 = (uint32_t *)realloc(ref_u, ref_cap * 4), *t2 = t1 ? (uint32_t *)realloc(ref_r, ref_cap * 4) : NULL;
                        if (t1) ref_u = t1;
                        if (t2) ref_r = t2;
                        if (!t1 || !t2) { rc = VC_ERR_OOM; goto done; }
                    }
                    ref_u[nref] = (uint32_t)uid[g];
                    ref_r[nref++] = slot;
                    ++ua[uid[g]].dst_end;   // count for now
                }
    }
    if (nreq) {
        // CSR of destinations per distinct atom; list offsets by capacity
        uint32_t *dst = (uint32_t *)malloc((nref ? nref : 1) * 4);
        uint64_t *off = (uint64_t *)malloc((nua ? nua : 1) * 8);
        if (!dst || !off) { free(dst); free(off); rc = VC_ERR_OOM; goto done; }
        uint32_t acc = 0;
        uint64_t cap = 0;
        for (size_t u = 0; u < nua; ++u) {
            const uint32_t c = ua[u].dst_end;
            ua[u].dst_begin = acc;
            ua[u].dst_end = acc;
            acc += c;
            off[u] = cap;
            const vcd_atom *t = &a->atoms[ua[u].idx];
            if (t->kind == VCD_PRESENT) cap += entry_cap(t);
        }
        for (size_t k = 0; k < nref; ++k) dst[ua[ref_u[k]].dst_end++] = ref_r[k];
        vcd_batch bt = {nreq, (uint32_t)nua, (uint32_t)nref, br, ua, dst, off, cap};
        uint8_t **hout = NULL;
        if (!out_on_device) {
            hout = (uint8_t **)malloc(nreq * sizeof(uint8_t *));
            if (!hout) { free(dst); free(off); rc = VC_ERR_OOM; goto done; }
            for (uint32_t s = 0; s < nreq; ++s) hout[s] = reqs[rmap[s]].out;
        }
        uint32_t *err = (uint32_t *)calloc(nreq, 4);
        int drc = err ? vcd_decode_batch(a->dev, &bt, hout, err) : VC_ERR_OOM;
        if (drc) {
            report("batched decode failed: %s", vcd_last_error());
            rc = (vc_status)drc;
        } else {
            for (uint32_t s = 0; s < nreq; ++s)
                if (err[s]) status[rmap[s]] = VC_ERR_FORMAT;
        }
        free(err);
        free(hout);
        free(dst);
        free(off);
    }
done:
    free(uid);
    free(br);
    free(rmap);
    free(ref_u);
    free(ref_r);
    free(ua);
    return rc;
}

VC_API vc_status vcg_make_resident(vc_archive *a) {
    VCD_SCOPE();
    if (!a) return VC_ERR_RANGE;
    return make_resident(a);
}

// ---------------------------------------------------------------------------
// Encode (the canonical vc_encode composition, see include/vc.h)
// ---------------------------------------------------------------------------
static int nlod_for(vc_dims d0) {   // src/vc/vc.c:1001-1006
    int nlod = 1;
    for (int l = 1; l < VC_NLOD; ++l) {
        vc_dims d = lod_dims_of(d0, l);
        nlod = l + 1;
        if (d.nx <= 1 && d.ny <= 1 && d.nz <= 1) break;
    }
    return nlod;
}

static vc_status encode_common(const uint8_t *vol, int on_device, vc_dims dims, float target,
                               const float *fixed_q, uint8_t **out, size_t *out_len, float *q0, int ds_method,
                               float ds_alpha) {
    if (!vol || !out || !out_len || !dims_valid(dims) || !(target >= 1.0f)) return VC_ERR_RANGE;
    if (vcd_init() != 0) { report("no usable CUDA device: %s", vcd_last_error()); return VC_ERR_IO; }
    vcd_encode_info info;
    memset(&info, 0, sizeof info);
    info.ds_method = ds_method;
    info.ds_alpha = ds_alpha;
    info.nx = dims.nx; info.ny = dims.ny; info.nz = dims.nz;
    info.target_ratio = target;
    info.nlod = nlod_for(dims);
    if (fixed_q) {
        info.fixed_q = 1;
        for (int l = 0; l < info.nlod; ++l) {
            if (!(fixed_q[l] > 0.0f)) return VC_ERR_RANGE;   // vc_append_atom needs a q (src/vc/vc.c:1100)
            info.q[l] = fixed_q[l];
        }
    }
    uint64_t max_regions = 0;   // src/vc/vc.c:1012-1021
    for (int l = 0; l < info.nlod; ++l) {
        uint32_t z, y, x;
        region_grid(dims, l, &z, &y, &x);
        max_regions += (uint64_t)z * y * x;
    }
    info.l1_cap = 1024;
    while (info.l1_cap < max_regions * 2) info.l1_cap <<= 1;
    int rc = vcd_encode(vol, on_device, &info, out, out_len);
    if (rc) { report("encode failed: %s", vcd_last_error()); return (vc_status)rc; }
    if (q0) *q0 = info.q0;
    return VC_OK;
}

VC_API vc_status vc_encode(const uint8_t *vol, vc_dims dims, float target_ratio, uint8_t **out_archive,
                           size_t *out_len) {
    VCD_SCOPE();
    return encode_common(vol, 0, dims, target_ratio, NULL, out_archive, out_len, NULL, VCG_DS_BOX, 0.0f);
}

VC_API vc_status vcg_encode_device(const uint8_t *vol_dev, vc_dims dims, float target_ratio,
                                   uint8_t **out_archive, size_t *out_len, float *q0) {
    VCD_SCOPE();
    return encode_common(vol_dev, 1, dims, target_ratio, NULL, out_archive, out_len, q0, VCG_DS_BOX, 0.0f);
}

VC_API vc_status vcg_encode_q(const uint8_t *vol, int vol_on_device, vc_dims dims, float target_ratio,
                              const float base_q[VC_NLOD], uint8_t **out_archive, size_t *out_len) {
    VCD_SCOPE();
    if (!base_q) return VC_ERR_RANGE;
    return encode_common(vol, vol_on_device, dims, target_ratio, base_q, out_archive, out_len, NULL, VCG_DS_BOX, 0.0f);
}

static int ds_args_ok(int method, float alpha) {
    return (method == VCG_DS_BOX || method == VCG_DS_CBOX) && isfinite(alpha);
}

VC_API vc_status vcg_encode_ds(const uint8_t *vol, int vol_on_device, vc_dims dims, float target_ratio,
                               const float base_q[VC_NLOD], int method, float alpha, uint8_t **out_archive,
                               size_t *out_len) {
    VCD_SCOPE();
    if (!ds_args_ok(method, alpha)) return VC_ERR_RANGE;
    return encode_common(vol, vol_on_device, dims, target_ratio, base_q, out_archive, out_len, NULL, method, alpha);
}

// ---------------------------------------------------------------------------
// Exporter 2x downscale (tools/downscale.h:48-93) on the device.
// ---------------------------------------------------------------------------
static vc_status downscale_common(const uint8_t *in, int on_device, vc_dims d, int method, float alpha, int levels,
                                  uint8_t *const *out) {
    if (!in || !out || levels < 1 || levels > 8 || !ds_args_ok(method, alpha)) return VC_ERR_RANGE;
    if (!d.nx || !d.ny || !d.nz || (uint64_t)d.nx * d.ny > (1ull << 40) / d.nz) return VC_ERR_RANGE;
    for (int l = 0; l < levels; ++l)
        if (!out[l]) return VC_ERR_RANGE;
    if (vcd_init() != 0) { report("no usable CUDA device: %s", vcd_last_error()); return VC_ERR_IO; }
    const uint32_t dims[3] = {d.nx, d.ny, d.nz};
    const int rc = vcd_downscale(in, on_device, dims, method, alpha, levels, out);
    if (rc) report("downscale failed: %s", vcd_last_error());
    return (vc_status)rc;
}

VC_API vc_status vcg_downscale2x(const uint8_t *in, int on_device, vc_dims dims, int method, float alpha, uint8_t *out,
                                 vc_dims *out_dims) {
    VCD_SCOPE();
    if (out_dims) {
        out_dims->nx = (dims.nx + 1) / 2;
        out_dims->ny = (dims.ny + 1) / 2;
        out_dims->nz = (dims.nz + 1) / 2;
    }
    return downscale_common(in, on_device, dims, method, alpha, 1, &out);
}

VC_API vc_status vcg_downscale_pyramid(const uint8_t *vol_dev, vc_dims dims, int method, float alpha, int levels,
                                       uint8_t *const *out_dev) {
    VCD_SCOPE();
    return downscale_common(vol_dev, 1, dims, method, alpha, levels, out_dev);
}

// ---------------------------------------------------------------------------
// Live view of a writer's image (vc_writer.c; src/vc/vc.c:1475-1530): a v1
// archive read through a callback over the image, whose length and base_q
// follow the writer. Only the writer changes it, while no reader uses it.
// ---------------------------------------------------------------------------
vc_archive *vch_view_new(vc_read_fn read, void *ud, vc_dims d0, int nlod, uint64_t l1_off, uint64_t l1_cap) {
    vc_archive *a = (vc_archive *)calloc(1, sizeof *a);
    if (!a) return NULL;
    a->read = read;
    a->ud = ud;
    a->d0 = d0;
    a->nlod = nlod;
    a->version = 1;
    a->l1_off = l1_off;
    a->l1_cap = l1_cap;
    a->view = 1;
    pthread_mutex_init(&a->mu, NULL);
    return a;
}

void vch_view_set(vc_archive *a, uint64_t len, const float *base_q) {
    a->len = len;
    if (memcmp(a->base_q, base_q, sizeof a->base_q)) {
        memcpy(a->base_q, base_q, sizeof a->base_q);
        if (a->sdev) { vcd_free_archive(a->sdev); a->sdev = NULL; }   // dequantisation tables follow base_q
    }
}

// src/vc/vc.c:1507-1530: the 8 atoms (dz, dy, dx) from (az0, ay0, ax0); atoms
// outside the LOD and atoms without a valid payload read as zeros.
vc_status vch_view_decode_2x2x2(vc_archive *a, int lod, uint32_t az0, uint32_t ay0, uint32_t ax0,
                                uint8_t out8[8][VC_ATOM3], int *any) {
    if (!a || lod < 0 || lod >= a->nlod || !out8) return VC_ERR_RANGE;
    const vc_dims d = lod_dims_of(a->d0, lod);
    const uint32_t acx = (d.nx + 31) / 32, acy = (d.ny + 31) / 32, acz = (d.nz + 31) / 32;
    memset(out8, 0, 8 * (size_t)VC_ATOM3);
    if (any) *any = 0;
    if (ax0 >= acx || ay0 >= acy || az0 >= acz) return VC_OK;
    const uint32_t nx = ax0 + 2 <= acx ? 2 : 1, ny = ay0 + 2 <= acy ? 2 : 1, nz = az0 + 2 <= acz ? 2 : 1;
    const vc_box b = {ax0 * 32, ay0 * 32, az0 * 32, (ax0 + nx) * 32, (ay0 + ny) * 32, (az0 + nz) * 32};
    uint8_t *box = (uint8_t *)malloc((size_t)nx * ny * nz * VC_ATOM3);
    if (!box) return VC_ERR_OOM;
    uint64_t present = 0;
    const vc_status s = decode_box_streamed(a, lod, b, box, NULL, 1, &present);
    if (s == VC_OK) {
        for (uint32_t dz = 0; dz < nz; ++dz)
            for (uint32_t dy = 0; dy < ny; ++dy)
                for (uint32_t dx = 0; dx < nx; ++dx)
                    for (uint32_t z = 0; z < 32; ++z)
                        for (uint32_t y = 0; y < 32; ++y)
                            memcpy(&out8[(dz * 2 + dy) * 2 + dx][(z * 32 + y) * 32],
                                   box + (((size_t)(dz * 32 + z) * ny * 32 + dy * 32 + y) * nx * 32 + dx * 32), 32);
        if (any) *any = present > 0;
    }
    free(box);
    return s;
}

// ---------------------------------------------------------------------------
// Repack into the v2 container (tools/vc_repack.c:96-177, layout
// src/vc/vc.c:706-718): [128-byte header][region directory, 16 B per region in
// canonical order][4 KiB-aligned blobs]. Regions are laid out coarse LOD first,
// raster order within a LOD; a region with a present atom gets a blob of its
// 512 KiB slot array followed by its payloads in slot order, copied verbatim.
// The image is assembled on the device from the resident archive.
// ---------------------------------------------------------------------------
VC_API vc_status vcg_repack_v2(vc_archive *a, uint8_t **out_archive, size_t *out_len) {
    VCD_SCOPE();
    if (!a || !out_archive || !out_len) return VC_ERR_RANGE;
    *out_archive = NULL;
    *out_len = 0;
    vc_status rs = make_resident(a);
    if (rs != VC_OK) return rs;
    uint64_t prefix[VC_NLOD + 1], total_regions = 0;
    for (int l = 0; l < a->nlod; ++l) {
        uint32_t z, y, x;
        region_grid(a->d0, l, &z, &y, &x);
        prefix[l] = total_regions;
        total_regions += (uint64_t)z * y * x;
    }
    const uint64_t dir_off = FILE_HDR, head_len = dir_off + total_regions * 16;
    const uint64_t blobs_off = (head_len + 4095) & ~4095ull;
    uint8_t *head = (uint8_t *)calloc(head_len, 1);
    uint64_t cap = 1024, n = 0;
    vcd_repack_rec *recs = (vcd_repack_rec *)malloc(cap * sizeof(vcd_repack_rec));
    if (!head || !recs) { free(head); free(recs); return VC_ERR_OOM; }
    vc_status rc = VC_OK;
    uint64_t cursor = blobs_off;
    for (int l = a->nlod - 1; l >= 0 && rc == VC_OK; --l) {
        uint32_t nrz, nry, nrx;
        region_grid(a->d0, l, &nrz, &nry, &nrx);
        for (uint32_t rz = 0; rz < nrz && rc == VC_OK; ++rz)
            for (uint32_t ry = 0; ry < nry && rc == VC_OK; ++ry)
                for (uint32_t rx = 0; rx < nrx && rc == VC_OK; ++rx) {
                    const uint64_t ri = prefix[l] + ((uint64_t)rz * nry + ry) * nrx + rx;
                    uint8_t *e = head + dir_off + ri * 16;
                    uint64_t pay = 0;
                    int any_present = 0, any_zero = 0;
                    for (uint32_t s = 0; s < R_ATOMS * R_ATOMS * R_ATOMS; ++s) {
                        const uint32_t az = rz * R_ATOMS + s / (R_ATOMS * R_ATOMS),
                                       ay = ry * R_ATOMS + (s / R_ATOMS) % R_ATOMS, ax = rx * R_ATOMS + s % R_ATOMS;
                        uint64_t off;
                        uint32_t len;
                        const vc_cover cov = vc_atom_payload_range(a, l, az, ay, ax, &off, &len);
                        if (cov == VC_PRESENT) {
                            if (len < 1 || off > a->len || len > a->len - off) { rc = VC_ERR_FORMAT; break; }
                            any_present = 1;
                            pay += len;
                        } else if (cov == VC_KNOWN_ZERO) {
                            any_zero = 1;
                        }
                    }
                    if (rc != VC_OK) break;
                    if (!any_present) {
                        const uint32_t fl = any_zero ? 1u : 0u;   // ZERO / ABSENT
                        memcpy(e + 12, &fl, 4);
                        continue;
                    }
                    const uint64_t blob = cursor, blen = L2_BYTES + pay;
                    const uint32_t blen32 = (uint32_t)blen, fl = 2u;   // DATA
                    memcpy(e, &blob, 8);
                    memcpy(e + 8, &blen32, 4);
                    memcpy(e + 12, &fl, 4);
                    uint64_t paycur = blob + L2_BYTES;
                    for (uint32_t s = 0; s < R_ATOMS * R_ATOMS * R_ATOMS; ++s) {
                        const uint32_t az = rz * R_ATOMS + s / (R_ATOMS * R_ATOMS),
                                       ay = ry * R_ATOMS + (s / R_ATOMS) % R_ATOMS, ax = rx * R_ATOMS + s % R_ATOMS;
                        uint64_t off;
                        uint32_t len;
                        const vc_cover cov = vc_atom_payload_range(a, l, az, ay, ax, &off, &len);
                        if (cov == VC_ABSENT) continue;
                        if (n == cap) {
                            vcd_repack_rec *t = (vcd_repack_rec *)realloc(recs, 2 * cap * sizeof(vcd_repack_rec));
                            if (!t) { rc = VC_ERR_OOM; break; }
                            recs = t;
                            cap *= 2;
                        }
                        vcd_repack_rec *r = &recs[n++];
                        r->slot_dst = blob + (uint64_t)s * 16;
                        if (cov == VC_PRESENT) {
                            r->src = off; r->pay_dst = paycur; r->len = len; r->flags = 1;
                            paycur += len;
                        } else {
                            r->src = 0; r->pay_dst = 0; r->len = 0; r->flags = 2;
                        }
                    }
                    cursor += blen;
                }
    }
    if (rc == VC_OK) {
        const uint32_t w[6] = {MAGIC, 2u, 32u, 0u, R_ATOMS, (uint32_t)a->nlod};
        memcpy(head, w, sizeof w);
        const uint32_t dims[3] = {a->d0.nx, a->d0.ny, a->d0.nz};
        memcpy(head + 24, dims, sizeof dims);
        memcpy(head + 36, a->hdr + 36, 4);   // target ratio
        const uint64_t h64[3] = {dir_off, total_regions, cursor};
        memcpy(head + 40, h64, sizeof h64);
        memcpy(head + 72, a->hdr + 72, 4 * VC_NLOD);   // base_q per LOD
        uint8_t *res = (uint8_t *)malloc(cursor);
        if (!res) {
            rc = VC_ERR_OOM;
        } else {
            const int e = vcd_repack(a->dev, head, head_len, cursor, recs, n, res);
            if (e) { free(res); rc = (vc_status)e; report("repack: %s", vcd_last_error()); }
            else { *out_archive = res; *out_len = cursor; }
        }
    }
    free(head);
    free(recs);
    return rc;
}

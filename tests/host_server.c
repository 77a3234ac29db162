// Host build of the decode server (volume-compressor_gb300/csrc/vc_server.c)
// against stand-ins for the two decode calls it makes (vc_decode_region for a
// batch of one, vcg_decode_regions for larger batches). Test infrastructure
// for tests/test_host_server.py: the stand-ins record every call (its requests,
// class, device bytes, start and end), sleep in proportion to the box size and
// write a pattern that belongs to the request into its output, so that the
// scenarios below check the server's rules without a GPU:
//   every request decoded once, into its own output, with its own status (or
//   the status of a whole batched call that failed); batches homogeneous in
//   class and within max_batch; requests in flight within the device budget
//   (a request larger than the budget alone); small requests served while large
//   ones run; ticket slots recycled past the initial 1024; a ticket waited for
//   twice refused; destroy finishing every queued request.
// Prints one line per scenario and exits 0 when all hold.
#include <pthread.h>
#include <signal.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include "vcg.h"

#define MAXREQ 8192
#define BIG_VOXELS (32ull << 20)   // the server's large-request size

static int g_fail = 0;
#define CHECK(c, ...)                                   \
    do {                                                \
        if (!(c)) {                                     \
            fprintf(stderr, "FAIL %s:%d ", __FILE__, __LINE__); \
            fprintf(stderr, __VA_ARGS__);               \
            fprintf(stderr, "\n");                      \
            g_fail = 1;                                 \
        }                                               \
    } while (0)

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + ts.tv_nsec * 1e-9;
}

static uint64_t voxels(vc_box b) { return (uint64_t)(b.x1 - b.x0) * (b.y1 - b.y0) * (b.z1 - b.z0); }
static int is_big(vc_box b) { return voxels(b) >= BIG_VOXELS; }
// device bytes of a request as the server's contract states them: its output
// plus 32 KiB of list scratch per atom it overlaps
static uint64_t cost_of(vc_box b) {
    uint64_t atoms = (uint64_t)((b.x1 - 1) / 32 - b.x0 / 32 + 1) * ((b.y1 - 1) / 32 - b.y0 / 32 + 1) *
                     ((b.z1 - 1) / 32 - b.z0 / 32 + 1);
    return voxels(b) + atoms * 32768ull;
}
static uint8_t tag_of(int lod, vc_box b) {
    return (uint8_t)(lod * 31 + b.x0 * 7 + b.y0 * 13 + b.z0 * 17 + b.x1 * 3 + b.y1 * 5 + b.z1 * 11 + 1);
}
// per-request status of the stand-in decoder
static vc_status status_of(int lod, vc_box b) {
    if (lod == 7) return VC_ERR_RANGE;
    if (b.x0 % 97 == 13) return VC_ERR_FORMAT;
    return VC_OK;
}

// ---------------------------------------------------------------- stand-in decoder
typedef struct {
    int n, big, failed;
    double t0, t1;
    uint8_t *outs[1024];
} call_rec;

static pthread_mutex_t g_mu = PTHREAD_MUTEX_INITIALIZER;
static call_rec *g_calls;
static int g_ncalls;
static int g_in_big, g_in_small;
static uint64_t g_in_cost, g_budget;
static uint32_t g_max_batch;
static int g_fail_lod = -1;        // a request of this LOD fails its whole call with VC_ERR_OOM
static double g_us_per_mvox = 20;  // stand-in decode time: 30 us + this per Mi voxels
static int g_over_budget_not_alone;

static void fill(int lod, vc_box b, uint8_t *out) {
    const uint64_t n = voxels(b);
    const uint8_t t = tag_of(lod, b);
    for (uint64_t i = 0; i < n && i < 64; ++i) out[i] = (uint8_t)(t + i);
    out[n - 1] = (uint8_t)(t ^ 0x5A);
}

static vc_status decode_call(uint32_t n, const vcg_region_request *reqs, vc_status *st) {
    int big = is_big(reqs[0].box), fails = 0;
    uint64_t cost = 0, vox = 0;
    for (uint32_t i = 0; i < n; ++i) {
        CHECK(is_big(reqs[i].box) == big, "batch mixes large and small requests");
        cost += cost_of(reqs[i].box);
        vox += voxels(reqs[i].box);
        fails |= reqs[i].lod == g_fail_lod;
    }
    CHECK(n <= g_max_batch, "batch of %u over max_batch %u", n, g_max_batch);
    pthread_mutex_lock(&g_mu);
    const int k = g_ncalls++;
    call_rec *c = &g_calls[k];
    c->n = (int)n;
    c->big = big;
    c->failed = fails;
    c->t0 = now_s();
    for (uint32_t i = 0; i < n && i < 1024; ++i) c->outs[i] = reqs[i].out;
    if (big) ++g_in_big;
    else ++g_in_small;
    g_in_cost += cost;
    if (g_in_cost > g_budget && !(n == 1 && g_in_big + g_in_small == 1)) g_over_budget_not_alone = 1;
    pthread_mutex_unlock(&g_mu);
    struct timespec d;
    const double us = 30.0 + g_us_per_mvox * (double)vox / (1 << 20);
    d.tv_sec = (time_t)(us / 1e6);
    d.tv_nsec = (long)((us - d.tv_sec * 1e6) * 1e3);
    nanosleep(&d, NULL);
    for (uint32_t i = 0; i < n; ++i) {
        fill(reqs[i].lod, reqs[i].box, reqs[i].out);
        if (st) st[i] = status_of(reqs[i].lod, reqs[i].box);
    }
    pthread_mutex_lock(&g_mu);
    c->t1 = now_s();
    if (big) --g_in_big;
    else --g_in_small;
    g_in_cost -= cost;
    pthread_mutex_unlock(&g_mu);
    return fails ? VC_ERR_OOM : VC_OK;
}

vc_status vc_decode_region(vc_archive *a, int lod, vc_box box, uint8_t *out) {
    (void)a;
    vcg_region_request r = {lod, box, out};
    vc_status st;
    vc_status rc = decode_call(1, &r, &st);
    return rc != VC_OK ? rc : st;
}

vc_status vcg_decode_regions(vc_archive *a, uint32_t n, const vcg_region_request *reqs, int out_on_device,
                             vc_status *status) {
    (void)a;
    CHECK(out_on_device == 0, "server asked for device outputs");
    return decode_call(n, reqs, status);
}

// ---------------------------------------------------------------- requests
typedef struct {
    int lod;
    vc_box box;
    uint8_t *out;
    int64_t ticket;
} req;

static req g_req[MAXREQ];
static uint64_t g_rng = 0x9E3779B97F4A7C15ull;
static uint32_t rnd(uint32_t n) {
    g_rng ^= g_rng << 13;
    g_rng ^= g_rng >> 7;
    g_rng ^= g_rng << 17;
    return (uint32_t)(g_rng % n);
}

// 70 % single atoms, 25 % boxes with edges 64..128, 5 % large boxes (32 Mi voxels)
static void make_req(req *r, int i) {
    const uint32_t u = rnd(100);
    uint32_t ex, ey, ez;
    if (u < 70) ex = ey = ez = 32;
    else if (u < 95) { ex = 64 + rnd(65); ey = 64 + rnd(65); ez = 64 + rnd(65); }
    else { ex = 512; ey = 256; ez = 256; }
    r->lod = (i % 53 == 0) ? 7 : (int)rnd(4);
    r->box.x0 = 32 * rnd(64) + (u < 70 ? 0 : rnd(32));
    r->box.y0 = 32 * rnd(64);
    r->box.z0 = 32 * rnd(64);
    r->box.x1 = r->box.x0 + ex;
    r->box.y1 = r->box.y0 + ey;
    r->box.z1 = r->box.z0 + ez;
    r->out = (uint8_t *)malloc(voxels(r->box));   // large ones: only a few pages are touched
}

static int call_of(const uint8_t *out) {
    for (int k = 0; k < g_ncalls; ++k)
        for (int i = 0; i < g_calls[k].n && i < 1024; ++i)
            if (g_calls[k].outs[i] == out) return k;
    return -1;
}

static void check_outputs(int n, const vc_status *got, const char *name) {
    int bad_out = 0, bad_st = 0, missing = 0;
    for (int i = 0; i < n; ++i) {
        const req *r = &g_req[i];
        const int k = call_of(r->out);
        if (k < 0) { ++missing; continue; }
        const uint8_t t = tag_of(r->lod, r->box);
        const uint64_t v = voxels(r->box);
        for (uint64_t j = 0; j < v && j < 64; ++j) bad_out += r->out[j] != (uint8_t)(t + j);
        bad_out += r->out[v - 1] != (uint8_t)(t ^ 0x5A);
        if (got) {
            const vc_status want = g_calls[k].failed ? VC_ERR_OOM : status_of(r->lod, r->box);
            bad_st += got[i] != want;
        }
    }
    int decoded = 0;
    for (int k = 0; k < g_ncalls; ++k) decoded += g_calls[k].n;
    CHECK(missing == 0, "%s: %d requests never decoded", name, missing);
    CHECK(decoded == n, "%s: %d requests decoded for %d submitted", name, decoded, n);
    CHECK(bad_out == 0, "%s: %d output bytes wrong", name, bad_out);
    CHECK(bad_st == 0, "%s: %d statuses wrong", name, bad_st);
}

static void reset(uint64_t budget, uint32_t max_batch) {
    g_ncalls = 0;
    g_budget = budget;
    g_max_batch = max_batch;
    g_over_budget_not_alone = 0;
    g_fail_lod = -1;
}

static void free_reqs(int n) {
    for (int i = 0; i < n; ++i) free(g_req[i].out);
}

// A stream of mixed requests, waited for about 300 tickets behind the
// submissions (the ticket slots recycle), then the ticket rules.
static void scenario_mixed(int workers, uint64_t budget, uint32_t max_batch, int n, int fail_lod, const char *name) {
    reset(budget, max_batch);
    g_fail_lod = fail_lod;
    vc_archive *a = (vc_archive *)&g_req;   // opaque to the server
    vcg_server *s = vcg_server_create(a, budget, max_batch, workers);
    CHECK(s != NULL, "%s: create", name);
    static vc_status st[MAXREQ];
    double lat;
    for (int i = 0; i < n; ++i) {
        make_req(&g_req[i], i);
        g_req[i].ticket = vcg_server_submit(s, g_req[i].lod, g_req[i].box, g_req[i].out);
        CHECK(g_req[i].ticket == i, "%s: ticket %lld for request %d", name, (long long)g_req[i].ticket, i);
        if (rnd(4) == 0) usleep(rnd(150));
        if (i >= 300) {
            st[i - 300] = vcg_server_wait(s, g_req[i - 300].ticket, &lat);
            CHECK(lat >= 0, "%s: latency %f", name, lat);
        }
    }
    for (int i = n > 300 ? n - 300 : 0; i < n; ++i) st[i] = vcg_server_wait(s, g_req[i].ticket, &lat);
    CHECK(vcg_server_wait(s, g_req[0].ticket, NULL) == VC_ERR_RANGE, "%s: second wait accepted", name);
    CHECK(vcg_server_wait(s, n + 5, NULL) == VC_ERR_RANGE, "%s: wait on an unissued ticket accepted", name);
    CHECK(vcg_server_wait(s, -1, NULL) == VC_ERR_RANGE, "%s: wait on ticket -1 accepted", name);
    uint64_t batches = 0, requests = 0;
    vcg_server_stats(s, &batches, &requests);
    CHECK(requests == (uint64_t)n && batches == (uint64_t)g_ncalls, "%s: stats %llu / %llu", name,
          (unsigned long long)batches, (unsigned long long)requests);
    vcg_server_destroy(s);
    check_outputs(n, st, name);
    CHECK(!g_over_budget_not_alone, "%s: device budget exceeded by more than one request", name);
    int maxn = 0, batched = 0;
    for (int k = 0; k < g_ncalls; ++k) {
        maxn = g_calls[k].n > maxn ? g_calls[k].n : maxn;
        batched += g_calls[k].n > 1;
    }
    printf("%s: %d requests, %d calls (%d batched, largest %d)%s\n", name, n, g_ncalls, batched, maxn,
           g_fail ? " FAILED" : " ok");
    free_reqs(n);
}

// Large requests queued behind two running ones, then a small request: the
// first worker to free up takes the small one (one worker is kept for small
// requests while any waits), so no large request still queued when it arrived
// starts before it.
static void scenario_small_not_starved(void) {
    reset(64ull << 30, 1024);
    g_us_per_mvox = 4000;   // a 32 Mi-voxel request takes about 0.13 s
    vcg_server *s = vcg_server_create((vc_archive *)&g_req, 64ull << 30, 1024, 2);
    const int nb = 6;
    static vc_status st[16];
    for (int i = 0; i < nb; ++i) {
        req *r = &g_req[i];
        r->lod = 0;
        const uint32_t ez = i == 1 ? 512 : 256;   // the second runs twice as long
        r->box = (vc_box){0, 0, (uint32_t)(512 * i), 512, 256, (uint32_t)(512 * i) + ez};
        r->out = (uint8_t *)malloc(voxels(r->box));
        r->ticket = vcg_server_submit(s, r->lod, r->box, r->out);
        for (int w = 0; i < 2 && w < 5000; ++w) {   // running on its own worker before the next one arrives
            pthread_mutex_lock(&g_mu);
            const int in = g_in_big;
            pthread_mutex_unlock(&g_mu);
            if (in > i) break;
            usleep(1000);
        }
    }
    req *q = &g_req[nb];
    q->lod = 0;
    q->box = (vc_box){32, 32, 32, 64, 64, 64};
    q->out = (uint8_t *)malloc(voxels(q->box));
    const double t_sub = now_s();
    q->ticket = vcg_server_submit(s, q->lod, q->box, q->out);
    double lat_small = 0;
    st[nb] = vcg_server_wait(s, q->ticket, &lat_small);
    for (int i = 0; i < nb; ++i) st[i] = vcg_server_wait(s, g_req[i].ticket, NULL);
    vcg_server_destroy(s);
    check_outputs(nb + 1, st, "small_not_starved");
    const double t_small = g_calls[call_of(q->out)].t0;
    int running = 0, overtaking = 0, after = 0;
    for (int k = 0; k < g_ncalls; ++k) {
        if (!g_calls[k].big) continue;
        if (g_calls[k].t0 < t_sub) running += g_calls[k].n;
        else if (g_calls[k].t0 < t_small) overtaking += g_calls[k].n;
        else after += g_calls[k].n;
    }
    CHECK(running == 2 && overtaking == 0 && after == nb - 2,
          "small_not_starved: %d large running at its arrival, %d queued ones started before it, %d after", running,
          overtaking, after);
    printf("small_not_starved: small %.0f us; large: %d running at its arrival, %d started before it, %d after%s\n",
           lat_small, running, overtaking, after, g_fail ? " FAILED" : " ok");
    free_reqs(nb + 1);
    g_us_per_mvox = 20;
}

// Every request costs more than the budget: each runs alone, none is stuck.
static void scenario_over_budget(void) {
    const uint64_t budget = 1 << 20;
    reset(budget, 64);
    vcg_server *s = vcg_server_create((vc_archive *)&g_req, budget, 64, 3);
    const int n = 40;
    static vc_status st[64];
    for (int i = 0; i < n; ++i) {
        req *r = &g_req[i];
        r->lod = 1;
        r->box = (vc_box){(uint32_t)(32 * i), 0, 0, (uint32_t)(32 * i + 128), 128, 128};   // 2 MiB + scratch
        r->out = (uint8_t *)malloc(voxels(r->box));
        r->ticket = vcg_server_submit(s, r->lod, r->box, r->out);
    }
    for (int i = 0; i < n; ++i) st[i] = vcg_server_wait(s, g_req[i].ticket, NULL);
    vcg_server_destroy(s);
    check_outputs(n, st, "over_budget");
    int most = 0;
    for (int k = 0; k < g_ncalls; ++k) most = g_calls[k].n > most ? g_calls[k].n : most;
    CHECK(most == 1 && g_ncalls == n, "over_budget: %d calls, largest batch %d", g_ncalls, most);
    CHECK(!g_over_budget_not_alone, "over_budget: two requests over the budget in flight together");
    printf("over_budget: %d calls%s\n", g_ncalls, g_fail ? " FAILED" : " ok");
    free_reqs(n);
}

// Destroy right after the submissions: every queued request is still decoded.
static void scenario_destroy_drains(void) {
    reset(256ull << 20, 32);
    vcg_server *s = vcg_server_create((vc_archive *)&g_req, 256ull << 20, 32, 4);
    const int n = 500;
    for (int i = 0; i < n; ++i) {
        make_req(&g_req[i], i + 1);
        g_req[i].ticket = vcg_server_submit(s, g_req[i].lod, g_req[i].box, g_req[i].out);
    }
    vcg_server_destroy(s);
    check_outputs(n, NULL, "destroy_drains");
    printf("destroy_drains: %d calls%s\n", g_ncalls, g_fail ? " FAILED" : " ok");
    free_reqs(n);
}

int main(void) {
    alarm(120);   // a deadlock ends the run instead of hanging it
    g_calls = (call_rec *)calloc(MAXREQ, sizeof(call_rec));
    CHECK(vcg_server_create(NULL, 1, 1, 1) == NULL, "create without an archive");
    CHECK(vcg_server_create((vc_archive *)&g_req, 1, 1, 9) == NULL, "create with 9 workers");
    CHECK(vcg_server_submit(NULL, 0, (vc_box){0, 0, 0, 1, 1, 1}, NULL) == -1, "submit to no server");
    scenario_mixed(3, 2ull << 30, 1024, 3000, -1, "mixed_3_workers");
    scenario_mixed(1, 256ull << 20, 8, 1500, -1, "mixed_1_worker_small_budget");
    scenario_mixed(8, 64ull << 20, 64, 3000, -1, "mixed_8_workers_tight_budget");
    scenario_mixed(3, 2ull << 30, 256, 2000, 2, "mixed_failed_calls");
    scenario_small_not_starved();
    scenario_over_budget();
    scenario_destroy_drains();
    free(g_calls);
    return g_fail;
}

// Concurrent writer sessions on the host build of the writer (tests/
// host_writer.c: the writer and reader with the oracle's atom encoder standing
// in for the device). Test infrastructure for tests/test_host_writer.py.
//
//   host_writer_mt <file> <threads>
//
// Threads append every atom of a 2100 x 72 x 64 volume (three regions along x
// at LOD0) and of its LOD1, in interleaved and shuffled orders: synchronous
// appends, queued appends (flushed by each thread at its end), all-zero atoms
// and zero marks, while other calls ask for coverage. After the close, the
// file is opened with the oracle's reader, and every atom must have the
// coverage it was given and decode to what the oracle's own encode and decode
// of its source give. Prints "atoms <n> wrong <k>"; exits 0 when k is 0.
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "vcg.h"
#include "vc_oracle.h"

#define NX 2100u
#define NY 72u
#define NZ 64u
#define NLOD 2

static const float kQ[NLOD] = {1.7f, 1.02f};
static vc_writer *g_w;
static int g_threads;

typedef struct {
    int lod;
    uint32_t az, ay, ax;
    int kind;   // 0 content, 1 all-zero content, 2 zero mark
    int async;
} job;

static job *g_jobs;
static uint32_t g_njobs;

static uint32_t atoms_of(uint32_t d) { return (d + 31) / 32; }
static uint32_t dim_of(uint32_t d, int lod) { return lod ? (d + 1) / 2 : d; }

static uint64_t mix(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// the source voxels of an atom: smooth ramps plus noise, zero past the LOD's edge
static void source(const job *j, uint8_t *v) {
    const uint32_t nx = dim_of(NX, j->lod), ny = dim_of(NY, j->lod), nz = dim_of(NZ, j->lod);
    for (uint32_t z = 0; z < 32; ++z)
        for (uint32_t y = 0; y < 32; ++y)
            for (uint32_t x = 0; x < 32; ++x) {
                const uint32_t gx = j->ax * 32 + x, gy = j->ay * 32 + y, gz = j->az * 32 + z;
                uint8_t b = 0;
                if (j->kind == 0 && gx < nx && gy < ny && gz < nz) {
                    const uint64_t h = mix(((uint64_t)j->lod << 48) ^ ((uint64_t)gz << 32) ^ ((uint64_t)gy << 16) ^ gx);
                    b = (uint8_t)(((gx * 3 + gy * 5 + gz * 7) & 0xFF) / 2 + (h & 31));
                }
                v[(z * 32 + y) * 32 + x] = b;
            }
}

static void *appender(void *arg) {
    const int t = (int)(intptr_t)arg;
    uint8_t v[32768];
    int queued = 0;
    for (uint32_t i = (uint32_t)t; i < g_njobs; i += (uint32_t)g_threads) {
        const job *j = &g_jobs[i];
        vc_status s;
        if (j->kind == 2) {
            s = vc_mark_zero_atom(g_w, j->lod, j->az, j->ay, j->ax);
        } else {
            source(j, v);
            s = j->async ? vcg_append_atom_async(g_w, j->lod, j->az, j->ay, j->ax, v)
                         : vc_append_atom(g_w, j->lod, j->az, j->ay, j->ax, v);
            queued |= j->async;
        }
        if (s != VC_OK) fprintf(stderr, "append %u: status %d\n", i, (int)s);
        if ((i / (uint32_t)g_threads) % 7 == 3)   // coverage queries between the appends
            (void)vc_writer_coverage(g_w, j->lod, j->az, j->ay, j->ax);
    }
    if (queued) {
        uint64_t failed = 0;
        const vc_status s = vcg_writer_flush(g_w, &failed);
        if (s != VC_OK || failed) fprintf(stderr, "flush: status %d, %llu failed\n", (int)s, (unsigned long long)failed);
    }
    return NULL;
}

int main(int argc, char **argv) {
    if (argc != 3) return 2;
    g_threads = atoi(argv[2]);
    if (g_threads < 1 || g_threads > 64) return 2;
    for (int l = 0; l < NLOD; ++l) g_njobs += atoms_of(dim_of(NX, l)) * atoms_of(dim_of(NY, l)) * atoms_of(dim_of(NZ, l));
    g_jobs = (job *)calloc(g_njobs, sizeof(job));
    uint32_t n = 0;
    for (int l = 0; l < NLOD; ++l)
        for (uint32_t az = 0; az < atoms_of(dim_of(NZ, l)); ++az)
            for (uint32_t ay = 0; ay < atoms_of(dim_of(NY, l)); ++ay)
                for (uint32_t ax = 0; ax < atoms_of(dim_of(NX, l)); ++ax) {
                    job *j = &g_jobs[n];
                    const uint64_t h = mix(n * 977u + 5);
                    j->lod = l; j->az = az; j->ay = ay; j->ax = ax;
                    j->kind = (h & 15) == 0 ? 1 : (h & 15) == 1 ? 2 : 0;
                    j->async = (h >> 8) & 1;
                    ++n;
                }
    for (uint32_t i = n - 1; i > 0; --i) {   // shuffled order
        const uint32_t k = (uint32_t)(mix(i) % (i + 1));
        const job tmp = g_jobs[i];
        g_jobs[i] = g_jobs[k];
        g_jobs[k] = tmp;
    }
    g_w = vc_create(argv[1], (vc_dims){NX, NY, NZ}, 10.0f);
    if (!g_w) return 3;
    for (int l = 0; l < NLOD; ++l) vc_set_base_q(g_w, l, kQ[l]);
    pthread_t th[64];
    for (int t = 0; t < g_threads; ++t) pthread_create(&th[t], NULL, appender, (void *)(intptr_t)t);
    for (int t = 0; t < g_threads; ++t) pthread_join(th[t], NULL);
    vc_writer_close(g_w);

    // read back with the oracle
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 4;
    fseek(f, 0, SEEK_END);
    const long len = ftell(f);
    fseek(f, 0, SEEK_SET);
    uint8_t *buf = (uint8_t *)malloc((size_t)len);
    if (fread(buf, 1, (size_t)len, f) != (size_t)len) return 4;
    fclose(f);
    orc_archive *a = orc_open(buf, (size_t)len);
    if (!a) return 5;
    uint32_t wrong = 0;
    uint8_t src[32768], got[32768], want[32768], pay[131136];
    for (uint32_t i = 0; i < n; ++i) {
        const job *j = &g_jobs[i];
        const int cov = orc_atom_coverage(a, j->lod, j->az, j->ay, j->ax);
        if (orc_decode_atom(a, j->lod, (int)j->ax, (int)j->ay, (int)j->az, got) != 0) { ++wrong; continue; }
        source(j, src);
        int is_zero = 0;
        uint8_t dc = 0;
        const uint32_t pl = j->kind == 2 ? 0 : orc_encode_atom(src, kQ[j->lod], pay, sizeof pay, &is_zero, &dc);
        if (j->kind == 2 || is_zero) {
            memset(want, 0, sizeof want);
            wrong += cov != VC_KNOWN_ZERO;
        } else {
            if (orc_decode_atom_payload(pay, pl, kQ[j->lod], want) != 0) { ++wrong; continue; }
            wrong += cov != VC_PRESENT;
        }
        wrong += memcmp(got, want, sizeof want) != 0;
    }
    orc_close(a);
    printf("atoms %u wrong %u\n", n, wrong);
    free(buf);
    free(g_jobs);
    return wrong ? 1 : 0;
}

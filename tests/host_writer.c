// Host build of the writer (volume-compressor_gb300/csrc/vc_writer.c) and the
// host reader (vc_host.c) with a stand-in for the device layer. Test
// infrastructure for tests/test_host_writer.py: the writer's batches of atoms
// are encoded by the oracle's atom encoder (oracle/vc_oracle.c
// orc_encode_atom, whose payloads are the reference's), and every other device
// call reports that there is no device. Built as a shared library exporting
// the vc.h writer API, so that writer sessions run on it as on the reference's
// writer: the file layout, the region index, the slot blocks, the zero marks,
// the coverage reads and the close are this library's own host code.
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "vcg.h"
#include "vc_internal.h"
#include "vc_oracle.h"

// ---- the stand-in encoder: vcd_encode_segments (vc_internal.h) on the host.
// Each thread's payload buffer lives until the thread ends (as the device
// layer's per-thread buffer does).
static __thread uint8_t *g_pay;
static __thread uint64_t g_pay_cap;
static pthread_key_t g_pay_key;
static pthread_once_t g_pay_once = PTHREAD_ONCE_INIT;
static void pay_free(void *p) { free(p); }
static void pay_key(void) { pthread_key_create(&g_pay_key, pay_free); }

int vcd_encode_segments(const vcd_seg *segs, int nseg, const float *qs, int nq, uint8_t **pay, uint64_t *pay_bytes) {
    (void)nq;
    uint64_t used = 0;
    uint8_t vox[32768];
    uint8_t out[131136];
    for (int s = 0; s < nseg; ++s) {
        const vcd_seg *S = &segs[s];
        const uint32_t anx = S->nx / 32, any = S->ny / 32, anz = S->nz / 32;
        for (uint32_t az = 0, i = 0; az < anz; ++az)
            for (uint32_t ay = 0; ay < any; ++ay)
                for (uint32_t ax = 0; ax < anx; ++ax, ++i) {
                    for (uint32_t z = 0; z < 32; ++z)
                        for (uint32_t y = 0; y < 32; ++y)
                            memcpy(vox + (z * 32 + y) * 32,
                                   S->vox + ((uint64_t)(az * 32 + z) * S->ny + ay * 32 + y) * S->nx + ax * 32, 32);
                    int is_zero = 0;
                    uint8_t dc = 0;
                    const uint32_t n = orc_encode_atom(vox, qs[S->qsel[i]], out, sizeof out, &is_zero, &dc);
                    const uint32_t len = is_zero ? 0u : n;
                    if (used + len > g_pay_cap) {
                        const uint64_t cap = 2 * (used + len) + 65536;
                        uint8_t *p = (uint8_t *)realloc(g_pay, cap);
                        if (!p) return VC_ERR_OOM;
                        g_pay = p;
                        g_pay_cap = cap;
                        pthread_once(&g_pay_once, pay_key);
                        pthread_setspecific(g_pay_key, p);
                    }
                    if (len) memcpy(g_pay + used, out, len);
                    S->len[i] = len;
                    S->off[i] = used;
                    used += len;
                }
    }
    *pay = g_pay;
    *pay_bytes = used;
    return 0;
}

// ---- the rest of the device layer: no device
int vcd_init(void) { return 0; }
int vcd_enter(void) { return -1; }
void vcd_leave(int *prev) { (void)prev; }
const char *vcd_last_error(void) { return "no device (host build)"; }
int vcd_upload_begin(vcd_archive **out, const uint8_t *buf, size_t len) { (void)out; (void)buf; (void)len; return VC_ERR_IO; }
int vcd_upload_finish(vcd_archive *d, const vcd_atom *atoms, uint64_t n_atoms, const vcd_dq *dq, int nlod) {
    (void)d; (void)atoms; (void)n_atoms; (void)dq; (void)nlod;
    return VC_ERR_IO;
}
void vcd_free_archive(vcd_archive *d) { (void)d; }
int vcd_decode_region(vcd_archive *d, const vcd_region *r, uint8_t *out_dev, uint8_t *out_host, size_t out_bytes) {
    (void)d; (void)r; (void)out_dev; (void)out_host; (void)out_bytes;
    return VC_ERR_IO;
}
int vcd_upload_dq(vcd_archive **out, const vcd_dq *dq, int nlod) { (void)out; (void)dq; (void)nlod; return VC_ERR_IO; }
int vcd_stage_reserve(size_t bytes, uint8_t **host) { (void)bytes; (void)host; return VC_ERR_IO; }
int vcd_stage_push(size_t off, size_t bytes) { (void)off; (void)bytes; return VC_ERR_IO; }
int vcd_decode_staged(vcd_archive *d, const vcd_region *r, size_t table_off, size_t arena_off, size_t arena_bytes,
                      uint8_t *out_dev, uint8_t *out_host, size_t out_bytes) {
    (void)d; (void)r; (void)table_off; (void)arena_off; (void)arena_bytes; (void)out_dev; (void)out_host;
    (void)out_bytes;
    return VC_ERR_IO;
}
int vcd_decode_batch(vcd_archive *d, const vcd_batch *b, uint8_t *const *host_out, uint32_t *req_err) {
    (void)d; (void)b; (void)host_out; (void)req_err;
    return VC_ERR_IO;
}
int vcd_encode(const uint8_t *vol, int vol_on_device, vcd_encode_info *info, uint8_t **out, size_t *out_len) {
    (void)vol; (void)vol_on_device; (void)info; (void)out; (void)out_len;
    return VC_ERR_IO;
}
int vcd_downscale(const uint8_t *in, int on_device, const uint32_t dims[3], int method, float alpha, int levels,
                  uint8_t *const *out) {
    (void)in; (void)on_device; (void)dims; (void)method; (void)alpha; (void)levels; (void)out;
    return VC_ERR_IO;
}
int vcd_repack(vcd_archive *d, const uint8_t *head, uint64_t head_len, uint64_t total_len, const vcd_repack_rec *recs,
               uint64_t n_recs, uint8_t *host_out) {
    (void)d; (void)head; (void)head_len; (void)total_len; (void)recs; (void)n_recs; (void)host_out;
    return VC_ERR_IO;
}

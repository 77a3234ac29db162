// CPU ORACLE — test infrastructure only (see vc_oracle.h). A restatement of the
// reference codec's per-atom path and v1/v2 archive format in portable C with
// strict IEEE float (built with -fno-fast-math -ffp-contract=off), so that it
// gives the same bytes on x86-64 and AArch64. Each function names the reference
// lines (src/vc/vc.c) it restates.
#include "vc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../volume-compressor_gb300/csrc/vc_release_tables.h"

#define N 32u
#define N3 32768u
#define L2_BYTES (32768ull * 16ull)
#define FILE_HDR 128u
#define NO_OFFSET 0xFFFFFFFFFFFFFFFFull

// ---------------------------------------------------------------------------
// Tables (src/vc/vc.c:75-88 CMATA, :266-290 g_step + scan, :462-468 band_of)
// ---------------------------------------------------------------------------
static int32_t g_cm[N][N];       // Q14 orthonormal DCT-II matrix, row = frequency
static float g_stepv[N3];        // release-build HF-boost steps per raster index
static uint16_t g_scan[N3];      // scan position -> raster index
static int g_ready;

static inline uint32_t freq_of(uint32_t r) { return (r >> 10) + ((r >> 5) & 31u) + (r & 31u); }

static float f_from_bits(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static uint32_t bits_of(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

static void tables_init(void) {
    if (__atomic_load_n(&g_ready, __ATOMIC_ACQUIRE)) return;
    for (uint32_t k = 0; k < N; ++k) {
        double ck = k ? sqrt(2.0 / 32.0) : sqrt(1.0 / 32.0);
        for (uint32_t n = 0; n < N; ++n)
            g_cm[k][n] = (int32_t)llround(ck * cos(M_PI * (2.0 * n + 1.0) * k / 64.0) * 16384.0);
    }
    for (uint32_t r = 0; r < N3; ++r) {
        uint32_t f = freq_of(r);
        int alt = (vc_step_alt_mask[r >> 5] >> (r & 31u)) & 1u;
        g_stepv[r] = f_from_bits(alt ? vc_step_alt_bits[f] : vc_step_base_bits[f]);
    }
    // ascending L1 frequency, ties by raster index (the qsort comparator at :258-264)
    uint32_t p = 0;
    for (uint32_t f = 0; f <= 93; ++f)
        for (uint32_t r = 0; r < N3; ++r)
            if (freq_of(r) == f) g_scan[p++] = (uint16_t)r;
    __atomic_store_n(&g_ready, 1, __ATOMIC_RELEASE);
}

void orc_tables(int32_t *cmat, float *step, uint16_t *scan) {
    tables_init();
    if (cmat) memcpy(cmat, g_cm, sizeof g_cm);
    if (step) memcpy(step, g_stepv, sizeof g_stepv);
    if (scan) memcpy(scan, g_scan, sizeof g_scan);
}

// band = floor(freq * 8 / 96) capped at 7 (:462-468)
int orc_band_of(uint32_t raster) {
    uint32_t b = freq_of(raster) * 8u / 96u;
    return b > 7u ? 7 : (int)b;
}

// ---------------------------------------------------------------------------
// Integer DCT-32 (:96-229). All products and sums are i32 with wrap-around, as
// the reference's vectorised i32 lanes behave; the even/odd split is exact.
// ---------------------------------------------------------------------------
static inline int32_t rnd14(uint32_t acc) { return (int32_t)(acc + 8192u) >> 14; }

// forward line: out[k] = (sum_n C[k][n] v[n] + 2^13) >> 14 via sums/differences (:142-171)
static void line_fwd(const int32_t *v, size_t vs, int32_t *o, size_t os) {
    uint32_t s[16], d[16];
    int any = 0;
    for (uint32_t n = 0; n < N; ++n) any |= v[n * vs] != 0;
    if (!any) { for (uint32_t k = 0; k < N; ++k) o[k * os] = 0; return; }
    for (uint32_t n = 0; n < 16; ++n) {
        s[n] = (uint32_t)v[n * vs] + (uint32_t)v[(31 - n) * vs];
        d[n] = (uint32_t)v[n * vs] - (uint32_t)v[(31 - n) * vs];
    }
    for (uint32_t k = 0; k < N; ++k) {
        const uint32_t *src = (k & 1u) ? d : s;
        uint32_t acc = 0;
        for (uint32_t n = 0; n < 16; ++n) acc += (uint32_t)g_cm[k][n] * src[n];
        o[k * os] = rnd14(acc);
    }
}

// inverse line: out[n] = (sum_k C[k][n] v[k] + 2^13) >> 14 via even/odd halves (:172-205)
static void line_inv(const int32_t *v, size_t vs, int32_t *o, size_t os) {
    int any = 0;
    for (uint32_t k = 0; k < N; ++k) any |= v[k * vs] != 0;
    if (!any) { for (uint32_t n = 0; n < N; ++n) o[n * os] = 0; return; }
    for (uint32_t n = 0; n < 16; ++n) {
        uint32_t ev = 0, od = 0;
        for (uint32_t k = 0; k < N; k += 2) ev += (uint32_t)g_cm[k][n] * (uint32_t)v[k * vs];
        for (uint32_t k = 1; k < N; k += 2) od += (uint32_t)g_cm[k][n] * (uint32_t)v[k * vs];
        o[n * os] = rnd14(ev + od);
        o[(31 - n) * os] = rnd14(ev - od);
    }
}

// Three passes in the reference's order (x, then y, then z) with rounding after
// each; the reference's axis rotations (:206-211) only relayout lines, so the
// passes are expressed here with strides. Output raster is [kz][ky][kx].
void orc_fdct(const uint8_t *vox, int32_t dc, int32_t *coef) {
    tables_init();
    int32_t *a = (int32_t *)malloc(N3 * sizeof(int32_t));
    int32_t *b = (int32_t *)malloc(N3 * sizeof(int32_t));
    for (uint32_t i = 0; i < N3; ++i) a[i] = (int32_t)vox[i] - dc;
    for (uint32_t zy = 0; zy < N * N; ++zy) line_fwd(a + zy * N, 1, b + zy * N, 1);          // x
    for (uint32_t z = 0; z < N; ++z)
        for (uint32_t kx = 0; kx < N; ++kx) line_fwd(b + z * 1024 + kx, N, a + z * 1024 + kx, N);  // y
    for (uint32_t yx = 0; yx < N * N; ++yx) line_fwd(a + yx, 1024, coef + yx, 1024);       // z
    free(a); free(b);
}

// :219-229 — inverse passes along kx, ky, kz, then +dc and clamp to u8.
void orc_idct(const int32_t *coef, int32_t dc, uint8_t *vox) {
    tables_init();
    int32_t *a = (int32_t *)malloc(N3 * sizeof(int32_t));
    int32_t *b = (int32_t *)malloc(N3 * sizeof(int32_t));
    for (uint32_t zy = 0; zy < N * N; ++zy) line_inv(coef + zy * N, 1, a + zy * N, 1);
    for (uint32_t z = 0; z < N; ++z)
        for (uint32_t x = 0; x < N; ++x) line_inv(a + z * 1024 + x, N, b + z * 1024 + x, N);
    for (uint32_t yx = 0; yx < N * N; ++yx) line_inv(b + yx, 1024, a + yx, 1024);
    for (uint32_t i = 0; i < N3; ++i) {
        int32_t v = (int32_t)((uint32_t)a[i] + (uint32_t)dc);
        vox[i] = (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v);
    }
    free(a); free(b);
}

// ---------------------------------------------------------------------------
// Quantizer (:293-306) as the release build evaluates it: the division by the
// step is RCPPS(step) refined by one Newton step, r' = 2r - r*(r*step).
// ---------------------------------------------------------------------------
static float rcp_est(float x) {
    uint32_t b = bits_of(x);
    uint32_t e = (b >> 23) & 0xFFu;
    uint32_t r = vc_rcp_est_bits[(b >> 12) & 0x7FFu];
    uint32_t re = ((r >> 23) & 0xFFu) - (e - 127u);
    return f_from_bits((b & 0x80000000u) | (re << 23) | (r & 0x7FFFFFu));
}

static int32_t quant_one(int32_t c, float base_q, float g) {
    float step = base_q * g;
    float dz = 0.8f * step;
    uint32_t mag = c < 0 ? 0u - (uint32_t)c : (uint32_t)c;
    float a = (float)(int32_t)mag;
    int32_t level = 0;
    if (a >= dz) {
        float r = rcp_est(step);
        float rr = (r + r) - r * (r * step);
        level = (int32_t)((a - dz) * rr + 1.0f);
    }
    if (level > 32767) level = 32767;
    return c < 0 ? -level : level;
}

void orc_quantize(const int32_t *coef, float base_q, int16_t *lv) {
    tables_init();
    for (uint32_t i = 0; i < N3; ++i) lv[i] = (int16_t)quant_one(coef[i], base_q, g_stepv[i]);
}

// Dequant tables (:314-326): step*2^8 and (0.4-1+0.8)*step*2^8, rounded to nearest even.
void orc_dq_tables(float base_q, int32_t *dq_step, int32_t *dq_bias) {
    tables_init();
    const float c = (0.4f - 1.0f) + 0.8f;
    for (uint32_t i = 0; i < N3; ++i) {
        float step = base_q * g_stepv[i];
        dq_step[i] = (int32_t)lrintf(step * 256.0f);
        dq_bias[i] = (int32_t)lrintf(c * step * 256.0f);
    }
}

// :327-338 — r = (|lv|*dq_step + dq_bias + 128) >> 8 with the sign restored (i32 wrap).
void orc_dequantize(const int16_t *lv, float base_q, int32_t *coef) {
    int32_t *ds = (int32_t *)malloc(N3 * sizeof(int32_t)), *db = (int32_t *)malloc(N3 * sizeof(int32_t));
    orc_dq_tables(base_q, ds, db);
    for (uint32_t i = 0; i < N3; ++i) {
        int32_t l = lv[i];
        uint32_t m = (uint32_t)(l < 0 ? -l : l);
        int32_t r = (int32_t)(m * (uint32_t)ds[i] + (uint32_t)db[i] + 128u) >> 8;
        coef[i] = l == 0 ? 0 : (l < 0 ? (int32_t)(0u - (uint32_t)r) : r);
    }
    free(ds); free(db);
}

// ---------------------------------------------------------------------------
// Adaptive binary range coder (:344-441) and coefficient context coder
// (:448-560): 12-bit P(0), shift-5 adaptation, carry-less-low LZMA-style output.
// ---------------------------------------------------------------------------
typedef struct {
    uint8_t *out; uint32_t cap, len; int overflow;
    uint64_t low; uint32_t range; uint8_t cache; uint64_t pending;
    uint32_t shifts;
} renc;

static void renc_init(renc *e, uint8_t *out, uint32_t cap) {
    memset(e, 0, sizeof *e);
    e->out = out; e->cap = cap; e->range = 0xFFFFFFFFu; e->pending = 1;
}
static void renc_emit(renc *e, uint8_t b) {
    if (!e->out) { e->len++; return; }
    if (e->len >= e->cap) { e->overflow = 1; return; }
    e->out[e->len++] = b;
}
static void renc_shift(renc *e) {   // :369-380
    e->shifts++;
    if ((uint32_t)(e->low >> 32) != 0 || e->low < 0xFF000000ull) {
        uint8_t carry = (uint8_t)(e->low >> 32);
        uint8_t c = e->cache;
        do { renc_emit(e, (uint8_t)(c + carry)); c = 0xFF; } while (--e->pending);
        e->cache = (uint8_t)(e->low >> 24);
    }
    e->pending++;
    e->low = (e->low << 8) & 0xFFFFFFFFull;
}
static void renc_norm(renc *e) { while (e->range < (1u << 24)) { renc_shift(e); e->range <<= 8; } }
static void renc_bit(renc *e, uint16_t *p0, int bit) {   // :381-393
    uint32_t r0 = (uint32_t)(((uint64_t)e->range * *p0) >> 12);
    if (!bit) { e->range = r0; *p0 = (uint16_t)(*p0 + ((4096u - *p0) >> 5)); }
    else { e->low += r0; e->range -= r0; *p0 = (uint16_t)(*p0 - (*p0 >> 5)); }
    renc_norm(e);
}
static void renc_bypass(renc *e, int bit) {   // :394-398
    e->range >>= 1;
    if (bit) e->low += e->range;
    renc_norm(e);
}

typedef struct { uint16_t sig[8], mag[12]; } ctxset;
static void ctx_reset(ctxset *c) {
    for (int i = 0; i < 8; ++i) c->sig[i] = 2048;
    for (int i = 0; i < 12; ++i) c->mag[i] = 2048;
}

// magnitude m >= 1: unary over mag[0..11], then EG0 of the rest in bypass (:471-490)
static void enc_mag(renc *e, ctxset *c, uint32_t m) {
    uint32_t v = m - 1, k = 0;
    while (k < 11 && v > 0) {
        renc_bit(e, &c->mag[k], 1);
        --v; ++k;
        if (v == 0) { renc_bit(e, &c->mag[k], 0); return; }
    }
    if (v == 0) { renc_bit(e, &c->mag[k], 0); return; }
    renc_bit(e, &c->mag[k], 1);
    uint32_t x1 = v + 1, nb = 0;
    for (uint32_t t = x1; t > 1; t >>= 1) ++nb;
    for (uint32_t i = 0; i < nb; ++i) renc_bypass(e, 1);
    renc_bypass(e, 0);
    for (int i = (int)nb - 1; i >= 0; --i) renc_bypass(e, (x1 >> i) & 1u);
}

static void enc_levels(renc *e, const int16_t *lv) {   // :528-544
    tables_init();
    ctxset c; ctx_reset(&c);
    uint32_t eob = 0;
    for (uint32_t p = N3; p-- > 0;) if (lv[g_scan[p]]) { eob = p + 1; break; }
    for (int i = 15; i >= 0; --i) renc_bypass(e, (eob >> i) & 1u);   // 16-bit EOB (:512-519)
    for (uint32_t p = 0; p < eob; ++p) {
        uint32_t r = g_scan[p];
        int16_t v = lv[r];
        uint16_t *sig = &c.sig[orc_band_of(r)];
        if (!v) { renc_bit(e, sig, 0); continue; }
        renc_bit(e, sig, 1);
        enc_mag(e, &c, (uint32_t)(v < 0 ? -(int32_t)v : v));
        renc_bypass(e, v < 0);
    }
    for (int i = 0; i < 5; ++i) renc_shift(e);   // flush (:399-401)
}

uint32_t orc_enc_levels(const int16_t *lv, uint8_t *out, uint32_t cap) {
    renc e; renc_init(&e, out, cap);
    enc_levels(&e, lv);
    return e.overflow ? 0 : e.len;
}

uint32_t orc_rc_size(const int16_t *lv) {
    renc e; renc_init(&e, NULL, 0);
    enc_levels(&e, lv);
    return e.len;
}

typedef struct { const uint8_t *buf; uint32_t len, pos; uint32_t code, range; } rdec;

static inline uint8_t rdec_byte(rdec *d) { return d->pos < d->len ? d->buf[d->pos++] : 0; }
static void rdec_init(rdec *d, const uint8_t *buf, uint32_t len) {   // :403-413
    d->buf = buf; d->len = len; d->pos = 0; d->code = 0; d->range = 0xFFFFFFFFu;
    for (int i = 0; i < 5; ++i) d->code = (d->code << 8) | rdec_byte(d);
}
static void rdec_norm(rdec *d) {
    while (d->range < (1u << 24)) { d->code = (d->code << 8) | rdec_byte(d); d->range <<= 8; }
}
static int rdec_bit(rdec *d, uint16_t *p0) {   // :414-430
    uint32_t r0 = (uint32_t)(((uint64_t)d->range * *p0) >> 12);
    int bit;
    if (d->code < r0) { d->range = r0; bit = 0; *p0 = (uint16_t)(*p0 + ((4096u - *p0) >> 5)); }
    else { d->code -= r0; d->range -= r0; bit = 1; *p0 = (uint16_t)(*p0 - (*p0 >> 5)); }
    rdec_norm(d);
    return bit;
}
static int rdec_bypass(rdec *d) {   // :431-441
    d->range >>= 1;
    int bit = d->code >= d->range;
    if (bit) d->code -= d->range;
    rdec_norm(d);
    return bit;
}

// Returns 1 (malformed) when the EG0 prefix runs past 32 ones: no legitimate
// level needs more than 15, and the reference's loop (:501) would not terminate
// on some hostile streams.
int orc_dec_levels(const uint8_t *buf, uint32_t len, int16_t *lv) {   // :545-560
    tables_init();
    rdec d; rdec_init(&d, buf, len);
    ctxset c; ctx_reset(&c);
    memset(lv, 0, N3 * sizeof(int16_t));
    uint32_t eob = 0;
    for (int i = 0; i < 16; ++i) eob = (eob << 1) | (uint32_t)rdec_bypass(&d);
    if (eob > N3) eob = N3;
    for (uint32_t p = 0; p < eob; ++p) {
        uint32_t r = g_scan[p];
        if (!rdec_bit(&d, &c.sig[orc_band_of(r)])) continue;
        uint32_t v = 0, k = 0, m;   // :491-506
        for (;;) {
            if (k == 11) {
                if (!rdec_bit(&d, &c.mag[11])) { m = v + 1; break; }
                uint32_t nb = 0;
                while (rdec_bypass(&d)) { if (++nb > 32) return 1; }
                uint32_t x = 1;
                for (uint32_t i = 0; i < nb; ++i) x = (x << 1) | (uint32_t)rdec_bypass(&d);
                m = v + (x - 1) + 1;
                break;
            }
            if (rdec_bit(&d, &c.mag[k])) { ++v; ++k; } else { m = v + 1; break; }
        }
        int neg = rdec_bypass(&d);
        lv[r] = (int16_t)(uint16_t)(neg ? 0u - m : m);
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Atom payload (:595-633): [dc u8][range-coder bytes]; an all-zero atom has none.
// ---------------------------------------------------------------------------
uint32_t orc_encode_atom(const uint8_t *vox, float base_q, uint8_t *out, uint32_t cap,
                         int *is_zero, uint8_t *dcv) {
    uint32_t sum = 0;
    for (uint32_t i = 0; i < N3; ++i) sum += vox[i];
    if (!sum) { *is_zero = 1; *dcv = 0; return 0; }
    *is_zero = 0;
    int32_t dc = (int32_t)((sum + N3 / 2) / N3);
    *dcv = (uint8_t)dc;
    int32_t *coef = (int32_t *)malloc(N3 * sizeof(int32_t));
    int16_t *lv = (int16_t *)malloc(N3 * sizeof(int16_t));
    orc_fdct(vox, dc, coef);
    orc_quantize(coef, base_q, lv);
    uint32_t n;
    if (out) {
        if (cap < 1) { free(coef); free(lv); return 0; }
        out[0] = (uint8_t)dc;
        n = orc_enc_levels(lv, out + 1, cap - 1);
        n = n ? n + 1 : 0;
    } else {
        n = orc_rc_size(lv) + 1;
    }
    free(coef); free(lv);
    return n;
}

int orc_decode_atom_payload(const uint8_t *pay, uint32_t len, float base_q, uint8_t *vox) {
    int16_t *lv = (int16_t *)malloc(N3 * sizeof(int16_t));
    int32_t *coef = (int32_t *)malloc(N3 * sizeof(int32_t));
    int bad = orc_dec_levels(pay + 1, len - 1, lv);
    if (!bad) {
        orc_dequantize(lv, base_q, coef);
        orc_idct(coef, pay[0], vox);
    } else {
        memset(vox, 0, N3);
    }
    free(lv); free(coef);
    return bad;
}

// ---------------------------------------------------------------------------
// Pyramid (:733-739 lod dims; :1001-1006 nlod; :1562-1577 downsample)
// ---------------------------------------------------------------------------
orc_dims orc_lod_dims_of(orc_dims d, int lod) {
    for (int i = 0; i < lod; ++i) { d.nx = (d.nx + 1) / 2; d.ny = (d.ny + 1) / 2; d.nz = (d.nz + 1) / 2; }
    return d;
}
int orc_nlod(orc_dims d0) {
    int nlod = 1;
    for (int l = 1; l < 8; ++l) {
        orc_dims d = orc_lod_dims_of(d0, l);
        nlod = l + 1;
        if (d.nx <= 1 && d.ny <= 1 && d.nz <= 1) break;
    }
    return nlod;
}
void orc_downsample2x(const uint8_t *in, orc_dims d, uint8_t *out) {
    uint32_t ox = (d.nx + 1) / 2, oy = (d.ny + 1) / 2, oz = (d.nz + 1) / 2;
    #pragma omp parallel for schedule(static)
    for (uint32_t z = 0; z < oz; ++z)
        for (uint32_t y = 0; y < oy; ++y)
            for (uint32_t x = 0; x < ox; ++x) {
                uint32_t acc = 0, n = 0;
                for (uint32_t zz = 2 * z; zz < 2 * z + 2 && zz < d.nz; ++zz)
                    for (uint32_t yy = 2 * y; yy < 2 * y + 2 && yy < d.ny; ++yy)
                        for (uint32_t xx = 2 * x; xx < 2 * x + 2 && xx < d.nx; ++xx) {
                            acc += in[((size_t)zz * d.ny + yy) * d.nx + xx];
                            ++n;
                        }
                out[((size_t)z * oy + y) * ox + x] = (uint8_t)((acc + n / 2) / n);
            }
}

// gather atom (az,ay,ax) of a volume, zero outside the extent
static void gather_atom(const uint8_t *vol, orc_dims d, uint32_t az, uint32_t ay, uint32_t ax,
                        uint8_t *atom) {
    memset(atom, 0, N3);
    for (uint32_t z = 0; z < N; ++z) {
        uint32_t vz = az * N + z;
        if (vz >= d.nz) break;
        for (uint32_t y = 0; y < N; ++y) {
            uint32_t vy = ay * N + y;
            if (vy >= d.ny) break;
            uint32_t x0 = ax * N, cnt = d.nx - x0 < N ? d.nx - x0 : N;
            memcpy(atom + (z * N + y) * N, vol + ((size_t)vz * d.ny + vy) * d.nx + x0, cnt);
        }
    }
}

// ---------------------------------------------------------------------------
// Canonical writer: vc_create (:995-1068) + vc_set_base_q (:1070-1079) +
// append_one (:1082-1159) for every atom of every LOD in raster order from one
// thread + vc_writer_close (:1231-1245).
// ---------------------------------------------------------------------------
static inline uint64_t mix64(uint64_t x) {   // :721-726
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
static inline uint64_t region_key(int lod, uint32_t rz, uint32_t ry, uint32_t rx) {
    return ((uint64_t)(lod & 7) << 45) | ((uint64_t)(rz & 0x7FFF) << 30) |
           ((uint64_t)(ry & 0x7FFF) << 15) | (uint64_t)(rx & 0x7FFF);
}
static inline void wr32(uint8_t *p, uint32_t v) { memcpy(p, &v, 4); }
static inline void wr64(uint8_t *p, uint64_t v) { memcpy(p, &v, 8); }
static inline uint32_t rd32(const uint8_t *p) { uint32_t v; memcpy(&v, p, 4); return v; }
static inline uint64_t rd64(const uint8_t *p) { uint64_t v; memcpy(&v, p, 8); return v; }

typedef struct { uint8_t *buf; size_t cap, cursor; uint64_t l1_cap; } owriter;

static int ow_reserve(owriter *w, size_t need) {
    if (need <= w->cap) return 0;
    size_t nc = w->cap ? w->cap : 1u << 20;
    while (nc < need) nc *= 2;
    uint8_t *nb = (uint8_t *)realloc(w->buf, nc);
    if (!nb) return -1;
    memset(nb + w->cap, 0, nc - w->cap);
    w->buf = nb; w->cap = nc;
    return 0;
}

// find-or-create the region's L2 block (:900-955 single-threaded)
static uint64_t ow_region(owriter *w, uint64_t key) {
    uint64_t mask = w->l1_cap - 1, i = mix64(key) & mask;
    for (;;) {
        uint8_t *e = w->buf + FILE_HDR + i * 16;
        uint64_t bref = rd64(e + 8);
        if (bref && rd64(e) == key) return bref;
        if (!bref) break;
        i = (i + 1) & mask;
    }
    uint64_t blk = w->cursor;
    if (ow_reserve(w, blk + L2_BYTES)) return 0;
    w->cursor += L2_BYTES;
    uint8_t *e = w->buf + FILE_HDR + i * 16;
    wr64(e, key); wr64(e + 8, blk);
    wr64(w->buf + 48, rd64(w->buf + 48) + 1);
    return blk;
}

int orc_encode_fixed_q(const uint8_t *vol, orc_dims d0, float target_ratio, const float *base_q,
                       int nthreads, uint8_t **out, size_t *out_len) {
    tables_init();
    if (!d0.nx || !d0.ny || !d0.nz || d0.nx > (1u << 20) || d0.ny > (1u << 20) || d0.nz > (1u << 20) ||
        !(target_ratio >= 1.0f))
        return ORC_ERR_RANGE;
    int nlod = orc_nlod(d0);
    uint64_t max_regions = 0;
    for (int l = 0; l < nlod; ++l) {
        orc_dims d = orc_lod_dims_of(d0, l);
        uint64_t rx = ((d.nx + 31) / 32 + 31) / 32, ry = ((d.ny + 31) / 32 + 31) / 32,
                 rz = ((d.nz + 31) / 32 + 31) / 32;
        max_regions += rx * ry * rz;
    }
    owriter w = {0};
    w.l1_cap = 1024;
    while (w.l1_cap < max_regions * 2) w.l1_cap <<= 1;
    w.cursor = FILE_HDR + w.l1_cap * 16;
    if (ow_reserve(&w, w.cursor)) return ORC_ERR_OOM;
    uint8_t *h = w.buf;
    wr32(h + 0, 0x00314356u); wr32(h + 4, 1); wr32(h + 8, 32); wr32(h + 12, 1); wr32(h + 16, 32);
    wr32(h + 20, (uint32_t)nlod); wr32(h + 24, d0.nx); wr32(h + 28, d0.ny); wr32(h + 32, d0.nz);
    memcpy(h + 36, &target_ratio, 4);
    wr64(h + 40, w.l1_cap); wr64(h + 48, 0); wr64(h + 56, FILE_HDR);
    float qs[8] = {0};
    for (int l = 0; l < nlod; ++l) {
        float q = base_q[l];
        if (q < 0.05f) q = 0.05f;
        if (q > 4096.0f) q = 4096.0f;
        qs[l] = q;
        memcpy(w.buf + 72 + 4 * l, &q, 4);
    }

    const uint8_t *cur = vol;
    uint8_t *own = NULL;
    for (int l = 0; l < nlod; ++l) {
        orc_dims d = orc_lod_dims_of(d0, l);
        if (l > 0) {
            orc_dims pd = orc_lod_dims_of(d0, l - 1);
            uint8_t *nxt = (uint8_t *)malloc((size_t)d.nx * d.ny * d.nz);
            if (!nxt) { free(own); free(w.buf); return ORC_ERR_OOM; }
            orc_downsample2x(cur, pd, nxt);
            free(own);
            own = nxt; cur = nxt;
        }
        uint32_t acx = (d.nx + 31) / 32, acy = (d.ny + 31) / 32, acz = (d.nz + 31) / 32;
        uint64_t na = (uint64_t)acx * acy * acz;
        // payloads are a pure function of (atom, q): compute them in parallel, then
        // lay them out strictly in append order.
        uint8_t **pays = (uint8_t **)calloc(na, sizeof(uint8_t *));
        uint32_t *lens = (uint32_t *)calloc(na, sizeof(uint32_t));
        uint8_t *dcs = (uint8_t *)calloc(na, 1);
        if (!pays || !lens || !dcs) { free(pays); free(lens); free(dcs); free(own); free(w.buf); return ORC_ERR_OOM; }
        #pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads > 0 ? nthreads : 1)
        for (uint64_t t = 0; t < na; ++t) {
            uint32_t ax = (uint32_t)(t % acx), ay = (uint32_t)((t / acx) % acy), az = (uint32_t)(t / ((uint64_t)acx * acy));
            uint8_t *atom = (uint8_t *)malloc(N3);
            uint8_t *buf = (uint8_t *)malloc(N3 * 4 + 64);
            gather_atom(cur, d, az, ay, ax, atom);
            int z = 0; uint8_t dc = 0;
            uint32_t n = orc_encode_atom(atom, qs[l], buf, N3 * 4 + 64, &z, &dc);
            if (!z) { pays[t] = buf; lens[t] = n; dcs[t] = dc; } else free(buf);
            free(atom);
        }
        int err = 0;
        for (uint64_t t = 0; t < na && !err; ++t) {
            uint32_t ax = (uint32_t)(t % acx), ay = (uint32_t)((t / acx) % acy), az = (uint32_t)(t / ((uint64_t)acx * acy));
            uint64_t blk = ow_region(&w, region_key(l, az / 32, ay / 32, ax / 32));
            if (!blk) { err = 1; break; }
            uint64_t slot = blk + ((((uint64_t)(az & 31) * 32 + (ay & 31)) * 32 + (ax & 31)) * 16);
            if (!pays[t]) {
                wr64(w.buf + slot, NO_OFFSET); wr32(w.buf + slot + 8, 0); w.buf[slot + 13] = 0;
                w.buf[slot + 12] = 2;
                continue;
            }
            uint64_t poff = w.cursor;
            if (ow_reserve(&w, poff + lens[t])) { err = 1; break; }
            w.cursor += lens[t];
            memcpy(w.buf + poff, pays[t], lens[t]);
            wr32(w.buf + slot + 8, lens[t]); w.buf[slot + 12] = 1; w.buf[slot + 13] = dcs[t];
            wr64(w.buf + slot, poff);
        }
        for (uint64_t t = 0; t < na; ++t) free(pays[t]);
        free(pays); free(lens); free(dcs);
        if (err) { free(own); free(w.buf); return ORC_ERR_OOM; }
    }
    free(own);
    wr64(w.buf + 64, w.cursor);
    *out = w.buf;
    *out_len = w.cursor;
    return ORC_OK;
}

// ---------------------------------------------------------------------------
// Rate control. The reference leaves q to the caller (vc.h:56-61, docs/SPEC.md
// §9) and states the intent as a bisection on measured size
// (docs/DO_NOT_IMPLEMENT.md:40-41); this is the deterministic rule both the
// oracle and the GPU path implement: bisect q0 over the IEEE-754 bit patterns of
// [0.05f, 4096.0f] (monotone in value, roughly log-spaced) for 24 steps, each
// measuring the present-atom ratio of LOD0 (32768 * present atoms / payload
// bytes); keep the q whose ratio is closest to the target (ties: larger q).
// ---------------------------------------------------------------------------
uint64_t orc_encode_sizes_mt(const uint8_t *vol, orc_dims d, float base_q, const uint32_t *atom_ids,
                             uint32_t n_atoms, uint32_t *lens, int nthreads) {
    tables_init();
    uint32_t acx = (d.nx + 31) / 32, acy = (d.ny + 31) / 32;
    uint64_t total = 0;
    #pragma omp parallel for schedule(dynamic, 2) reduction(+ : total) num_threads(nthreads > 0 ? nthreads : 1)
    for (uint32_t i = 0; i < n_atoms; ++i) {
        uint32_t t = atom_ids[i];
        uint32_t ax = t % acx, ay = (t / acx) % acy, az = t / (acx * acy);
        uint8_t *atom = (uint8_t *)malloc(N3);
        gather_atom(vol, d, az, ay, ax, atom);
        int z = 0; uint8_t dc = 0;
        uint32_t n = orc_encode_atom(atom, base_q, NULL, 0, &z, &dc);
        if (lens) lens[i] = n;
        total += n;
        free(atom);
    }
    return total;
}

float orc_rate_control(const uint8_t *vol, orc_dims d, float target, int nthreads,
                       uint64_t *present_out, uint64_t *bytes_out) {
    uint32_t acx = (d.nx + 31) / 32, acy = (d.ny + 31) / 32, acz = (d.nz + 31) / 32;
    uint64_t na = (uint64_t)acx * acy * acz;
    uint32_t *ids = (uint32_t *)malloc(na * sizeof(uint32_t));
    uint32_t np = 0;
    uint8_t *atom = (uint8_t *)malloc(N3);
    for (uint64_t t = 0; t < na; ++t) {
        uint32_t ax = (uint32_t)(t % acx), ay = (uint32_t)((t / acx) % acy), az = (uint32_t)(t / ((uint64_t)acx * acy));
        gather_atom(vol, d, az, ay, ax, atom);
        uint32_t s = 0;
        for (uint32_t i = 0; i < N3; ++i) s |= atom[i];
        if (s) ids[np++] = (uint32_t)t;
    }
    free(atom);
    float best_q = 1.0f;
    uint64_t best_bytes = 0;
    if (np) {
        uint32_t lo = bits_of(0.05f), hi = bits_of(4096.0f);
        double best_err = INFINITY;
        for (int it = 0; it < 24; ++it) {
            uint32_t mid = lo + (hi - lo) / 2;
            float q = f_from_bits(mid);
            uint64_t bytes = orc_encode_sizes_mt(vol, d, q, ids, np, NULL, nthreads);
            double ratio = (double)(32768ull * np) / (double)bytes;
            double err = fabs(ratio - (double)target);
            if (err < best_err || (err == best_err && q > best_q)) { best_err = err; best_q = q; best_bytes = bytes; }
            if (ratio < (double)target) lo = mid; else hi = mid;
        }
    }
    if (present_out) *present_out = np;
    if (bytes_out) *bytes_out = best_bytes;
    free(ids);
    return best_q;
}

int orc_encode(const uint8_t *vol, orc_dims d, float target, int nthreads, uint8_t **out, size_t *out_len) {
    if (!d.nx || !d.ny || !d.nz || d.nx > (1u << 20) || d.ny > (1u << 20) || d.nz > (1u << 20) ||
        !(target >= 1.0f))
        return ORC_ERR_RANGE;
    float q0 = orc_rate_control(vol, d, target, nthreads, NULL, NULL);
    float qs[8];
    float q = q0;
    for (int l = 0; l < 8; ++l) { qs[l] = q < 0.05f ? 0.05f : q; q = q * 0.6f; }
    return orc_encode_fixed_q(vol, d, target, qs, nthreads, out, out_len);
}

void orc_free(void *p) { free(p); }

// ---------------------------------------------------------------------------
// Exporter 2x downscale (tools/downscale.h:29-93), strictly within the 2x2x2
// cell, odd boundaries edge-replicated. DS_BOX is the cell mean rounded half
// up; DS_CBOX moves the mean toward the cell's voxel of largest deviation
// (the first one in (dz, dy, dx) order on ties) by alpha. The deviations are
// compared exactly as integers |8c - sum| (the reference's float differences
// are exact). The push mean + alpha * (best - mean) is evaluated as the
// reference's release build (gcc -O3 -ffast-math -ffp-contract=fast
// -march=native) evaluates it: one fused multiply-add, except in the 8-lane
// vector body of the nz == 2 fast path (tools/downscale.h:62-79; the first
// 8 * floor(ox / 8) outputs of each row), where it multiplies and adds
// separately. Pinned against that build cell by cell.
// ---------------------------------------------------------------------------
static int g_ds_fused = 1;
void orc_ds_set_fused(int fused) { g_ds_fused = fused; }

static uint8_t ds_cell_rule(const uint8_t *c8, int method, float alpha, int fused) {
    uint32_t sum = 0;
    for (int i = 0; i < 8; ++i) sum += c8[i];
    if (sum == 0) return 0;
    if (method == 0) return (uint8_t)((sum + 4) >> 3);
    int best = c8[0], bestdev = -1;
    for (int i = 0; i < 8; ++i) {
        int d = 8 * (int)c8[i] - (int)sum;
        if (d < 0) d = -d;
        if (d > bestdev) { bestdev = d; best = c8[i]; }
    }
    const float mean = (float)sum * 0.125f, dlt = (float)best - mean;
    const float v = fused ? fmaf(alpha, dlt, mean) : mean + alpha * dlt;
    if (v < 0.0f) return 0;
    if (v > 255.0f) return 255;
    return (uint8_t)(v + 0.5f);
}

uint8_t orc_ds_cell(const uint8_t *c8, int method, float alpha) {   // :38-46
    return ds_cell_rule(c8, method, alpha, g_ds_fused);
}

void orc_ds_downscale2x(const uint8_t *in, orc_dims d, int method, float alpha, uint8_t *out, orc_dims *od) {   // :48-93
    orc_dims o = {(d.nx + 1) / 2, (d.ny + 1) / 2, (d.nz + 1) / 2};
    if (o.nx < 1) o.nx = 1;
    if (o.ny < 1) o.ny = 1;
    if (o.nz < 1) o.nz = 1;
    if (od) *od = o;
    const int fast = d.nz == 2 && d.nx % 2 == 0 && d.ny % 2 == 0;   // :62
    const uint32_t vec_end = fast ? o.nx & ~7u : 0;
    for (uint32_t z = 0; z < o.nz; ++z)
        for (uint32_t y = 0; y < o.ny; ++y)
            for (uint32_t x = 0; x < o.nx; ++x) {
                uint8_t c8[8];
                int n = 0;
                for (uint32_t dz = 0; dz < 2; ++dz)
                    for (uint32_t dy = 0; dy < 2; ++dy)
                        for (uint32_t dx = 0; dx < 2; ++dx) {
                            uint32_t z2 = 2 * z + dz, y2 = 2 * y + dy, x2 = 2 * x + dx;
                            if (z2 >= d.nz) z2 = d.nz - 1;
                            if (y2 >= d.ny) y2 = d.ny - 1;
                            if (x2 >= d.nx) x2 = d.nx - 1;
                            c8[n++] = in[((size_t)z2 * d.ny + y2) * d.nx + x2];
                        }
                out[((size_t)z * o.ny + y) * o.nx + x] = ds_cell_rule(c8, method, alpha, x >= vec_end);
            }
}


// ---------------------------------------------------------------------------
// Reader (:1247-1555)
// ---------------------------------------------------------------------------
struct orc_archive {
    const uint8_t *buf; size_t len;     // buf == NULL: streaming (read / ud)
    orc_read_fn read; void *ud;
    orc_dims d0; int nlod, version;
    uint64_t l1_off, l1_cap, dir_off, region_prefix[9];
    float base_q[8];
};

static void region_grid(orc_dims d0, int lod, uint32_t *nrz, uint32_t *nry, uint32_t *nrx) {
    orc_dims d = orc_lod_dims_of(d0, lod);
    *nrx = ((d.nx + 31) / 32 + 31) / 32; *nry = ((d.ny + 31) / 32 + 31) / 32; *nrz = ((d.nz + 31) / 32 + 31) / 32;
}

// Streaming open (:1329-1338): the header through the callback, then the same
// validation as orc_open; every later read goes through rd().
orc_archive *orc_open_streaming(orc_read_fn read, void *ud, uint64_t total_len) {
    if (!read || total_len < FILE_HDR) return NULL;
    uint8_t hdr[FILE_HDR];
    if (read(ud, 0, FILE_HDR, hdr) != ORC_OK) return NULL;
    orc_archive *a = orc_open(hdr, total_len);
    if (!a) return NULL;
    a->buf = NULL;
    a->read = read;
    a->ud = ud;
    return a;
}

orc_archive *orc_open(const uint8_t *buf, size_t len) {   // :1285-1323
    tables_init();
    if (!buf || len < FILE_HDR) return NULL;
    if (rd32(buf) != 0x00314356u || rd32(buf + 8) != 32 || rd32(buf + 16) != 32) return NULL;
    uint32_t ver = rd32(buf + 4), nlod = rd32(buf + 20);
    if (nlod == 0 || nlod > 8) return NULL;
    orc_archive *a = (orc_archive *)calloc(1, sizeof *a);
    a->buf = buf; a->len = len; a->nlod = (int)nlod;
    a->d0.nx = rd32(buf + 24); a->d0.ny = rd32(buf + 28); a->d0.nz = rd32(buf + 32);
    memcpy(a->base_q, buf + 72, 32);
    if (ver == 2) {
        a->version = 2;
        a->dir_off = rd64(buf + 40);
        uint64_t cnt = rd64(buf + 48);
        if (a->dir_off > len || cnt > (len - a->dir_off) / 16) { free(a); return NULL; }
        uint64_t acc = 0;
        for (int l = 0; l < a->nlod; ++l) {
            a->region_prefix[l] = acc;
            uint32_t z, y, x; region_grid(a->d0, l, &z, &y, &x);
            acc += (uint64_t)z * y * x;
        }
        a->region_prefix[a->nlod] = acc;
        if (acc != cnt) { free(a); return NULL; }
        return a;
    }
    if (ver != 1 || rd32(buf + 12) != 1) { free(a); return NULL; }
    a->version = 1;
    a->l1_off = rd64(buf + 56); a->l1_cap = rd64(buf + 40);
    if (!a->l1_cap || (a->l1_cap & (a->l1_cap - 1)) || a->l1_off > len ||
        a->l1_cap > (len - a->l1_off) / 16) { free(a); return NULL; }
    return a;
}
void orc_close(orc_archive *a) { free(a); }
int orc_nlod_of(const orc_archive *a) { return a ? a->nlod : 0; }
float orc_base_q(const orc_archive *a, int lod) { return a->base_q[lod]; }

int orc_lod_dims(const orc_archive *a, int lod, orc_dims *out) {
    if (!a || lod < 0 || lod >= a->nlod || !out) return ORC_ERR_RANGE;
    *out = orc_lod_dims_of(a->d0, lod);
    return ORC_OK;
}

// bytes [off, off+n) inside the archive (the reference's test at :1266)
static int in_file(const orc_archive *a, uint64_t off, uint64_t n) { return off + n <= a->len; }

// Fetch [off, off + n) (:1262-1267): a flat archive copies from its buffer, a
// streaming one asks the callback. 0 on success.
static int rd(const orc_archive *a, uint64_t off, uint32_t n, uint8_t *dst) {
    if (a->read) return a->read(a->ud, off, n, dst) == ORC_OK ? 0 : -1;
    if (!in_file(a, off, n)) return -1;
    memcpy(dst, a->buf + off, n);
    return 0;
}

static int resolve(const orc_archive *a, int lod, uint32_t az, uint32_t ay, uint32_t ax,
                   uint64_t *off, uint32_t *len, uint8_t *dc) {   // :1349-1402
    uint64_t slot_idx = (((uint64_t)(az & 31) * 32 + (ay & 31)) * 32 + (ax & 31));
    uint64_t blk;
    if (a->version == 2) {
        uint32_t nrz, nry, nrx; region_grid(a->d0, lod, &nrz, &nry, &nrx);
        uint32_t rz = az / 32, ry = ay / 32, rx = ax / 32;
        if (rz >= nrz || ry >= nry || rx >= nrx) return 0;
        uint64_t ri = a->region_prefix[lod] + ((uint64_t)rz * nry + ry) * nrx + rx;
        if (ri >= a->region_prefix[a->nlod]) return 0;
        uint8_t e[16];
        if (rd(a, a->dir_off + ri * 16, 16, e)) return 0;
        uint32_t fl = rd32(e + 12);
        if (fl == 0) return 0;
        if (fl == 1) return 2;
        blk = rd64(e);
    } else {
        uint64_t key = region_key(lod, az / 32, ay / 32, ax / 32);
        uint64_t mask = a->l1_cap - 1, i = mix64(key) & mask;
        // bounded probe: a table with no empty bucket and no match is treated as absent
        for (uint64_t step = 0;; ++step) {
            if (step >= a->l1_cap) return 0;
            uint8_t e[16];
            if (rd(a, a->l1_off + i * 16, 16, e)) return 0;
            uint64_t bref = rd64(e + 8);
            if (!bref) return 0;
            if (rd64(e) == key) { blk = bref; break; }
            i = (i + 1) & mask;
        }
        if (blk == 1) return 2;
    }
    if (blk + L2_BYTES > a->len || blk > a->len) return 0;
    uint8_t sl[16];
    if (rd(a, blk + slot_idx * 16, 16, sl)) return 0;   // :1367
    uint8_t fl = sl[12];
    if (fl == 1) { *off = rd64(sl); *len = rd32(sl + 8); *dc = sl[13]; }
    return fl;
}

static int decode_atom_raw(orc_archive *a, int lod, uint32_t ax, uint32_t ay, uint32_t az, uint8_t *out) {
    uint64_t off = 0; uint32_t len = 0; uint8_t dc = 0;
    int fl = resolve(a, lod, az, ay, ax, &off, &len, &dc);
    if (fl == 1) {
        if (off == NO_OFFSET || len < 1 || off > a->len || len > a->len - off) {
            memset(out, 0, N3);
            return ORC_ERR_FORMAT;
        }
        if (!a->read) {
            if (orc_decode_atom_payload(a->buf + off, len, a->base_q[lod], out)) return ORC_ERR_FORMAT;
            return ORC_OK;
        }
        // streaming payload (:1274-1280): at most the reference's scratch of 4 * 32768 + 64 bytes
        uint8_t *pay = len <= 4u * N3 + 64u ? (uint8_t *)malloc(len) : NULL;
        if (!pay || rd(a, off, len, pay)) {
            free(pay);
            memset(out, 0, N3);
            return ORC_ERR_FORMAT;
        }
        int bad = orc_decode_atom_payload(pay, len, a->base_q[lod], out);
        free(pay);
        return bad ? ORC_ERR_FORMAT : ORC_OK;
    }
    memset(out, 0, N3);
    return ORC_OK;
}

int orc_decode_atom(orc_archive *a, int lod, int ax, int ay, int az, uint8_t *out) {   // :1404-1421
    if (!a || lod < 0 || lod >= a->nlod || !out) return ORC_ERR_RANGE;
    orc_dims d = orc_lod_dims_of(a->d0, lod);
    uint32_t acx = (d.nx + 31) / 32, acy = (d.ny + 31) / 32, acz = (d.nz + 31) / 32;
    if ((uint32_t)ax >= acx || (uint32_t)ay >= acy || (uint32_t)az >= acz) return ORC_ERR_RANGE;
    return decode_atom_raw(a, lod, (uint32_t)ax, (uint32_t)ay, (uint32_t)az, out);
}

int orc_decode_region(orc_archive *a, int lod, orc_box b, uint8_t *out) {   // :1535-1555
    if (!a || lod < 0 || lod >= a->nlod || !out) return ORC_ERR_RANGE;
    orc_dims d = orc_lod_dims_of(a->d0, lod);
    if (b.x1 > d.nx || b.y1 > d.ny || b.z1 > d.nz) return ORC_ERR_RANGE;
    if (b.x0 >= b.x1 || b.y0 >= b.y1 || b.z0 >= b.z1) return ORC_ERR_RANGE;
    uint32_t ox = b.x1 - b.x0, oy = b.y1 - b.y0;
    uint8_t *atom = (uint8_t *)malloc(N3);
    for (uint32_t az = b.z0 / 32; az <= (b.z1 - 1) / 32; ++az)
        for (uint32_t ay = b.y0 / 32; ay <= (b.y1 - 1) / 32; ++ay)
            for (uint32_t ax = b.x0 / 32; ax <= (b.x1 - 1) / 32; ++ax) {
                int s = orc_decode_atom(a, lod, (int)ax, (int)ay, (int)az, atom);
                if (s) { free(atom); return s; }
                uint32_t z0 = az * 32 < b.z0 ? b.z0 : az * 32, z1 = az * 32 + 32 > b.z1 ? b.z1 : az * 32 + 32;
                uint32_t y0 = ay * 32 < b.y0 ? b.y0 : ay * 32, y1 = ay * 32 + 32 > b.y1 ? b.y1 : ay * 32 + 32;
                uint32_t x0 = ax * 32 < b.x0 ? b.x0 : ax * 32, x1 = ax * 32 + 32 > b.x1 ? b.x1 : ax * 32 + 32;
                for (uint32_t z = z0; z < z1; ++z)
                    for (uint32_t y = y0; y < y1; ++y)
                        memcpy(out + ((size_t)(z - b.z0) * oy + (y - b.y0)) * ox + (x0 - b.x0),
                               atom + ((z - az * 32) * 32 + (y - ay * 32)) * 32 + (x0 - ax * 32), x1 - x0);
            }
    free(atom);
    return ORC_OK;
}

int orc_decode_lod(orc_archive *a, int lod, uint8_t *out, orc_dims *od) {
    orc_dims d;
    int s = orc_lod_dims(a, lod, &d);
    if (s) return s;
    if (od) *od = d;
    orc_box b = {0, 0, 0, d.nx, d.ny, d.nz};
    return orc_decode_region(a, lod, b, out);
}

int orc_atom_coverage(const orc_archive *a, int lod, uint32_t az, uint32_t ay, uint32_t ax) {
    if (!a || lod < 0 || lod >= a->nlod) return 0;
    uint64_t off; uint32_t len; uint8_t dc;
    int fl = resolve(a, lod, az, ay, ax, &off, &len, &dc);
    return fl == 1 ? 2 : fl == 2 ? 1 : 0;
}

int orc_atom_payload_range(const orc_archive *a, int lod, uint32_t az, uint32_t ay, uint32_t ax,
                           uint64_t *off, uint32_t *len) {
    if (off) *off = 0;
    if (len) *len = 0;
    if (!a || lod < 0 || lod >= a->nlod) return 0;
    uint64_t o = 0; uint32_t l = 0; uint8_t dc = 0;
    int fl = resolve(a, lod, az, ay, ax, &o, &l, &dc);
    if (fl == 1) { if (off) *off = o; if (len) *len = l; return 2; }
    return fl == 2 ? 1 : 0;
}

int orc_archive_version(const orc_archive *a) { return a ? a->version : 0; }

// Whole-LOD decode with a parallel-for over atoms: each atom decoded independently
// into the full LOD raster (the caller-side parallelism the reference relies on).
int orc_decode_lod_mt(orc_archive *a, int lod, uint8_t *out, int nthreads) {
    orc_dims d;
    int s = orc_lod_dims(a, lod, &d);
    if (s) return s;
    uint32_t acx = (d.nx + 31) / 32, acy = (d.ny + 31) / 32, acz = (d.nz + 31) / 32;
    uint64_t na = (uint64_t)acx * acy * acz;
    int err = 0;
    #pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
    for (uint64_t t = 0; t < na; ++t) {
        uint32_t ax = (uint32_t)(t % acx), ay = (uint32_t)((t / acx) % acy), az = (uint32_t)(t / ((uint64_t)acx * acy));
        uint8_t atom[N3];
        if (decode_atom_raw(a, lod, ax, ay, az, atom)) {
            #pragma omp atomic write
            err = 1;
        }
        for (uint32_t z = 0; z < N && az * N + z < d.nz; ++z)
            for (uint32_t y = 0; y < N && ay * N + y < d.ny; ++y) {
                uint32_t x0 = ax * N, cnt = d.nx - x0 < N ? d.nx - x0 : N;
                memcpy(out + ((size_t)(az * N + z) * d.ny + ay * N + y) * d.nx + x0, atom + (z * N + y) * N, cnt);
            }
    }
    return err ? ORC_ERR_FORMAT : ORC_OK;
}

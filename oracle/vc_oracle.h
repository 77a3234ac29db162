// CPU ORACLE — test infrastructure only. A plain-C restatement of the reference
// codec's per-atom path and archive format (src/vc/vc.c of
// SuperOptimizer/volume-compressor), used as the checker in the parity tests and
// as the timed CPU baseline. It is never linked into, loaded by, or called from
// the product library.
//
// Parity pins: every kernel here is checked bit-for-bit against the reference's
// own code compiled with its release flags (oracle/_ref, tests/test_oracle_*.py)
// and against golden archives generated by that build (tests/golden/).
// Float behaviour follows the reference's release build exactly (step table,
// RCPPS-based quantizer; see vc_release_tables.h).
#ifndef VC_ORACLE_H
#define VC_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { uint32_t nx, ny, nz; } orc_dims;
typedef struct { uint32_t x0, y0, z0, x1, y1, z1; } orc_box;

enum { ORC_OK = 0, ORC_ERR_FORMAT = 1, ORC_ERR_RANGE = 2, ORC_ERR_OOM = 3, ORC_ERR_IO = 4 };

// ---- tables (src/vc/vc.c:75-88, 266-290, 462-468)
void     orc_tables(int32_t *cmat /*1024*/, float *step /*32768*/, uint16_t *scan /*32768*/);
int      orc_band_of(uint32_t raster);

// ---- per-atom kernels
void     orc_fdct(const uint8_t *vox, int32_t dc, int32_t *coef);
void     orc_idct(const int32_t *coef, int32_t dc, uint8_t *vox);
void     orc_quantize(const int32_t *coef, float base_q, int16_t *lv);
void     orc_dq_tables(float base_q, int32_t *dq_step, int32_t *dq_bias);
void     orc_dequantize(const int16_t *lv, float base_q, int32_t *coef);
uint32_t orc_enc_levels(const int16_t *lv, uint8_t *out, uint32_t cap);
// returns 0, or 1 when the stream is malformed (escape prefix longer than 32 bits)
int      orc_dec_levels(const uint8_t *buf, uint32_t len, int16_t *lv);
uint32_t orc_rc_size(const int16_t *lv);   // byte count of orc_enc_levels without output
uint32_t orc_encode_atom(const uint8_t *vox, float base_q, uint8_t *out, uint32_t cap,
                         int *is_zero, uint8_t *dc);
int      orc_decode_atom_payload(const uint8_t *pay, uint32_t len, float base_q, uint8_t *vox);

// ---- pyramid (src/vc/vc.c:1562-1577)
void     orc_downsample2x(const uint8_t *in, orc_dims d, uint8_t *out);
// exporter downscale (tools/downscale.h): method 0 = DS_BOX, 1 = DS_CBOX
uint8_t  orc_ds_cell(const uint8_t *c8, int method, float alpha);
void     orc_ds_downscale2x(const uint8_t *in, orc_dims d, int method, float alpha, uint8_t *out, orc_dims *od);
void     orc_ds_set_fused(int fused);   // CBOX push as one fma (default) or multiply + add
int      orc_nlod(orc_dims d0);
orc_dims orc_lod_dims_of(orc_dims d0, int lod);

// ---- whole-volume encode (canonical single-threaded append order)
float    orc_rate_control(const uint8_t *vol, orc_dims d, float target_ratio,
                          int nthreads, uint64_t *present, uint64_t *bytes);
int      orc_encode_fixed_q(const uint8_t *vol, orc_dims d, float target_ratio,
                            const float *base_q /*nlod*/, int nthreads,
                            uint8_t **out, size_t *out_len);
int      orc_encode(const uint8_t *vol, orc_dims d, float target_ratio, int nthreads,
                    uint8_t **out, size_t *out_len);
void     orc_free(void *p);

// ---- reader (src/vc/vc.c:1285-1555)
typedef struct orc_archive orc_archive;
orc_archive *orc_open(const uint8_t *buf, size_t len);
typedef int (*orc_read_fn)(void *ud, uint64_t off, uint32_t len, uint8_t *dst);   // 0 = ok
orc_archive *orc_open_streaming(orc_read_fn read, void *ud, uint64_t total_len);
void     orc_close(orc_archive *a);
int      orc_lod_dims(const orc_archive *a, int lod, orc_dims *out);
int      orc_nlod_of(const orc_archive *a);
float    orc_base_q(const orc_archive *a, int lod);
int      orc_decode_atom(orc_archive *a, int lod, int ax, int ay, int az, uint8_t *out);
int      orc_decode_region(orc_archive *a, int lod, orc_box box, uint8_t *out);
int      orc_decode_lod(orc_archive *a, int lod, uint8_t *out, orc_dims *out_dims);
int      orc_atom_coverage(const orc_archive *a, int lod, uint32_t az, uint32_t ay, uint32_t ax);
int      orc_atom_payload_range(const orc_archive *a, int lod, uint32_t az, uint32_t ay, uint32_t ax,
                                uint64_t *off, uint32_t *len);
int      orc_archive_version(const orc_archive *a);

// ---- multi-threaded CPU baselines (caller-side parallel-for over atoms, as the
// reference's callers do; plan.txt:38-39)
int      orc_decode_lod_mt(orc_archive *a, int lod, uint8_t *out, int nthreads);
uint64_t orc_encode_sizes_mt(const uint8_t *vol, orc_dims d, float base_q,
                             const uint32_t *atom_ids, uint32_t n_atoms, uint32_t *lens,
                             int nthreads);

#ifdef __cplusplus
}
#endif
#endif

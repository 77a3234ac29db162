// Internal interface between the C host library (vc_host.c) and the CUDA
// device layer (*.cu): plain C structs and extern "C" functions, no CUDA or
// torch types. Not installed; the public boundary is include/vc.h + vcg.h.
#ifndef VC_INTERNAL_H
#define VC_INTERNAL_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VCD_NCLASS 188          // quantizer step classes: L1 frequency f (0..93) + 94 * alt bit
#define VCD_MAX_ENTRIES 32768u  // one atom's coefficients

// Kinds in the resolved atom table.
enum { VCD_EMPTY = 0, VCD_PRESENT = 1, VCD_BAD = 2 };

// One atom of an archive, resolved on the host from the v1 hash index / v2
// directory plus its L2 slot (src/vc/vc.c:1349-1402), with the payload range
// already checked against the archive length.
typedef struct {
    uint64_t off;   // payload byte offset in the archive (PRESENT)
    uint32_t len;   // payload bytes, >= 1 (PRESENT)
    uint8_t kind;   // VCD_EMPTY (absent or known-zero), VCD_PRESENT, VCD_BAD
    uint8_t dc;     // slot dc byte (informational; decode uses payload byte 0)
    uint16_t rsv;
} vcd_atom;

// Per-LOD dequantisation tables by step class (src/vc/vc.c:314-326).
typedef struct {
    int32_t step[VCD_NCLASS];
    int32_t bias[VCD_NCLASS];
} vcd_dq;

// Per-q quantiser constants by step class (src/vc/vc.c:293-306 as the release
// build evaluates it): step, dead zone 0.8*step, refined reciprocal of step.
typedef struct {
    float step[VCD_NCLASS];
    float dz[VCD_NCLASS];
    float rr[VCD_NCLASS];
} vcd_quant;

// Constant tables shared by every kernel.
typedef struct {
    uint32_t alt_mask[1024];   // bit i: raster index i uses the alternate step value
    uint16_t scan[32768];      // scan position -> raster index
    uint16_t rank_base[94 * 32];  // scan position of (f, kz, ky = max(0, f-kz-31))
    uint32_t band_start[9];    // first scan position of each significance band, [8] = 32768
} vcd_tables;

// Region / LOD decode request, resolved on the host.
typedef struct {
    const vcd_atom *atoms;      // host table of this LOD (raster az, ay, ax)
    uint64_t atom_base;         // index of this LOD's first atom in the device table
    uint32_t acx, acy, acz;     // LOD atom grid
    uint32_t x0, y0, z0, x1, y1, z1;   // box (voxels)
    uint32_t bax, bay, baz;     // first atom of the box
    uint32_t bnx, bny, bnz;     // atoms of the box per axis
    uint64_t n_atoms;           // atoms to decode (box order z, y, x), stops at the first bad
    uint64_t cap_total;         // sum of entry capacities of those atoms
    uint64_t payload_bytes;     // sum of their payload lengths (for profiling)
    uint64_t present;           // PRESENT atoms among them
    int lod;
} vcd_region;

// Batched region decode, built on the host.
typedef struct {         // one request box (device view)
    uint8_t *out;        // box raster, device memory (filled in by the device layer for host outputs)
    uint32_t x0, y0, z0, x1, y1, z1;
    uint32_t lod, rsv;
} vcd_boxreq;
typedef struct {         // one distinct atom of a batch
    uint64_t idx;        // index in the archive's atom table (all LODs)
    uint32_t lod, az, ay, ax;
    uint32_t dst_begin, dst_end;   // the requests it feeds: dst[dst_begin .. dst_end)
    uint32_t rsv;
} vcd_uatom;
typedef struct {
    uint32_t n_req, n_ua, n_dst;
    vcd_boxreq *reqs;
    const vcd_uatom *ua;
    const uint32_t *dst;
    const uint64_t *ent_off;  // per distinct atom
    uint64_t cap_total;       // list entries in total
} vcd_batch;

typedef struct vcd_archive vcd_archive;   // device residency of one archive

// ---- device layer (vc_device.cu) ------------------------------------------
int  vcd_init(void);                        // 0 ok; -1 no usable device; makes the library's device current
// The library runs on one device (VC_DEVICE, default 0). A public entry point
// that uses the GPU opens with VCD_SCOPE(): the library's device is made current
// for the call (once the library is initialised; the first vcd_init selects it)
// and the caller's current device is current again when the call returns.
int  vcd_enter(void);                       // the caller's current device, or -1
void vcd_leave(int *prev);
#define VCD_SCOPE() int vcd_prev_ __attribute__((cleanup(vcd_leave))) = vcd_enter()
const char *vcd_last_error(void);
// residency: begin starts the copy of the archive bytes, finish adds the atom
// table and the dequantisation tables and waits (the caller frees on failure)
int  vcd_upload_begin(vcd_archive **out, const uint8_t *buf, size_t len);
int  vcd_upload_finish(vcd_archive *d, const vcd_atom *atoms, uint64_t n_atoms, const vcd_dq *dq /*nlod*/, int nlod);
void vcd_free_archive(vcd_archive *d);
// decode into a device buffer (out_dev, box bytes) or, when out_dev is NULL, into
// the host buffer out_host (box raster); returns 0 or a vc_status
int  vcd_decode_region(vcd_archive *d, const vcd_region *r, uint8_t *out_dev, uint8_t *out_host,
                       size_t out_bytes);

// Streamed decode (archives opened on a read callback). The archive's device
// side holds only the dequantisation tables. Per call, the host fills a pinned
// staging area: a box-local atom table (one vcd_atom per box atom, box order
// z, y, x, offsets relative to the payload area) and the payloads packed after
// it; uploads of finished pieces overlap the filling of the next.
int  vcd_upload_dq(vcd_archive **out, const vcd_dq *dq /*nlod*/, int nlod);
int  vcd_stage_reserve(size_t bytes, uint8_t **host);          // pinned staging of >= bytes
int  vcd_stage_push(size_t off, size_t bytes);                 // async upload of [off, off+bytes)
int  vcd_decode_staged(vcd_archive *d, const vcd_region *r, size_t table_off, size_t arena_off,
                       size_t arena_bytes, uint8_t *out_dev, uint8_t *out_host, size_t out_bytes);

// Batched decode. Outputs: reqs[i].out (device) when host_out is NULL, else
// host_out[i] (the device layer stages through its own buffer). req_err[i] is
// set to 1 for requests that met a malformed stream.
int  vcd_decode_batch(vcd_archive *d, const vcd_batch *b, uint8_t *const *host_out, uint32_t *req_err);

// Encode: volume (device or host) -> canonical archive (host malloc).
typedef struct {
    uint32_t nx, ny, nz;
    float target_ratio;
    int nlod;
    uint64_t l1_cap;
    int fixed_q;        // 1: use q[] as given (no rate control)
    float q[8];         // per-LOD base_q when fixed_q
    float q0;           // chosen LOD0 base_q (output)
    uint64_t present0;  // present LOD0 atoms (output)
    uint64_t bytes0;    // LOD0 payload bytes at q0 (output)
    int ds_method;      // pyramid: 0 the codec's rule (= DS_BOX), 1 DS_CBOX
    float ds_alpha;     // DS_CBOX push
} vcd_encode_info;
int  vcd_encode(const uint8_t *vol, int vol_on_device, vcd_encode_info *info, uint8_t **out,
                size_t *out_len);

// Writer batches: independent atoms encoded on the device. A segment is a host
// raster (x fastest) of nx x ny x nz voxels, each a multiple of 32, whose atoms
// (raster order of its atom grid) are encoded each with the quantiser qs[qsel[i]]
// (src/vc/vc.c:595-622). len[i] receives the payload bytes ([dc][coder bytes];
// 0 for an all-zero atom) and off[i] the payload's offset in *pay, where all
// payloads of all segments are packed in segment order (a pinned buffer owned by
// the calling thread, valid until its next call).
typedef struct {
    const uint8_t *vox;
    uint32_t nx, ny, nz;
    const uint8_t *qsel;
    uint32_t *len;
    uint64_t *off;
} vcd_seg;
int  vcd_encode_segments(const vcd_seg *segs, int nseg, const float *qs, int nq, uint8_t **pay, uint64_t *pay_bytes);

// Exporter 2x downscale (tools/downscale.h): levels 1..levels of the cascade
// from in; level l into out[l-1]. Device pointers when on_device, else host
// pointers (staged through device memory).
int  vcd_downscale(const uint8_t *in, int on_device, const uint32_t dims[3], int method, float alpha, int levels,
                   uint8_t *const *out);

// Repack into the v2 container (device): one record per non-absent atom slot of
// the output. flags 1 = present (slot [pay_dst][len][1][dc = first payload
// byte], payload src..src+len of the resident archive copied to pay_dst),
// flags 2 = known zero (slot byte 12 = 2). head (header + region directory,
// head_len bytes) goes to offset 0; everything else of the total_len-byte image
// is zero. The image is copied into host_out.
typedef struct {
    uint64_t slot_dst, src, pay_dst;
    uint32_t len, flags;
} vcd_repack_rec;
int  vcd_repack(vcd_archive *d, const uint8_t *head, uint64_t head_len, uint64_t total_len,
                const vcd_repack_rec *recs, uint64_t n_recs, uint8_t *host_out);

// ---- host helpers shared with the device layer (vc_host.c) ----------------
void vch_tables(vcd_tables *t);
void vch_quant_consts(float base_q, vcd_quant *q);
void vch_dq_consts(float base_q, vcd_dq *dq);
float vch_clamp_q(float q);
uint64_t vch_region_key(int lod, uint32_t rz, uint32_t ry, uint32_t rx);
uint64_t vch_mix64(uint64_t x);

#ifdef __cplusplus
}
#endif
#endif

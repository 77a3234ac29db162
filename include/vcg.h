// vcg.h — GB300 extensions to the vc.h C API (no counterpart in the reference
// unless stated). Plain C types only: device buffers are passed as pointers
// returned by vcg_alloc (or any CUDA device allocation on the same device).
#ifndef VCG_H
#define VCG_H

#include <stddef.h>
#include <stdint.h>

#include "vc.h"

#ifdef __cplusplus
extern "C" {
#endif

// Decode into device memory instead of a host buffer (same results and
// statuses as vc_decode_region / vc_decode_lod). On VC_ERR_FORMAT the contents
// of out_dev are unspecified.
vc_status vcg_decode_region_device(vc_archive *a, int lod, vc_box box, uint8_t *out_dev);
vc_status vcg_decode_lod_device(vc_archive *a, int lod, uint8_t *out_dev, vc_dims *out_dims);

// Batched region decode: many boxes (any LODs, sizes and offsets) of one
// archive in one device pass. Every distinct atom the batch touches is decoded
// once and cropped into each box that overlaps it. status[i] is what
// vc_decode_region would return for request i, and outputs follow its rules
// (a request that meets a bad atom gets only the atoms before it, z-y-x order).
// out_on_device != 0: every out is device memory; else host memory. The launch
// shape is autotuned on the process's first batch; a thread's later batches
// replay one CUDA graph while the batch buffers keep their addresses.
typedef struct {
    int32_t lod;
    vc_box box;
    uint8_t *out;   // (x1-x0)*(y1-y0)*(z1-z0) bytes, raster (z, y, x)
} vcg_region_request;
vc_status vcg_decode_regions(vc_archive *a, uint32_t n, const vcg_region_request *reqs, int out_on_device,
                             vc_status *status);
// Launch shape the calling thread uses (0 before its first batch): range-decoder
// policy (warps per SM sub-partition that decode one atom each before atoms
// share warps in lockstep; see vcg_set_rc_scalar_warps), transform CTA size
// (32 x warps per atom) and transform form (0 butterfly on the CUDA cores,
// 1 int8 tensor cores). The autotuner times every combination on the process's
// first batch; all give identical bytes.
void vcg_batch_shape(int *rc_scalar_warps, int *transform_threads, int *transform_imma);
// Fix the shape of every later batch instead of autotuning (rc_scalar_warps 1,
// 4 or 16; transform_threads 256 or 512 for the butterfly, 256 for the tensor
// cores); rc_scalar_warps = 0 returns to the tuned shape. VC_ERR_RANGE for a
// shape that is not a candidate.
vc_status vcg_set_batch_shape(int rc_scalar_warps, int transform_threads, int transform_imma);

// Range-decoder policy of vc_decode_region / vc_decode_lod / vc_decode_atom and
// the device-output variants (process-wide; results do not depend on it). Up
// to one atom per SM sub-partition (4 per SM) each atom has a warp running the
// latency-tuned scalar decoder; up to w warps per sub-partition, one atom per
// warp with the plain scalar decoder, longest payloads first; above that the
// per-lane decoder (every lane of a warp decodes its own atom, atoms in order
// of payload length). w = 0: no atom keeps a warp to itself (above one atom
// per sub-partition the per-lane decoder, below it atoms share warps in
// lockstep); w < 0 restores the default (8: measured on GB300, the per-lane
// decoder wins from 3,000-5,000 atoms on, depending on the atoms' sizes).
void vcg_set_rc_scalar_warps(int w);
// The per-lane decoder's n longest atoms (by payload length) each get a warp of
// their own running the latency-tuned decoder, on a second stream beside it
// (process-wide; results do not depend on it). The longest atoms set the
// per-lane decoder's time, and the latency decoder takes about half the time
// per decision; whether that shortens the decode depends on which SM
// sub-partitions the solo warps land on, which the launch does not control.
// n = 0 (the default): none; n < 0 restores the default.
void vcg_set_rc_solo(int n);

// Decode server: continuous batching against one resident archive. Requests
// queue with vcg_server_submit; `workers` threads (each with its own stream)
// take waiting requests in arrival order, as many as fit `device_budget` bytes
// (box output + list scratch) and `max_batch`, decode them with
// vcg_decode_regions and release their memory; requests that arrive while
// batches run join the next batch, and batches of different workers overlap on
// the device. Results and statuses equal vc_decode_region's for each request.
typedef struct vcg_server vcg_server;
vcg_server *vcg_server_create(vc_archive *a, uint64_t device_budget, uint32_t max_batch, int workers);
// out: host memory of the box's size, valid until the ticket completes; returns a ticket >= 0, or -1
int64_t vcg_server_submit(vcg_server *s, int lod, vc_box box, uint8_t *out);
// blocks until the ticket is done; latency_us (optional) = submit-to-completion
// time. Each ticket is waited for once (its slot is then recycled; a second wait
// is VC_ERR_RANGE); tickets that are never waited for keep their slots.
vc_status vcg_server_wait(vcg_server *s, int64_t ticket, double *latency_us);
void vcg_server_stats(vcg_server *s, uint64_t *batches, uint64_t *requests);
// finishes all queued requests, then stops the workers
void vcg_server_destroy(vcg_server *s);

// Rewrite an archive (v1 or v2) into the v2 container, byte-identical to the
// reference's repack tool (tools/vc_repack.c): region directory + one
// contiguous blob per region with a present atom, coarse LOD first, payloads
// copied verbatim. The image is assembled on the device from the resident
// archive; *out_archive is malloc'd. VC_ERR_FORMAT for an archive with a payload
// range outside the file.
vc_status vcg_repack_v2(vc_archive *a, uint8_t **out_archive, size_t *out_len);

// Resolve the archive's atom table and copy archive + table into device
// memory now (otherwise done on the first decode). A streaming archive is
// first pulled whole through its read callback (VC_ERR_IO if a read fails; it
// then stays streaming); batched decode, the server and repack make it
// resident this way on their first call, while vc_decode_* of a streaming
// archive that is not resident pull only what the box needs.
vc_status vcg_make_resident(vc_archive *a);

// Host threads that call a streaming archive's read callback during one
// decode: 1 (the default) keeps every call on the decoding thread; up to 64
// for callbacks that are safe to call concurrently. Returns the previous value.
int vcg_set_stream_threads(int n);

// A vc_read_fn byte source over a host buffer (tests, benchmarks): ud points
// to a vcg_memory_source; reads and bytes count the calls and bytes served.
// A range outside [0, len) returns VC_ERR_FORMAT.
typedef struct {
    const uint8_t *buf;
    uint64_t len;
    uint64_t reads, bytes;
} vcg_memory_source;
vc_status vcg_memory_read(void *ud, uint64_t off, uint32_t len, uint8_t *dst);

// vc_encode with the volume already in device memory; *q0 (optional)
// receives the LOD0 base_q chosen by rate control.
vc_status vcg_encode_device(const uint8_t *vol_dev, vc_dims dims, float target_ratio,
                            uint8_t **out_archive, size_t *out_len, float *q0);

// Encode with an explicit base_q per LOD (the reference's vc_set_base_q
// semantics: each q is clamped to [0.05, 4096]; q <= 0 for a LOD below the
// volume's LOD count is VC_ERR_RANGE) instead of rate control. vol is host
// memory, or device memory when vol_on_device is nonzero.
vc_status vcg_encode_q(const uint8_t *vol, int vol_on_device, vc_dims dims, float target_ratio,
                       const float base_q[VC_NLOD], uint8_t **out_archive, size_t *out_len);

// Asynchronous appends (no counterpart in the reference). vc_append_atom
// returns once its atom is in the image, which on the GPU costs one pass of the
// serial range coder per call; a caller that appends many atoms queues them
// with vcg_append_atom_async (the atom is copied; argument errors return at
// once) and they are encoded in batches of thousands. Every 8192 queued atoms
// the appending caller commits them; vcg_writer_flush commits the rest and
// returns VC_OK or the first failure among the appends queued since the last
// flush (*failed: how many). Order with the other calls is kept; the readers
// see a queued atom after the flush; vc_writer_close flushes.
vc_status vcg_append_atom_async(vc_writer *w, int lod, uint32_t az, uint32_t ay, uint32_t ax,
                                const uint8_t vox[VC_ATOM3]);
vc_status vcg_writer_flush(vc_writer *w, uint64_t *failed);

// The exporter's 2x downscale (tools/downscale.h:29-93) on the GPU. Every
// output voxel is a function of its own 2x2x2 cell; odd boundaries replicate
// the edge voxel; output dims are (n + 1) / 2 per axis.
//   VCG_DS_BOX   rounded mean, (sum + 4) >> 3 (the codec's own pyramid rule)
//   VCG_DS_CBOX  the mean pushed by alpha toward the cell's voxel of largest
//                deviation; the exporter's default, alpha 0.5
// alpha must be finite; method anything else is VC_ERR_RANGE.
#define VCG_DS_BOX 0
#define VCG_DS_CBOX 1
// One level: in and out both in device memory (on_device != 0) or both host.
vc_status vcg_downscale2x(const uint8_t *in, int on_device, vc_dims dims, int method, float alpha, uint8_t *out,
                          vc_dims *out_dims);
// Levels 1..levels (at most 8) of the cascade of a device volume: out_dev[l-1]
// receives level l, each level the downscale of the one before.
vc_status vcg_downscale_pyramid(const uint8_t *vol_dev, vc_dims dims, int method, float alpha, int levels,
                                uint8_t *const *out_dev);
// vc_encode (base_q NULL: rate control) or vcg_encode_q (base_q given) with the
// LOD pyramid built by the exporter's downscale instead of the codec's rule.
// VCG_DS_BOX gives exactly the archive of vc_encode / vcg_encode_q.
vc_status vcg_encode_ds(const uint8_t *vol, int vol_on_device, vc_dims dims, float target_ratio,
                        const float base_q[VC_NLOD], int method, float alpha, uint8_t **out_archive,
                        size_t *out_len);

// Decode without allocating (no counterpart in the reference). For callers
// that cannot let a library allocate device memory: applications that reserve
// the whole GPU for their own pool up front, so a library cudaMalloc would
// fail, and latency-bound pipelines that cannot take the device-wide
// synchronisation that cudaMalloc / cudaFree may cause. Decodes up to
// VCG_NOALLOC_MAX_ATOMS atom payloads already in device memory: payload i is
// payload_dev[offsets[i], offsets[i] + lengths[i]) ([dc byte][coder bytes] as
// stored in an archive, e.g. from vc_atom_payload_range; length 0 = all-zero
// atom); offsets and lengths are host arrays; base_q is the LOD's base_q. Atom
// i goes to out_dev + i * VC_ATOM3 (raster z, y, x). payload_dev must be
// 4-byte aligned and payload_bytes is its size. Returns VC_ERR_RANGE for more
// than VCG_NOALLOC_MAX_ATOMS atoms, VC_ERR_FORMAT for a range outside the
// buffer or a malformed payload.
// Scratch is one fixed device array (about 8 MiB) that every GPU using this
// library keeps until the process exits; all calls share it and it keeps the
// last call's contents, so calls whose GPU work overlaps race and must be
// serialised by the caller. The first call on a device sets the array up
// (with that device current). Runs on the calling thread's default stream.
#define VCG_NOALLOC_MAX_ATOMS 64
vc_status vcg_decode_atoms_noalloc(const uint8_t *payload_dev, size_t payload_bytes, const uint64_t *offsets,
                                   const uint32_t *lengths, uint32_t n_atoms, float base_q, uint8_t *out_dev);

// Exact integer 3-D DCT-32 of every atom of a volume in device memory (no
// counterpart in the reference's API: the reference's per-atom transform,
// src/vc/vc.c:212-229). `centre` is subtracted from every voxel (0..255, e.g.
// 128 for u8 centred to signed) or, with VCG_DCT_ATOM_DC, each atom's dc
// = (sum of its voxels + 16384) / 32768 as the codec uses (src/vc/vc.c:603):
// the forward writes it to dc_dev[atom], the inverse reads it from there
// (dc_dev: device memory, one byte per atom; ignored otherwise). dims must be
// multiples of 32; coef_dev / vol_dev 16-byte aligned device memory. Atoms are
// taken in raster order (az, ay, ax); atom i's coefficients are
// coef[i*32768 ...] in (kz, ky, kx) raster order. The inverse applies the
// reference's inverse transform and adds the centre back, clamped to [0, 255].
// Both forms give the reference's bits for every input: VCG_DCT_BUTTERFLY runs
// the even/odd butterfly on the CUDA cores, VCG_DCT_IMMA runs each pass as int8
// tensor-core matrix products over hi/lo pieces; *redone (optional) receives
// the number of atoms the IMMA form handed to the butterfly because an
// intermediate left its piece range (always 0 for the forward transform).
enum { VCG_DCT_BUTTERFLY = 0, VCG_DCT_IMMA = 1 };
#define VCG_DCT_ATOM_DC (-1)
vc_status vcg_dct_forward(const uint8_t *vol_dev, vc_dims dims, int centre, int form, int32_t *coef_dev,
                          uint8_t *dc_dev, uint32_t *redone);
vc_status vcg_dct_inverse(const int32_t *coef_dev, const uint8_t *dc_dev, vc_dims dims, int centre, int form,
                          uint8_t *vol_dev, uint32_t *redone);

// Seeded synthetic scroll-sheet volume (the benchmark workload) generated on
// the device; byte-identical to the host generator in libvcsynth.
int vcg_synth_volume_device(uint32_t nx, uint32_t ny, uint32_t nz, uint64_t seed, uint8_t *out_dev);

// Measurement. Each decode / encode call brackets its kernels with CUDA events
// on its own stream; vcg_last_call_ms returns that device time for the calling
// thread's last call. With profiling enabled, per-stage device times, launch
// counts, algorithmic bytes read / written and work units are accumulated per
// kernel stage and read back (and optionally reset) with vcg_profile_read.
// Enabling it changes two schedules so that each stage can be timed alone: a
// batch of regions runs its two kernels without the CUDA graph, and an encode
// runs the coarser LODs after LOD0 rather than beside it on a second stream.
typedef struct {
    char name[32];
    double ms;
    uint64_t launches;
    uint64_t bytes_read;
    uint64_t bytes_written;
    uint64_t units;
} vcg_kernel_stat;
void   vcg_profile_enable(int on);
int    vcg_profile_read(vcg_kernel_stat *out, int max, int reset);
double vcg_last_call_ms(void);

// Device / pinned memory helpers (cudaMalloc / cudaMallocHost / cudaMemcpy
// with direction inferred).
void *vcg_alloc(size_t bytes);
void  vcg_free(void *p);
void *vcg_alloc_host(size_t bytes);
void  vcg_free_host(void *p);
int   vcg_copy(void *dst, const void *src, size_t bytes);
int   vcg_memset(void *dst, int v, size_t bytes);
int   vcg_sync(void);
int   vcg_device_info(int *num_sms, int *cc_major, int *cc_minor);
int   vcg_device_memory(size_t *free_bytes, size_t *total_bytes);   // cudaMemGetInfo of the library's device

// Allocation-failure injection, for tests: with n > 0, the n-th device or
// pinned-host allocation the library makes from now on fails as if the device
// were out of memory (once); n <= 0 turns it off. Returns the previous state:
// allocations still to go before the failure, -1 if the failure happened, 0
// if off. Arming (n > 0) also frees the device blocks kept from closed
// archives. A call that meets the failure returns VC_ERR_OOM (or NULL / -1 where
// it returns a handle or ticket), or succeeds where it has a path that needs no
// new allocation, and leaves the library usable.
int64_t vcg_debug_fail_alloc(int64_t n);
const char *vcg_last_error(void);

#ifdef __cplusplus
}
#endif
#endif // VCG_H

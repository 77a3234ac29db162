// vc.h — drop-in C API of the GB300 volume codec.
//
// Same names, types, enum values, macros and coordinate orders as the reference
// library's public header (src/vc/vc.h of SuperOptimizer/volume-compressor), for
// the per-atom codec path: reading archives (v1 sparse-hash and v2
// region-directory containers) and encoding whole volumes. Every decode and
// encode runs on the GPU (hand-written CUDA for sm_103a); there is no CPU
// fallback — without a usable CUDA device these calls return VC_ERR_IO.
//
// Two entry points that the reference documents (README.md:51-58,
// plan.txt:206-211) but no longer ships are defined here as compositions of the
// reference semantics: vc_encode and vc_decode_lod.
#ifndef VC_H
#define VC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// src/vc/vc.h:15-21
typedef enum {
    VC_OK = 0,
    VC_ERR_FORMAT = 1,
    VC_ERR_RANGE = 2,
    VC_ERR_OOM = 3,
    VC_ERR_IO = 4,
} vc_status;

// src/vc/vc.h:23-30 — extents are x fastest, z slowest; boxes are half-open.
typedef struct {
    uint32_t nx, ny, nz;
} vc_dims;

typedef struct {
    uint32_t x0, y0, z0;
    uint32_t x1, y1, z1;
} vc_box;

// src/vc/vc.h:32-35
#define VC_ATOM    32u
#define VC_ATOM3   (32u*32u*32u)
#define VC_NLOD    8
#define VC_MAX_DIM (1u<<20)

// src/vc/vc.h:40 — ABSENT: never written; KNOWN_ZERO: written as all-zero.
typedef enum { VC_ABSENT = 0, VC_KNOWN_ZERO = 1, VC_PRESENT = 2 } vc_cover;

typedef struct vc_archive vc_archive;

// Encode a whole volume (x fastest, dims.nx*dims.ny*dims.nz bytes) into a v1
// archive held in memory. Builds the 2x LOD pyramid (src/vc/vc.c:1562-1577),
// picks base_q for LOD0 by bisection on the measured present-atom ratio
// (32768 * present atoms / payload bytes, closest to target_ratio) and uses
// base_q * 0.6^l (floored at 0.05) for coarser LODs, then lays the archive out
// exactly as vc_create + vc_set_base_q + vc_append_atom (every atom of every
// LOD in raster order, from one thread) + vc_writer_close would
// (src/vc/vc.c:995-1245). *out_archive is malloc'd; the caller free()s it.
// Returns VC_ERR_RANGE for invalid dims or target_ratio < 1 (or NaN).
vc_status vc_encode(const uint8_t *vol, vc_dims dims, float target_ratio,
                    uint8_t **out_archive, size_t *out_len);

// ---------------------------------------------------------------------------
// Writer (src/vc/vc.h:42-95, src/vc/vc.c:995-1245): builds a v1 archive file by
// appending atoms. Atoms are encoded on the GPU; a call returns when its atoms
// are in the image, as in the reference, and concurrent calls from several
// threads are encoded together in one device batch. The file layout follows
// the order in which calls are laid out: a single thread gets exactly the
// reference's bytes. Thread-safe: many readers and writers may share one handle.
// ---------------------------------------------------------------------------
typedef struct vc_writer vc_writer;

// src/vc/vc.h:56 — create (or truncate) the archive file at path for a volume
// whose LOD0 is lod0_dims. NULL on invalid dims, target_ratio < 1 or an I/O error.
vc_writer *vc_create(const char *path, vc_dims lod0_dims, float target_ratio);

// src/vc/vc.h:63 — base_q of a LOD, clamped to [0.05, 4096]; an append reads it
// when it is called. VC_ERR_RANGE for a LOD outside the archive.
vc_status vc_set_base_q(vc_writer *w, int lod, float q);

// src/vc/vc.h:66 — append one atom. VC_ERR_RANGE for a LOD or atom outside the
// archive, or a nonzero atom of a LOD without base_q; an all-zero atom is
// stored KNOWN_ZERO. Appending an atom again replaces it.
vc_status vc_append_atom(vc_writer *w, int lod, uint32_t az, uint32_t ay, uint32_t ax,
                         const uint8_t vox[VC_ATOM3]);

// src/vc/vc.h:73 — append a box of whole atoms (origin and size multiples of
// 32), raster (z, y, x) order, x fastest; atoms go in (z, y, x) order and the
// call stops at the first that fails.
vc_status vc_append_box(vc_writer *w, int lod, vc_box voxel_box, const uint8_t *voxels);

// src/vc/vc.h:78-79 — mark an atom / an index region (atom coords / 32)
// KNOWN_ZERO without a payload. A region that has a block keeps it.
vc_status vc_mark_zero_atom(vc_writer *w, int lod, uint32_t az, uint32_t ay, uint32_t ax);
vc_status vc_mark_zero_region(vc_writer *w, int lod, uint32_t rz, uint32_t ry, uint32_t rx);

// src/vc/vc.h:84-92 — read back from the writer (decoded on the GPU with the
// current base_q): an atom as vc_decode_atom would, its coverage, or the 8 atoms
// of a 2x2x2 block in (dz, dy, dx) order (absent, zero, invalid or outside the
// LOD: zeros; *any set if one was present).
vc_status vc_writer_decode_atom(vc_writer *w, int lod, uint32_t az, uint32_t ay, uint32_t ax,
                                uint8_t out[VC_ATOM3]);
vc_cover  vc_writer_coverage(vc_writer *w, int lod, uint32_t az, uint32_t ay, uint32_t ax);
vc_status vc_writer_decode_2x2x2(vc_writer *w, int lod, uint32_t az0, uint32_t ay0, uint32_t ax0,
                                 uint8_t out8[8][VC_ATOM3], int *any);

// src/vc/vc.h:95 — trim the file to its used length and close it (no unlink).
void vc_writer_close(vc_writer *w);

// src/vc/vc.h:106 — open an archive held in memory. Borrows the buffer: it must
// outlive the handle. Returns NULL if the header is not a valid v1/v2 header.
// The archive bytes are copied into device memory on first decode.
vc_archive *vc_open(const uint8_t *archive, size_t len);

// src/vc/vc.h:108-112 — byte source of a streaming archive: fill dst with
// exactly len bytes from archive offset off; return VC_OK on success.
typedef vc_status (*vc_read_fn)(void *ud, uint64_t off, uint32_t len, uint8_t *dst);

// src/vc/vc.h:118 — open an archive without holding it: the header here, and
// the index entries, slots and payloads each decode needs, are pulled through
// read on demand. total_len is the archive's size. Results equal vc_open's on
// the same bytes. As in the reference, an index entry or slot whose read fails
// is absent, and a payload whose read fails, or that is longer than 131136
// bytes, makes its atom VC_ERR_FORMAT. read is called only from the decoding
// thread unless vcg_set_stream_threads allows more; it must outlive the handle.
vc_archive *vc_open_streaming(vc_read_fn read, void *ud, uint64_t total_len);

// src/vc/vc.h:120 — NULL is allowed.
void vc_close(vc_archive *a);

// src/vc/vc.h:123 — dims of any LOD (strict 2x pyramid from LOD0).
vc_status vc_lod_dims(const vc_archive *a, int lod, vc_dims *out);

// Decode a whole LOD into out_vol (out_dims.nx*ny*nz bytes, x fastest):
// vc_lod_dims followed by vc_decode_region over the full box.
vc_status vc_decode_lod(vc_archive *a, int lod, uint8_t *out_vol, vc_dims *out_dims);

// src/vc/vc.h:126 — one 32^3 atom; note the (ax, ay, az) argument order.
// ABSENT and KNOWN_ZERO atoms decode to zeros.
vc_status vc_decode_atom(vc_archive *a, int lod, int ax, int ay, int az,
                         uint8_t out[VC_ATOM3]);

// src/vc/vc.h:130 — decode the voxels of box (half-open, inside the LOD) into
// out, raster (z - z0, y - y0, x - x0). On VC_ERR_FORMAT the atoms before the
// first bad atom (z, y, x order) are written and the rest of out is untouched,
// as in the reference.
vc_status vc_decode_region(vc_archive *a, int lod, vc_box box, uint8_t *out);

// src/vc/vc.h:133 — coverage without decoding.
vc_cover vc_atom_coverage(const vc_archive *a, int lod,
                          uint32_t az, uint32_t ay, uint32_t ax);

// src/vc/vc.h:139 — payload byte range of a PRESENT atom (0,0 otherwise).
vc_cover vc_atom_payload_range(const vc_archive *a, int lod,
                               uint32_t az, uint32_t ay, uint32_t ax,
                               uint64_t *off, uint32_t *len);

// src/vc/vc.h:145 — 1 (v1), 2 (v2), 0 for NULL.
int vc_archive_version(const vc_archive *a);

// src/vc/vc.h:151 — v2 only: a region's contiguous blob.
vc_cover vc_region_blob_range(const vc_archive *a, int lod,
                              uint32_t rz, uint32_t ry, uint32_t rx,
                              uint64_t *off, uint64_t *len);

// src/vc/vc.h:97 — index-region edge in atoms (32).
uint32_t vc_region_atoms(void);

// src/vc/vc.h:156 — called with a message before this library gives up on an
// unrecoverable condition. Unlike the reference, the library never aborts:
// device and allocation failures are returned as VC_ERR_IO / VC_ERR_OOM and the
// hook is only informed.
void vc_set_panic_hook(void (*hook)(const char *msg));

#ifdef __cplusplus
}
#endif
#endif // VC_H

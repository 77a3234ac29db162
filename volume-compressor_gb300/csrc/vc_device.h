// Private device-runtime state shared by the CUDA translation units.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "vc_internal.h"

enum {
    VCD_BUF_CNT = 0, VCD_BUF_OFF, VCD_BUF_ENT, VCD_BUF_OUT,   // decode
    VCD_BUF_VOL, VCD_BUF_PYR, VCD_BUF_EENT, VCD_BUF_EMETA, VCD_BUF_LEN, VCD_BUF_POS, VCD_BUF_ARC,
    VCD_BUF_BEST, VCD_BUF_RED,
    VCD_BUF_BUA, VCD_BUF_BDST, VCD_BUF_BREQ, VCD_BUF_BOFF, VCD_BUF_BCNT, VCD_BUF_BENT, VCD_BUF_BCTL, VCD_BUF_BOUT,
    VCD_BUF_BPIN, VCD_BUF_COEF, VCD_BUF_RPK, VCD_BUF_RPKREC, VCD_BUF_STG, VCD_BUF_WPACK,
    VCD_BUF_EENT2, VCD_BUF_EMETA2,   // encode: lists and metadata of the coarser LODs (second stream)
    VCD_BUF_ORD,                     // decode: atom order of the per-lane range decoder + sort counters
    VCD_BUF_BORD,                    // batched decode: the same for the distinct atoms
    VCD_NBUF
};

constexpr int VCD_SLABS = 32;   // copy-out slabs of a large host-output decode

struct vcd_ctx {
    cudaStream_t stream;
    void *buf[VCD_NBUF];
    size_t cap[VCD_NBUF];
    void *pinned;
    size_t pinned_cap;
    cudaEvent_t ev[8];           // stage events of the last call on this thread
    double last_ms;              // device time of the last decode / encode call (start..end events)
    // batched decode: autotuned launch shape and the CUDA graph of its launches
    int batch_rc_scalar_warps, batch_tx_threads, batch_imma, batch_forced;
    cudaGraphExec_t batch_graph;
    unsigned char batch_key[512];   // kernel parameters + shape + grid capacity the graph was captured with
    // second stream (created on first use, vcd_side_stream): copy-out overlapped
    // with the inverse transform; the coarser LODs' coder passes beside LOD0's
    cudaStream_t copy_stream;
    cudaEvent_t chunk_ev[VCD_SLABS];
    cudaEvent_t ring_ev[4];      // pinned bounce slots of a copy-out into pageable memory
    // streamed decode: pinned staging filled by the read callback, copied to VCD_BUF_STG
    uint8_t *stage_host;
    size_t stage_cap;
    int stage_started;           // an upload of the current call was issued (ev[4] recorded)
    // writer batches: payloads copied back from the device
    uint8_t *wpin;
    size_t wpin_cap;
};

// Kernel statistics, accumulated while profiling is enabled (vcg_profile_enable).
int vcd_prof_on(void);
void vcd_prof_add(const char *name, double ms, uint64_t launches, uint64_t bytes_read, uint64_t bytes_written,
                  uint64_t units);
float vcd_elapsed(cudaEvent_t a, cudaEvent_t b);

struct vcd_archive {
    uint8_t *arc;       // archive bytes (+16 slack)
    size_t len;
    vcd_atom *atoms;    // all LODs
    vcd_dq *dq;         // per LOD
    int nlod;
    size_t arc_cap, atoms_cap, dq_cap;   // bytes of the blocks (from the residency block cache; 0: cudaMalloc'd)
};

struct vcd_device {
    int device, num_sms;
    vcd_tables *tables;          // device copy
    uint32_t band_start[9];
};

extern vcd_device g_dev;
vcd_ctx *vcd_thread_ctx(void);
cudaError_t vcd_scratch(vcd_ctx *c, int slot, size_t bytes, void **out);
// cudaMalloc / cudaMallocHost of the library, through the allocation-failure
// injector (vcg_debug_fail_alloc)
cudaError_t vcd_malloc(void **p, size_t bytes);
cudaError_t vcd_malloc_host(void **p, size_t bytes);
cudaError_t vcd_pinned(vcd_ctx *c, size_t bytes, void **out);
// the context's second stream with its slab and bounce-slot events, created on first use; NULL if that fails
cudaStream_t vcd_side_stream(vcd_ctx *c);
// Synchronous copies between device memory and host memory of any kind on the
// context's stream (queued work first): pageable buffers of 16 MiB or more go
// through pinned 32 MiB chunks copied by host threads, others in one copy.
cudaError_t vcd_copy_to_host(vcd_ctx *c, void *dst, const void *src_dev, size_t bytes);
cudaError_t vcd_copy_from_host(vcd_ctx *c, void *dst_dev, const void *src, size_t bytes);
void vcd_set_error(const char *what, cudaError_t e);
int vcd_status_of(cudaError_t e);

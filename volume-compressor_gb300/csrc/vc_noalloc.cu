// vcg_decode_atoms_noalloc: atom decode that allocates no memory.
//
// Some callers cannot let a library allocate device memory: host applications
// that reserve the whole GPU for their own memory pool up front (a library
// cudaMalloc then fails), and latency-bound pipelines that cannot afford the
// device-wide synchronisation cudaMalloc / cudaFree may perform. This entry
// point serves them: the caller passes inputs (payload bytes already in device
// memory) and outputs (a device buffer), and every byte of scratch the decode
// needs lives in one file-scope device array of fixed size, held by every GPU
// that loads the library until the process exits.
#include <cuda_runtime.h>
#include <pthread.h>
#include <stdint.h>
#include <string.h>

#include "kernels.cuh"
#include "vc_device.h"

using namespace vcg;

#define VC_API extern "C" __attribute__((visibility("default")))

#define NA_MAX_ATOMS 64u   // VCG_NOALLOC_MAX_ATOMS in include/vcg.h
#define NA_MAX_DEVICES 64

// Layout of the scratch array (byte offsets, each 256-aligned).
constexpr size_t kNaEnt = 0;                                               // lists: 64 x 32768 x u32
constexpr size_t kNaOff = kNaEnt + (size_t)NA_MAX_ATOMS * VCD_MAX_ENTRIES * 4;   // list offsets: 64 x u64
constexpr size_t kNaCnt = kNaOff + 512;                                    // entry counts: 64 x u32
constexpr size_t kNaCtl = kNaCnt + 256;                                    // [u32 err][u32][u64 entries]
constexpr size_t kNaAtoms = kNaCtl + 256;                                  // 64 x vcd_atom
constexpr size_t kNaDq = kNaAtoms + NA_MAX_ATOMS * sizeof(vcd_atom);       // vcd_dq
constexpr size_t kNaScan = kNaDq + ((sizeof(vcd_dq) + 255) / 256) * 256;   // scan order: 32768 x u16
constexpr size_t kNaAlt = kNaScan + 32768 * 2;                             // step-class bits: 1024 x u32
constexpr size_t kNaBytes = kNaAlt + 4096;                                 // ~8.07 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

// Per device: the array's device address (obtained once, with that device
// current) and the SM count.
static uint8_t *g_na_base[NA_MAX_DEVICES];
static int g_na_sms[NA_MAX_DEVICES];
static uint32_t g_na_band[9];   // first scan position of each significance band
static pthread_mutex_t g_na_mu = PTHREAD_MUTEX_INITIALIZER;

static int na_setup(int dev, uint8_t **base, int *sms) {
    pthread_mutex_lock(&g_na_mu);
    if (!g_na_base[dev]) {
        void *p = NULL;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        int n = 0;
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) {
            // constant parts: scan order, step-class bits, fixed list offsets
            static vcd_tables t;   // host staging (68 KiB), filled once
            vch_tables(&t);
            memcpy(g_na_band, t.band_start, sizeof g_na_band);
            uint64_t offs[NA_MAX_ATOMS];
            for (uint32_t i = 0; i < NA_MAX_ATOMS; ++i) offs[i] = (uint64_t)i * VCD_MAX_ENTRIES;
            uint8_t *b = (uint8_t *)p;
            e = cudaMemcpy(b + kNaScan, t.scan, sizeof t.scan, cudaMemcpyHostToDevice);
            if (e == cudaSuccess) e = cudaMemcpy(b + kNaAlt, t.alt_mask, sizeof t.alt_mask, cudaMemcpyHostToDevice);
            if (e == cudaSuccess) e = cudaMemcpy(b + kNaOff, offs, sizeof offs, cudaMemcpyHostToDevice);
        }
        if (e != cudaSuccess) {
            pthread_mutex_unlock(&g_na_mu);
            vcd_set_error("no-alloc decode: scratch set-up", e);
            return e == cudaErrorMemoryAllocation ? 3 : 4;
        }
        g_na_sms[dev] = n;
        g_na_base[dev] = (uint8_t *)p;
    }
    *base = g_na_base[dev];
    *sms = g_na_sms[dev];
    pthread_mutex_unlock(&g_na_mu);
    return 0;
}

// Decode n_atoms (<= 64) atom payloads held in device memory. Payload i is
// payload_dev[offsets[i], offsets[i] + lengths[i]) ([dc byte][range-coder
// bytes], as stored in an archive; lengths[i] == 0 means an all-zero atom);
// offsets / lengths are host arrays. base_q is the LOD's base_q from the
// archive header. Atom i is written to out_dev + i * 32768 (raster z, y, x).
// payload_dev must be 4-byte aligned (device allocations are) and
// payload_bytes is the size of that buffer.
//
// No memory is allocated: scratch is a fixed device array shared by every call
// in the process and left holding the last call's data. Calls whose work
// overlaps on the GPU (from several host threads, say) race on it and must be
// serialised by the caller. The first call on each device sets the array up
// (address lookup and constant tables) with that device current.
VC_API int vcg_decode_atoms_noalloc(const uint8_t *payload_dev, size_t payload_bytes, const uint64_t *offsets,
                                    const uint32_t *lengths, uint32_t n_atoms, float base_q, uint8_t *out_dev) {
    if (n_atoms > NA_MAX_ATOMS || (n_atoms && (!payload_dev || !offsets || !lengths || !out_dev)))
        return 2;   // VC_ERR_RANGE
    if (((uintptr_t)payload_dev & 3u) != 0) return 2;
    if (n_atoms == 0) return 0;
    vcd_atom atoms[NA_MAX_ATOMS];
    memset(atoms, 0, sizeof atoms);
    for (uint32_t i = 0; i < n_atoms; ++i) {
        if (lengths[i] == 0) { atoms[i].kind = VCD_EMPTY; continue; }
        if (offsets[i] > payload_bytes || lengths[i] > payload_bytes - offsets[i]) return 1;   // VC_ERR_FORMAT
        atoms[i].kind = VCD_PRESENT;
        atoms[i].off = offsets[i];
        atoms[i].len = lengths[i];
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) {
        vcd_set_error("no-alloc decode: current device", e);
        return 4;
    }
    uint8_t *base = NULL;
    int sms = 0;
    int rc = na_setup(dev, &base, &sms);
    if (rc) return rc;
    vcd_dq dq;
    vch_dq_consts(base_q, &dq);
    cudaStream_t st = cudaStreamPerThread;
    e = cudaMemcpyAsync(base + kNaAtoms, atoms, n_atoms * sizeof(vcd_atom), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(base + kNaDq, &dq, sizeof dq, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(base + kNaCtl, 0, 16, st);          // entry total starts at zero
    if (e == cudaSuccess) e = cudaMemsetAsync(base + kNaCtl, 0xFF, 4, st);        // no malformed atom yet
    if (e != cudaSuccess) {
        vcd_set_error("no-alloc decode: upload of the atom table", e);
        return 4;
    }
    DecodeJob J;
    memset(&J, 0, sizeof J);
    J.arc = payload_dev;
    J.atoms = reinterpret_cast<const vcd_atom *>(base + kNaAtoms);
    J.acx = 1; J.acy = 1;                       // atoms stacked along z: atom i = voxels z in [32i, 32i+32)
    J.bnx = 1; J.bny = 1;
    J.n_atoms = n_atoms;
    J.x1 = 32; J.y1 = 32; J.z1 = 32 * n_atoms;
    J.out = out_dev;
    J.ox = 32; J.oy = 32;
    J.ent = reinterpret_cast<uint32_t *>(base + kNaEnt);
    J.ent_off = reinterpret_cast<uint64_t *>(base + kNaOff);
    J.cnt = reinterpret_cast<uint32_t *>(base + kNaCnt);
    J.dq = reinterpret_cast<const vcd_dq *>(base + kNaDq);
    J.alt_mask = reinterpret_cast<const uint32_t *>(base + kNaAlt);
    J.scan = reinterpret_cast<const uint16_t *>(base + kNaScan);
    J.err = reinterpret_cast<uint32_t *>(base + kNaCtl);
    J.nnz_total = reinterpret_cast<unsigned long long *>(base + kNaCtl + 8);
    memcpy(J.band_start, g_na_band, sizeof J.band_start);
    launch_decode_lists(J, sms, st);
    if ((e = cudaGetLastError()) != cudaSuccess) {   // the launches of this call
        vcd_set_error("no-alloc decode: kernel launch", e);
        return 4;
    }
    uint32_t err = 0xFFFFFFFFu;
    e = cudaMemcpyAsync(&err, base + kNaCtl, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        vcd_set_error("no-alloc decode", e);
        return 4;
    }
    if (err < n_atoms) {
        vcd_set_error("no-alloc decode: malformed payload", cudaSuccess);
        return 1;
    }
    return 0;
}

// Repack into the v2 container on the device (tools/vc_repack.c:96-177 defines
// the layout): the image is zeroed, the header and region directory are written
// from the host, and one warp per record writes an atom's 16-byte slot and
// copies its payload from the resident archive to its place in the region blob.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "vc_device.h"

namespace {

__global__ void k_repack(const uint8_t *arc, const vcd_repack_rec *recs, uint64_t n, uint8_t *out) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x / 32);
    for (uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nw) {
        const vcd_repack_rec r = recs[i];
        uint8_t *slot = out + r.slot_dst;   // any byte offset: bytewise
        if (r.flags == 1u) {
            if (lane < 16) {
                uint8_t b = 0;
                if (lane < 8) b = (uint8_t)(r.pay_dst >> (8 * lane));
                else if (lane < 12) b = (uint8_t)(r.len >> (8 * (lane - 8)));
                else if (lane == 12) b = 1;
                else if (lane == 13) b = arc[r.src];   // dc = first payload byte
                slot[lane] = b;
            }
            const uint8_t *src = arc + r.src;
            uint8_t *dst = out + r.pay_dst;
            for (uint32_t k = lane; k < r.len; k += 32) dst[k] = src[k];
        } else if (lane == 0) {
            slot[12] = 2;   // known zero
        }
    }
}

}  // namespace

extern "C" int vcd_repack(vcd_archive *d, const uint8_t *head, uint64_t head_len, uint64_t total_len,
                          const vcd_repack_rec *recs, uint64_t n_recs, uint8_t *host_out) {
    vcd_ctx *c = vcd_thread_ctx();
    if (!c) return 4;
    cudaStream_t st = c->stream;
    void *p_out, *p_rec;
    cudaError_t e;
    if ((e = vcd_scratch(c, VCD_BUF_RPK, total_len + 16, &p_out)) != cudaSuccess ||
        (e = vcd_scratch(c, VCD_BUF_RPKREC, n_recs * sizeof(vcd_repack_rec) + 16, &p_rec)) != cudaSuccess) {
        vcd_set_error("repack buffers", e);
        return vcd_status_of(e);
    }
    cudaEventRecord(c->ev[0], st);
    cudaMemsetAsync(p_out, 0, total_len, st);
    cudaMemcpyAsync(p_out, head, head_len, cudaMemcpyHostToDevice, st);
    if (n_recs) {
        cudaMemcpyAsync(p_rec, recs, n_recs * sizeof(vcd_repack_rec), cudaMemcpyHostToDevice, st);
        const uint64_t warps = n_recs < (uint64_t)g_dev.num_sms * 64 ? n_recs : (uint64_t)g_dev.num_sms * 64;
        k_repack<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, st>>>(d->arc, (const vcd_repack_rec *)p_rec, n_recs,
                                                                      (uint8_t *)p_out);
    }
    cudaEventRecord(c->ev[1], st);
    if ((e = vcd_copy_to_host(c, host_out, p_out, total_len)) != cudaSuccess || (e = cudaGetLastError()) != cudaSuccess) {
        vcd_set_error("repack", e);
        return vcd_status_of(e);
    }
    c->last_ms = vcd_elapsed(c->ev[0], c->ev[1]);
    if (vcd_prof_on()) {
        uint64_t pay = 0;
        for (uint64_t i = 0; i < n_recs; ++i) pay += recs[i].len;
        vcd_prof_add("repack_v2", c->last_ms, 2, pay + n_recs * 32, total_len + pay, n_recs);
    }
    return 0;
}

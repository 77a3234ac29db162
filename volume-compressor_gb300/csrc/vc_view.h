// Private: the live view of a writer's image that the reader code in
// vc_host.c provides to the writer (vc_writer.c).
#ifndef VC_VIEW_H
#define VC_VIEW_H
#include "../../include/vc.h"

vc_archive *vch_view_new(vc_read_fn read, void *ud, vc_dims d0, int nlod, uint64_t l1_off, uint64_t l1_cap);
void vch_view_set(vc_archive *a, uint64_t len, const float *base_q /*VC_NLOD*/);
vc_status vch_view_decode_2x2x2(vc_archive *a, int lod, uint32_t az0, uint32_t ay0, uint32_t ax0,
                                uint8_t out8[8][VC_ATOM3], int *any);
#endif

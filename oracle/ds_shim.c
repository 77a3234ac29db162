// Test infrastructure only: exports the reference exporter's 2x downscale
// (tools/downscale.h, included from the reference checkout by oracle/Makefile)
// compiled with the reference's release flags, so that the oracle's
// restatement can be pinned against it. Nothing in the product loads it.
//   dsref_cell        -> ds_cell()          tools/downscale.h:38-46
//   dsref_downscale2x -> ds_downscale2x()   tools/downscale.h:48-93
#include "downscale.h"

#define SHIM __attribute__((visibility("default")))

SHIM unsigned dsref_cell(const unsigned char *c8, int method, float alpha) {
    unsigned acc = 0;
    for (int i = 0; i < 8; ++i) acc |= c8[i];
    return ds_cell(c8, acc, (ds_method)method, alpha);
}

SHIM void dsref_downscale2x(const uint8_t *in, int nx, int ny, int nz, uint8_t *out, int *ox, int *oy, int *oz,
                            int method, float alpha) {
    ds_downscale2x(in, nx, ny, nz, out, ox, oy, oz, (ds_method)method, alpha);
}

// Exporter 2x downscale (DS_BOX / DS_CBOX) launches, shared by the encoder's
// pyramid and the downscale entry points.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace vcg {
// method 0 = DS_BOX (also the codec's pyramid rule), 1 = DS_CBOX
void launch_ds2x(const uint8_t *in, uint32_t nx, uint32_t ny, uint32_t nz, uint8_t *out, int method, float alpha,
                 int num_sms, cudaStream_t s);
}  // namespace vcg

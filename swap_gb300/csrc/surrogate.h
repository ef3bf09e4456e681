// surrogate.h -- the network's side of the surrogate field step, used by
// the FP32 form (swap_f32.cu).
#pragma once

#include <cuda_runtime.h>

#include "../../include/swap_gpu.h"

namespace surr {
// The correction to E0 per interior node (FP32 [V][3], device) from the
// inputs [V][11]: B, u_p, n_p, p_e and E0, the plain E at the step's start.
int predict_e(swap_surrogate* net, int nx, int ny, int nz, const float* vin, float* ve, cudaStream_t st);
// Append one training pair (device inputs [V][11], target [V][3]: the mean
// corrector E minus E0).
int add_sample(swap_surrogate* net, int nx, int ny, int nz, const float* vin, const float* ve, cudaStream_t st);
const char* last_error(swap_surrogate* net);
}  // namespace surr

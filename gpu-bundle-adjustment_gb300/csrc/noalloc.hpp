#pragma once
// FP64 reprojection cost without device allocation (noalloc.cu).

#include <cuda_runtime.h>

namespace gba {

// Largest observation count gba_cost_noalloc accepts (its fixed scratch).
long long cost_noalloc_max_observations();

// SSE of the Snavely residuals of E observations (device pointers, BAL
// layout, observation order) into *out_sse and the number of non-finite
// residuals into *out_bad (device outputs; out_bad may be null). Allocates
// nothing; throws std::invalid_argument above the scratch limit.
void cost_noalloc(const double* cams, const double* pts, const int* oc, const int* op, const double* px, int E,
                  double* out_sse, unsigned long long* out_bad, cudaStream_t s);

}  // namespace gba

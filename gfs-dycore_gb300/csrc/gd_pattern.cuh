// gd_pattern.cuh -- internal interface of the stochastic pattern generator
// (gd_pattern.cu) for the dycore's stochastically perturbed physics.
#pragma once
#include <cuda_runtime.h>

#include "gd_api.h"

namespace gd {
// nsteps AR(1) steps of every field, enqueued on stream s (the generator's own
// stream is not used); the launches also count in the caller's launch count
void pattern_advance_on(gd_pattern* p, int nsteps, cudaStream_t s);
// device coefficients [nfields][nlm(jcap)], m-major triangular, FP32
const float2* pattern_spec(const gd_pattern* p);
int pattern_jcap(const gd_pattern* p);
int pattern_device(const gd_pattern* p);
int pattern_nfields(const gd_pattern* p);
}  // namespace gd

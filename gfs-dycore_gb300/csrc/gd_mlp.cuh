// gd_mlp.cuh -- the closure network (gd_mlp.cu) as the dycore uses it: the
// forward pass on a given stream, the normalisation, and the column kernels
// that turn the grid state into network inputs and the network's output
// into grid increments.
#pragma once
#include "gd_api.h"
#include "gd_common.cuh"
#include "gd_grid.cuh"

namespace gd {

void mlp_reserve(gd_mlp* p, int ncols);
void mlp_forward_on(gd_mlp* p, const float* x, int n, float* y, cudaStream_t s);
// throws when a bounded wait of the tensor-core forward timed out
void mlp_check(gd_mlp* p, cudaStream_t s);
int mlp_nin(const gd_mlp* p);
int mlp_nout(const gd_mlp* p);
int mlp_device(const gd_mlp* p);
// device normalisation arrays; false until gd_mlp_set_norm was called
bool mlp_norm(const gd_mlp* p, const float** in_mu, const float** in_sd, const float** out_mu,
              const float** out_sd);

// Closure inputs of every grid column p: x[p][0, L) = u, [L, 2L) = v,
// [2L, 3L) = Tv (levels bottom to top, rows of the synthesis buffer gS), x[p][3L]
// = ps = exp(ln ps).  Normalised (x - mu) / sd when mu is given, raw otherwise.
template <typename R>
void launch_closure_in(const R* gS, const SynthRows& s, int L, long ng, const float* mu, const float* sd, float* x,
                       cudaStream_t st);
// The network's output y[p][0, 3L) (normalised du/dt, dv/dt, dTv/dt) to
// increments over dt in the grid rows of the column-physics update: Tv
// [0, L), q [L, 2L) (zero), u [2L, 3L), v [3L, 4L).
template <typename R>
void launch_closure_out(const float* y, int L, long ng, const float* mu, const float* sd, R dt, R* gA,
                        cudaStream_t st);

}  // namespace gd

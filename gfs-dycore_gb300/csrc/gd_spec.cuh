// gd_spec.cuh -- spectral-space kernels (declarations).
#pragma once
#include "gd_common.cuh"

namespace gd {

// Complex-column layout of the spectral state buffer S[nlm][ncol]:
// vrt | div | tv | trc (ntrac*L) | s = a invlap vrt | c = a invlap div | lnps
struct SpecCols {
  int vrt, div, tv, trc, s, c, lnps, ncol;
};
// Per-stage tendency buffer TD[nlm][ncol]: nonlinear tendencies (after the
// linear gravity-wave terms are removed) and the linear terms themselves.
struct TendCols {
  int dvrt, ddiv, dtv, dtrc, dlnps, ddl, dtl, dpl, ncol;
};
// Analysis outputs: AP = P^T-analysis columns, AH = dP/dphi^T-analysis.
struct APCols {
  int ttend, ke, qtend, dlnps, imfv, imfu, ncol;
};
struct AHCols {
  int fu, mfv, ncol;
};

template <typename R>
struct StageArgs {
  int L, nt, T, stage, explicit_, final_;
  const int4* items;  // (n, m0, count)
  int nitems;
  const long* moff;
  R* S;
  const R* S0;
  long ldS;  // reals per spectral row
  const R* AP;
  long ldAP;
  const R* AH;
  long ldAH;
  R* TD0;
  R* TD1;
  R* TD2;
  long ldTD;
  const R* amhyb;  // [L][L] transposed: amhyb[j][k] = A(k, j), k = output level
  const R* bmhyb;  // transposed likewise
  const R* svhyb;  // [L]
  const R* tor;    // [L]
  const R* dhyb;   // [3][T+1][L][L], each matrix transposed
  const R* disspec;
  const R* diff_prof;
  const R* dmp_prof;
  R dt, ainv, ainv2, rerth;
  R ce[3], ci[3], cimp;
  // IAU forcing in the state's columns (vrt, div, tv, trc, lnps), added to the
  // explicit tendencies of every stage (run.f90:301-308, 362-369, 428-435);
  // null without IAU
  const R* F;
  SpecCols sc;
  TendCols tc;
  APCols ap;
  AHCols ah;
};
// coefficients of one degree per stage CTA, and the FP32 stage kernel's resident CTAs per SM
#ifndef GD_STAGE_QC
#define GD_STAGE_QC 16
#endif
#ifndef GD_STAGE_MINB
#define GD_STAGE_MINB 4
#endif
std::vector<int4> make_stage_items(int T, int qc);
template <typename R>
void launch_stage(const StageArgs<R>& a, cudaStream_t s);

// Tendencies of getdyntend (no linear terms removed) into TD columns.
template <typename R>
void launch_assemble(const StageArgs<R>& a, R* TD, cudaStream_t s);

// Physics adjustment (run.f90:526-538): state += dt * HS tendencies in AP
// columns [0,L) tv, [L,2L) vrt, [2L,3L) div; lnps from the dry-mass fixer
// analysis in AP column 3L (or unchanged); recomputes s, c.
template <typename R>
void launch_phys_update(R* S, long ldS, const SpecCols& sc, int L, int nt, int nlm, const R* AP, long ldAP,
                        int massfix, int heldsuarez, R dt, const R* lapv, R rerth, cudaStream_t s);

// Physics adjustment for the DCMIP simple physics (phy_run_simple.f90:145-160
// then run.f90:526-538): analyses of the grid increments in AP columns [0,L)
// Tv, [L,2L) q, 2L dry-mass fixer, [2L+1,3L+1) and [3L+1,4L+1) the
// i m/cos parts of vorticity and divergence, AH columns [0,L) and [L,2L)
// their d/dphi parts; tendency = analysis / dt (vorticity, divergence scaled
// by 1/a), state += dt * tendency for Tv, tracer 1 (hasq), vorticity, divergence;
// lnps from the fixer (or unchanged); recomputes s, c.
template <typename R>
void launch_simple_update(R* S, long ldS, const SpecCols& sc, int L, int nlm, const R* AP, long ldAP, const R* AH,
                          long ldAH, int massfix, int hasq, R dt, R ainv, const R* lapv, R rerth, cudaStream_t s);

// IAU forcing of one step (iau_module.f90:88-135): F = (ca inc[ia] + cb
// inc[ib]) / dtiau over the prognostic columns of the state layout (the
// (3+nt) L columns from vrt and the lnps column); ca = cb = 0 gives zero.
// inc holds nfiles arrays of nlm rows with the state's pitch.
template <typename R>
void launch_iau_forcing(R* F, const R* inc, long ldS, const SpecCols& sc, int ncs, int nlm, int ia, double ca,
                        int ib, double cb, double dtiau, cudaStream_t s);
// Digital filter (run.f90:58-91): acc = w S (first) or acc += w S, over the
// prognostic columns, acc in FP64 [nlm][ncs+1] complex.
template <typename R>
void launch_dfi_acc(double* acc, const R* S, long ldS, const SpecCols& sc, int ncs, int nlm, double w, int first,
                    cudaStream_t s);
// S = acc over the prognostic columns (run.f90:116-117).
template <typename R>
void launch_dfi_set(R* S, long ldS, const SpecCols& sc, int ncs, int nlm, const double* acc, cudaStream_t s);

// s = a invlap vrt, c = a invlap div for all coefficients.
template <typename R>
void launch_sc(R* S, long ldS, const SpecCols& sc, int L, int nlm, const R* lapv, R rerth, cudaStream_t s);

// Layout conversion: ref [nb][nlm] complex H (double, or float for the
// single-precision host entry points) <-> internal [nlm][ld] R.
template <typename R, typename H = double>
void launch_ref2int(const H* ref, int nb, int nlm, R* dst, long ld, int col0, cudaStream_t s);
template <typename R, typename H = double>
void launch_int2ref(const R* src, long ld, int col0, int nb, int nlm, H* ref, cudaStream_t s);
// out[c] = scale * (X[c] + Y[c]) on [nlm][nb] complex columns
template <typename R>
void launch_combine(const R* X, long ldX, int cx, const R* Y, long ldY, int cy, R* O, long ldO, int co, int nb,
                    int nlm, R scale, cudaStream_t s);
// columns c0..c0+nb of X scaled by f[idx] * scale
template <typename R>
void launch_scale_cols(R* X, long ldX, int c0, int nb, int nlm, const R* f, R scale, cudaStream_t s);
template <typename R>
void launch_to_double(const R* src, double* dst, long n, cudaStream_t s);

// FP64 batched inversion of nmat LxL row-major matrices (in place).
void launch_batched_inverse(double* mats, int nmat, int L, cudaStream_t s);

}  // namespace gd

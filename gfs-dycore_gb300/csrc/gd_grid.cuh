// gd_grid.cuh -- grid-space column kernels (declarations).
#pragma once
#include "gd_common.cuh"

namespace gd {

// Row offsets (in units of nlat*nlon) of the synthesis output grid buffer.
struct SynthRows {
  int vrt, div, tv, trc, u, v, dtvdx, dtvdy, dqdx, dqdy, lnps, dlnpsdx, dlnpsdy, total;
};
// Row offsets of the analysis input grid buffer.
struct AnalRows {
  int ttend, ke, qtend, dlnps, fu, fv, total;
};

template <typename R>
struct ColumnArgs {
  int L, nt, nlon, nlat, dry;
  const R* ak;    // [L+1] top to bottom
  const R* bk;    // [L+1]
  const R* dbk;   // [L]
  const R* ck;    // [L]
  const R* sinlat;  // [nlat]
  const R* coslat;  // [nlat]
  const R* gS;    // synthesis output rows
  SynthRows s;
  const R* dphisdx;  // [nlat*nlon]
  const R* dphisdy;
  R* gA;          // analysis input rows
  AnalRows a;
  R* psg;         // [nlat*nlon] out
  R* dlnpsdt;     // [nlat*nlon] out
  R* dlnpdtg;     // [L][nlat*nlon] out (may be null)
  R* etadot;      // [L+1][nlat*nlon] out (may be null)
  R* prs;         // [L][nlat*nlon] out (may be null)
  R kappa, rd, cvap_cp, omega2, log2sp, rlnp_top;
};

template <typename R>
// lb: levels per warp, 4 or 8 (0: 4 up to 64 levels, else 8)
void launch_dyn_columns(const ColumnArgs<R>& a, bool inverse_only, cudaStream_t s, int lb = 0);

template <typename R>
struct HsArgs {
  int L, nlon, nlat;
  const R* ak;
  const R* bk;
  const R* sinlat;
  const R* coslat;
  const R* gS;
  SynthRows s;
  R* gA;  // rows: dtv [0,L), dvrt [L,2L), ddiv [2L,3L)
  // stochastically perturbed tendencies (phy_run_gfs.f90:617-620 applied to
  // the HS forcing): x (1 + vfact[b] sppt[p]); sppt null: unperturbed
  const R* sppt;  // [nlat*nlon]
  const R* vfact;  // [L] bottom to top
  R kappa;
  R sigbot, kdrag, krada, kradb, expo;
};
template <typename R>
void launch_hs_forcing(const HsArgs<R>& a, cudaStream_t s);

// FP64 deterministic area-weighted sums.  rowsum[j] = w_j/(2 nlon) sum_i f
template <typename R>
void launch_area_mean_ps(const R* psg, const double* w, int nlat, int nlon, double* rowsum, double* out,
                         cudaStream_t s);
// pdry on stage 1: sets *pdryini if it is 0 (dyn_run.f90:135-153)
// pdryini = pmean - pmoist when pdryini is 0 (dyn_run.f90:146-150); pmoist
// may be null (dry runs)
void launch_pdry_init(const double* pmean, const double* pmoist, double* pdryini, cudaStream_t s);
// grid row log(ps*pcorr), pcorr = pdryini / pmean (dyn_run.f90:626-631)
template <typename R>
// log(ps pcorr), pcorr = (pdryini + grav pwatg) / pmean (dyn_run.f90:621-631);
// pwatg may be null (no precipitable water)
void launch_massfix_grid(const R* psg, const double* pdryini, const double* pmean, const double* pwatg, double grav,
                         int ng, R* out, cudaStream_t s);
// diagnostics of run.f90:159-161 -> out[0..3]
template <typename R>
void launch_diag(const R* u, const R* v, int L, const R* psg, const R* dlnpsdt, const double* w, int nlat, int nlon,
                 double* scratch, double* out, cudaStream_t s);

}  // namespace gd

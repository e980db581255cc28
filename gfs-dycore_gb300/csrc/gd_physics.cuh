// gd_physics.cuh -- column physics on the grid: DCMIP simple physics and the
// moist dry-mass bookkeeping (declarations).
#pragma once
#include "gd_common.cuh"
#include "gd_grid.cuh"

namespace gd {

// DCMIP simple physics (src/phy_run_simple.f90:26-176 around
// src/simple_physics_v5_1.f90), one thread per grid column.
template <typename R>
struct SimpleArgs {
  int L, nlon, nlat;
  const R* ak;   // [L+1] interfaces top to bottom
  const R* bk;   // [L+1]
  const R* dbk;  // [L] bk(k+1) - bk(k), differenced in FP64
  const R* lat;  // [nlat] latitude (radians)
  const R* gS;   // synthesis rows of the last inverse transform: Tv, tracer 1, u, v
  SynthRows s;
  const R* psg;  // [nlat*nlon] surface pressure (Pa)
  R* gA;         // out, grid increments over the step: Tv [0,L), q [L,2L), u [2L,3L), v [3L,4L), bottom to top
  R* precip;     // [nlat*nlon] out: precipitation rate (mm/s)
  R* pwat;       // [nlat*nlon] out: precipitable water after the physics (kg/m^2)
  R* apcp;       // [nlat*nlon] in/out: accumulated precipitation (mm), += precip * dt
  R dt;
  int test;      // 1: latitude-dependent SST (dcmip 4x); 0: constant SST (5x)
  int turbflux;  // surface fluxes and boundary-layer mixing (dcmip 43 and 5x)
  R fvirt, qmin, grav, kappa;  // con_fvirt, qmin of phy_run_simple.f90:38, con_g, con_rocp
};
template <typename R>
void launch_simple_physics(const SimpleArgs<R>& a, cudaStream_t s);

// pmoist of dyn_run.f90:135-145: sum over the grid of areawts * dpk * q over
// levels and the first ntuse tracers (trcg rows [ntuse*L] bottom to top),
// with pk = ak + bk ps top to bottom; FP64 row sums then one total in *out.
template <typename R>
void launch_area_pmoist(const R* trcg, int ntuse, int L, const R* psg, const R* ak, const R* bk, const double* w,
                        int nlat, int nlon, double* rowsum, double* out, cudaStream_t s);

}  // namespace gd

// gd_dcmip.h -- DCMIP-2012 analytic initial states at one point (host code).
#pragma once

namespace gd {
namespace dcmip {

// Test 4 (moist baroclinic instability, src/dcmip_initial_conditions_test_4_v3.f90)
// at pressure p (zcoords = 0): surface pressure 1e5 Pa, eta = p / ps.  moist
// selects the humidity field (and converts the formula's virtual
// temperature to temperature with 0.608 q).  q1 is potential temperature,
// q2 |Ertel PV| (unscaled, X = 1).
struct Point4 {
  double u, v, t, phis, ps, q, q1, q2;
};
Point4 test4(bool moist, double lon, double lat, double p);

// Test 5 (tropical cyclone, src/dcmip_initial_conditions_test_5_v1.f90) at
// pressure p (zcoords = 0): the height comes from inverting the pressure
// profile by Newton iteration within 1000 km of the vortex centre.
struct Point5 {
  double u, v, t, phis, ps, q;
};
Point5 test5(double lon, double lat, double p);

}  // namespace dcmip
}  // namespace gd

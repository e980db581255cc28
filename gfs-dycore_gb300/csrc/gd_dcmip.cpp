// gd_dcmip.cpp -- DCMIP-2012 analytic initial states (host code).
//
// Test 4: the moist baroclinic instability of the DCMIP-2012 test-case
// document (Jablonowski-Williamson jet with a Gaussian u perturbation at
// 20E 40N, humidity q0 exp(-(lat/40deg)^4) exp(-((eta-1) p0/34000 Pa)^2),
// potential temperature and Ertel PV as passive tracers), as
// src/dcmip_initial_conditions_test_4_v3.f90 evaluates it on pressure
// levels.  Test 5: the Reed-Jablonowski analytic tropical cyclone (vortex at
// 180E 10N, radius 282 km, pressure deficit 1115 Pa) of
// src/dcmip_initial_conditions_test_5_v1.f90.  Double precision throughout,
// with those routines' own constants (not the model's).
#include "gd_dcmip.h"

#include <algorithm>
#include <cmath>

namespace gd {
namespace dcmip {

namespace {

const double kPi = 4.0 * std::atan(1.0);
const double kA = 6371220.0, kRd = 287.0, kG = 9.80616, kOmega = 7.29212e-5;

double ipow(double x, int n) {  // x**n for an integer n
  double r = 1.0;
  for (int i = 0; i < n; ++i) r *= x;
  return r;
}

// ---------------------------------------------------------------- test 4
namespace t4 {
const double p0 = 100000.0, kappa = 2.0 / 7.0;
const double eta_tropo = 0.2, u0 = 35.0, T0 = 288.0, eta0 = 0.252, radius = 10.0, pert_amp = 1.0;
const double pert_lon = 20.0 * kPi / 180.0, pert_lat = 40.0 * kPi / 180.0, eta_sfc = 1.0;
const double delta_T = 480000.0, gamma = 0.005, a_omega = kA * kOmega, expo = kRd * gamma / kG;
const double q0 = 0.021, lat_hw = 2.0 * kPi / 9.0, p_hw = 34000.0;

// the latitude factor shared by temperature, geopotential and theta
double lat_poly(double lat) { return -2.0 * ipow(std::sin(lat), 6) * (ipow(std::cos(lat), 2) + 1.0 / 3.0) + 10.0 / 63.0; }
double lat_poly2(double lat) {
  return 8.0 / 5.0 * ipow(std::cos(lat), 3) * (ipow(std::sin(lat), 2) + 2.0 / 3.0) - kPi / 4.0;
}
double t_mean(double eta) {
  double t = T0 * std::pow(eta, expo);
  if (eta < eta_tropo) t += delta_T * ipow(eta_tropo - eta, 5);
  return t;
}
double t_deviation(double lat, double eta) {
  const double factor = eta * kPi * u0 / kRd, phv = (eta - eta0) * 0.5 * kPi;
  return factor * 1.5 * std::sin(phv) * std::pow(std::cos(phv), 0.5) *
         (lat_poly(lat) * u0 * std::pow(std::cos(phv), 1.5) + lat_poly2(lat) * a_omega * 0.5);
}
double surface_geopotential(double lat) {
  const double ct = u0 * std::pow(std::cos((eta_sfc - eta0) * kPi * 0.5), 1.5);
  return (lat_poly(lat) * ct + lat_poly2(lat) * a_omega) * ct;
}
double u_wind(double lon, double lat, double eta) {
  const double phv = (eta - eta0) * 0.5 * kPi;
  double u = std::pow(std::cos(phv), 1.5) * 4.0 * u0 * ipow(std::sin(lat), 2) * ipow(std::cos(lat), 2);
  const double r = std::acos(std::sin(pert_lat) * std::sin(lat) + std::cos(pert_lat) * std::cos(lat) * std::cos(lon - pert_lon));
  return pert_amp * std::exp(-ipow(r * radius, 2)) + u;
}
double theta(double lat, double eta) {
  const double enu = (eta - eta0) * kPi * 0.5, ct = u0 * std::pow(std::cos(enu), 1.5);
  const double Y = lat_poly(lat) * 2.0 * ct + lat_poly2(lat) * a_omega;
  return t_mean(eta) * std::pow(eta, -kappa) +
         3.0 / 4.0 * kPi * u0 / kRd * std::pow(eta, 1.0 - kappa) * std::sin(enu) * std::sqrt(std::cos(enu)) * Y;
}
double epv(double lon, double lat, double eta) {
  const double eps = 1.e-6;
  const double enu = (eta - eta0) * kPi * 0.5, ct = u0 * std::pow(std::cos(enu), 1.5);
  const double sl = std::sin(lat), cl = std::cos(lat);
  const double Y = lat_poly(lat) * 2.0 * ct + lat_poly2(lat) * a_omega;
  const double K = std::sin(pert_lat) * sl + std::cos(pert_lat) * cl * std::cos(lon - pert_lon);
  const double DK = std::sin(pert_lat) * cl - std::cos(pert_lat) * sl * std::cos(lon - pert_lon);
  const double r = std::acos(K);
  const double zeta_bg = -4.0 / kA * ct * sl * cl * (2.0 - 5.0 * ipow(sl, 2));
  double zeta;
  if (std::fabs(lat - pert_lat) <= eps && std::fabs(lon - pert_lon) <= eps) {  // at the perturbation centre
    zeta = zeta_bg + pert_amp / kA * std::tan(lat);
  } else if ((std::fabs(lat + pert_lat) <= eps && std::fabs(lon - (pert_lon + kPi)) <= eps) ||
             std::fabs(lat - kPi * 0.5) <= eps || std::fabs(lat + kPi * 0.5) <= eps) {  // antipode, poles
    zeta = zeta_bg;
  } else {
    zeta = zeta_bg + pert_amp / kA * std::exp(-ipow(r * radius, 2)) *
                         (std::tan(lat) - 2.0 * ipow(radius, 2) * std::acos(K) * DK / std::sqrt(1.0 - ipow(K, 2)));
  }
  const double dudeta =
      -u0 * ipow(std::sin(2.0 * lat), 2) * 3.0 * kPi / 4.0 * std::sqrt(std::cos(enu)) * std::sin(enu);
  double dmt = T0 * (expo - kappa) * std::pow(eta, expo - kappa - 1.0);
  if (eta < eta_tropo)
    dmt -= delta_T * (5.0 * ipow(eta_tropo - eta, 4) * std::pow(eta, -kappa) +
                      kappa * ipow(eta_tropo - eta, 5) * std::pow(eta, -kappa - 1.0));
  const double dthetadeta =
      dmt + 3.0 / 4.0 * kPi * u0 / kRd * (1.0 - kappa) * std::pow(eta, -kappa) * std::sin(enu) * std::sqrt(std::cos(enu)) * Y +
      3.0 / 8.0 * kPi * kPi / kRd * std::pow(eta, 1.0 - kappa) * ct * Y -
      3.0 / 16.0 * kPi * kPi * u0 / kRd * std::pow(eta, 1.0 - kappa) * ipow(std::sin(enu), 2) *
          std::pow(std::cos(enu), -0.5) * Y -
      9.0 / 8.0 * kPi * kPi * u0 * u0 / kRd * std::pow(eta, 1.0 - kappa) * ipow(std::sin(enu), 2) * std::cos(enu) *
          lat_poly(lat);
  const double d1 = 2.0 * ct * (-12.0 * cl * ipow(sl, 5) * (ipow(cl, 2) + 1.0 / 3.0) + 4.0 * cl * ipow(sl, 7));
  const double d2 =
      a_omega * (-24.0 / 5.0 * sl * ipow(cl, 2) * (ipow(sl, 2) + 2.0 / 3.0) + 16.0 / 5.0 * ipow(cl, 4) * sl);
  const double dthetadphi =
      3.0 / 4.0 * kPi * u0 / kRd * std::pow(eta, 1.0 - kappa) * std::sin(enu) * std::sqrt(std::cos(enu)) * (d1 + d2);
  const double f = 2.0 * kOmega * sl;
  return kG / p0 * (-dudeta * dthetadphi / kA - (zeta + f) * dthetadeta);
}
}  // namespace t4

// ---------------------------------------------------------------- test 5
namespace t5 {
const double omega = 7.292115e-5;  // this routine's own rotation rate
const double deg = 180.0 / kPi;
const double rp = 282000.0, dp = 1115.0, zp = 7000.0, q0 = 0.021, gamma = 0.007, Ts0 = 302.15, p00 = 101500.0;
const double cen_lat = 10.0, cen_lon = 180.0, zq1 = 3000.0, zq2 = 8000.0, exppr = 1.5, exppz = 2.0;
const double ztrop = 15000.0, qtrop = 1.e-11, rfpi = 1000000.0, constTv = 0.608, deltaz = 1.e-11, epsilon = 1.e-25;
const double expo = kRd * gamma / kG;
const double T0 = Ts0 * (1.0 + constTv * q0);
const double Ttrop = T0 - gamma * ztrop;

// pressure at height z minus p, and its z derivative (the Newton pair)
double fpi_f(double p, double gr, double z) {
  return p - (p00 - dp * std::exp(-std::pow(gr / rp, exppr)) * std::exp(-std::pow(z / zp, exppz))) *
                 std::pow((T0 - gamma * z) / T0, kG / (kRd * gamma));
}
double fpi_dfdz(double gr, double z) {
  const double e = std::exp(-std::pow(gr / rp, exppr)) * std::exp(-std::pow(z / zp, exppz));
  return -exppz * z * dp * e / (zp * zp) * std::pow((T0 - gamma * z) / T0, kG / (kRd * gamma)) +
         kG / (kRd * T0) * (p00 - dp * e) * std::pow((T0 - gamma * z) / T0, kG / (kRd * gamma) - 1.0);
}
}  // namespace t5

}  // namespace

Point4 test4(bool moist, double lon, double lat, double p) {
  using namespace t4;
  Point4 o;
  o.ps = p0;
  const double eta = p / o.ps;
  o.u = u_wind(lon, lat, eta);
  o.v = 0.0;
  o.t = t_mean(eta) + t_deviation(lat, eta);
  o.phis = surface_geopotential(lat);
  if (moist) {
    o.q = q0 * std::exp(-ipow(lat / lat_hw, 4)) * std::exp(-ipow((eta - 1.0) * p0 / p_hw, 2));
    o.t = o.t / (1.0 + 0.608 * o.q);
  } else {
    o.q = 0.0;
  }
  o.q1 = theta(lat, eta);
  o.q2 = std::fabs(epv(lon, lat, eta));
  return o;
}

Point5 test5(double lon, double lat, double p) {
  using namespace t5;
  Point5 o;
  const double f = 2.0 * omega * std::sin(cen_lat / deg);
  const double gr = kA * std::acos(std::sin(cen_lat / deg) * std::sin(lat) +
                                   std::cos(cen_lat / deg) * std::cos(lat) * std::cos(lon - cen_lon / deg));
  o.ps = p00 - dp * std::exp(-std::pow(gr / rp, exppr));
  double h = (T0 / gamma) * (1.0 - std::pow(p / o.ps, expo));
  if (gr < rfpi) {  // Newton iteration, at most 19 updates, to relative change deltaz
    double zhere = h, zn = h;
    for (int n = 2;; ++n) {
      zn = zhere - fpi_f(p, gr, zhere) / fpi_dfdz(gr, zhere);
      if (n > 20 || !(std::fabs(zn - zhere) / std::fabs(zn) > deltaz)) break;
      zhere = zn;
    }
    h = zn;
  }
  const double d1 = std::sin(cen_lat / deg) * std::cos(lat) - std::cos(cen_lat / deg) * std::sin(lat) * std::cos(lon - cen_lon / deg);
  const double d2 = std::cos(cen_lat / deg) * std::sin(lon - cen_lon / deg);
  const double d = std::max(epsilon, std::sqrt(d1 * d1 + d2 * d2));
  const double ufac = d1 / d, vfac = d2 / d;
  const double er = std::exp(std::pow(gr / rp, exppr)), ez = std::exp(std::pow(h / zp, exppz));
  if (h > ztrop) {
    o.u = o.v = 0.0;
    o.q = qtrop;
    o.t = Ttrop;
  } else {
    const double vt = -f * gr / 2.0 +
                      std::sqrt(std::pow(f * gr / 2.0, 2.0) -
                                exppr * std::pow(gr / rp, exppr) * kRd * (T0 - gamma * h) /
                                    (exppz * h * kRd * (T0 - gamma * h) / (kG * std::pow(zp, exppz)) +
                                     (1.0 - p00 / dp * er * ez)));
    o.v = vfac * vt;
    o.u = ufac * vt;
    o.q = q0 * std::exp(-h / zq1) * std::exp(-std::pow(h / zq2, exppz));
    o.t = (T0 - gamma * h) / (1.0 + constTv * o.q) /
          (1.0 + exppz * kRd * (T0 - gamma * h) * h / (kG * std::pow(zp, exppz) * (1.0 - p00 / dp * er * ez)));
  }
  o.phis = 0.0;
  return o;
}

}  // namespace dcmip
}  // namespace gd

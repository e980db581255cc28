// gd_physics.cu -- column physics on the grid.
//
// DCMIP simple physics (src/phy_run_simple.f90:26-176 around
// src/simple_physics_v5_1.f90, Reed and Jablonowski 2012): large-scale
// condensation; with turbulent fluxes, implicit surface fluxes at the lowest
// level and implicit boundary-layer diffusion of u, v, potential temperature
// and q.  One thread per grid column (consecutive threads take consecutive
// longitudes, so every level's load and store is coalesced).  The diffusion
// is the reference's tridiagonal elimination: a bottom-up sweep that streams
// the levels through a three-level window (condensing each level as it
// enters) and keeps the elimination coefficients in per-thread arrays, then
// a top-down substitution that writes the increments.  Arithmetic is in the
// state precision (the reference computes this routine in real(8); the FP64
// mode does too).
//
// The moist pmoist sum of dyn_run.f90:135-145 is here as well.
#include "gd_physics.cuh"

namespace gd {

namespace {

__device__ double phys_block_sum(double v) {
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x + 31) / 32; ++i) r += sh[i];
  return r;  // valid in thread 0
}

__global__ void k_phys_final_sum(const double* rowsum, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += rowsum[i];
    *out = s;
  }
}

template <typename R>
__device__ __forceinline__ R ipow_d(R x, int n) {  // x**n for an integer n
  R r = R(1);
  for (int i = 0; i < n; ++i) r *= x;
  return r;
}

// simple_physics_v5_1.f90:168-210
template <typename R>
struct SimpleConst {
  static constexpr double gravit = 9.80616, rair = 287.0, cpair = 1.0045e3, latvap = 2.5e6, rh2o = 461.5;
  static constexpr double C = 0.0011, SST_tc = 302.15, T0 = 273.16, e0 = 610.78, rhow = 1000.0;
  static constexpr double Cd0 = 0.0007, Cd1 = 0.000065, Cm = 0.002, v20 = 20.0, p0 = 100000.0;
  static constexpr double pbltop = 85000., pblconst = 10000., T00 = 288.0, u0 = 35.0;
  static constexpr double pi = 3.14159265358979323846, a = 6371220.0, omega = 7.29212e-5;
};

}  // namespace

// Thread per column; LMAX bounds the level count of the per-thread arrays.
// The sweeps are dependent chains per thread, so the kernel lives on
// occupancy: 16 CTAs of 128 threads per SM for the FP32 state (32
// registers), 5 for FP64.
template <typename R, int LMAX>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? 16 : 5) k_simple_physics(SimpleArgs<R> a) {
  typedef SimpleConst<R> K;
  const long ng = (long)a.nlon * a.nlat;
  const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ng) return;
  const int L = a.L, j = (int)(p / a.nlon), nb = L - 1;
  const R gravit = R(K::gravit), rair = R(K::rair), cpair = R(K::cpair), latvap = R(K::latvap), rh2o = R(K::rh2o);
  const R epsilo = rair / rh2o, zvir = (rh2o / rair) - R(1);
  const R C = R(K::C), T0 = R(K::T0), e0 = R(K::e0), rhow = R(K::rhow), p0 = R(K::p0);
  const R rk = rair / cpair, dt = a.dt;
  const R ps = a.psg[p];
  const R* gS = a.gS;
  auto IN = [&](int row, int t) -> R { return gS[(long)(row + (L - 1 - t)) * ng + p]; };  // top-down t
  auto PK = [&](int t) -> R { return a.ak[t] + a.bk[t] * ps; };
  auto PMID = [&](int t) -> R {  // prs of calc_pressdata (pressure_data.f90:87-88)
    const R pu = PK(t), pl = PK(t + 1);
    return pow((pow(pl, a.kappa) * pl - pow(pu, a.kappa) * pu) / ((a.kappa + R(1)) * (pl - pu)), R(1) / a.kappa);
  };
  // Layer thickness: the reference differences interface pressures; in
  // FP32 that cancels (ulp(ps) against 10^2-10^3 Pa), so the FP32 state
  // takes ak(k+1) - ak(k) + dbk(k) ps instead.
  auto PDEL = [&](int t) -> R {
    if (sizeof(R) == 4) return (a.ak[t + 1] - a.ak[t]) + a.dbk[t] * ps;
    return PK(t + 1) - PK(t);
  };
  auto PDELX = [&](int t) -> R { return PK(t + 1) - PK(t); };  // as in PMID
  auto TEMP = [&](R tv, R q) -> R { return tv / (R(1) + a.fvirt * max(a.qmin, q)); };
  // large-scale condensation of one level (simple_physics_v5_1.f90:226-255)
  R precl = R(0);
  auto condense = [&](R& t, R& q, R pm, R pdel) {
    const R qsat = epsilo * e0 / pm * exp(-latvap / rh2o * ((R(1) / t) - R(1) / T0));
    if (q > qsat) {
      const R tmp = R(1) / dt * (q - qsat) / (R(1) + (latvap / cpair) * (epsilo * latvap * qsat / (rair * (t * t))));
      t = t + (latvap / cpair * tmp) * dt;
      q = q + (-tmp) * dt;
      precl = precl + tmp * pdel / (gravit * rhow);
    }
  };
  R pw = R(0);
  auto emit = [&](int t, R tn, R qn, R un, R vn) {  // increments at bottom-up level L-1-t
    const long b = L - 1 - t;
    const R qi = IN(a.s.trc, t);
    const R dq = qn - qi;
    a.gA[b * ng + p] = tn * (R(1) + a.fvirt * max(a.qmin, qn)) - IN(a.s.tv, t);
    a.gA[(L + b) * ng + p] = dq;
    a.gA[(2 * L + b) * ng + p] = un - IN(a.s.u, t);
    a.gA[(3 * L + b) * ng + p] = vn - IN(a.s.v, t);
    pw += PDEL(t) * (dq + qi);
  };

  if (!a.turbflux) {
    for (int t = 0; t < L; ++t) {
      R q = IN(a.s.trc, t), tt = TEMP(IN(a.s.tv, t), q);
      condense(tt, q, PMID(t), PDEL(t));
      emit(t, tt, q, IN(a.s.u, t), IN(a.s.v, t));
    }
  } else {
    // the lowest level before any update: height, wind, exchange coefficients
    const R qb = IN(a.s.trc, nb), tb = TEMP(IN(a.s.tv, nb), qb);
    // ln(ps / pint) across the lowest layer; log1p of the thickness ratio in
    // FP32, where log(ps) - log(pint) would cancel to ~1e-4
    const R dlnpint = sizeof(R) == 4 ? log1p(PDEL(nb) / PK(nb)) : log(ps) - log(PK(nb));
    const R za = rair / gravit * tb * (R(1) + zvir * qb) * R(0.5) * dlnpint;
    R Tsurf;
    if (a.test == 1) {
      const R pi = R(K::pi), u0 = R(K::u0), lat = a.lat[j];
      const R latw = R(2) * pi / R(9), eta0 = R(0.252), etav = (R(1) - eta0) * R(0.5) * pi;
      const R q0 = R((double)0.021f);  // a literal without a kind suffix
      const R sl = sin(lat), cl = cos(lat);
      Tsurf = (R(K::T00) + pi * u0 / rair * R(1.5) * sin(etav) * pow(cos(etav), R(0.5)) *
                               ((R(-2) * ipow_d(sl, 6) * (cl * cl + R(1) / R(3)) + R(10) / R(63)) * u0 *
                                    pow(cos(etav), R(1.5)) +
                                (R(8) / R(5) * ipow_d(cl, 3) * (sl * sl + R(2) / R(3)) - pi / R(4)) * R(K::a) *
                                    R(K::omega) * R(0.5))) /
              (R(1) + zvir * q0 * exp(-ipow_d(lat / latw, 4)));
    } else {
      Tsurf = R(K::SST_tc);
    }
    const R ub = IN(a.s.u, nb), vb = IN(a.s.v, nb);
    const R wind = sqrt(ub * ub + vb * vb);
    const R Ken = C * wind * za;
    R Cd, Kmn;
    if (wind < R(K::v20)) {
      Cd = R(K::Cd0) + R(K::Cd1) * wind;
      Kmn = Cd * wind * za;
    } else {
      Cd = R(K::Cm);
      Kmn = R(K::Cm) * wind * za;
    }
    // interface i (top-down): the vertical taper of the exchange coefficients
    // above pbltop, shared by Km and Ke
    auto TAPER = [&](int i) -> R {
      const R pint = PK(i);
      if (pint >= R(K::pbltop)) return R(1);
      const R x = R(K::pbltop) - pint;
      return exp(-(x * x) / (R(K::pblconst) * R(K::pblconst)));
    };
    const R qsats = epsilo * e0 / ps * exp(-latvap / rh2o * ((R(1) / Tsurf) - R(1) / T0));
    // pk^kappa pk at interface i, each computed once (layer pressures of two layers)
    auto PKK = [&](int i) -> R {
      const R pk = PK(i);
      return pow(pk, a.kappa) * pk;
    };
    auto PMID2 = [&](int t, R kku, R kkl) -> R {  // Phillips layer pressure from the interface terms
      return pow((kkl - kku) / ((a.kappa + R(1)) * PDELX(t)), R(1) / a.kappa);
    };
    // sweep 1: bottom to top, level k with the level below (k+1) and above (k-1)
    R ce[LMAX], cem[LMAX], cfu[LMAX], cfv[LMAX], cft[LMAX], cfq[LMAX], exv[LMAX];
    R kkl = PKK(nb + 1), kku = PKK(nb);
    R tk = tb, qk = qb, uk = ub, vk = vb, pmk = PMID2(nb, kku, kkl), pdk = PDEL(nb);
    condense(tk, qk, pmk, pdk);
    uk = uk / (R(1) + Cd * wind * dt / za);
    vk = vk / (R(1) + Cd * wind * dt / za);
    tk = (tk + C * wind * Tsurf * dt / za) / (R(1) + C * wind * dt / za);
    qk = (qk + C * wind * qsats * dt / za) / (R(1) + C * wind * dt / za);
    // the interface below the current level: dt g^2 K rho^2 / dpm for Km and Ke
    R xm1 = R(0), xe1 = R(0);
    R ce1 = R(0), cem1 = R(0), fu1 = R(0), fv1 = R(0), ft1 = R(0), fq1 = R(0);
    for (int k = nb; k >= 0; --k) {
      R tu = R(0), qu = R(0), uu = R(0), vu = R(0), pmu = R(0), pdu = R(0), xm = R(0), xe = R(0);
      if (k > 0) {
        qu = IN(a.s.trc, k - 1);
        tu = TEMP(IN(a.s.tv, k - 1), qu);
        uu = IN(a.s.u, k - 1);
        vu = IN(a.s.v, k - 1);
        const R kkn = PKK(k - 1);
        pmu = PMID2(k - 1, kkn, kku);
        kku = kkn;
        pdu = PDEL(k - 1);
        condense(tu, qu, pmu, pdu);
        // interface k, between k-1 and k
        const R rho = (PK(k) / (rair * (tk + tu) / R(2)));
        const R x = dt * gravit * gravit * rho * rho / (pmk - pmu);
        const R tp = TAPER(k);
        xm = x * (Kmn * tp);
        xe = x * (Ken * tp);
      }
      const R rpd = R(1) / pdk;
      const R CAm = rpd * xm1, CA = rpd * xe1, CCm = rpd * xm, CC = rpd * xe;
      const R de = R(1) + CA + CC - CA * ce1;
      const R dm = R(1) + CAm + CCm - CAm * cem1;
      const R ex = pow(p0 / pmk, rk);
      ce[k] = CC / de;
      cem[k] = CCm / dm;
      cfu[k] = (uk + CAm * fu1) / dm;
      cfv[k] = (vk + CAm * fv1) / dm;
      cft[k] = (ex * tk + CA * ft1) / de;
      cfq[k] = (qk + CA * fq1) / de;
      exv[k] = ex;
      xm1 = xm, xe1 = xe;
      ce1 = ce[k], cem1 = cem[k], fu1 = cfu[k], fv1 = cfv[k], ft1 = cft[k], fq1 = cfq[k];
      tk = tu, qk = qu, uk = uu, vk = vu, pmk = pmu, pdk = pdu;
    }
    // sweep 2: top to bottom, potential temperature back to temperature
    R un = cfu[0], vn = cfv[0], tn = cft[0] / exv[0], qn = cfq[0];
    emit(0, tn, qn, un, vn);
    for (int k = 1; k < L; ++k) {
      un = cem[k] * un + cfu[k];
      vn = cem[k] * vn + cfv[k];
      tn = (ce[k] * tn * exv[k - 1] + cft[k]) / exv[k];
      qn = ce[k] * qn + cfq[k];
      emit(k, tn, qn, un, vn);
    }
  }
  a.pwat[p] = pw / a.grav;
  const R pr = precl * R(1000);
  a.precip[p] = pr;
  a.apcp[p] = a.apcp[p] + pr * dt;
}

template <typename R>
void launch_simple_physics(const SimpleArgs<R>& a, cudaStream_t s) {
  const long ng = (long)a.nlon * a.nlat;
  const int nblk = ceil_div(ng, 128);
  if (a.L <= 32)
    k_simple_physics<R, 32><<<nblk, 128, 0, s>>>(a);
  else if (a.L <= 64)
    k_simple_physics<R, 64><<<nblk, 128, 0, s>>>(a);
  else if (a.L <= 128)
    k_simple_physics<R, 128><<<nblk, 128, 0, s>>>(a);
  else
    throw std::invalid_argument("simple physics: more than 128 levels");
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_simple_physics<double>(const SimpleArgs<double>&, cudaStream_t);
template void launch_simple_physics<float>(const SimpleArgs<float>&, cudaStream_t);

template <typename R>
__global__ void k_rowsum_pmoist(const R* trcg, int ntuse, int L, const R* psg, const R* ak, const R* bk,
                                const double* w, int nlon, long ng, double* rowsum) {
  const int j = blockIdx.x;
  double s = 0;
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
    const long p = (long)j * nlon + i;
    const R ps = psg[p];
    for (int k = 0; k < L; ++k) {  // bottom-up level k is top-down layer L-1-k
      const int t = L - 1 - k;
      const R dpk = (ak[t + 1] + bk[t + 1] * ps) - (ak[t] + bk[t] * ps);
      for (int n = 0; n < ntuse; ++n) s += (double)dpk * (double)trcg[((long)n * L + k) * ng + p];
    }
  }
  s = phys_block_sum(s);
  if (threadIdx.x == 0) rowsum[j] = s * (w[j] / (2.0 * nlon));
}
template <typename R>
void launch_area_pmoist(const R* trcg, int ntuse, int L, const R* psg, const R* ak, const R* bk, const double* w,
                        int nlat, int nlon, double* rowsum, double* out, cudaStream_t s) {
  k_rowsum_pmoist<R><<<nlat, 256, 0, s>>>(trcg, ntuse, L, psg, ak, bk, w, nlon, (long)nlat * nlon, rowsum);
  k_phys_final_sum<<<1, 32, 0, s>>>(rowsum, nlat, out);
  count_launch(2);
  GD_LAUNCH_CHECK();
}
template void launch_area_pmoist<double>(const double*, int, int, const double*, const double*, const double*,
                                         const double*, int, int, double*, double*, cudaStream_t);
template void launch_area_pmoist<float>(const float*, int, int, const float*, const float*, const float*,
                                        const double*, int, int, double*, double*, cudaStream_t);

}  // namespace gd

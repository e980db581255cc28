// gd_grid.cu -- grid-space column kernels of the GFS spectral dycore step.
//
// One thread per grid column; all vertical recurrences of one column run in
// that thread, reads and writes are coalesced along longitude.  Restates
// src/pressure_data.f90:58-100 (calc_pressdata), src/dyn_run.f90:307-373
// (getomega), :375-451 (getpresgrad), :453-476 (getvadv), :478-603
// (getvadv_tracers, Thuburn limiter), the tendency assembly of
// :190-292, and src/phy_run_hs.f90:42-77 (Held-Suarez forcing).
// Vertical order as in the reference: 3-D fields bottom (b=0) to top,
// interface quantities (ak, bk, pk, dpk, rlnp, alfa, etadot) top (t=0) to
// bottom; b = L-1-t.
#include <cfloat>

#include "gd_grid.cuh"

namespace gd {

template <typename R>
__device__ __forceinline__ R epstiny_of();
template <>
__device__ __forceinline__ double epstiny_of<double>() {
  return DBL_MIN;
}
template <>
__device__ __forceinline__ float epstiny_of<float>() {
  return FLT_MIN;
}

constexpr int LMAX = 128;

template <typename R>
__global__ void __launch_bounds__(128) k_dyn_columns(ColumnArgs<R> a, int inverse_only) {
  const long ng = (long)a.nlon * a.nlat;
  const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ng) return;
  const int j = (int)(p / a.nlon);
  const int L = a.L;
  const R* gS = a.gS;
  auto S = [&](int row) -> R { return gS[(long)row * ng + p]; };
  const R* ak = a.ak;
  const R* bk = a.bk;
  const R* dbk = a.dbk;
  const R rd = a.rd;

  const R ps = exp(S(a.s.lnps));
  const R dlx = S(a.s.dlnpsdx), dly = S(a.s.dlnpsdy);
  R DB[LMAX], CB[LMAX], CG[LMAX], RL[LMAX], AL[LMAX];

  // calc_pressdata + getomega prefix sums (top to bottom)
  R pk_t = ak[0] + bk[0] * ps;
  R db = R(0), cb = R(0);
  for (int t = 0; t < L; ++t) {
    const int b = L - 1 - t;
    const R pk_t1 = ak[t + 1] + bk[t + 1] * ps;
    const R dp = pk_t1 - pk_t;
    const R rl = (t == 0) ? a.rlnp_top : log(pk_t1 / pk_t);
    const R al = (t == 0) ? a.log2sp : R(1) - (pk_t / dp) * rl;
    const R u = S(a.s.u + b), v = S(a.s.v + b), dv = S(a.s.div + b);
    const R cg = u * dlx + v * dly;
    if (t == 0) {
      db = dv * dp;
      cb = cg * dbk[0];
    } else {
      db = db + dv * dp;
      cb = cb + cg * dbk[t];
    }
    DB[t] = db;
    CB[t] = cb;
    CG[t] = cg;
    RL[t] = rl;
    AL[t] = al;
    pk_t = pk_t1;
    if (a.prs) {  // Phillips layer pressure (pressure_data.f90:87-88)
      const R pkt = ak[t] + bk[t] * ps;
      a.prs[(long)b * ng + p] =
          pow((pow(pk_t1, a.kappa) * pk_t1 - pow(pkt, a.kappa) * pkt) / ((a.kappa + R(1)) * dp), R(1) / a.kappa);
    }
  }
  const R dlnpsdt = -DB[L - 1] / ps - CB[L - 1];
  a.psg[p] = ps;
  a.dlnpsdt[p] = dlnpsdt;
  auto etadot = [&](int t) -> R {
    if (t == 0 || t == L) return R(0);
    return -ps * (bk[t] * dlnpsdt + CB[t - 1]) - DB[t - 1];
  };
  auto dlnpdt = [&](int t, R dv_b) -> R {
    const R pkt = ak[t] + bk[t] * ps, pkt1 = ak[t + 1] + bk[t + 1] * ps;
    const R dp = pkt1 - pkt;
    R wb, wc;
    if (t == 0) {
      wb = AL[0] * (dv_b * dp + ps * CB[0] * dbk[0]);
      wc = ps * CG[0] * dbk[0];
    } else {
      wb = RL[t] * (DB[t - 1] + ps * CB[t - 1]) + AL[t] * (dv_b * dp + ps * CG[t] * dbk[t]);
      wc = ps * CG[t] * (dbk[t] + a.ck[t] * RL[t] / dp);
    }
    return (wc - wb) / dp;
  };
  if (a.etadot)
    for (int t = 0; t <= L; ++t) a.etadot[(long)t * ng + p] = etadot(t);
  if (a.dlnpdtg)
    for (int t = 0; t < L; ++t) a.dlnpdtg[(long)(L - 1 - t) * ng + p] = dlnpdt(t, S(a.s.div + L - 1 - t));
  if (inverse_only) return;

  R* gA = a.gA;
  auto A = [&](int row) -> R& { return gA[(long)row * ng + p]; };
  const R fcor = a.omega2 * a.sinlat[j];
  const R dphx = a.dphisdx[p], dphy = a.dphisdy[p];
  // getpresgrad suffix recurrences, vertical advection and tendencies,
  // bottom to top
  R cofb2 = R(0), px3u = R(0), px3v = R(0);
  R um = R(0), vm = R(0), tm = R(0), dxm = R(0), dym = R(0);  // level b-1
  R uc = S(a.s.u), vc = S(a.s.v), tc = S(a.s.tv);
  for (int b = 0; b < L; ++b) {
    const int t = L - 1 - b;
    const R dtx = S(a.s.dtvdx + b), dty = S(a.s.dtvdy + b);
    if (b > 0) {
      const R pk2 = ak[t + 2] + bk[t + 2] * ps, pk1 = ak[t + 1] + bk[t + 1] * ps;
      cofb2 = cofb2 - rd * (bk[t + 2] / pk2 - bk[t + 1] / pk1) * tm;
      px3u = px3u - rd * RL[t + 1] * dxm;
      px3v = px3v - rd * RL[t + 1] * dym;
    }
    const R pkt = ak[t] + bk[t] * ps, pkt1 = ak[t + 1] + bk[t + 1] * ps;
    const R dp = pkt1 - pkt;
    const R cofb1 = (t == 0) ? -(R(1) / dp) * (AL[0] * dbk[0]) : -(R(1) / dp) * (bk[t] * RL[t] + AL[t] * dbk[t]);
    const R cofa = -(R(1) / dp) * (bk[t + 1] * pkt / pkt1 - bk[t] + RL[t] * (bk[t] - pkt * dbk[t] / dp));
    const R prsgx = cofb1 * rd * tc * ps * dlx - dphx + cofb2 * ps * dlx + px3u - rd * AL[t] * dtx -
                    cofa * rd * tc * ps * dlx;
    const R prsgy = cofb1 * rd * tc * ps * dly - dphy + cofb2 * ps * dly + px3v - rd * AL[t] * dty -
                    cofa * rd * tc * ps * dly;
    R up = R(0), vp = R(0), tp = R(0);
    if (b + 1 < L) {
      up = S(a.s.u + b + 1);
      vp = S(a.s.v + b + 1);
      tp = S(a.s.tv + b + 1);
    }
    const R e1 = etadot(t + 1), e0 = etadot(t);
    const R h = R(0.5) / dp;
    R vu = R(0), vv = R(0), vt = R(0);
    if (b > 0) {
      vu += e1 * (um - uc);
      vv += e1 * (vm - vc);
      vt += e1 * (tm - tc);
    }
    if (b + 1 < L) {
      vu += e0 * (uc - up);
      vv += e0 * (vc - vp);
      vt += e0 * (tc - tp);
    }
    vu *= h;
    vv *= h;
    vt *= h;
    const R dv_b = S(a.s.div + b);
    R vq = a.kappa * dlnpdt(t, dv_b) * tc;
    if (a.nt > 0) vq = vq / (R(1) + a.cvap_cp * S(a.s.trc + b));
    const R vadvv = vv - prsgy, vadvu = vu - prsgx;
    const R vr = S(a.s.vrt + b);
    A(a.a.ttend + b) = -uc * dtx - vc * dty - vt + vq;
    A(a.a.fu + b) = uc * (vr + fcor) + vadvv;
    A(a.a.fv + b) = vc * (vr + fcor) - vadvu;
    A(a.a.ke + b) = R(0.5) * (uc * uc + vc * vc);
    um = uc;
    vm = vc;
    tm = tc;
    dxm = dtx;
    dym = dty;
    uc = up;
    vc = vp;
    tc = tp;
  }
  A(a.a.dlnps) = dlnpsdt;

  // tracers: Thuburn (1993) flux-limited vertical advection + horizontal
  // advection (dyn_run.f90:279-292, :478-603)
  const R eps = epstiny_of<R>();
  R DDs[LMAX + 1];
  for (int iq = 0; iq < a.nt; ++iq) {
    const int q0 = a.s.trc + iq * L;
    auto Q = [&](int b) -> R { return S(q0 + b); };
    for (int k = 1; k <= L - 1; ++k) DDs[k] = Q(L - k - 1) - Q(L - k);
    {
      const R qt = Q(L - 1), qt1 = Q(L - 2);
      DDs[0] = (qt >= R(0)) ? qt - fmax(R(0), R(2) * qt - qt1) : qt - fmin(R(0), R(2) * qt - qt1);
      const R qb = Q(0), qb1 = Q(1);
      DDs[L] = (qb >= R(0)) ? fmax(R(0), R(2) * qb - qb1) - qb : fmin(R(0), R(2) * qb - qb1) - qb;
    }
    for (int k = 1; k <= L - 1; ++k)
      if (fabs(DDs[k]) < eps) DDs[k] = copysign(eps, DDs[k]);
    R hprev = Q(L - 1);
    for (int k = 1; k <= L; ++k) {
      R hk;
      const R qk = Q(L - k);
      if (k <= L - 1) {
        const R qk1 = Q(L - k - 1);
        hk = R(0.5) * (qk1 + qk);
        if (etadot(k) > R(0)) {
          const R phi = DDs[k - 1] / DDs[k];
          hk = qk + (phi + fabs(phi)) / (R(1) + fabs(phi)) * (hk - qk);
        } else {
          const R phi = DDs[k + 1] / DDs[k];
          hk = qk1 + (phi + fabs(phi)) / (R(1) + fabs(phi)) * (hk - qk1);
        }
      } else {
        hk = Q(0);
      }
      const int t = k - 1, b = L - k;
      const R pkt = ak[t] + bk[t] * ps, pkt1 = ak[t + 1] + bk[t + 1] * ps;
      const R ek = etadot(k), ek1 = etadot(k - 1);
      const R vadv = (R(1) / (pkt1 - pkt)) * ((hk * ek - hprev * ek1) + (qk * (ek1 - ek)));
      const int qd = a.s.dqdx + iq * L + b, qy = a.s.dqdy + iq * L + b;
      A(a.a.qtend + iq * L + b) = -S(a.s.u + b) * S(qd) - S(a.s.v + b) * S(qy) - vadv;
      hprev = hk;
    }
  }
}

template <typename R>
void launch_dyn_columns(const ColumnArgs<R>& a, bool inverse_only, cudaStream_t s) {
  if (a.L > LMAX - 1) throw std::runtime_error("nlev too large for the column kernel");
  long ng = (long)a.nlon * a.nlat;
  k_dyn_columns<R><<<ceil_div(ng, 128), 128, 0, s>>>(a, inverse_only ? 1 : 0);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_dyn_columns<double>(const ColumnArgs<double>&, bool, cudaStream_t);
template void launch_dyn_columns<float>(const ColumnArgs<float>&, bool, cudaStream_t);

// Held-Suarez forcing on the grid (phy_run_hs.f90:42-77); prs and psg are
// recomputed from ln(ps) as in calc_pressdata.
template <typename R>
__global__ void __launch_bounds__(256) k_hs(HsArgs<R> a) {
  const long ng = (long)a.nlon * a.nlat;
  const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ng) return;
  const int j = (int)(p / a.nlon);
  const int L = a.L;
  const R ps = exp(a.gS[(long)a.s.lnps * ng + p]);
  const R sl = a.sinlat[j], cl = a.coslat[j];
  const R s2 = sl * sl, c2 = cl * cl, c4 = c2 * c2;
  const R p0 = R(1.e5);
  for (int b = 0; b < L; ++b) {
    const int t = L - 1 - b;
    const R pkt = a.ak[t] + a.bk[t] * ps, pkt1 = a.ak[t + 1] + a.bk[t + 1] * ps;
    const R prs =
        pow((pow(pkt1, a.kappa) * pkt1 - pow(pkt, a.kappa) * pkt) / ((a.kappa + R(1)) * (pkt1 - pkt)), R(1) / a.kappa);
    R bl = prs / ps;
    R teq = pow(prs / p0, a.expo) * (R(315) - R(60) * s2 - R(10) * log(prs / p0) * c2);
    bl = (bl - a.sigbot) / (R(1) - a.sigbot);
    if (bl < R(0)) bl = R(0);
    if (teq < R(200)) teq = R(200);
    const R tv = a.gS[(long)(a.s.tv + b) * ng + p];
    const R vr = a.gS[(long)(a.s.vrt + b) * ng + p];
    const R dv = a.gS[(long)(a.s.div + b) * ng + p];
    a.gA[(long)b * ng + p] = (a.krada + (a.kradb - a.krada) * bl * c4) * (teq - tv);
    a.gA[(long)(L + b) * ng + p] = -(bl * a.kdrag) * vr;
    a.gA[(long)(2 * L + b) * ng + p] = -(bl * a.kdrag) * dv;
  }
}
template <typename R>
void launch_hs_forcing(const HsArgs<R>& a, cudaStream_t s) {
  long ng = (long)a.nlon * a.nlat;
  k_hs<R><<<ceil_div(ng, 256), 256, 0, s>>>(a);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_hs_forcing<double>(const HsArgs<double>&, cudaStream_t);
template void launch_hs_forcing<float>(const HsArgs<float>&, cudaStream_t);

// ------------------------------------------------------------ reductions --
__device__ double block_sum(double v) {
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

template <typename R>
__global__ void k_rowsum_ps(const R* psg, const double* w, int nlon, double* rowsum) {
  const int j = blockIdx.x;
  double s = 0;
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) s += (double)psg[(long)j * nlon + i];
  s = block_sum(s);
  if (threadIdx.x == 0) rowsum[j] = s * (w[j] / (2.0 * nlon));
}
__global__ void k_final_sum(const double* rowsum, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += rowsum[i];
    *out = s;
  }
}
template <typename R>
void launch_area_mean_ps(const R* psg, const double* w, int nlat, int nlon, double* rowsum, double* out,
                         cudaStream_t s) {
  k_rowsum_ps<R><<<nlat, 256, 0, s>>>(psg, w, nlon, rowsum);
  k_final_sum<<<1, 32, 0, s>>>(rowsum, nlat, out);
  count_launch(2);
  GD_LAUNCH_CHECK();
}
template void launch_area_mean_ps<double>(const double*, const double*, int, int, double*, double*, cudaStream_t);
template void launch_area_mean_ps<float>(const float*, const double*, int, int, double*, double*, cudaStream_t);

__global__ void k_pdry_init(const double* pmean, double* pdryini) {
  if (threadIdx.x == 0 && *pdryini == 0.0) *pdryini = *pmean;
}
void launch_pdry_init(const double* pmean, double* pdryini, cudaStream_t s) {
  k_pdry_init<<<1, 32, 0, s>>>(pmean, pdryini);
  count_launch();
  GD_LAUNCH_CHECK();
}

template <typename R>
__global__ void k_massfix_grid(const R* psg, const double* pdryini, const double* pmean, long ng, R* out) {
  const R pcorr = (R)(*pdryini / *pmean);
  for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < ng; p += (long)gridDim.x * blockDim.x)
    out[p] = log(psg[p] * pcorr);
}
template <typename R>
void launch_massfix_grid(const R* psg, const double* pdryini, const double* pmean, int ng, R* out, cudaStream_t s) {
  k_massfix_grid<R><<<ceil_div(ng, 256), 256, 0, s>>>(psg, pdryini, pmean, ng, out);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_massfix_grid<double>(const double*, const double*, const double*, int, double*, cudaStream_t);
template void launch_massfix_grid<float>(const float*, const double*, const double*, int, float*, cudaStream_t);

// per latitude: max wind speed over levels, min/max ps, area-weighted sum of
// (36 ps dlnps/dt)^2
template <typename R>
__global__ void k_diag_rows(const R* u, const R* v, int L, const R* psg, const R* dl, const double* w, int nlat,
                            int nlon, double* part) {
  const int j = blockIdx.x;
  const long ng = (long)nlat * nlon;
  double smax = 0, pmin = 1e300, pmax = -1e300, pt = 0;
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
    const long p = (long)j * nlon + i;
    for (int k = 0; k < L; ++k) {
      double uu = u[k * ng + p], vv = v[k * ng + p];
      smax = fmax(smax, sqrt(uu * uu + vv * vv));
    }
    double ps = psg[p];
    pmin = fmin(pmin, ps / 100.);
    pmax = fmax(pmax, ps / 100.);
    double x = 36. * ps * (double)dl[p];
    pt += x * x;
  }
  __shared__ double a[256], b[256], c[256], d[256];
  a[threadIdx.x] = smax;
  b[threadIdx.x] = pmin;
  c[threadIdx.x] = pmax;
  d[threadIdx.x] = pt;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      a[threadIdx.x] = fmax(a[threadIdx.x], a[threadIdx.x + o]);
      b[threadIdx.x] = fmin(b[threadIdx.x], b[threadIdx.x + o]);
      c[threadIdx.x] = fmax(c[threadIdx.x], c[threadIdx.x + o]);
      d[threadIdx.x] += d[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[4 * j + 0] = a[0];
    part[4 * j + 1] = b[0];
    part[4 * j + 2] = c[0];
    part[4 * j + 3] = d[0] * (w[j] / (2.0 * nlon));
  }
}
__global__ void k_diag_final(const double* part, int nlat, double* out) {
  if (threadIdx.x != 0) return;
  double smax = 0, pmin = 1e300, pmax = -1e300, pt = 0;
  for (int j = 0; j < nlat; ++j) {
    smax = fmax(smax, part[4 * j]);
    pmin = fmin(pmin, part[4 * j + 1]);
    pmax = fmax(pmax, part[4 * j + 2]);
    pt += part[4 * j + 3];
  }
  out[0] = smax;
  out[1] = pmin;
  out[2] = pmax;
  out[3] = sqrt(pt);
}
template <typename R>
void launch_diag(const R* u, const R* v, int L, const R* psg, const R* dlnpsdt, const double* w, int nlat, int nlon,
                 double* scratch, double* out, cudaStream_t s) {
  k_diag_rows<R><<<nlat, 256, 0, s>>>(u, v, L, psg, dlnpsdt, w, nlat, nlon, scratch);
  k_diag_final<<<1, 32, 0, s>>>(scratch, nlat, out);
  count_launch(2);
  GD_LAUNCH_CHECK();
}
template void launch_diag<double>(const double*, const double*, int, const double*, const double*, const double*,
                                  int, int, double*, double*, cudaStream_t);
template void launch_diag<float>(const float*, const float*, int, const float*, const float*, const double*, int,
                                 int, double*, double*, cudaStream_t);

}  // namespace gd

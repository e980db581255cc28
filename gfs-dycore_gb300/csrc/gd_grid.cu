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
constexpr int NTMAX = 8;  // tracers handled in registers by the column kernel

// Division and logarithm of the column kernel: IEEE for the FP64 path (the
// reference restated exactly), the hardware approximations for the FP32
// state (relative error ~1e-7, below the FP32 state's own rounding).
__device__ __forceinline__ double cdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float cdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double clog(double a) { return log(a); }
__device__ __forceinline__ float clog(float a) { return __logf(a); }

// Thuburn (1993) limited half-level value at interior interface k
// (dyn_run.f90:574-590): qa = level above the interface, qb = level below,
// dm = dd[k-1], d0 = dd[k], dp = dd[k+1], upwind by the sign of etadot.
template <typename R>
__device__ __forceinline__ R thuburn_half(R qa, R qb, R dm, R d0, R dp, R eta) {
  R h = R(0.5) * (qb + qa);
  if (eta > R(0)) {
    const R phi = cdiv(dm, d0);
    h = qa + cdiv(phi + fabs(phi), R(1) + fabs(phi)) * (h - qa);
  } else {
    const R phi = cdiv(dp, d0);
    h = qb + cdiv(phi + fabs(phi), R(1) + fabs(phi)) * (h - qb);
  }
  return h;
}

template <typename R>
__global__ void __launch_bounds__(128) k_dyn_columns(ColumnArgs<R> a, int inverse_only) {
  extern __shared__ __align__(16) unsigned char smcol[];
  const long ng = (long)a.nlon * a.nlat;
  const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ng) return;
  const int j = (int)(p / a.nlon);
  const int L = a.L;
  const R* gS = a.gS;
  // inputs through the read-only path: loads may be issued ahead of the
  // stores to the (disjoint) analysis rows
  auto S = [&](int row) -> R { return __ldg(gS + (long)row * ng + p); };
  const R* ak = a.ak;
  const R* bk = a.bk;
  const R* dbk = a.dbk;
  const R rd = a.rd;

  const R ps = exp(S(a.s.lnps));
  const R dlx = S(a.s.dlnpsdx), dly = S(a.s.dlnpsdy);
  auto PK = [&](int t) -> R { return ak[t] + bk[t] * ps; };
  // rlnp and alfa of the top-down layer t (pressure_data.f90:89-96)
  auto RLN = [&](int t, R pkt, R pkt1) -> R { return (t == 0) ? a.rlnp_top : clog(cdiv(pkt1, pkt)); };
  // getomega prefix sums in shared memory, [t][thread]
  R* DBs = reinterpret_cast<R*>(smcol);
  R* CBs = DBs + (long)L * blockDim.x;
  auto DB = [&](int t) -> R& { return DBs[t * blockDim.x + threadIdx.x]; };
  auto CB = [&](int t) -> R& { return CBs[t * blockDim.x + threadIdx.x]; };

  // pass 1, top to bottom: getomega prefix sums (dyn_run.f90:327-337)
  R pk_t = PK(0);
  R db = R(0), cb = R(0);
#pragma unroll 4
  for (int t = 0; t < L; ++t) {
    const int b = L - 1 - t;
    const R pk_t1 = PK(t + 1);
    const R dp = pk_t1 - pk_t;
    const R cg = S(a.s.u + b) * dlx + S(a.s.v + b) * dly;
    const R dv = S(a.s.div + b);
    if (t == 0) {
      db = dv * dp;
      cb = cg * dbk[0];
    } else {
      db = db + dv * dp;
      cb = cb + cg * dbk[t];
    }
    DB(t) = db;
    CB(t) = cb;
    if (a.prs)  // Phillips layer pressure (pressure_data.f90:87-88)
      a.prs[(long)b * ng + p] =
          pow((pow(pk_t1, a.kappa) * pk_t1 - pow(pk_t, a.kappa) * pk_t) / ((a.kappa + R(1)) * dp), R(1) / a.kappa);
    pk_t = pk_t1;
  }
  const R dlnpsdt = -DB(L - 1) / ps - CB(L - 1);
  a.psg[p] = ps;
  a.dlnpsdt[p] = dlnpsdt;
  auto etadot = [&](int t) -> R {  // dyn_run.f90:340-344
    if (t == 0 || t == L) return R(0);
    return -ps * (bk[t] * dlnpsdt + CB(t - 1)) - DB(t - 1);
  };
  // omega/p of layer t (dyn_run.f90:347-368) from its cg, divergence, rlnp, alfa
  auto dlnpdt = [&](int t, R cg, R dv, R dp, R idp, R rl, R al) -> R {
    R wb, wc;
    if (t == 0) {
      wb = al * (dv * dp + ps * CB(0) * dbk[0]);
      wc = ps * cg * dbk[0];
    } else {
      wb = rl * (DB(t - 1) + ps * CB(t - 1)) + al * (dv * dp + ps * cg * dbk[t]);
      wc = ps * cg * (dbk[t] + a.ck[t] * rl * idp);
    }
    return (wc - wb) * idp;
  };
  if (a.etadot)
    for (int t = 0; t <= L; ++t) a.etadot[(long)t * ng + p] = etadot(t);
  if (a.dlnpdtg)
    for (int t = 0; t < L; ++t) {
      const int b = L - 1 - t;
      const R pkt = PK(t), pkt1 = PK(t + 1), dp = pkt1 - pkt, idp = R(1) / dp;
      const R rl = RLN(t, pkt, pkt1), al = (t == 0) ? a.log2sp : R(1) - (pkt * idp) * rl;
      const R cg = S(a.s.u + b) * dlx + S(a.s.v + b) * dly;
      a.dlnpdtg[(long)b * ng + p] = dlnpdt(t, cg, S(a.s.div + b), dp, idp, rl, al);
    }
  if (inverse_only) return;

  R* gA = a.gA;
  auto A = [&](int row) -> R& { return gA[(long)row * ng + p]; };
  const R fcor = a.omega2 * a.sinlat[j];
  const R dphx = a.dphisdx[p], dphy = a.dphisdy[p];
  const int nt = min(a.nt, NTMAX);
  const R eps = epstiny_of<R>();
  // tracer windows q[b-1..b+2], carried limited half-level value at the
  // bottom interface of the current level (half[L] = q[0])
  R qm1[NTMAX], q0[NTMAX], q1[NTMAX], q2[NTMAX], hb[NTMAX];
#pragma unroll
  for (int iq = 0; iq < NTMAX; ++iq)
    if (iq < nt) {
      const int r0 = a.s.trc + iq * L;
      qm1[iq] = R(0);
      q0[iq] = S(r0);
      q1[iq] = (L > 1) ? S(r0 + 1) : R(0);
      q2[iq] = (L > 2) ? S(r0 + 2) : R(0);
      hb[iq] = q0[iq];
    }
  // pass 2, bottom to top: getpresgrad suffix recurrences (dyn_run.f90:416-434),
  // vertical advection (getvadv, :453-476; getvadv_tracers, :478-603) and the
  // tendencies (:190-292)
  R cofb2 = R(0), px3u = R(0), px3v = R(0);
  R um = R(0), vm = R(0), tm = R(0), dxm = R(0), dym = R(0), rlm = R(0);  // layer below
  R uc = S(a.s.u), vc = S(a.s.v), tc = S(a.s.tv);
  // pressure at the interfaces below the current layer, carried upward
  bool ipk_valid = false;
  R pk_below = R(0), ipk_below = R(0), ipk2 = R(0);
  // inputs of the current level, loaded one level ahead
  R n_dtx = S(a.s.dtvdx), n_dty = S(a.s.dtvdy), n_dv = S(a.s.div), n_vr = S(a.s.vrt);
  R n_up = (L > 1) ? S(a.s.u + 1) : R(0), n_vp = (L > 1) ? S(a.s.v + 1) : R(0), n_tp = (L > 1) ? S(a.s.tv + 1) : R(0);
  for (int b = 0; b < L; ++b) {
    const int t = L - 1 - b;
    const R dtx = n_dtx, dty = n_dty, dv_b = n_dv, vr = n_vr, up = n_up, vp = n_vp, tp = n_tp;
    if (b + 1 < L) {
      n_dtx = S(a.s.dtvdx + b + 1);
      n_dty = S(a.s.dtvdy + b + 1);
      n_dv = S(a.s.div + b + 1);
      n_vr = S(a.s.vrt + b + 1);
      n_up = (b + 2 < L) ? S(a.s.u + b + 2) : R(0);
      n_vp = (b + 2 < L) ? S(a.s.v + b + 2) : R(0);
      n_tp = (b + 2 < L) ? S(a.s.tv + b + 2) : R(0);
    }
    const R pkt = PK(t), pkt1 = ipk_valid ? pk_below : PK(t + 1);
    const R ipk1 = ipk_valid ? ipk_below : R(1) / pkt1;  // 1 / pk(t+1), carried from below
    const R ipkt = R(1) / pkt;                           // inf at the model top (pk = 0), unused there
    const R dp = pkt1 - pkt, idp = R(1) / dp;
    const R rl = (t == 0) ? a.rlnp_top : clog(pkt1 * ipkt);
    const R al = (t == 0) ? a.log2sp : R(1) - (pkt * idp) * rl;
    if (b > 0) cofb2 = cofb2 - rd * (bk[t + 2] * ipk2 - bk[t + 1] * ipk1) * tm;
    if (b > 0) {
      px3u = px3u - rd * rlm * dxm;
      px3v = px3v - rd * rlm * dym;
    }
    const R cofb1 = (t == 0) ? -idp * (al * dbk[0]) : -idp * (bk[t] * rl + al * dbk[t]);
    const R cofa = -idp * (bk[t + 1] * pkt * ipk1 - bk[t] + rl * (bk[t] - pkt * dbk[t] * idp));
    const R prsgx =
        cofb1 * rd * tc * ps * dlx - dphx + cofb2 * ps * dlx + px3u - rd * al * dtx - cofa * rd * tc * ps * dlx;
    const R prsgy =
        cofb1 * rd * tc * ps * dly - dphy + cofb2 * ps * dly + px3v - rd * al * dty - cofa * rd * tc * ps * dly;
    const R e1 = etadot(t + 1), e0 = etadot(t);
    const R h = R(0.5) * idp;
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
    const R cg = uc * dlx + vc * dly;
    R vq = a.kappa * dlnpdt(t, cg, dv_b, dp, idp, rl, al) * tc;
    if (a.nt > 0) vq = cdiv(vq, R(1) + a.cvap_cp * q0[0]);
    const R vadvv = vv - prsgy, vadvu = vu - prsgx;
    A(a.a.ttend + b) = -uc * dtx - vc * dty - vt + vq;
    A(a.a.fu + b) = uc * (vr + fcor) + vadvv;
    A(a.a.fv + b) = vc * (vr + fcor) - vadvu;
    A(a.a.ke + b) = R(0.5) * (uc * uc + vc * vc);
    // tracers at level b: top interface kt = t (= L-1-b), bottom kb = t + 1
#pragma unroll
    for (int iq = 0; iq < NTMAX; ++iq) {
      if (iq >= nt) continue;
      R ht;
      if (t == 0) {
        ht = q0[iq];  // half[0] = q at the top level
      } else {
        // dd[k] = q(level below k) - q(level above k); interfaces kt-1, kt, kt+1
        R dm, d0, dpp;
        if (t - 1 == 0) {  // dd[0], top boundary (dyn_run.f90:507-513)
          const R qt = q1[iq], qt1 = q0[iq];  // q[L-1] = q[b+1], q[L-2] = q[b]
          dm = (qt >= R(0)) ? qt - fmax(R(0), R(2) * qt - qt1) : qt - fmin(R(0), R(2) * qt - qt1);
        } else {
          dm = q1[iq] - q2[iq];
          if (fabs(dm) < eps) dm = copysign(eps, dm);
        }
        d0 = q0[iq] - q1[iq];
        if (fabs(d0) < eps) d0 = copysign(eps, d0);
        if (t + 1 == L) {  // dd[L], bottom boundary (dyn_run.f90:514-518)
          const R qb = q0[iq], qb1 = q1[iq];
          dpp = (qb >= R(0)) ? fmax(R(0), R(2) * qb - qb1) - qb : fmin(R(0), R(2) * qb - qb1) - qb;
        } else {
          dpp = qm1[iq] - q0[iq];
          if (fabs(dpp) < eps) dpp = copysign(eps, dpp);
        }
        ht = thuburn_half(q1[iq], q0[iq], dm, d0, dpp, e0);
      }
      const R vadq = idp * ((hb[iq] * e1 - ht * e0) + (q0[iq] * (e0 - e1)));
      const int qd = a.s.dqdx + iq * L + b, qy = a.s.dqdy + iq * L + b;
      A(a.a.qtend + iq * L + b) = -uc * S(qd) - vc * S(qy) - vadq;
      hb[iq] = ht;
      qm1[iq] = q0[iq];
      q0[iq] = q1[iq];
      q1[iq] = q2[iq];
      q2[iq] = (b + 3 < L) ? S(a.s.trc + iq * L + b + 3) : R(0);
    }
    um = uc;
    vm = vc;
    tm = tc;
    dxm = dtx;
    dym = dty;
    rlm = rl;
    ipk2 = ipk1;  // 1 / pk(t+1) becomes 1 / pk(t'+2) for the layer above
    pk_below = pkt;
    ipk_below = ipkt;
    ipk_valid = true;
    uc = up;
    vc = vp;
    tc = tp;
  }
  A(a.a.dlnps) = dlnpsdt;
}

template <typename R>
void launch_dyn_columns(const ColumnArgs<R>& a, bool inverse_only, cudaStream_t s) {
  if (a.L > LMAX - 1) throw std::runtime_error("nlev too large for the column kernel");
  if (a.nt > NTMAX) throw std::runtime_error("ntrac too large for the column kernel");
  long ng = (long)a.nlon * a.nlat;
  const size_t sm = 2 * (size_t)a.L * 128 * sizeof(R);
  static bool attr = false;
  if (!attr) {
    GD_CUDA(cudaFuncSetAttribute(k_dyn_columns<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr = true;
  }
  k_dyn_columns<R><<<ceil_div(ng, 128), 128, sm, s>>>(a, inverse_only ? 1 : 0);
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

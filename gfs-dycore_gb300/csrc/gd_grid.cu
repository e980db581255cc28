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

// Division and logarithm of the column kernel: IEEE for the FP64 path (the
// reference restated exactly), the hardware approximations for the FP32
// state (relative error ~1e-7, below the FP32 state's own rounding).
__device__ __forceinline__ double cdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float cdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double clog(double a) { return log(a); }
__device__ __forceinline__ double crcp(double a) { return 1.0 / a; }
__device__ __forceinline__ float crcp(float a) { return __fdividef(1.f, a); }
__device__ __forceinline__ float clog(float a) { return __logf(a); }

// Thuburn (1993) limited half-level value at interior interface k
// (dyn_run.f90:574-590): qa = level above the interface, qb = level below,
// dm = dd[k-1], d0 = dd[k], dp = dd[k+1], upwind by the sign of etadot.
// Both upwind cases in one path: the columns of a warp differ in the sign.
// The limiter (phi + |phi|) / (1 + |phi|) of phi = r / d0 (r = dm or dp) is
// 2 phi / (1 + phi) = 2 r / (d0 + r) when r and d0 have one sign and 0
// otherwise: one division instead of two, and finite where r / d0 would
// overflow (d0 is clamped to the smallest normal, not to zero).
template <typename R>
__device__ __forceinline__ R thuburn_half(R qa, R qb, R dm, R d0, R dp, R eta) {
  const R h = R(0.5) * (qb + qa);
  const bool up = eta > R(0);
  const R qu = up ? qa : qb;
  const R r = up ? dm : dp;
  const bool same = (r > R(0)) == (d0 > R(0)) && r != R(0);
  const R lim = same ? cdiv(R(2) * r, d0 + r) : R(0);
  return qu + lim * (h - qu);
}

// dd[k] = q(level below k) - q(level above k) at interior interface k,
// clamped away from zero (dyn_run.f90:519-524)
template <typename R>
__device__ __forceinline__ R dd_mid(R qbelow, R qabove) {
  const R eps = epstiny_of<R>();
  const R d = qbelow - qabove;
  return (fabs(d) < eps) ? copysign(eps, d) : d;
}
// one-sided boundary differences (dyn_run.f90:507-518): dd[0] from the top
// level qt and the one below it, dd[L] from the bottom level qb and the one
// above it
template <typename R>
__device__ __forceinline__ R dd_top(R qt, R qn) {
  return (qt >= R(0)) ? qt - fmax(R(0), R(2) * qt - qn) : qt - fmin(R(0), R(2) * qt - qn);
}
template <typename R>
__device__ __forceinline__ R dd_bottom(R qb, R qn) {
  return (qb >= R(0)) ? fmax(R(0), R(2) * qb - qn) - qb : fmin(R(0), R(2) * qb - qn) - qb;
}

// Level-parallel column kernel.  A CTA owns 32 adjacent grid columns (one per
// lane, so every load and store is a 128-byte row segment) and splits the L
// levels into blocks of LB, one block per warp.  The vertical recurrences
// are scans: each thread sums its block, the block sums meet in shared
// memory, and every thread adds the sums of the blocks above it (getomega's
// top-down prefix sums, dyn_run.f90:327-337) or below it (getpresgrad's
// bottom-up sums, :416-434).  etadot at the interfaces goes through shared
// memory to the two levels that use it.  Phases:
//   1. block sums of div dp, cg dbk (top-down) and of the pressure-gradient
//      terms (bottom-up); Phillips layer pressure (pressure_data.f90:87-88);
//   2. block offsets, dlnps/dt, etadot at the block's interfaces
//      (dyn_run.f90:340-344);
//   3. omega/p (:347-368), pressure gradient, vertical advection of u, v,
//      Tv (getvadv, :453-476) and the tendencies (:190-292);
//   4. tracers, one at a time: Thuburn-limited vertical advection
//      (getvadv_tracers, :478-603) and horizontal advection.
// Levels are indexed b bottom (0) to top; interface quantities t top (0)
// to bottom; layer t = L-1-b.
// at most NWM warps (LB is chosen so); 1024 resident threads per SM for the
// FP32 state (64 registers), 512 for FP64
template <typename R, int LB, int NWM>
__global__ void __launch_bounds__(32 * NWM, (sizeof(R) == 4 ? 32 : 16) / NWM)
    k_dyn_columns(ColumnArgs<R> a, int inverse_only) {
  extern __shared__ __align__(16) unsigned char smcol[];
  // the warp's level block: the same for all its lanes (blockDim.x is 32);
  // taken through a warp reduction so that the compiler knows it too, and
  // every level index, row offset and branch on a level is warp-uniform
  const int lane = threadIdx.x, w = (int)__reduce_min_sync(0xffffffffu, threadIdx.y), NW = blockDim.y;
  const int L = a.L;
  const long ng = (long)a.nlon * a.nlat;
  const long pq = (long)blockIdx.x * 32 + lane;
  const bool valid = pq < ng;
  const long p = valid ? pq : ng - 1;  // lanes past the end compute a copy and store nothing
  const int j = (int)(p / a.nlon);
  R* part = reinterpret_cast<R*>(smcol);  // [5][NW][32] block sums, then [2][32] column totals
  R* etas = part + (5 * NW + 2) * 32;      // [L+1][32] etadot
  // FP64: ln(p(t+1)/p(t)) and 1/p(t) of every layer from phase 1 for phase 3
  // (each thread reads back only what it wrote: no barrier).  Its log and
  // reciprocals are the costly FP64 operations of the level loop; the FP32
  // kernel recomputes them (hardware approximations).
  constexpr bool kKeep = sizeof(R) == 8;
  R* rls = etas + (L + 1) * 32;  // [L][32] (FP64 only)
  R* ipks = rls + L * 32;        // [L][32] (FP64 only)
  auto PART = [&](int q, int ww) -> R& { return part[(q * NW + ww) * 32 + lane]; };
  auto ETA = [&](int t) -> R& { return etas[t * 32 + lane]; };
  const R* gS = a.gS;
  auto S = [&](int row) -> R { return __ldg(gS + (long)row * ng + p); };
  const R* ak = a.ak;
  const R* bk = a.bk;
  const R* dbk = a.dbk;
  const R rd = a.rd;
  const R ps = exp(S(a.s.lnps));
  const R dlx = S(a.s.dlnpsdx), dly = S(a.s.dlnpsdy);
  auto PK = [&](int t) -> R { return __ldg(ak + t) + __ldg(bk + t) * ps; };
  auto RLN = [&](int t, R pkt, R pkt1) -> R { return (t == 0) ? a.rlnp_top : clog(cdiv(pkt1, pkt)); };
  const int b0 = w * LB;
  const int nb = max(0, min(LB, L - b0));

  // phase 1
  R xdb[LB], xcb[LB];
  R s2 = R(0), su = R(0), sv = R(0);
  // pressure and its reciprocal at the bottom interface of the current level,
  // carried upward (the top interface of level i is the bottom one of i + 1)
  R pkb = PK(L - b0), ipkb = crcp(pkb);
  // the block's inputs, all loads issued before the arithmetic (levels past
  // the block's end load its last level again and are not used)
  R lu[LB], lv[LB], ldv[LB], ltv[LB], ltx[LB], lty[LB];
#pragma unroll
  for (int i = 0; i < LB; ++i) {
    const int b = b0 + min(i, nb - 1);
    lu[i] = S(a.s.u + b);
    lv[i] = S(a.s.v + b);
    ldv[i] = S(a.s.div + b);
    ltv[i] = S(a.s.tv + b);
    ltx[i] = S(a.s.dtvdx + b);
    lty[i] = S(a.s.dtvdy + b);
  }
#pragma unroll
  for (int i = 0; i < LB; ++i) {
    xdb[i] = R(0);
    xcb[i] = R(0);
    if (i < nb) {
      const int b = b0 + i, t = L - 1 - b;
      const R pkt = PK(t), pkt1 = pkb, dp = pkt1 - pkt;
      const R ipkt = t > 0 ? crcp(pkt) : R(0), ipk1 = ipkb;
      pkb = pkt;
      ipkb = ipkt;
      const R cg = lu[i] * dlx + lv[i] * dly;
      xdb[i] = ldv[i] * dp;
      xcb[i] = cg * __ldg(dbk + t);
      if (t > 0) {  // terms of the sums over the layers below a layer
        const R rl = clog(cdiv(pkt1, pkt));
        s2 += (__ldg(bk + t + 1) * ipk1 - __ldg(bk + t) * ipkt) * ltv[i];
        su += rl * ltx[i];
        sv += rl * lty[i];
        if (kKeep) rls[t * 32 + lane] = rl;
      } else if (kKeep) {
        rls[lane] = a.rlnp_top;
      }
      if (kKeep) ipks[t * 32 + lane] = ipkt;
      if (a.prs && valid)
        a.prs[(long)b * ng + p] =
            pow((pow(pkt1, a.kappa) * pkt1 - pow(pkt, a.kappa) * pkt) / ((a.kappa + R(1)) * dp), R(1) / a.kappa);
    }
  }
  // exclusive top-down prefix within the block (its top level is i = nb-1)
  R dbs = R(0), cbs = R(0);
#pragma unroll
  for (int i = LB - 1; i >= 0; --i) {
    const R d = xdb[i], c = xcb[i];
    xdb[i] = dbs;
    xcb[i] = cbs;
    dbs += d;
    cbs += c;
  }
  PART(0, w) = dbs;
  PART(1, w) = cbs;
  PART(2, w) = s2;
  PART(3, w) = su;
  PART(4, w) = sv;
  __syncthreads();

  // phase 2: offsets from the blocks above (DB, CB) and below (the rest).
  // Warp q scans quantity q over the blocks in place (exclusive sums; DB
  // and CB also keep their column totals), then every warp reads its own.
  for (int q = w; q < 5; q += NW) {
    R run = R(0);
    for (int k = 0; k < NW; ++k) {
      const int ww = q < 2 ? NW - 1 - k : k;
      const R v = PART(q, ww);
      PART(q, ww) = run;
      run += v;
    }
    if (q < 2) part[(5 * NW + q) * 32 + lane] = run;
  }
  __syncthreads();
  const R dbo = PART(0, w), cbo = PART(1, w);
  const R dbt = part[5 * NW * 32 + lane], cbt = part[(5 * NW + 1) * 32 + lane];
  R S2 = PART(2, w), SU = PART(3, w), SV = PART(4, w);
  const R dlnpsdt = -dbt / ps - cbt;
#pragma unroll
  for (int i = 0; i < LB; ++i) {
    xdb[i] += dbo;  // DB(t-1), CB(t-1) of layer t
    xcb[i] += cbo;
    if (i < nb) {
      const int t = L - 1 - (b0 + i);
      const R e = (t == 0) ? R(0) : -ps * (__ldg(bk + t) * dlnpsdt + xcb[i]) - xdb[i];
      ETA(t) = e;
      if (a.etadot && valid) a.etadot[(long)t * ng + p] = e;
    }
  }
  if (w == 0) {
    ETA(L) = R(0);
    if (valid) {
      if (a.etadot) a.etadot[(long)L * ng + p] = R(0);
      a.psg[p] = ps;
      a.dlnpsdt[p] = dlnpsdt;
      if (!inverse_only) a.gA[(long)a.a.dlnps * ng + p] = dlnpsdt;
    }
  }
  if (inverse_only && !a.dlnpdtg) return;  // uniform over the CTA
  __syncthreads();

  // phase 3
  R* gA = a.gA;
  auto A = [&](int row, R v) {
    if (valid) gA[(long)row * ng + p] = v;
  };
  const R fcor = a.omega2 * a.sinlat[j];
  const R dphx = a.dphisdx[p], dphy = a.dphisdy[p];
  R uu[LB], vv[LB], idpa[LB];
  R pkb3 = PK(L - b0), ipkb3 = crcp(pkb3);
  R um = R(0), vm = R(0), tm = R(0);
  R uc = R(0), vc = R(0), tc = R(0);
  if (nb > 0) {
    if (b0 > 0) {
      um = S(a.s.u + b0 - 1);
      vm = S(a.s.v + b0 - 1);
      tm = S(a.s.tv + b0 - 1);
    }
    uc = S(a.s.u + b0);
    vc = S(a.s.v + b0);
    tc = S(a.s.tv + b0);
  }
#pragma unroll
  for (int i = 0; i < LB; ++i) {
    uu[i] = uc;
    vv[i] = vc;
    idpa[i] = R(0);
    if (i >= nb) continue;
    const int b = b0 + i, t = L - 1 - b;
    R up = R(0), vp = R(0), tp = R(0);
    if (b + 1 < L) {
      up = S(a.s.u + b + 1);
      vp = S(a.s.v + b + 1);
      tp = S(a.s.tv + b + 1);
    }
    const R pkt = PK(t), pkt1 = pkb3, dp = pkt1 - pkt, idp = crcp(dp);
    // 1/pk(t) is unused at the model top (pk = 0)
    const R ipkt = kKeep ? ipks[t * 32 + lane] : (t > 0 ? crcp(pkt) : R(0)), ipk1 = ipkb3;
    pkb3 = pkt;
    ipkb3 = ipkt;
    idpa[i] = idp;
    const R rl = kKeep ? rls[t * 32 + lane] : RLN(t, pkt, pkt1);
    const R al = (t == 0) ? a.log2sp : R(1) - (pkt * idp) * rl;
    const R cg = uc * dlx + vc * dly;
    const R dv = S(a.s.div + b);
    const R dbkt = __ldg(dbk + t);
    R wb, wc;
    if (t == 0) {
      wb = al * (dv * dp + ps * (cg * dbkt) * dbkt);
      wc = ps * cg * dbkt;
    } else {
      wb = rl * (xdb[i] + ps * xcb[i]) + al * (dv * dp + ps * cg * dbkt);
      wc = ps * cg * (dbkt + __ldg(a.ck + t) * rl * idp);
    }
    const R dlnpdt = (wc - wb) * idp;  // omega / p
    if (a.dlnpdtg && valid) a.dlnpdtg[(long)b * ng + p] = dlnpdt;
    if (!inverse_only) {
      const R dtx = S(a.s.dtvdx + b), dty = S(a.s.dtvdy + b);
      const R bkt = __ldg(bk + t), bkt1 = __ldg(bk + t + 1);
      const R cofb2 = -rd * S2, px3u = -rd * SU, px3v = -rd * SV;
      const R cofb1 = (t == 0) ? -idp * (al * dbkt) : -idp * (bkt * rl + al * dbkt);
      const R cofa = -idp * (bkt1 * pkt * ipk1 - bkt + rl * (bkt - pkt * dbkt * idp));
      const R prsgx =
          cofb1 * rd * tc * ps * dlx - dphx + cofb2 * ps * dlx + px3u - rd * al * dtx - cofa * rd * tc * ps * dlx;
      const R prsgy =
          cofb1 * rd * tc * ps * dly - dphy + cofb2 * ps * dly + px3v - rd * al * dty - cofa * rd * tc * ps * dly;
      const R e1 = ETA(t + 1), e0 = ETA(t);
      const R h = R(0.5) * idp;
      R vu = R(0), vvv = R(0), vt = R(0);
      if (b > 0) {
        vu += e1 * (um - uc);
        vvv += e1 * (vm - vc);
        vt += e1 * (tm - tc);
      }
      if (b + 1 < L) {
        vu += e0 * (uc - up);
        vvv += e0 * (vc - vp);
        vt += e0 * (tc - tp);
      }
      vu *= h;
      vvv *= h;
      vt *= h;
      R vq = a.kappa * dlnpdt * tc;
      if (a.nt > 0) vq = cdiv(vq, R(1) + a.cvap_cp * S(a.s.trc + b));
      const R vr = S(a.s.vrt + b);
      A(a.a.ttend + b, -uc * dtx - vc * dty - vt + vq);
      A(a.a.fu + b, uc * (vr + fcor) + (vvv - prsgy));
      A(a.a.fv + b, vc * (vr + fcor) - (vu - prsgx));
      A(a.a.ke + b, R(0.5) * (uc * uc + vc * vc));
      if (t > 0) {
        S2 += (bkt1 * ipk1 - bkt * ipkt) * tc;
        SU += rl * dtx;
        SV += rl * dty;
      }
    }
    um = uc;
    vm = vc;
    tm = tc;
    uc = up;
    vc = vp;
    tc = tp;
  }
  if (inverse_only) return;

  // phase 4: tracers, one at a time.  Interface t (top of level b = L-1-t)
  // has dd[t] = q[b] - q[b+1]; the limited value at t uses dd[t-1], dd[t],
  // dd[t+1], so each level computes one new difference and carries two.
  for (int iq = 0; iq < a.nt; ++iq) {
    const int r0 = a.s.trc + iq * L;
    auto Q = [&](int b) -> R { return (b >= 0 && b < L) ? S(r0 + b) : R(0); };
    // the horizontal gradients of the block's levels, loaded ahead of their use
    R gqx[LB], gqy[LB];
#pragma unroll
    for (int i = 0; i < LB; ++i) {
      gqx[i] = gqy[i] = R(0);
      if (i < nb) {
        gqx[i] = S(a.s.dqdx + iq * L + b0 + i);
        gqy[i] = S(a.s.dqdy + iq * L + b0 + i);
      }
    }
    const int t0 = L - 1 - b0;
    R q0 = Q(b0), q1 = Q(b0 + 1), q2 = Q(b0 + 2);
    // dA = dd[t], dB = dd[t+1] for the level about to be processed; hb =
    // limited value at its bottom interface t+1 (half[L] = q[0])
    R dA, dB, hb;
    if (b0 == 0) {
      hb = q0;
      dA = dd_mid(q0, q1);  // unused when L = 1
      dB = dd_bottom(q0, q1);
    } else {
      const R qm = Q(b0 - 1), qmm = Q(b0 - 2);
      dA = (t0 == 0) ? dd_top(q0, qm) : dd_mid(q0, q1);
      dB = dd_mid(qm, q0);
      const R dC = (b0 == 1) ? dd_bottom(qm, q0) : dd_mid(qmm, qm);
      hb = thuburn_half(q0, qm, dA, dB, dC, ETA(t0 + 1));
    }
    R e1 = ETA(t0 + 1);
#pragma unroll
    for (int i = 0; i < LB; ++i) {
      if (i >= nb) continue;
      const int b = b0 + i, t = L - 1 - b;
      const R e0 = ETA(t);
      R ht = q0;  // half[0] = q at the top level
      if (t > 0) {
        const R dN = (t == 1) ? dd_top(q1, q0) : dd_mid(q1, q2);  // dd[t-1]
        ht = thuburn_half(q1, q0, dN, dA, dB, e0);
        dB = dA;
        dA = dN;
      }
      const R idp = idpa[i];
      const R vadq = idp * ((hb * e1 - ht * e0) + (q0 * (e0 - e1)));
      A(a.a.qtend + iq * L + b, -uu[i] * gqx[i] - vv[i] * gqy[i] - vadq);
      hb = ht;
      e1 = e0;
      q0 = q1;
      q1 = q2;
      q2 = Q(b + 3);
    }
  }
}

template <typename R, int LB, int NWM>
static void launch_cols_lb(const ColumnArgs<R>& a, bool inverse_only, cudaStream_t s) {
  const long ng = (long)a.nlon * a.nlat;
  const int nw = ceil_div(a.L, LB);
  const size_t sm = (size_t)(5 * nw + 2 + a.L + 1 + (sizeof(R) == 8 ? 2 * a.L : 0)) * 32 * sizeof(R);
  if (sm > 48 * 1024)
    GD_CUDA(cudaFuncSetAttribute(k_dyn_columns<R, LB, NWM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  k_dyn_columns<R, LB, NWM><<<(unsigned)ceil_div(ng, 32), dim3(32, nw), sm, s>>>(a, inverse_only ? 1 : 0);
}

template <typename R>
void launch_dyn_columns(const ColumnArgs<R>& a, bool inverse_only, cudaStream_t s, int lb) {
  if (a.L < 1 || a.L > LMAX) throw std::runtime_error("nlev out of range for the column kernel");
  // levels per warp (at most 16 warps per CTA): 4, or 8 when asked or above 64 levels
  if (a.L <= 64 && lb != 8)
    launch_cols_lb<R, 4, 16>(a, inverse_only, s);
  else
    launch_cols_lb<R, 8, 16>(a, inverse_only, s);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_dyn_columns<double>(const ColumnArgs<double>&, bool, cudaStream_t, int);
template void launch_dyn_columns<float>(const ColumnArgs<float>&, bool, cudaStream_t, int);

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
  const R p0 = R(1.e5), logp0 = log(p0);
  // levels in groups of four: the group's grid loads are issued before its
  // arithmetic, and pk^kappa of an interface is carried from the level below
  // (the bottom interface of a level is the top one of the level under it)
  constexpr int G = 4;
  R pw1 = pow(a.ak[L] + a.bk[L] * ps, a.kappa);
  for (int b0 = 0; b0 < L; b0 += G) {
    R tvv[G], vrv[G], dvv[G];
#pragma unroll
    for (int u = 0; u < G; ++u) {
      const int b = min(b0 + u, L - 1);
      tvv[u] = a.gS[(long)(a.s.tv + b) * ng + p];
      vrv[u] = a.gS[(long)(a.s.vrt + b) * ng + p];
      dvv[u] = a.gS[(long)(a.s.div + b) * ng + p];
    }
#pragma unroll
    for (int u = 0; u < G; ++u) {
      const int b = b0 + u;
      if (b >= L) break;
      const int t = L - 1 - b;
      const R pkt = a.ak[t] + a.bk[t] * ps, pkt1 = a.ak[t + 1] + a.bk[t + 1] * ps;
      const R pw0 = pow(pkt, a.kappa);
      // Phillips layer pressure prs = X^(1/kappa) and ln(prs/p0) from one
      // logarithm of X: three logarithms and two powers fewer per level than
      // pow(X, 1/kappa), pow(prs/p0, expo) and log(prs/p0) (the level loop's
      // FP64 cost; the results agree to ~1e-14 relative)
      const R lx = log((pw1 * pkt1 - pw0 * pkt) / ((a.kappa + R(1)) * (pkt1 - pkt))) / a.kappa;
      const R prs = exp(lx);
      const R lp = lx - logp0;
      pw1 = pw0;
      R bl = prs / ps;
      R teq = exp(a.expo * lp) * (R(315) - R(60) * s2 - R(10) * lp * c2);
      bl = (bl - a.sigbot) / (R(1) - a.sigbot);
      if (bl < R(0)) bl = R(0);
      if (teq < R(200)) teq = R(200);
      const R tv = tvv[u], vr = vrv[u], dv = dvv[u];
      const R f = a.sppt ? R(1) + a.vfact[b] * a.sppt[p] : R(1);
      a.gA[(long)b * ng + p] = f * ((a.krada + (a.kradb - a.krada) * bl * c4) * (teq - tv));
      a.gA[(long)(L + b) * ng + p] = f * (-(bl * a.kdrag) * vr);
      a.gA[(long)(2 * L + b) * ng + p] = f * (-(bl * a.kdrag) * dv);
    }
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

__global__ void k_pdry_init(const double* pmean, const double* pmoist, double* pdryini) {
  if (threadIdx.x == 0 && *pdryini == 0.0) *pdryini = *pmean - (pmoist ? *pmoist : 0.0);
}
void launch_pdry_init(const double* pmean, const double* pmoist, double* pdryini, cudaStream_t s) {
  k_pdry_init<<<1, 32, 0, s>>>(pmean, pmoist, pdryini);
  count_launch();
  GD_LAUNCH_CHECK();
}

template <typename R>
__global__ void k_massfix_grid(const R* psg, const double* pdryini, const double* pmean, const double* pwatg,
                               double grav, long ng, R* out) {
  const R pcorr = (R)((*pdryini + grav * (pwatg ? *pwatg : 0.0)) / *pmean);
  for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < ng; p += (long)gridDim.x * blockDim.x)
    out[p] = log(psg[p] * pcorr);
}
template <typename R>
void launch_massfix_grid(const R* psg, const double* pdryini, const double* pmean, const double* pwatg, double grav,
                         int ng, R* out, cudaStream_t s) {
  k_massfix_grid<R><<<ceil_div(ng, 256), 256, 0, s>>>(psg, pdryini, pmean, pwatg, grav, ng, out);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_massfix_grid<double>(const double*, const double*, const double*, const double*, double, int,
                                          double*, cudaStream_t);
template void launch_massfix_grid<float>(const float*, const double*, const double*, const double*, double, int,
                                         float*, cudaStream_t);

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

// gd_spec.cu -- spectral-space kernels of the GFS spectral dycore step:
// the per-degree semi-implicit IMEX RK3 stage update (src/run.f90:312-490),
// implicit hyperdiffusion (run.f90:493-501), the time-split physics update
// (run.f90:526-538), the batched FP64 inversion of the semi-implicit
// matrices (semimp_data.f90:238-253) and layout conversions.
#include <vector>

#include "gd_spec.cuh"

namespace gd {

constexpr int QC = GD_STAGE_QC;  // spectral coefficients (same degree n) per CTA
static_assert(QC % 4 == 0, "the matvec works on groups of four coefficients");

std::vector<int4> make_stage_items(int T, int qc) {
  std::vector<int4> it;
  for (int n = T; n >= 0; --n)
    for (int m0 = 0; m0 <= n; m0 += qc) it.push_back(make_int4(n, m0, std::min(qc, n + 1 - m0), 0));
  return it;
}

template <typename V>
__device__ __forceinline__ V vz() {
  V v;
  v.x = 0;
  v.y = 0;
  return v;
}

// even-L product on two adjacent levels x Q coefficients per thread
template <typename R, typename V, int Q, typename St>
__device__ __forceinline__ void smem_matvec_even(const R* __restrict__ AT, const V* X, St st, int L, int cnt, int t,
                                                 int nt) {
  const int Lh = L >> 1, nqq = (cnt + Q - 1) / Q;
  for (int e = t; e < Lh * nqq; e += nt) {
    const int q = e / Lh, k = 2 * (e - q * Lh);
    const int i0 = Q * q;
    R ax0[Q], ay0[Q], ax1[Q], ay1[Q];
#pragma unroll
    for (int u = 0; u < Q; ++u) ax0[u] = ay0[u] = ax1[u] = ay1[u] = R(0);
    const V* X0 = X + i0 * L;
#pragma unroll 16
    for (int j = 0; j < L; ++j) {
      const V aj = __ldg(reinterpret_cast<const V*>(AT + j * L + k));  // A[k][j], A[k+1][j]
#pragma unroll
      for (int u = 0; u < Q; ++u) {
        const V x = X0[u * L + j];
        ax0[u] += aj.x * x.x;
        ay0[u] += aj.x * x.y;
        ax1[u] += aj.y * x.x;
        ay1[u] += aj.y * x.y;
      }
    }
#pragma unroll
    for (int u = 0; u < Q; ++u)
      if (i0 + u < cnt) {
        V y0, y1;
        y0.x = ax0[u];
        y0.y = ay0[u];
        y1.x = ax1[u];
        y1.y = ay1[u];
        st(i0 + u, k, y0);
        st(i0 + u, k + 1, y1);
      }
  }
}

// Y[i][k] = sum_j A[k][j] X[i][j] for i < cnt (complex X, real A).  AT
// holds A transposed (AT[j][k] = A[k][j]) so a warp's loads of one j are
// contiguous over k; the L x L matrices stay L1-resident.  X, Y index-major
// with QC rows.  For even L a thread owns two adjacent output levels of four
// coefficients: one paired matrix load and four broadcast reads of X feed
// sixteen FMAs (the shared-memory pipe, not the FMA pipe, bounds this loop);
// of two coefficients when four would leave threads of the group idle.
// Odd L: one level per thread.  Rows past cnt are computed from unused
// shared memory and not stored.  Every output sums over j in order, so both
// forms give the same bits.  Threads t = 0 .. nt-1 of a group share the work
// (two independent products run side by side on the two halves of a CTA).
// st(i, k, y) takes output (i, k): stores it, or folds the step that uses it
// into the product's epilogue
template <typename V>
struct MvStore {
  V* Y;
  int L;
  __device__ __forceinline__ void operator()(int i, int k, V y) const { Y[i * L + k] = y; }
};
template <typename R, typename V, typename St>
__device__ __forceinline__ void smem_matvec(const R* __restrict__ AT, const V* X, St st, int L, int cnt, int t, int nt) {
  const int nq = (cnt + 3) >> 2;
  if (L & 1) {
    for (int e = t; e < L * nq; e += nt) {
      const int q = e / L, k = e - q * L;
      const int i0 = 4 * q;
      R ax[4], ay[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) ax[u] = ay[u] = R(0);
      const V* X0 = X + i0 * L;
#pragma unroll 4
      for (int j = 0; j < L; ++j) {
        const R aj = __ldg(AT + j * L + k);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const V x = X0[u * L + j];
          ax[u] += aj * x.x;
          ay[u] += aj * x.y;
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (i0 + u < cnt) {
          V y;
          y.x = ax[u];
          y.y = ay[u];
          st(i0 + u, k, y);
        }
    }
    return;
  }
  // four coefficients per thread while that leaves no thread of the group
  // idle, else two (one more thread's worth of loads per FMA, twice the threads)
  const int Lh = L >> 1;
  if (Lh * nq >= nt) {
    smem_matvec_even<R, V, 4>(AT, X, st, L, cnt, t, nt);
  } else {
    smem_matvec_even<R, V, 2>(AT, X, st, L, cnt, t, nt);
  }
}

// Y3[i] = sum_k w[k] X[i][k] for i < cnt: eight threads per coefficient, each
// summing every eighth level, then a shuffle tree over the eight.  The group
// (nt threads, a multiple of 32) runs whole warps, all of them to the end.
template <typename R, typename V, typename St>
__device__ __forceinline__ void smem_dot(const R* __restrict__ w, const V* X, St st, int L, int cnt, int t, int nt) {
  const int g = t & 7, per = nt >> 3;
  for (int base = 0; base < cnt; base += per) {
    const int i = base + (t >> 3);
    R sx = R(0), sy = R(0);
    if (i < cnt)
      for (int k = g; k < L; k += 8) {
        const R wk = __ldg(w + k);
        sx += wk * X[i * L + k].x;
        sy += wk * X[i * L + k].y;
      }
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {
      sx += __shfl_xor_sync(0xffffffffu, sx, o);
      sy += __shfl_xor_sync(0xffffffffu, sy, o);
    }
    if (g == 0 && i < cnt) {
      V y;
      y.x = sx;
      y.y = sy;
      st(i, 0, y);
    }
  }
}

template <typename R>
__device__ __forceinline__ typename C2<R>::T ld2(const R* base, long row, long ld, int col) {
  return *reinterpret_cast<const typename C2<R>::T*>(base + row * ld + 2 * col);
}
// read-only path for arrays no thread of the launch writes
template <typename R>
__device__ __forceinline__ typename C2<R>::T ldg2(const R* base, long row, long ld, int col) {
  return __ldg(reinterpret_cast<const typename C2<R>::T*>(base + row * ld + 2 * col));
}
template <typename R>
__device__ __forceinline__ void st2(R* base, long row, long ld, int col, typename C2<R>::T v) {
  *reinterpret_cast<typename C2<R>::T*>(base + row * ld + 2 * col) = v;
}

// Raw tendencies of getdyntend (dyn_run.f90:229-271) from the analyses:
// ddiv = curl(F)/a - lap/a^2 KE, dvrt = -div(F)/a with F = (Fu, Fv).
template <typename R>
__device__ __forceinline__ void raw_tend(const StageArgs<R>& a, long idx, int k, R lap, typename C2<R>::T& dvrt,
                                         typename C2<R>::T& ddiv, typename C2<R>::T& dtv) {
  typedef typename C2<R>::T V;
  const V imfv = ldg2(a.AP, idx, a.ldAP, a.ap.imfv + k), imfu = ldg2(a.AP, idx, a.ldAP, a.ap.imfu + k);
  const V fu = ldg2(a.AH, idx, a.ldAH, a.ah.fu + k), mfv = ldg2(a.AH, idx, a.ldAH, a.ah.mfv + k);
  const V ke = ldg2(a.AP, idx, a.ldAP, a.ap.ke + k);
  dvrt.x = -(imfu.x + mfv.x) * a.ainv;
  dvrt.y = -(imfu.y + mfv.y) * a.ainv;
  ddiv.x = (imfv.x + fu.x) * a.ainv - (lap * a.ainv2) * ke.x;
  ddiv.y = (imfv.y + fu.y) * a.ainv - (lap * a.ainv2) * ke.y;
  dtv = ldg2(a.AP, idx, a.ldAP, a.ap.ttend + k);
}

template <typename R>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? GD_STAGE_MINB : 2) k_stage(StageArgs<R> a) {
  typedef typename C2<R>::T V;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int L = a.L;
  V* TV = reinterpret_cast<V*>(smraw);  // [QC][L], index-major
  V* DV = TV + L * QC;
  V* Y = DV + L * QC;
  V* Y2 = Y + L * QC;
  V* LN = Y2 + L * QC;  // [QC]
  V* Y3 = LN + QC;      // [QC]
  const int4 it = a.items[blockIdx.x];
  const int n = it.x, m0 = it.y, cnt = it.z;
  const R lap = -(R)n * ((R)n + R(1));
  const R il = (n == 0) ? R(0) : R(1) / lap;
  const int s = a.stage;
  R* TDs = s == 0 ? a.TD0 : (s == 1 ? a.TD1 : a.TD2);
  auto TDr = [&](int r) -> const R* { return r == 0 ? a.TD0 : (r == 1 ? a.TD1 : a.TD2); };
  auto IDX = [&](int i) -> long { return a.moff[m0 + i] + (n - m0 - i); };

  for (int e = threadIdx.x; e < L * cnt; e += blockDim.x) {
    const int i = e / L, k = e - i * L;
    const long idx = IDX(i);
    TV[i * L + k] = ld2(a.S, idx, a.ldS, a.sc.tv + k);
    DV[i * L + k] = ld2(a.S, idx, a.ldS, a.sc.div + k);
  }
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) LN[i] = ld2(a.S, IDX(i), a.ldS, a.sc.lnps);
  __syncthreads();
  const int th = (int)blockDim.x >> 1;  // half of the CTA, whole warps
  if (!a.explicit_) {  // linear terms on the current state (run.f90:329-335)
    if ((int)threadIdx.x < th) {
      smem_matvec<R, V>(a.amhyb, TV, MvStore<V>{Y, L}, L, cnt, threadIdx.x, th);
    } else {
      smem_matvec<R, V>(a.bmhyb, DV, MvStore<V>{Y2, L}, L, cnt, threadIdx.x - th, th);
      smem_dot<R, V>(a.svhyb, DV, MvStore<V>{Y3, 1}, L, cnt, threadIdx.x - th, th);  // Y3[i]
    }
  }
  __syncthreads();
  const R dt = a.dt;
  // nonlinear tendencies, explicit part of the update
  for (int e = threadIdx.x; e < L * cnt; e += blockDim.x) {
    const int i = e / L, k = e - i * L;
    const long idx = IDX(i);
    V dvrt, ddiv, dtv;
    raw_tend(a, idx, k, lap, dvrt, ddiv, dtv);
    if (a.F) {  // IAU forcing, before the linear terms are taken out
      const V fv = ldg2(a.F, idx, a.ldS, a.sc.vrt + k), fd = ldg2(a.F, idx, a.ldS, a.sc.div + k),
              ft = ldg2(a.F, idx, a.ldS, a.sc.tv + k);
      dvrt.x += fv.x, dvrt.y += fv.y;
      ddiv.x += fd.x, ddiv.y += fd.y;
      dtv.x += ft.x, dtv.y += ft.y;
    }
    V ddl = vz<V>(), dtl = vz<V>();
    if (!a.explicit_) {
      ddl.x = -lap * (Y[i * L + k].x + a.tor[k] * LN[i].x);
      ddl.y = -lap * (Y[i * L + k].y + a.tor[k] * LN[i].y);
      dtl.x = -Y2[i * L + k].x;
      dtl.y = -Y2[i * L + k].y;
      ddiv.x -= ddl.x;
      ddiv.y -= ddl.y;
      dtv.x -= dtl.x;
      dtv.y -= dtl.y;
    }
    if (!a.final_) {  // the last stage's tendencies feed no later stage
      st2(TDs, idx, a.ldTD, a.tc.dvrt + k, dvrt);
      st2(TDs, idx, a.ldTD, a.tc.ddiv + k, ddiv);
      st2(TDs, idx, a.ldTD, a.tc.dtv + k, dtv);
      st2(TDs, idx, a.ldTD, a.tc.ddl + k, ddl);
      st2(TDs, idx, a.ldTD, a.tc.dtl + k, dtl);
    }
    V vr = ldg2(a.S0, idx, a.ldS, a.sc.vrt + k), dv = ldg2(a.S0, idx, a.ldS, a.sc.div + k),
      tv = ldg2(a.S0, idx, a.ldS, a.sc.tv + k);
    V svr = vz<V>(), sdv = vz<V>(), stv = vz<V>();
    for (int r = 0; r <= s; ++r) {
      V x_vr = dvrt, x_dv = ddiv, x_tv = dtv, x_dl = ddl, x_tl = dtl;
      if (r < s) {
        x_vr = ldg2(TDr(r), idx, a.ldTD, a.tc.dvrt + k);
        x_dv = ldg2(TDr(r), idx, a.ldTD, a.tc.ddiv + k);
        x_tv = ldg2(TDr(r), idx, a.ldTD, a.tc.dtv + k);
        x_dl = ldg2(TDr(r), idx, a.ldTD, a.tc.ddl + k);
        x_tl = ldg2(TDr(r), idx, a.ldTD, a.tc.dtl + k);
      }
      svr.x += a.ce[r] * x_vr.x;
      svr.y += a.ce[r] * x_vr.y;
      sdv.x += a.ce[r] * x_dv.x + a.ci[r] * x_dl.x;
      sdv.y += a.ce[r] * x_dv.y + a.ci[r] * x_dl.y;
      stv.x += a.ce[r] * x_tv.x + a.ci[r] * x_tl.x;
      stv.y += a.ce[r] * x_tv.y + a.ci[r] * x_tl.y;
    }
    vr.x += dt * svr.x;
    vr.y += dt * svr.y;
    dv.x += dt * sdv.x;
    dv.y += dt * sdv.y;
    tv.x += dt * stv.x;
    tv.y += dt * stv.y;
    R fd = R(1), ft = R(1);
    if (a.final_) {  // implicit hyperdiffusion / drag (run.f90:493-501)
      fd = R(1) - (a.disspec[idx] * a.diff_prof[k] - a.dmp_prof[k]) * dt;
      ft = R(1) - a.disspec[idx] * a.diff_prof[k] * dt;
      vr.x /= fd;
      vr.y /= fd;
    }
    st2(a.S, idx, a.ldS, a.sc.vrt + k, vr);
    V svv;
    svv.x = a.rerth * il * vr.x;
    svv.y = a.rerth * il * vr.y;
    st2(a.S, idx, a.ldS, a.sc.s + k, svv);
    DV[i * L + k] = dv;
    TV[i * L + k] = tv;
    for (int iq = 0; iq < a.nt; ++iq) {  // tracers, always explicit
      const int col = iq * L + k;
      V dq = ldg2(a.AP, idx, a.ldAP, a.ap.qtend + col);
      if (a.F) {
        const V fq = ldg2(a.F, idx, a.ldS, a.sc.trc + col);
        dq.x += fq.x, dq.y += fq.y;
      }
      if (!a.final_) st2(TDs, idx, a.ldTD, a.tc.dtrc + col, dq);
      V q = ldg2(a.S0, idx, a.ldS, a.sc.trc + col);
      V sq = vz<V>();
      for (int r = 0; r <= s; ++r) {
        V x = (r < s) ? ldg2(TDr(r), idx, a.ldTD, a.tc.dtrc + col) : dq;
        sq.x += a.ce[r] * x.x;
        sq.y += a.ce[r] * x.y;
      }
      q.x += dt * sq.x;
      q.y += dt * sq.y;
      if (a.final_) {
        q.x /= ft;
        q.y /= ft;
      }
      st2(a.S, idx, a.ldS, a.sc.trc + col, q);
    }
  }
  __syncthreads();  // LN (current ln ps) is read above and replaced below
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
    const long idx = IDX(i);
    V dl = ldg2(a.AP, idx, a.ldAP, a.ap.dlnps);
    if (a.F) {
      const V fl = ldg2(a.F, idx, a.ldS, a.sc.lnps);
      dl.x += fl.x, dl.y += fl.y;
    }
    V dpl = vz<V>();
    if (!a.explicit_) {
      dpl.x = -Y3[i].x;
      dpl.y = -Y3[i].y;
      dl.x -= dpl.x;
      dl.y -= dpl.y;
    }
    if (!a.final_) {
      st2(TDs, idx, a.ldTD, a.tc.dlnps, dl);
      st2(TDs, idx, a.ldTD, a.tc.dpl, dpl);
    }
    V ln = ldg2(a.S0, idx, a.ldS, a.sc.lnps);
    V sl = vz<V>();
    for (int r = 0; r <= s; ++r) {
      V x = dl, xp = dpl;
      if (r < s) {
        x = ldg2(TDr(r), idx, a.ldTD, a.tc.dlnps);
        xp = ldg2(TDr(r), idx, a.ldTD, a.tc.dpl);
      }
      sl.x += a.ce[r] * x.x + a.ci[r] * xp.x;
      sl.y += a.ce[r] * x.y + a.ci[r] * xp.y;
    }
    ln.x += dt * sl.x;
    ln.y += dt * sl.y;
    LN[i] = ln;
  }
  __syncthreads();
  if (!a.explicit_ && a.cimp != R(0)) {  // implicit solve for divergence
    const R c = a.cimp;
    // right-hand side r = D - c lap dt (A T + tor ln ps), formed in the
    // epilogue of the A T product
    smem_matvec<R, V>(
        a.amhyb, TV,
        [&](int i, int k, V y) {
          V r;
          r.x = DV[i * L + k].x - c * lap * dt * (y.x + a.tor[k] * LN[i].x);
          r.y = DV[i * L + k].y - c * lap * dt * (y.y + a.tor[k] * LN[i].y);
          Y2[i * L + k] = r;
        },
        L, cnt, threadIdx.x, blockDim.x);
    __syncthreads();
    const R* D = a.dhyb + ((long)s * (a.T + 1) + n) * L * L;
    smem_matvec<R, V>(D, Y2, MvStore<V>{DV, L}, L, cnt, threadIdx.x, blockDim.x);
    __syncthreads();
    // back-substitution into T and ln ps in the epilogues of B D and sv . D
    if ((int)threadIdx.x < th)
      smem_matvec<R, V>(
          a.bmhyb, DV,
          [&](int i, int k, V y) {
            TV[i * L + k].x -= c * dt * y.x;
            TV[i * L + k].y -= c * dt * y.y;
          },
          L, cnt, threadIdx.x, th);
    else
      smem_dot<R, V>(
          a.svhyb, DV,
          [&](int i, int, V y) {
            LN[i].x -= c * dt * y.x;
            LN[i].y -= c * dt * y.y;
          },
          L, cnt, threadIdx.x - th, th);
    __syncthreads();
  }
  for (int e = threadIdx.x; e < L * cnt; e += blockDim.x) {
    const int i = e / L, k = e - i * L;
    const long idx = IDX(i);
    V dv = DV[i * L + k], tv = TV[i * L + k];
    if (a.final_) {
      const R fd = R(1) - (a.disspec[idx] * a.diff_prof[k] - a.dmp_prof[k]) * dt;
      const R ft = R(1) - a.disspec[idx] * a.diff_prof[k] * dt;
      dv.x /= fd;
      dv.y /= fd;
      tv.x /= ft;
      tv.y /= ft;
    }
    st2(a.S, idx, a.ldS, a.sc.div + k, dv);
    st2(a.S, idx, a.ldS, a.sc.tv + k, tv);
    V cc;
    cc.x = a.rerth * il * dv.x;
    cc.y = a.rerth * il * dv.y;
    st2(a.S, idx, a.ldS, a.sc.c + k, cc);
  }
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) st2(a.S, IDX(i), a.ldS, a.sc.lnps, LN[i]);
}

template <typename R>
void launch_stage(const StageArgs<R>& a, cudaStream_t s) {
  size_t sm = (4 * (size_t)a.L * QC + 2 * QC) * sizeof(typename C2<R>::T);
  static bool attr = false;
  if (!attr) {
    GD_CUDA(cudaFuncSetAttribute(k_stage<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr = true;
  }
  k_stage<R><<<a.nitems, 256, sm, s>>>(a);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_stage<double>(const StageArgs<double>&, cudaStream_t);
template void launch_stage<float>(const StageArgs<float>&, cudaStream_t);

template <typename R>
__global__ void k_assemble(StageArgs<R> a, R* TD, int nlm) {
  typedef typename C2<R>::T V;
  const long total = (long)nlm * a.L;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long idx = e / a.L;
    const int k = (int)(e - idx * a.L);
    // degree of idx: find m with moff[m] <= idx < moff[m+1]
    int lo = 0, hi = a.T;
    while (lo < hi) {
      int mid = (lo + hi + 1) / 2;
      if (a.moff[mid] <= idx) lo = mid;
      else hi = mid - 1;
    }
    const int n = lo + (int)(idx - a.moff[lo]);
    const R lap = -(R)n * ((R)n + R(1));
    V dvrt, ddiv, dtv;
    raw_tend(a, idx, k, lap, dvrt, ddiv, dtv);
    st2(TD, idx, a.ldTD, a.tc.dvrt + k, dvrt);
    st2(TD, idx, a.ldTD, a.tc.ddiv + k, ddiv);
    st2(TD, idx, a.ldTD, a.tc.dtv + k, dtv);
    for (int iq = 0; iq < a.nt; ++iq)
      st2(TD, idx, a.ldTD, a.tc.dtrc + iq * a.L + k, ldg2(a.AP, idx, a.ldAP, a.ap.qtend + iq * a.L + k));
    if (k == 0) st2(TD, idx, a.ldTD, a.tc.dlnps, ldg2(a.AP, idx, a.ldAP, a.ap.dlnps));
  }
}
template <typename R>
void launch_assemble(const StageArgs<R>& a, R* TD, cudaStream_t s) {
  long nlm = (long)(a.T + 1) * (a.T + 2) / 2;
  k_assemble<R><<<std::min(ceil_div(nlm * a.L, 256), 4096), 256, 0, s>>>(a, TD, (int)nlm);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_assemble<double>(const StageArgs<double>&, double*, cudaStream_t);
template void launch_assemble<float>(const StageArgs<float>&, float*, cudaStream_t);

template <typename R>
__global__ void k_phys_update(R* S, long ldS, SpecCols sc, int L, int nt, int nlm, const R* AP, long ldAP,
                              int massfix, int heldsuarez, R dt, const R* lapv, R rerth) {
  typedef typename C2<R>::T V;
  const long total = (long)nlm * (L + 1);
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long idx = e / (L + 1);
    const int k = (int)(e - idx * (L + 1));
    const R lap = lapv[idx];
    const R il = (idx == 0) ? R(0) : R(1) / lap;
    if (k == L) {  // ln(ps): dry-mass fixer (dyn_run.f90:633, run.f90:538)
      if (massfix) {
        V ln = ld2(S, idx, ldS, sc.lnps);
        V ws = ld2(AP, idx, ldAP, 3 * L);
        V d;
        d.x = (ws.x - ln.x) / dt;
        d.y = (ws.y - ln.y) / dt;
        ln.x = ln.x + dt * d.x;
        ln.y = ln.y + dt * d.y;
        st2(S, idx, ldS, sc.lnps, ln);
      }
      continue;
    }
    V vr = ld2(S, idx, ldS, sc.vrt + k), dv = ld2(S, idx, ldS, sc.div + k), tv = ld2(S, idx, ldS, sc.tv + k);
    if (heldsuarez) {
      V ft = ld2(AP, idx, ldAP, k), fv = ld2(AP, idx, ldAP, L + k), fd = ld2(AP, idx, ldAP, 2 * L + k);
      vr.x += dt * fv.x;
      vr.y += dt * fv.y;
      dv.x += dt * fd.x;
      dv.y += dt * fd.y;
      tv.x += dt * ft.x;
      tv.y += dt * ft.y;
    }
    st2(S, idx, ldS, sc.vrt + k, vr);
    st2(S, idx, ldS, sc.div + k, dv);
    st2(S, idx, ldS, sc.tv + k, tv);
    V s_, c_;
    s_.x = rerth * il * vr.x;
    s_.y = rerth * il * vr.y;
    c_.x = rerth * il * dv.x;
    c_.y = rerth * il * dv.y;
    st2(S, idx, ldS, sc.s + k, s_);
    st2(S, idx, ldS, sc.c + k, c_);
  }
}
template <typename R>
void launch_phys_update(R* S, long ldS, const SpecCols& sc, int L, int nt, int nlm, const R* AP, long ldAP,
                        int massfix, int heldsuarez, R dt, const R* lapv, R rerth, cudaStream_t s) {
  long total = (long)nlm * (L + 1);
  k_phys_update<R><<<std::min(ceil_div(total, 256), 8192), 256, 0, s>>>(S, ldS, sc, L, nt, nlm, AP, ldAP, massfix,
                                                                        heldsuarez, dt, lapv, rerth);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_phys_update<double>(double*, long, const SpecCols&, int, int, int, const double*, long, int,
                                         int, double, const double*, double, cudaStream_t);
template void launch_phys_update<float>(float*, long, const SpecCols&, int, int, int, const float*, long, int, int,
                                        float, const float*, float, cudaStream_t);

template <typename R>
__global__ void k_simple_update(R* S, long ldS, SpecCols sc, int L, int nlm, const R* AP, long ldAP, const R* AH,
                                long ldAH, int massfix, int hasq, R dt, R ainv, const R* lapv, R rerth) {
  typedef typename C2<R>::T V;
  const long total = (long)nlm * (L + 1);
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long idx = e / (L + 1);
    const int k = (int)(e - idx * (L + 1));
    if (k == L) {  // ln(ps): dry-mass fixer (dyn_run.f90:633, run.f90:538)
      if (massfix) {
        V ln = ld2(S, idx, ldS, sc.lnps);
        V ws = ld2(AP, idx, ldAP, 2 * L);
        V d;
        d.x = (ws.x - ln.x) / dt;
        d.y = (ws.y - ln.y) / dt;
        ln.x = ln.x + dt * d.x;
        ln.y = ln.y + dt * d.y;
        st2(S, idx, ldS, sc.lnps, ln);
      }
      continue;
    }
    const R lap = lapv[idx];
    const R il = (idx == 0) ? R(0) : R(1) / lap;
    V tv = ld2(S, idx, ldS, sc.tv + k);
    V vr = ld2(S, idx, ldS, sc.vrt + k), dv = ld2(S, idx, ldS, sc.div + k);
    const V at = ld2(AP, idx, ldAP, k);
    const V pv = ld2(AP, idx, ldAP, 2 * L + 1 + k), pd = ld2(AP, idx, ldAP, 3 * L + 1 + k);
    const V hv = ld2(AH, idx, ldAH, k), hd = ld2(AH, idx, ldAH, L + k);
    tv.x += dt * (at.x / dt);
    tv.y += dt * (at.y / dt);
    if (hasq) {  // the first tracer's increment (the learned closure has none)
      V q = ld2(S, idx, ldS, sc.trc + k);
      const V aq = ld2(AP, idx, ldAP, L + k);
      q.x += dt * (aq.x / dt);
      q.y += dt * (aq.y / dt);
      st2(S, idx, ldS, sc.trc + k, q);
    }
    vr.x += dt * ((pv.x + hv.x) * ainv / dt);
    vr.y += dt * ((pv.y + hv.y) * ainv / dt);
    dv.x += dt * ((pd.x + hd.x) * ainv / dt);
    dv.y += dt * ((pd.y + hd.y) * ainv / dt);
    st2(S, idx, ldS, sc.tv + k, tv);
    st2(S, idx, ldS, sc.vrt + k, vr);
    st2(S, idx, ldS, sc.div + k, dv);
    V s_, c_;
    s_.x = rerth * il * vr.x;
    s_.y = rerth * il * vr.y;
    c_.x = rerth * il * dv.x;
    c_.y = rerth * il * dv.y;
    st2(S, idx, ldS, sc.s + k, s_);
    st2(S, idx, ldS, sc.c + k, c_);
  }
}
template <typename R>
void launch_simple_update(R* S, long ldS, const SpecCols& sc, int L, int nlm, const R* AP, long ldAP, const R* AH,
                          long ldAH, int massfix, int hasq, R dt, R ainv, const R* lapv, R rerth, cudaStream_t s) {
  long total = (long)nlm * (L + 1);
  k_simple_update<R><<<std::min(ceil_div(total, 256), 8192), 256, 0, s>>>(S, ldS, sc, L, nlm, AP, ldAP, AH, ldAH,
                                                                         massfix, hasq, dt, ainv, lapv, rerth);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_simple_update<double>(double*, long, const SpecCols&, int, int, const double*, long,
                                           const double*, long, int, int, double, double, const double*, double,
                                           cudaStream_t);
template void launch_simple_update<float>(float*, long, const SpecCols&, int, int, const float*, long, const float*,
                                          long, int, int, float, float, const float*, float, cudaStream_t);

// prognostic column j of the state layout: the (3+nt) L columns from vrt, then lnps
__device__ __forceinline__ int prog_col(const SpecCols& sc, int ncs, int j) { return j < ncs ? sc.vrt + j : sc.lnps; }

template <typename R>
__global__ void k_iau_forcing(R* F, const R* inc, long ldS, SpecCols sc, int ncs, int nlm, int ia, double ca, int ib,
                              double cb, double dtiau) {
  const long per = (long)nlm * ldS;
  const long total = (long)nlm * (ncs + 1);
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long idx = e / (ncs + 1);
    const int col = prog_col(sc, ncs, (int)(e - idx * (ncs + 1)));
    typename C2<R>::T f;
    if (ca == 0.0 && cb == 0.0) {
      f.x = f.y = R(0);
    } else {
      const typename C2<R>::T x = ld2(inc + ia * per, idx, ldS, col), y = ld2(inc + ib * per, idx, ldS, col);
      f.x = (R(ca) * x.x + R(cb) * y.x) / R(dtiau);
      f.y = (R(ca) * x.y + R(cb) * y.y) / R(dtiau);
    }
    st2(F, idx, ldS, col, f);
  }
}
template <typename R>
void launch_iau_forcing(R* F, const R* inc, long ldS, const SpecCols& sc, int ncs, int nlm, int ia, double ca,
                        int ib, double cb, double dtiau, cudaStream_t s) {
  const long total = (long)nlm * (ncs + 1);
  k_iau_forcing<R><<<std::min(ceil_div(total, 256), 8192), 256, 0, s>>>(F, inc, ldS, sc, ncs, nlm, ia, ca, ib, cb,
                                                                        dtiau);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_iau_forcing<double>(double*, const double*, long, const SpecCols&, int, int, int, double, int,
                                         double, double, cudaStream_t);
template void launch_iau_forcing<float>(float*, const float*, long, const SpecCols&, int, int, int, double, int,
                                        double, double, cudaStream_t);

template <typename R>
__global__ void k_dfi_acc(double* acc, const R* S, long ldS, SpecCols sc, int ncs, int nlm, double w, int first) {
  const long total = (long)nlm * (ncs + 1);
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long idx = e / (ncs + 1);
    const int j = (int)(e - idx * (ncs + 1));
    const typename C2<R>::T x = ld2(S, idx, ldS, prog_col(sc, ncs, j));
    double* o = acc + 2 * e;
    if (first) {
      o[0] = w * (double)x.x;
      o[1] = w * (double)x.y;
    } else {
      o[0] = o[0] + w * (double)x.x;
      o[1] = o[1] + w * (double)x.y;
    }
  }
}
template <typename R>
void launch_dfi_acc(double* acc, const R* S, long ldS, const SpecCols& sc, int ncs, int nlm, double w, int first,
                    cudaStream_t s) {
  const long total = (long)nlm * (ncs + 1);
  k_dfi_acc<R><<<std::min(ceil_div(total, 256), 8192), 256, 0, s>>>(acc, S, ldS, sc, ncs, nlm, w, first);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_dfi_acc<double>(double*, const double*, long, const SpecCols&, int, int, double, int,
                                     cudaStream_t);
template void launch_dfi_acc<float>(double*, const float*, long, const SpecCols&, int, int, double, int, cudaStream_t);

template <typename R>
__global__ void k_dfi_set(R* S, long ldS, SpecCols sc, int ncs, int nlm, const double* acc) {
  const long total = (long)nlm * (ncs + 1);
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long idx = e / (ncs + 1);
    const int j = (int)(e - idx * (ncs + 1));
    st2(S, idx, ldS, prog_col(sc, ncs, j), mk2<R>((R)acc[2 * e], (R)acc[2 * e + 1]));
  }
}
template <typename R>
void launch_dfi_set(R* S, long ldS, const SpecCols& sc, int ncs, int nlm, const double* acc, cudaStream_t s) {
  const long total = (long)nlm * (ncs + 1);
  k_dfi_set<R><<<std::min(ceil_div(total, 256), 8192), 256, 0, s>>>(S, ldS, sc, ncs, nlm, acc);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_dfi_set<double>(double*, long, const SpecCols&, int, int, const double*, cudaStream_t);
template void launch_dfi_set<float>(float*, long, const SpecCols&, int, int, const double*, cudaStream_t);

template <typename R>
__global__ void k_sc(R* S, long ldS, SpecCols sc, int L, int nlm, const R* lapv, R rerth) {
  typedef typename C2<R>::T V;
  const long total = (long)nlm * L;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long idx = e / L;
    const int k = (int)(e - idx * L);
    const R il = (idx == 0) ? R(0) : R(1) / lapv[idx];
    V vr = ld2(S, idx, ldS, sc.vrt + k), dv = ld2(S, idx, ldS, sc.div + k);
    V s_, c_;
    s_.x = rerth * il * vr.x;
    s_.y = rerth * il * vr.y;
    c_.x = rerth * il * dv.x;
    c_.y = rerth * il * dv.y;
    st2(S, idx, ldS, sc.s + k, s_);
    st2(S, idx, ldS, sc.c + k, c_);
  }
}
template <typename R>
void launch_sc(R* S, long ldS, const SpecCols& sc, int L, int nlm, const R* lapv, R rerth, cudaStream_t s) {
  long total = (long)nlm * L;
  k_sc<R><<<std::min(ceil_div(total, 256), 8192), 256, 0, s>>>(S, ldS, sc, L, nlm, lapv, rerth);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_sc<double>(double*, long, const SpecCols&, int, int, const double*, double, cudaStream_t);
template void launch_sc<float>(float*, long, const SpecCols&, int, int, const float*, float, cudaStream_t);

// ---------------------------------------------------------------- layout --
// Reference layout H[nb][nlm] complex (H = double, or float for the
// single-precision host entry points) <-> the internal [nlm][ld] columns.
template <typename H>
__device__ __forceinline__ double2 ld_ref(const H* p) {
  if constexpr (sizeof(H) == 8) {
    return *reinterpret_cast<const double2*>(p);
  } else {
    const float2 v = *reinterpret_cast<const float2*>(p);
    return make_double2((double)v.x, (double)v.y);
  }
}
template <typename H>
__device__ __forceinline__ void st_ref(H* p, double2 v) {
  if constexpr (sizeof(H) == 8) {
    *reinterpret_cast<double2*>(p) = v;
  } else {
    *reinterpret_cast<float2*>(p) = make_float2((float)v.x, (float)v.y);
  }
}
template <typename H, typename R>
__global__ void k_ref2int(const H* __restrict__ ref, int nb, int nlm, R* __restrict__ dst, long ld, int col0) {
  __shared__ double2 tile[32][33];
  const int q0 = blockIdx.x * 32, b0 = blockIdx.y * 32;
  for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
    int b = b0 + yy, q = q0 + threadIdx.x;
    if (b < nb && q < nlm) tile[yy][threadIdx.x] = ld_ref<H>(ref + 2 * ((long)b * nlm + q));
  }
  __syncthreads();
  for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
    int q = q0 + yy, b = b0 + threadIdx.x;
    if (b < nb && q < nlm) {
      double2 v = tile[threadIdx.x][yy];
      dst[(long)q * ld + 2 * (col0 + b)] = (R)v.x;
      dst[(long)q * ld + 2 * (col0 + b) + 1] = (R)v.y;
    }
  }
}
template <typename R, typename H>
__global__ void k_int2ref(const R* __restrict__ src, long ld, int col0, int nb, int nlm, H* __restrict__ ref) {
  __shared__ double2 tile[32][33];
  const int q0 = blockIdx.x * 32, b0 = blockIdx.y * 32;
  for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
    int q = q0 + yy, b = b0 + threadIdx.x;
    if (b < nb && q < nlm)
      tile[yy][threadIdx.x] = make_double2((double)src[(long)q * ld + 2 * (col0 + b)],
                                           (double)src[(long)q * ld + 2 * (col0 + b) + 1]);
  }
  __syncthreads();
  for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
    int b = b0 + yy, q = q0 + threadIdx.x;
    if (b < nb && q < nlm) st_ref<H>(ref + 2 * ((long)b * nlm + q), tile[threadIdx.x][yy]);
  }
}
template <typename R, typename H>
void launch_ref2int(const H* ref, int nb, int nlm, R* dst, long ld, int col0, cudaStream_t s) {
  if (nb <= 0) return;
  dim3 g(ceil_div(nlm, 32), ceil_div(nb, 32)), b(32, 8);
  k_ref2int<H, R><<<g, b, 0, s>>>(ref, nb, nlm, dst, ld, col0);
  count_launch();
  GD_LAUNCH_CHECK();
}
template <typename R, typename H>
void launch_int2ref(const R* src, long ld, int col0, int nb, int nlm, H* ref, cudaStream_t s) {
  if (nb <= 0) return;
  dim3 g(ceil_div(nlm, 32), ceil_div(nb, 32)), b(32, 8);
  k_int2ref<R, H><<<g, b, 0, s>>>(src, ld, col0, nb, nlm, ref);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_ref2int<double, double>(const double*, int, int, double*, long, int, cudaStream_t);
template void launch_ref2int<float, double>(const double*, int, int, float*, long, int, cudaStream_t);
template void launch_ref2int<double, float>(const float*, int, int, double*, long, int, cudaStream_t);
template void launch_ref2int<float, float>(const float*, int, int, float*, long, int, cudaStream_t);
template void launch_int2ref<double, double>(const double*, long, int, int, int, double*, cudaStream_t);
template void launch_int2ref<float, double>(const float*, long, int, int, int, double*, cudaStream_t);
template void launch_int2ref<double, float>(const double*, long, int, int, int, float*, cudaStream_t);
template void launch_int2ref<float, float>(const float*, long, int, int, int, float*, cudaStream_t);

template <typename R>
__global__ void k_combine(const R* X, long ldX, int cx, const R* Y, long ldY, int cy, R* O, long ldO, int co, int nb,
                          int nlm, R scale) {
  const long total = (long)nlm * nb;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long q = e / nb;
    const int b = (int)(e - q * nb);
    for (int c = 0; c < 2; ++c)
      O[q * ldO + 2 * (co + b) + c] = scale * (X[q * ldX + 2 * (cx + b) + c] + Y[q * ldY + 2 * (cy + b) + c]);
  }
}
template <typename R>
void launch_combine(const R* X, long ldX, int cx, const R* Y, long ldY, int cy, R* O, long ldO, int co, int nb,
                    int nlm, R scale, cudaStream_t s) {
  long total = (long)nlm * nb;
  k_combine<R><<<std::min(ceil_div(total, 256), 8192), 256, 0, s>>>(X, ldX, cx, Y, ldY, cy, O, ldO, co, nb, nlm,
                                                                    scale);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_combine<double>(const double*, long, int, const double*, long, int, double*, long, int, int,
                                     int, double, cudaStream_t);
template void launch_combine<float>(const float*, long, int, const float*, long, int, float*, long, int, int, int,
                                    float, cudaStream_t);

template <typename R>
__global__ void k_scale_cols(R* X, long ldX, int c0, int nb, int nlm, const R* f, R scale) {
  const long total = (long)nlm * nb;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long q = e / nb;
    const int b = (int)(e - q * nb);
    const R g = f[q] * scale;
    X[q * ldX + 2 * (c0 + b)] *= g;
    X[q * ldX + 2 * (c0 + b) + 1] *= g;
  }
}
template <typename R>
void launch_scale_cols(R* X, long ldX, int c0, int nb, int nlm, const R* f, R scale, cudaStream_t s) {
  long total = (long)nlm * nb;
  k_scale_cols<R><<<std::min(ceil_div(total, 256), 8192), 256, 0, s>>>(X, ldX, c0, nb, nlm, f, scale);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_scale_cols<double>(double*, long, int, int, int, const double*, double, cudaStream_t);
template void launch_scale_cols<float>(float*, long, int, int, int, const float*, float, cudaStream_t);

template <typename R>
__global__ void k_to_double(const R* src, double* dst, long n) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}
template <typename R>
void launch_to_double(const R* src, double* dst, long n, cudaStream_t s) {
  k_to_double<R><<<std::min(ceil_div(n, 256), 8192), 256, 0, s>>>(src, dst, n);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_to_double<double>(const double*, double*, long, cudaStream_t);
template void launch_to_double<float>(const float*, double*, long, cudaStream_t);

// LU with partial pivoting, then inv(A) column by column, FP64, one CTA per
// matrix held in shared memory (role of dgetrf/dgetri, semimp_data.f90:248).
__global__ void k_inverse(double* mats, int L) {
  extern __shared__ double smd[];
  double* A = smd;                        // [L][L]
  int* piv = reinterpret_cast<int*>(A + (long)L * L);
  __shared__ int pk;
  double* g = mats + (long)blockIdx.x * L * L;
  for (int e = threadIdx.x; e < L * L; e += blockDim.x) A[e] = g[e];
  __syncthreads();
  for (int k = 0; k < L; ++k) {
    if (threadIdx.x == 0) {
      int p = k;
      for (int i = k + 1; i < L; ++i)
        if (fabs(A[i * L + k]) > fabs(A[p * L + k])) p = i;
      pk = p;
      piv[k] = p;
    }
    __syncthreads();
    const int p = pk;
    if (p != k)
      for (int jj = threadIdx.x; jj < L; jj += blockDim.x) {
        double t = A[k * L + jj];
        A[k * L + jj] = A[p * L + jj];
        A[p * L + jj] = t;
      }
    __syncthreads();
    const double d = A[k * L + k];
    for (int i = k + 1 + threadIdx.x; i < L; i += blockDim.x) A[i * L + k] /= d;
    __syncthreads();
    for (int e = threadIdx.x; e < (L - k - 1) * (L - k - 1); e += blockDim.x) {
      const int i = k + 1 + e / (L - k - 1), jj = k + 1 + e % (L - k - 1);
      A[i * L + jj] -= A[i * L + k] * A[k * L + jj];
    }
    __syncthreads();
  }
  // column c of the inverse: solve A x = e_c (row permutation, L, U)
  for (int c = threadIdx.x; c < L; c += blockDim.x) {
    double x[128];
    for (int i = 0; i < L; ++i) x[i] = (i == c) ? 1.0 : 0.0;
    for (int k = 0; k < L; ++k) {
      double t = x[k];
      x[k] = x[piv[k]];
      x[piv[k]] = t;
    }
    for (int i = 0; i < L; ++i)
      for (int k = 0; k < i; ++k) x[i] -= A[i * L + k] * x[k];
    for (int i = L - 1; i >= 0; --i) {
      for (int k = i + 1; k < L; ++k) x[i] -= A[i * L + k] * x[k];
      x[i] /= A[i * L + i];
    }
    for (int i = 0; i < L; ++i) g[(long)i * L + c] = x[i];
  }
}
void launch_batched_inverse(double* mats, int nmat, int L, cudaStream_t s) {
  if (L > 128) throw std::runtime_error("nlev too large for the batched inverse");
  size_t sm = (size_t)L * L * sizeof(double) + L * sizeof(int) + 16;
  GD_CUDA(cudaFuncSetAttribute(k_inverse, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  k_inverse<<<nmat, 128, sm, s>>>(mats, L);
  count_launch();
  GD_LAUNCH_CHECK();
}

}  // namespace gd

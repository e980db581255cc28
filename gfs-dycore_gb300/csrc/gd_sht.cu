// gd_sht.cu -- Gaussian-grid spherical harmonic transform kernels for
// sm_103a: FP64 grid/table construction, per-order Legendre GEMMs with the
// even/odd hemispheric split, and shared-memory Stockham FFTs along longitude.
//
// These take over the roles SHTns (+FFTW) plays behind src/shtns.f90 of
// jswhit/gfs-dycore: shtns_cos_array / shtns_gauss_wts (shtns.f90:125-126),
// the SHT_GAUSS_FLY Legendre recurrences, shtns_sh_to_spat /
// shtns_spat_to_sh (shtns.f90:195,199,225,229) and the vector forms
// (shtns.f90:261,270,303,308,341,348).  Convention: orthonormal harmonics
// without Condon-Shortley phase (shtns.f90:110), latitudes north to south.
#include <cstdlib>
#include <type_traits>
#include <vector>

#include "gd_kernels.h"

namespace gd {

long long g_launches = 0;

// ------------------------------------------------------------------ init --
// Gauss-Legendre nodes (north to south) and weights by Newton iteration on
// P_nlat, FP64.  One thread per northern node.
__global__ void k_gauss(int N, double* mu, double* w) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N / 2) return;
  double x = cos(3.14159265358979323846 * (j + 0.75) / (N + 0.5));
  double dp = 0.0;
  for (int it = 0; it < 100; ++it) {
    double p0 = 1.0, p1 = x;
    for (int k = 1; k < N; ++k) {
      double p2 = ((2 * k + 1) * x * p1 - k * p0) / (k + 1);
      p0 = p1;
      p1 = p2;
    }
    dp = N * (x * p1 - p0) / (x * x - 1.0);
    double dx = p1 / dp;
    x -= dx;
    if (fabs(dx) <= 1e-16) break;
  }
  double p0 = 1.0, p1 = x;
  for (int k = 1; k < N; ++k) {
    double p2 = ((2 * k + 1) * x * p1 - k * p0) / (k + 1);
    p0 = p1;
    p1 = p2;
  }
  dp = N * (x * p1 - p0) / (x * x - 1.0);
  double wj = 2.0 / ((1.0 - x) * (1.0 + x) * dp * dp);
  mu[j] = x;
  mu[N - 1 - j] = -x;
  w[j] = wj;
  w[N - 1 - j] = wj;
}

void launch_gauss(int nlat, double* mu, double* w, cudaStream_t s) {
  k_gauss<<<ceil_div(nlat / 2, 64), 64, 0, s>>>(nlat, mu, w);
  count_launch();
  GD_LAUNCH_CHECK();
}

// Orthonormal associated Legendre functions P_n^m(mu_j)/sqrt(2 pi) and their
// latitude derivative, by the three-term recurrence in n with exact binary
// rescaling (ldexp) so high orders near the poles neither underflow nor lose
// the recurrence.  FP64; one thread per (m, j).
__global__ void k_legendre(int T, int nh, const double* mu, const long* toff, double* P, double* H) {
  long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)(T + 1) * nh) return;
  const int m = (int)(t / nh), j = (int)(t % nh);
  const int K = T - m + 1;
  const double x = mu[j];
  const double s = sqrt((1.0 - x) * (1.0 + x));
  const double inv_s2pi = 0.39894228040143267794;  // 1/sqrt(2 pi)
  const int SC = 600;
  double v = 0.70710678118654752440;
  int c = 0;
  for (int k = 1; k <= m; ++k) {
    v *= sqrt((2.0 * k + 1.0) / (2.0 * k)) * s;
    if (fabs(v) < ldexp(1.0, -SC)) {
      v = ldexp(v, SC);
      ++c;
    }
  }
  double pm1 = 0.0, p = v;
  double* Pr = P + toff[m] + (long)j * K;
  double* Hr = H + toff[m] + (long)j * K;
  for (int n = m; n <= T; ++n) {
    if (n == m + 1) {
      double pn = sqrt(2.0 * m + 3.0) * x * p;
      pm1 = p;
      p = pn;
    } else if (n > m + 1) {
      double a = sqrt((4.0 * n * n - 1.0) / ((double)n * n - (double)m * m));
      double b = sqrt(((n - 1.0) * (n - 1.0) - (double)m * m) / (4.0 * (n - 1.0) * (n - 1.0) - 1.0));
      double pn = a * (x * p - b * pm1);
      pm1 = p;
      p = pn;
    }
    if (c > 0 && fabs(p) > ldexp(1.0, 300)) {
      p = ldexp(p, -SC);
      pm1 = ldexp(pm1, -SC);
      --c;
    }
    double cnm = (n > m) ? sqrt(((double)n * n - (double)m * m) * (2.0 * n + 1.0) / (2.0 * n - 1.0)) : 0.0;
    double h = (-n * x * p + cnm * pm1) / s;
    double pv = (c == 0) ? p : ldexp(p, -SC * c);
    double hv = (c == 0) ? h : ldexp(h, -SC * c);
    Pr[n - m] = pv * inv_s2pi;
    Hr[n - m] = hv * inv_s2pi;
  }
}

void launch_legendre_tables(int T, int nh, const double* mu, const long* toff, double* P64, double* H64,
                            cudaStream_t s) {
  long n = (long)(T + 1) * nh;
  k_legendre<<<ceil_div(n, 128), 128, 0, s>>>(T, nh, mu, toff, P64, H64);
  count_launch();
  GD_LAUNCH_CHECK();
}

template <typename R>
__global__ void k_convert(const double* src, R* dst, long n) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    dst[i] = (R)src[i];
}
template <typename R>
void launch_convert(const double* src, R* dst, long n, cudaStream_t s) {
  int blocks = (int)std::min<long>(ceil_div(n, 256), 152L * 16);
  k_convert<R><<<blocks, 256, 0, s>>>(src, dst, n);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_convert<double>(const double*, double*, long, cudaStream_t);
template void launch_convert<float>(const double*, float*, long, cudaStream_t);

// dst[r][c] = src[r][c] for r < rows, c < cols (row pitches lds, ldd), with
// the type change round-to-nearest; the staging copies of the FP64-state
// split-precision modes around the FP32 tensor-core Legendre GEMMs.  Rows
// hold real/imaginary pairs (even cols and pitches, pair-aligned bases), so
// each thread moves whole pairs; a CTA walks rows with a stride over the grid.
constexpr int kConvChunk = 1024;  // pairs per tile of the staging conversions
template <typename S, typename D>
__global__ void __launch_bounds__(256) k_convert2d(const S* __restrict__ src, long lds, D* __restrict__ dst,
                                                   long ldd, long rows, int cols) {
  typedef typename C2<S>::T VS;
  typedef typename C2<D>::T VD;
  const int np = cols >> 1, nchunk = (np + kConvChunk - 1) / kConvChunk;
  for (long t = blockIdx.x; t < rows * nchunk; t += gridDim.x) {  // tiles of (row, chunk of kConvChunk pairs)
    const long r = t / nchunk;
    const int q0 = (int)(t - r * nchunk) * kConvChunk, q1 = min(np, q0 + kConvChunk);
    const VS* sp = reinterpret_cast<const VS*>(src + r * lds);
    VD* dp = reinterpret_cast<VD*>(dst + r * ldd);
    for (int q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
      const VS v = sp[q];
      VD w;
      w.x = (D)v.x;
      w.y = (D)v.y;
      dp[q] = w;
    }
  }
}
template <typename S, typename D>
void launch_convert2d(const S* src, long lds, D* dst, long ldd, long rows, int cols, cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return;
  if ((cols | lds | ldd) & 1) throw CudaError("launch_convert2d: columns and pitches must be even");
  const long tiles = rows * (((cols >> 1) + kConvChunk - 1) / kConvChunk);
  const int blocks = (int)std::min<long>(tiles, 152L * 32);
  k_convert2d<S, D><<<blocks, 256, 0, s>>>(src, lds, dst, ldd, rows, cols);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_convert2d<double, float>(const double*, long, float*, long, long, int, cudaStream_t);
template void launch_convert2d<float, double>(const float*, long, double*, long, long, int, cudaStream_t);

// dst[r][c] = sum over q < nseg of src[q seg_stride + r lds + c], summed in
// FP64 in the order q = 0, 1, ...: the K-segmented tensor-core analysis's
// partial sums of the FP64-state modes (pairs per thread, rows per CTA)
__global__ void __launch_bounds__(256) k_sumconvert(const float* __restrict__ src, long lds, long seg_stride,
                                                    int nseg, double* __restrict__ dst, long ldd, long rows,
                                                    int cols) {
  const int np = cols >> 1, nchunk = (np + kConvChunk - 1) / kConvChunk;
  for (long t = blockIdx.x; t < rows * nchunk; t += gridDim.x) {
    const long r = t / nchunk;
    const int q0 = (int)(t - r * nchunk) * kConvChunk, q1 = min(np, q0 + kConvChunk);
    const float* sp = src + r * lds;
    double2* dp = reinterpret_cast<double2*>(dst + r * ldd);
    for (int q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
      double2 v = make_double2(0.0, 0.0);
      for (int k = 0; k < nseg; ++k) {
        const float2 f = reinterpret_cast<const float2*>(sp + k * seg_stride)[q];
        v.x += (double)f.x;
        v.y += (double)f.y;
      }
      dp[q] = v;
    }
  }
}
void launch_sumconvert(const float* src, long lds, long seg_stride, int nseg, double* dst, long ldd, long rows,
                       int cols, cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return;
  if ((cols | lds | ldd | seg_stride) & 1) throw CudaError("launch_sumconvert: columns and pitches must be even");
  const long tiles = rows * (((cols >> 1) + kConvChunk - 1) / kConvChunk);
  const int blocks = (int)std::min<long>(tiles, 152L * 32);
  k_sumconvert<<<blocks, 256, 0, s>>>(src, lds, seg_stride, nseg, dst, ldd, rows, cols);
  count_launch();
  GD_LAUNCH_CHECK();
}

// --------------------------------------------------------- Legendre GEMMs --
// Tiles: synthesis 32 latitude pairs x 64 real columns, analysis 32 degrees
// x 64 real columns; 256 threads, each 2 rows x 4 columns (columns strided
// by 16 for conflict-free shared reads and coalesced stores).
constexpr int GT_R = 32, GT_C = 64, GT_K = 16;

GemmPlan make_synth_plan(int T, int nh, int ncols_real, cudaStream_t s, int m_lo, int m_hi) {
  std::vector<int4> it;
  int tj = ceil_div(nh, GT_R), tc = ceil_div(ncols_real, GT_C);
  if (m_hi < 0) m_hi = T;
  for (int m = m_lo; m <= m_hi; ++m)  // longest K first for load balance
    for (int a = 0; a < tj; ++a)
      for (int b = 0; b < tc; ++b) it.push_back(make_int4(m, a, b, 0));
  GemmPlan p;
  p.nitems = (int)it.size();
  GD_CUDA(cudaMalloc(&p.items, sizeof(int4) * it.size()));
  GD_CUDA(cudaMemcpyAsync(p.items, it.data(), sizeof(int4) * it.size(), cudaMemcpyHostToDevice, s));
  GD_CUDA(cudaStreamSynchronize(s));
  return p;
}

GemmPlan make_anal_plan(int T, int ncols_real, cudaStream_t s, int m_lo, int m_hi) {
  std::vector<int4> it;
  int tc = ceil_div(ncols_real, GT_C);
  if (m_hi < 0) m_hi = T;
  for (int m = m_lo; m <= m_hi; ++m)
    for (int a = 0; a < ceil_div(T - m + 1, GT_R); ++a)
      for (int b = 0; b < tc; ++b) it.push_back(make_int4(m, a, b, 0));
  GemmPlan p;
  p.nitems = (int)it.size();
  GD_CUDA(cudaMalloc(&p.items, sizeof(int4) * it.size()));
  GD_CUDA(cudaMemcpyAsync(p.items, it.data(), sizeof(int4) * it.size(), cudaMemcpyHostToDevice, s));
  GD_CUDA(cudaStreamSynchronize(s));
  return p;
}

void free_plan(GemmPlan& p) {
  if (p.items) cudaFree(p.items);
  p.items = nullptr;
  p.nitems = 0;
}

template <typename R>
__global__ void __launch_bounds__(256) k_synth(const int4* __restrict__ items, int T, int nh, int nlat,
                                               const long* __restrict__ moff, const long* __restrict__ toff,
                                               const R* __restrict__ tab, const R* __restrict__ B, long ldB,
                                               int ncols, R* __restrict__ F, long ldF, int parityH) {
  __shared__ R sA[GT_K][GT_R];
  __shared__ R sB[GT_K][GT_C];
  const int4 it = items[blockIdx.x];
  const int m = it.x, j0 = it.y * GT_R, c0 = it.z * GT_C;
  const int K = T - m + 1;
  const R* A = tab + toff[m];
  const R* Bm = B + moff[m] * ldB;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  R ae[2][4], ao[2][4];
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int i = 0; i < 4; ++i) ae[r][i] = ao[r][i] = R(0);
  for (int q0 = 0; q0 < K; q0 += GT_K) {
    for (int e = threadIdx.x; e < GT_R * GT_K; e += 256) {
      int jj = e / GT_K, qq = e % GT_K;
      int j = j0 + jj, q = q0 + qq;
      sA[qq][jj] = (j < nh && q < K) ? A[(long)j * K + q] : R(0);
    }
    for (int e = threadIdx.x; e < GT_K * GT_C; e += 256) {
      int qq = e / GT_C, cc = e % GT_C;
      int q = q0 + qq, c = c0 + cc;
      sB[qq][cc] = (q < K && c < ncols) ? Bm[(long)q * ldB + c] : R(0);
    }
    __syncthreads();
#pragma unroll
    for (int qq = 0; qq < GT_K; qq += 2) {
      R a0 = sA[qq][2 * ty], a1 = sA[qq][2 * ty + 1];
      R b0 = sA[qq + 1][2 * ty], b1 = sA[qq + 1][2 * ty + 1];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        R be = sB[qq][tx + 16 * i], bo = sB[qq + 1][tx + 16 * i];
        ae[0][i] += a0 * be;
        ae[1][i] += a1 * be;
        ao[0][i] += b0 * bo;
        ao[1][i] += b1 * bo;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    int j = j0 + 2 * ty + r;
    if (j >= nh) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int c = c0 + tx + 16 * i;
      if (c >= ncols) continue;
      R E = ae[r][i], O = ao[r][i];
      F[((long)m * nlat + j) * ldF + c] = E + O;
      F[((long)m * nlat + (nlat - 1 - j)) * ldF + c] = parityH ? (O - E) : (E - O);
    }
  }
}

template <typename R>
__global__ void __launch_bounds__(256) k_anal(const int4* __restrict__ items, int T, int nh, int nlat,
                                              const long* __restrict__ moff, const long* __restrict__ toff,
                                              const R* __restrict__ tab, const R* __restrict__ G, long ldG,
                                              int ncols, R* __restrict__ A, long ldA, int parityH) {
  __shared__ R sT[GT_K][GT_R];
  __shared__ R sE[GT_K][GT_C];
  __shared__ R sO[GT_K][GT_C];
  const int4 it = items[blockIdx.x];
  const int m = it.x, q0 = it.y * GT_R, c0 = it.z * GT_C;
  const int K = T - m + 1;
  const R* Tm = tab + toff[m];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  R acc[2][4];
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int i = 0; i < 4; ++i) acc[r][i] = R(0);
  for (int jb = 0; jb < nh; jb += GT_K) {
    for (int e = threadIdx.x; e < GT_K * GT_R; e += 256) {
      int jl = e / GT_R, ql = e % GT_R;
      int j = jb + jl, q = q0 + ql;
      sT[jl][ql] = (j < nh && q < K) ? Tm[(long)j * K + q] : R(0);
    }
    for (int e = threadIdx.x; e < GT_K * GT_C; e += 256) {
      int jl = e / GT_C, cc = e % GT_C;
      int j = jb + jl, c = c0 + cc;
      R gn = R(0), gs = R(0);
      if (j < nh && c < ncols) {
        gn = G[((long)m * nlat + j) * ldG + c];
        gs = G[((long)m * nlat + (nlat - 1 - j)) * ldG + c];
      }
      // n-m even rows pair with (gn+gs) for P and (gn-gs) for dP/dphi
      sE[jl][cc] = parityH ? gn - gs : gn + gs;
      sO[jl][cc] = parityH ? gn + gs : gn - gs;
    }
    __syncthreads();
#pragma unroll
    for (int jl = 0; jl < GT_K; ++jl) {
      R t0 = sT[jl][2 * ty], t1 = sT[jl][2 * ty + 1];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        acc[0][i] += t0 * sE[jl][tx + 16 * i];
        acc[1][i] += t1 * sO[jl][tx + 16 * i];
      }
    }
    __syncthreads();
  }
  const long base = moff[m];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    int q = q0 + 2 * ty + r;
    if (q >= K) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int c = c0 + tx + 16 * i;
      if (c < ncols) A[(base + q) * ldA + c] = acc[r][i];
    }
  }
}

template <typename R>
void launch_synth(const ShtDev<R>& d, bool useH, const GemmPlan& plan, const R* B, long ldB, int ncols_real,
                  R* F, long ldF, cudaStream_t s) {
  if (plan.nitems == 0) return;
  k_synth<R><<<plan.nitems, 256, 0, s>>>(plan.items, d.T, d.nh, d.nlat, d.moff, d.toff, useH ? d.H : d.P, B, ldB,
                                         ncols_real, F, ldF, useH ? 1 : 0);
  count_launch();
  GD_LAUNCH_CHECK();
}
template <typename R>
void launch_anal(const ShtDev<R>& d, bool useH, const GemmPlan& plan, const R* G, long ldG, int ncols_real, R* A,
                 long ldA, cudaStream_t s) {
  if (plan.nitems == 0) return;
  k_anal<R><<<plan.nitems, 256, 0, s>>>(plan.items, d.T, d.nh, d.nlat, d.moff, d.toff, useH ? d.H : d.P, G, ldG,
                                        ncols_real, A, ldA, useH ? 1 : 0);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_synth<double>(const ShtDev<double>&, bool, const GemmPlan&, const double*, long, int, double*,
                                   long, cudaStream_t);
template void launch_synth<float>(const ShtDev<float>&, bool, const GemmPlan&, const float*, long, int, float*,
                                  long, cudaStream_t);
template void launch_anal<double>(const ShtDev<double>&, bool, const GemmPlan&, const double*, long, int, double*,
                                  long, cudaStream_t);
template void launch_anal<float>(const ShtDev<float>&, bool, const GemmPlan&, const float*, long, int, float*,
                                 long, cudaStream_t);

// -------------------------------------------------------------- FFTs ------
// Real transforms of length nlon = 2M through one complex Stockham FFT of
// length M per row, several rows per CTA, ping-pong buffers in shared memory.
void fft_radix_plan(int M, int* nrad, int* rad) {
  int n = 0, r = M;
  while (r % 4 == 0) {
    rad[n++] = 4;
    r /= 4;
  }
  while (r % 2 == 0) {
    rad[n++] = 2;
    r /= 2;
  }
  while (r % 3 == 0) {
    rad[n++] = 3;
    r /= 3;
  }
  if (r != 1) throw std::runtime_error("nlon/2 must be 2^a 3^b");
  *nrad = n;
}

template <typename R>
__global__ void k_fft_tables(int M, typename C2<R>::T* twM, typename C2<R>::T* twN) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < M) {
    double sn, cs;
    sincospi(-2.0 * k / M, &sn, &cs);
    twM[k] = mk2<R>((R)cs, (R)sn);
  }
  if (k <= M) {
    double sn, cs;
    sincospi(-1.0 * k / M, &sn, &cs);  // exp(-2 pi i k / (2M))
    twN[k] = mk2<R>((R)cs, (R)sn);
  }
}
template <typename R>
void fft_init_tables(int nlon, typename C2<R>::T* twM, typename C2<R>::T* twN, cudaStream_t s) {
  int M = nlon / 2;
  k_fft_tables<R><<<ceil_div(M + 1, 128), 128, 0, s>>>(M, twM, twN);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void fft_init_tables<double>(int, double2*, double2*, cudaStream_t);
template void fft_init_tables<float>(int, float2*, float2*, cudaStream_t);

// The stochastic-physics pattern on the grid (run.f90:277-281): spectogrd of
// a pattern truncated at pj <= T (coefficients m-major triangular at pj, FP32)
// with the model's own Legendre tables, then the logit transform
// 2 / (1 + exp(g)) - 1 that keeps perturbed tendencies from changing sign.
// One CTA per latitude: the orders' Fourier coefficients in shared memory,
// then the real Fourier sum g = F_0 + 2 sum_m Re(F_m e^{i m lambda}).
template <typename R>
__global__ void k_pattern_grid(ShtDev<R> d, const float2* __restrict__ spec, int pj, R* __restrict__ out) {
  typedef typename C2<R>::T V;
  extern __shared__ __align__(16) unsigned char smpg[];
  V* F = reinterpret_cast<V*>(smpg);
  const int j = blockIdx.x;
  const bool south = j >= d.nh;
  const int jh = south ? d.nlat - 1 - j : j;
  for (int m = threadIdx.x; m <= pj; m += blockDim.x) {
    const int K = d.T + 1 - m;
    const R* Pm = d.P + d.toff[m] + (long)jh * K;
    const long po = (long)m * (pj + 1) - (long)m * (m - 1) / 2;  // (n = m, m) in the pattern's layout
    R re = R(0), im = R(0);
    for (int n = m; n <= pj; ++n) {
      R pv = Pm[n - m];
      if (south && ((n - m) & 1)) pv = -pv;  // P_n^m(-mu) = (-1)^(n-m) P_n^m(mu)
      const float2 c = spec[po + n - m];
      re += pv * (R)c.x;
      im += pv * (R)c.y;
    }
    F[m] = mk2<R>(re, im);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < d.nlon; i += blockDim.x) {
    R g = F[0].x;
    for (int m = 1; m <= pj; ++m) {
      R sn, cs;
      sincospi(R(2) * (R)(((long)m * i) % d.nlon) / (R)d.nlon, &sn, &cs);
      g += R(2) * (F[m].x * cs - F[m].y * sn);
    }
    out[(long)j * d.nlon + i] = R(2) / (R(1) + exp(g)) - R(1);
  }
}
template <typename R>
void launch_pattern_grid(const ShtDev<R>& d, const float2* spec, int pj, R* out, cudaStream_t s) {
  if (pj < 0 || pj > d.T) throw std::invalid_argument("pattern truncation above the model's");
  k_pattern_grid<R><<<d.nlat, 128, (size_t)(pj + 1) * sizeof(typename C2<R>::T), s>>>(d, spec, pj, out);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_pattern_grid<double>(const ShtDev<double>&, const float2*, int, double*, cudaStream_t);
template void launch_pattern_grid<float>(const ShtDev<float>&, const float2*, int, float*, cudaStream_t);

template <typename V>
__device__ __forceinline__ V cmul(V a, V b) {
  V r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename V>
__device__ __forceinline__ V cadd(V a, V b) {
  a.x += b.x;
  a.y += b.y;
  return a;
}
template <typename V>
__device__ __forceinline__ V csub(V a, V b) {
  a.x -= b.x;
  a.y -= b.y;
  return a;
}
template <typename V>
__device__ __forceinline__ V cconj(V a) {
  a.y = -a.y;
  return a;
}

// In-shared-memory Stockham FFT of nr rows of length M; sign -1 forward,
// +1 inverse (unnormalised).  Returns the buffer holding the result.
template <typename R>
__device__ typename C2<R>::T* fft_rows(typename C2<R>::T* a, typename C2<R>::T* b, int M, int nr,
                                       const typename C2<R>::T* __restrict__ tw, int nrad, const int* rad,
                                       int sign) {
  typedef typename C2<R>::T V;
  int Ns = 1;
  for (int st = 0; st < nrad; ++st) {
    const int p = rad[st];
    const int nb = M / p;
    const int tstep = M / (Ns * p);
    for (int e = threadIdx.x; e < nr * nb; e += blockDim.x) {
      const int r = e / nb, jj = e - r * nb;
      const V* in = a + (long)r * M;
      V* out = b + (long)r * M;
      const int k = jj % Ns;
      V v[4];
      for (int q = 0; q < p; ++q) {
        V x = in[jj + q * nb];
        if (q > 0 && k > 0) {
          V w = tw[k * q * tstep];
          if (sign > 0) w = cconj(w);
          x = cmul(x, w);
        }
        v[q] = x;
      }
      if (p == 2) {
        V t = v[0];
        v[0] = cadd(t, v[1]);
        v[1] = csub(t, v[1]);
      } else if (p == 4) {
        V s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
        V s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
        V id13;  // sign * i * d13
        id13.x = -sign * d13.y;
        id13.y = sign * d13.x;
        v[0] = cadd(s02, s13);
        v[2] = csub(s02, s13);
        v[1] = cadd(d02, id13);
        v[3] = csub(d02, id13);
      } else {  // p == 3
        const R c3 = R(-0.5), s3 = R(0.86602540378443864676) * R(sign);
        V t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
        V y0 = cadd(v[0], t1);
        V m1;
        m1.x = v[0].x + c3 * t1.x;
        m1.y = v[0].y + c3 * t1.y;
        V m2;  // i s3 t2
        m2.x = -s3 * t2.y;
        m2.y = s3 * t2.x;
        v[0] = y0;
        v[1] = cadd(m1, m2);
        v[2] = csub(m1, m2);
      }
      const int od = (jj / Ns) * Ns * p + k;
      for (int q = 0; q < p; ++q) out[od + q * Ns] = v[q];
    }
    __syncthreads();
    V* t = a;
    a = b;
    b = t;
    Ns *= p;
  }
  return a;
}

template <typename R>
__host__ __device__ constexpr int nr_of() {
  return sizeof(R) == 8 ? 2 : 4;
}
// rows per CTA of the four-step kernels (64-byte contiguous Fourier chunks)
template <typename R>
__host__ __device__ constexpr int nr4_of() {
  return sizeof(R) == 8 ? 4 : 8;
}
static bool four_step_len(int M) { return M == 64 || M == 96 || M == 192 || M == 384 || M == 576; }
template <typename R>
int fft_rows_per_cta(int M) {
  return (four_step_len(M) && !getenv("GD_FFT_STOCKHAM")) ? nr4_of<R>() : nr_of<R>();
}
template int fft_rows_per_cta<double>(int);
template int fft_rows_per_cta<float>(int);

struct FftArgs {
  int nrad;
  int rad[12];
};

// Fourier -> grid for runs of rows described by SynthDesc.
template <typename R>
__global__ void __launch_bounds__(256) k_c2r(const int2* __restrict__ jobs, const SynthDesc* __restrict__ descs,
                                             ShtDev<R> d, FftArgs fa, const R* __restrict__ FP, long ldP,
                                             const R* __restrict__ FH, long ldH, R* __restrict__ grid) {
  typedef typename C2<R>::T V;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int NR = nr_of<R>();
  const int M = d.M, T = d.T, nlat = d.nlat, nlon = d.nlon;
  V* b0 = reinterpret_cast<V*>(smraw);
  V* b1 = b0 + (long)NR * M;
  const int2 jb = jobs[blockIdx.x];
  const SynthDesc ds = descs[jb.x];
  const int j = blockIdx.y;
  const int r0 = jb.y;
  const int nr = min(NR, ds.count - r0);
  const R rc = d.rcos[j];
  const R alpha = (R)ds.alpha, beta = (R)ds.beta;
  // gather X[r][k] = alpha A + beta (i k / cos) B, zero above T
  for (int e = threadIdx.x; e < nr * M; e += blockDim.x) {
    const int k = e / nr, r = e - k * nr;
    V x = mk2<R>(R(0), R(0));
    if (k <= T) {
      if (ds.srcA >= 0) {
        const R* src = ds.srcA == 0 ? FP : FH;
        const long ld = ds.srcA == 0 ? ldP : ldH;
        V a = *reinterpret_cast<const V*>(src + ((long)k * nlat + j) * ld + 2 * (ds.colA + r0 + r));
        x.x = alpha * a.x;
        x.y = alpha * a.y;
      }
      if (ds.srcB >= 0) {
        const R* src = ds.srcB == 0 ? FP : FH;
        const long ld = ds.srcB == 0 ? ldP : ldH;
        V bb = *reinterpret_cast<const V*>(src + ((long)k * nlat + j) * ld + 2 * (ds.colB + r0 + r));
        const R f = beta * (R)k * rc;  // i f bb
        x.x -= f * bb.y;
        x.y += f * bb.x;
      }
      if (k == 0) x.y = R(0);
    }
    b1[(long)r * M + k] = x;
  }
  __syncthreads();
  // Z[k] = (X[k] + conj X[M-k]) + i (X[k] - conj X[M-k]) exp(+2 pi i k / nlon)
  for (int e = threadIdx.x; e < nr * M; e += blockDim.x) {
    const int r = e / M, k = e - r * M;
    V xk = b1[(long)r * M + k];
    V xm = (k == 0) ? mk2<R>(R(0), R(0)) : cconj(b1[(long)r * M + (M - k)]);
    V A = cadd(xk, xm), B = csub(xk, xm);
    V w = cconj(d.twN[k]);
    V Bw = cmul(B, w);
    V z;
    z.x = A.x - Bw.y;
    z.y = A.y + Bw.x;
    b0[(long)r * M + k] = z;
  }
  __syncthreads();
  V* res = fft_rows<R>(b0, b1, M, nr, d.twM, fa.nrad, fa.rad, +1);
  for (int e = threadIdx.x; e < nr * M; e += blockDim.x) {
    const int r = e / M, n = e - r * M;
    *reinterpret_cast<V*>(grid + ((long)(ds.dst + r0 + r) * nlat + j) * nlon + 2 * n) = res[(long)r * M + n];
  }
}

// grid -> Fourier (scaled by the quadrature weight 2 pi w_j / nlon) for runs
// of rows described by AnalDesc.
template <typename R>
__global__ void __launch_bounds__(256) k_r2c(const int2* __restrict__ jobs, const AnalDesc* __restrict__ descs,
                                             ShtDev<R> d, FftArgs fa, const R* __restrict__ grid,
                                             R* __restrict__ GP, long ldP, R* __restrict__ GH, long ldH) {
  typedef typename C2<R>::T V;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int NR = nr_of<R>();
  const int M = d.M, T = d.T, nlat = d.nlat, nlon = d.nlon;
  V* b0 = reinterpret_cast<V*>(smraw);
  V* b1 = b0 + (long)NR * M;
  const int2 jb = jobs[blockIdx.x];
  const AnalDesc ds = descs[jb.x];
  const int j = blockIdx.y;
  const int r0 = jb.y;
  const int nr = min(NR, ds.count - r0);
  for (int e = threadIdx.x; e < nr * M; e += blockDim.x) {
    const int r = e / M, n = e - r * M;
    b0[(long)r * M + n] = *reinterpret_cast<const V*>(grid + ((long)(ds.src + r0 + r) * nlat + j) * nlon + 2 * n);
  }
  __syncthreads();
  V* Z = fft_rows<R>(b0, b1, M, nr, d.twM, fa.nrad, fa.rad, -1);
  const R wn = d.wn[j], rc = d.rcos[j];
  const R half = R(0.5);
  for (int e = threadIdx.x; e < nr * (T + 1); e += blockDim.x) {
    const int k = e / nr, r = e - k * nr;
    V zk = Z[(long)r * M + k];
    V zm = cconj(Z[(long)r * M + ((M - k) % M)]);
    V E = cadd(zk, zm), O = csub(zk, zm);  // 2E, 2iO
    // X = E + exp(-2 pi i k/nlon) O,  O = -i/2 (Z[k] - conj Z[M-k])
    V Oi;
    Oi.x = O.y;
    Oi.y = -O.x;
    V X = cadd(E, cmul(d.twN[k], Oi));
    X.x *= half * wn;
    X.y *= half * wn;
    const int col = r0 + r;
    if (ds.dstP >= 0) {
      V y = X;
      if (ds.imcosP) {
        const R f = (R)k * rc;
        y.x = -f * X.y;
        y.y = f * X.x;
      }
      y.x *= (R)ds.scaleP;
      y.y *= (R)ds.scaleP;
      *reinterpret_cast<V*>(GP + ((long)k * nlat + j) * ldP + 2 * (ds.dstP + col)) = y;
    }
    if (ds.dstH >= 0) {
      V y = X;
      y.x *= (R)ds.scaleH;
      y.y *= (R)ds.scaleH;
      *reinterpret_cast<V*>(GH + ((long)k * nlat + j) * ldH + 2 * (ds.dstH + col)) = y;
    }
  }
}

// ---- compile-time-planned FFT kernels (common lengths) -------------------
// One in-place shared-memory buffer per CTA (NR rows of M complex values);
// each Stockham stage stages its butterflies through registers, so a CTA
// needs NR*M*sizeof(complex) bytes and many CTAs fit on an SM.  Radix plan,
// strides and divisions are compile-time constants.
template <int M>
struct FftPlanC {
  static constexpr int count() {
    int n = 0, r = M;
    while (r % 4 == 0) r /= 4, ++n;
    while (r % 2 == 0) r /= 2, ++n;
    while (r % 3 == 0) r /= 3, ++n;
    return n;
  }
  static constexpr int radix(int s) {
    int r = M, i = 0;
    while (r % 4 == 0) {
      if (i == s) return 4;
      r /= 4, ++i;
    }
    while (r % 2 == 0) {
      if (i == s) return 2;
      r /= 2, ++i;
    }
    while (r % 3 == 0) {
      if (i == s) return 3;
      r /= 3, ++i;
    }
    return 1;
  }
  static constexpr int ns(int s) {
    int n = 1;
    for (int i = 0; i < s; ++i) n *= radix(i);
    return n;
  }
};

template <typename R, int M, int NR, int NT, int S, int SIGN>
__device__ __forceinline__ void stage_c(typename C2<R>::T* buf, const typename C2<R>::T* __restrict__ tw) {
  typedef typename C2<R>::T V;
  constexpr int p = FftPlanC<M>::radix(S), Ns = FftPlanC<M>::ns(S), nb = M / p, tstep = M / (Ns * p);
  constexpr int NB = NR * nb, PER = (NB + NT - 1) / NT;
  V v[PER][p];
  int od[PER];
#pragma unroll
  for (int u = 0; u < PER; ++u) {
    const int e = threadIdx.x + u * NT;
    od[u] = -1;
    if (e < NB) {
      const int r = e / nb, jj = e - r * nb, k = jj % Ns;
#pragma unroll
      for (int q = 0; q < p; ++q) {
        V x = buf[r * M + jj + q * nb];
        if (q > 0 && k > 0) {
          V w = tw[k * q * tstep];
          if (SIGN > 0) w.y = -w.y;
          x = cmul(x, w);
        }
        v[u][q] = x;
      }
      if (p == 2) {
        V t = v[u][0];
        v[u][0] = cadd(t, v[u][1]);
        v[u][1] = csub(t, v[u][1]);
      } else if (p == 4) {
        V s02 = cadd(v[u][0], v[u][2]), d02 = csub(v[u][0], v[u][2]);
        V s13 = cadd(v[u][1], v[u][3]), d13 = csub(v[u][1], v[u][3]);
        V id13;
        id13.x = -SIGN * d13.y;
        id13.y = SIGN * d13.x;
        v[u][0] = cadd(s02, s13);
        v[u][2] = csub(s02, s13);
        v[u][1] = cadd(d02, id13);
        v[u][3] = csub(d02, id13);
      } else if (p == 3) {
        const R c3 = R(-0.5), s3 = R(0.86602540378443864676) * R(SIGN);
        V t1 = cadd(v[u][1], v[u][2]), t2 = csub(v[u][1], v[u][2]);
        V m1, m2;
        m1.x = v[u][0].x + c3 * t1.x;
        m1.y = v[u][0].y + c3 * t1.y;
        m2.x = -s3 * t2.y;
        m2.y = s3 * t2.x;
        v[u][0] = cadd(v[u][0], t1);
        v[u][1] = cadd(m1, m2);
        v[u][2] = csub(m1, m2);
      }
      od[u] = r * M + (jj / Ns) * Ns * p + k;
    }
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < PER; ++u)
    if (od[u] >= 0) {
#pragma unroll
      for (int q = 0; q < p; ++q) buf[od[u] + q * Ns] = v[u][q];
    }
  __syncthreads();
}

template <typename R, int M, int NR, int NT, int S, int SIGN>
__device__ __forceinline__ void stages_c(typename C2<R>::T* buf, const typename C2<R>::T* __restrict__ tw) {
  if constexpr (S < FftPlanC<M>::count()) {
    stage_c<R, M, NR, NT, S, SIGN>(buf, tw);
    stages_c<R, M, NR, NT, S + 1, SIGN>(buf, tw);
  }
}

template <typename R>
__device__ __forceinline__ typename C2<R>::T synth_coef(const SynthDesc& ds, int k, int T, int j, int nlat, int col,
                                                      const R* __restrict__ FP, long ldP,
                                                      const R* __restrict__ FH, long ldH, R rc, R alpha,
                                                      R beta) {
  typedef typename C2<R>::T V;
  V x = mk2<R>(R(0), R(0));
  if (k > T) return x;
  if (ds.srcA >= 0) {
    const R* src = ds.srcA == 0 ? FP : FH;
    const long ld = ds.srcA == 0 ? ldP : ldH;
    V a = *reinterpret_cast<const V*>(src + ((long)k * nlat + j) * ld + 2 * (ds.colA + col));
    x.x = alpha * a.x;
    x.y = alpha * a.y;
  }
  if (ds.srcB >= 0) {
    const R* src = ds.srcB == 0 ? FP : FH;
    const long ld = ds.srcB == 0 ? ldP : ldH;
    V bb = *reinterpret_cast<const V*>(src + ((long)k * nlat + j) * ld + 2 * (ds.colB + col));
    const R f = beta * (R)k * rc;
    x.x -= f * bb.y;
    x.y += f * bb.x;
  }
  if (k == 0) x.y = R(0);
  return x;
}

template <typename R, int M>
__global__ void __launch_bounds__(128) k_c2r_t(const int2* __restrict__ jobs, const SynthDesc* __restrict__ descs,
                                               ShtDev<R> d, const R* __restrict__ FP, long ldP,
                                               const R* __restrict__ FH, long ldH, R* __restrict__ grid) {
  typedef typename C2<R>::T V;
  constexpr int NR = nr_of<R>(), NT = 128;
  __shared__ V buf[NR * M];
  const int T = d.T, nlat = d.nlat, nlon = d.nlon;
  const int2 jb = jobs[blockIdx.x];
  const SynthDesc ds = descs[jb.x];
  const int j = blockIdx.y, r0 = jb.y;
  const int nr = min(NR, ds.count - r0);
  const R rc = d.rcos[j], alpha = (R)ds.alpha, beta = (R)ds.beta;
  // gather X[k], X[M-k] and form the half-length spectrum Z in place:
  // Z[k] = (X[k] + conj X[M-k]) + i (X[k] - conj X[M-k]) exp(2 pi i k / nlon)
  for (int e = threadIdx.x; e < NR * (M / 2 + 1); e += NT) {
    const int kk = e / NR, r = e - kk * NR;
    V z1 = mk2<R>(R(0), R(0)), z2 = z1;
    if (r < nr) {
      const int k2 = M - kk;
      const V x1 = synth_coef<R>(ds, kk, T, j, nlat, r0 + r, FP, ldP, FH, ldH, rc, alpha, beta);
      const V x2 = (kk == 0) ? mk2<R>(R(0), R(0))
                             : synth_coef<R>(ds, k2, T, j, nlat, r0 + r, FP, ldP, FH, ldH, rc, alpha, beta);
      V A = cadd(x1, cconj(x2)), B = csub(x1, cconj(x2));
      V Bw = cmul(B, cconj(d.twN[kk]));
      z1.x = A.x - Bw.y;
      z1.y = A.y + Bw.x;
      if (kk > 0 && k2 != kk) {
        V A2 = cadd(x2, cconj(x1)), B2 = csub(x2, cconj(x1));
        V Bw2 = cmul(B2, cconj(d.twN[k2]));
        z2.x = A2.x - Bw2.y;
        z2.y = A2.y + Bw2.x;
      }
    }
    buf[r * M + kk] = z1;
    if (kk > 0 && M - kk != kk) buf[r * M + (M - kk)] = z2;
  }
  __syncthreads();
  stages_c<R, M, NR, NT, 0, +1>(buf, d.twM);
  for (int e = threadIdx.x; e < nr * M; e += NT) {
    const int r = e / M, n = e - r * M;
    *reinterpret_cast<V*>(grid + ((long)(ds.dst + r0 + r) * nlat + j) * nlon + 2 * n) = buf[r * M + n];
  }
}

template <typename R, int M>
__global__ void __launch_bounds__(128) k_r2c_t(const int2* __restrict__ jobs, const AnalDesc* __restrict__ descs,
                                               ShtDev<R> d, const R* __restrict__ grid, R* __restrict__ GP,
                                               long ldP, R* __restrict__ GH, long ldH) {
  typedef typename C2<R>::T V;
  constexpr int NR = nr_of<R>(), NT = 128;
  __shared__ V buf[NR * M];
  const int T = d.T, nlat = d.nlat, nlon = d.nlon;
  const int2 jb = jobs[blockIdx.x];
  const AnalDesc ds = descs[jb.x];
  const int j = blockIdx.y, r0 = jb.y;
  const int nr = min(NR, ds.count - r0);
  for (int e = threadIdx.x; e < NR * M; e += NT) {
    const int r = e / M, n = e - r * M;
    V z = mk2<R>(R(0), R(0));
    if (r < nr) z = *reinterpret_cast<const V*>(grid + ((long)(ds.src + r0 + r) * nlat + j) * nlon + 2 * n);
    buf[e] = z;
  }
  __syncthreads();
  stages_c<R, M, NR, NT, 0, -1>(buf, d.twM);
  const R wn = d.wn[j] * R(0.5), rc = d.rcos[j];
  for (int e = threadIdx.x; e < nr * (M / 2 + 1); e += NT) {
    const int kk = e / nr, r = e - kk * nr;
    const V Z1 = buf[r * M + kk], Z2 = buf[r * M + (M - kk) % M];
    for (int h = 0; h < 2; ++h) {
      const int k = h ? M - kk : kk;
      if (k > T || (h && (kk == 0 || M - kk == kk))) continue;
      const V za = h ? Z2 : Z1, zb = h ? Z1 : Z2;
      V E = cadd(za, cconj(zb)), O = csub(za, cconj(zb));
      V Oi;
      Oi.x = O.y;
      Oi.y = -O.x;
      V X = cadd(E, cmul(d.twN[k], Oi));
      X.x *= wn;
      X.y *= wn;
      const int col = r0 + r;
      if (ds.dstP >= 0) {
        V y = X;
        if (ds.imcosP) {
          const R f = (R)k * rc;
          y.x = -f * X.y;
          y.y = f * X.x;
        }
        y.x *= (R)ds.scaleP;
        y.y *= (R)ds.scaleP;
        *reinterpret_cast<V*>(GP + ((long)k * nlat + j) * ldP + 2 * (ds.dstP + col)) = y;
      }
      if (ds.dstH >= 0) {
        V y = X;
        y.x *= (R)ds.scaleH;
        y.y *= (R)ds.scaleH;
        *reinterpret_cast<V*>(GH + ((long)k * nlat + j) * ldH + 2 * (ds.dstH + col)) = y;
      }
    }
  }
}

// ---- four-step register FFTs (M = M1 * M2) --------------------------------
// Step A: M1 independent M2-point DFTs (stride M1) in registers, then the
// twiddle W_M^(n1 k2); one shared-memory exchange; step B: M2 independent
// M1-point DFTs in registers.  Rows live in shared memory with one pad
// element after every M1 values so the strided exchanges are bank-conflict
// free.  The in-register DFTs are fully unrolled Stockham passes over the
// compile-time radix plan with compile-time twiddles; the twiddle between
// the steps comes from the length-M table.
template <int M, int M1>
__device__ __forceinline__ int pad_addr(int n) {
  return n + n / M1;
}
// Row pitch (complex elements): the padded length plus an extra offset chosen
// by counting shared-memory wavefronts of all four phases (gather, step A,
// step B, store) for 8 rows of float2 per CTA.
template <int M, int M1>
constexpr int row_pitch4() {
  return M + M / M1 + (M == 192 ? 12 : M == 384 ? 10 : M == 576 ? 2 : 0);
}

// cos and sin of 2 pi a / b at compile time: exact octant reduction in
// integers, then Taylor series on an angle of at most pi/4 (the terms fall
// below 1e-17 of the sum after 12 of them).  Used for the twiddles of the
// in-register DFTs, which become immediate operands.
struct CtCS {
  double c, s;
};
constexpr double ct_taylor_cos(double t) {
  double term = 1.0, sum = 1.0;
  for (int i = 1; i <= 14; ++i) {
    term *= -t * t / ((2.0 * i - 1.0) * (2.0 * i));
    sum += term;
  }
  return sum;
}
constexpr double ct_taylor_sin(double t) {
  double term = t, sum = t;
  for (int i = 1; i <= 14; ++i) {
    term *= -t * t / ((2.0 * i) * (2.0 * i + 1.0));
    sum += term;
  }
  return sum;
}
constexpr CtCS ct_cs_turn(long a, long b) {  // angle 2 pi a / b
  long r = a % b;
  if (r < 0) r += b;
  // fraction f = r / b of a turn; reduce to [0, 1/8] with exact rationals
  // in units of 1 / (8 b)
  long u = 8 * r;  // f * 8b
  const long B8 = 8 * b;
  double sc = 1.0, ss = 1.0;
  bool swap = false;
  if (u > B8 / 2) {  // f in (1/2, 1): cos(2pi - x) = cos x, sin = -sin
    u = B8 - u;
    ss = -ss;
  }
  if (u > B8 / 4) {  // f in (1/4, 1/2]: cos(pi - x) = -cos x, sin = sin
    u = B8 / 2 - u;
    sc = -sc;
  }
  if (u > B8 / 8) {  // f in (1/8, 1/4]: cos x = sin(pi/2 - x)
    u = B8 / 4 - u;
    swap = true;
  }
  const double t = 2.0 * 3.14159265358979323846264338327950288 * (double)u / (double)B8;
  const double c0 = ct_taylor_cos(t), s0 = ct_taylor_sin(t);
  return CtCS{sc * (swap ? s0 : c0), ss * (swap ? c0 : s0)};
}
// x * W_M^E for SIGN < 0 (W = exp(-2 pi i / M)), x * conj(W_M^E) for SIGN > 0
template <typename R, int SIGN, long E, long M>
__device__ __forceinline__ typename C2<R>::T ct_twiddle(typename C2<R>::T x) {
  if constexpr (E % M == 0) {
    return x;
  } else {
    constexpr CtCS cs = ct_cs_turn(E, M);
    constexpr R wc = (R)cs.c, ws = (R)(SIGN > 0 ? cs.s : -cs.s);
    typename C2<R>::T r;
    r.x = x.x * wc - x.y * ws;
    r.y = x.x * ws + x.y * wc;
    return r;
  }
}

// one radix-p butterfly (index JJ of the stage) and the rest of the stage
template <typename R, int N, int M, int SIGN, int S, int JJ>
__device__ __forceinline__ void reg_bfly(const typename C2<R>::T* x, typename C2<R>::T* y) {
  typedef typename C2<R>::T V;
  constexpr int p = FftPlanC<N>::radix(S), Ns = FftPlanC<N>::ns(S), nb = N / p;
  if constexpr (JJ < nb) {
    constexpr int k = JJ % Ns;
    constexpr long tstep = (M / N) * (N / (Ns * p));  // W_{Ns p} = W_M^(M/(Ns p))
    V v[4];
    v[0] = x[JJ];
    v[1] = ct_twiddle<R, SIGN, 1L * k * tstep, M>(x[JJ + nb]);
    if constexpr (p > 2) v[2] = ct_twiddle<R, SIGN, 2L * k * tstep, M>(x[JJ + 2 * nb]);
    if constexpr (p > 3) v[3] = ct_twiddle<R, SIGN, 3L * k * tstep, M>(x[JJ + 3 * nb]);
    if constexpr (p == 2) {
      V t = v[0];
      v[0] = cadd(t, v[1]);
      v[1] = csub(t, v[1]);
    } else if constexpr (p == 4) {
      V s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
      V s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
      V id13;
      id13.x = -SIGN * d13.y;
      id13.y = SIGN * d13.x;
      v[0] = cadd(s02, s13);
      v[2] = csub(s02, s13);
      v[1] = cadd(d02, id13);
      v[3] = csub(d02, id13);
    } else {
      const R c3 = R(-0.5), s3 = R(0.86602540378443864676) * R(SIGN);
      V t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
      V m1, m2;
      m1.x = v[0].x + c3 * t1.x;
      m1.y = v[0].y + c3 * t1.y;
      m2.x = -s3 * t2.y;
      m2.y = s3 * t2.x;
      v[0] = cadd(v[0], t1);
      v[1] = cadd(m1, m2);
      v[2] = csub(m1, m2);
    }
    constexpr int od = (JJ / Ns) * Ns * p + k;
#pragma unroll
    for (int q = 0; q < p; ++q) y[od + q * Ns] = v[q];
    reg_bfly<R, N, M, SIGN, S, JJ + 1>(x, y);
  }
}
template <typename R, int N, int M, int SIGN, int S>
__device__ __forceinline__ void reg_stages(typename C2<R>::T* x, typename C2<R>::T* y) {
  if constexpr (S < FftPlanC<N>::count()) {
    reg_bfly<R, N, M, SIGN, S, 0>(x, y);
    reg_stages<R, N, M, SIGN, S + 1>(y, x);
  }
}
// in-register N-point DFT of x (y is scratch); the result is left in x
template <typename R, int N, int M, int SIGN>
__device__ __forceinline__ void reg_fft(typename C2<R>::T* x, typename C2<R>::T* y) {
  reg_stages<R, N, M, SIGN, 0>(x, y);
  if constexpr (FftPlanC<N>::count() % 2 == 1) {
#pragma unroll
    for (int i = 0; i < N; ++i) x[i] = y[i];
  }
}

// four-step FFT of NR rows held in buf (padded addressing), sign SIGN.
// LoadA(r, n1, x) fills x[n2] = row r's x[n1 + M1 n2] for step A: from buf
// (nullptr: the rows are already there) or straight from global memory;
// StoreB(r, k2, x) takes the outputs X[k2 + M2 k1] of step B (nullptr: back
// into buf).  Going straight to or from global memory saves one pass over
// shared memory and one barrier.
struct Fft4InBuf {};
template <typename R, int M, int M1, int M2, int NR, int NT, int SIGN, typename LoadA, typename StoreB>
__device__ __forceinline__ void fft4x(typename C2<R>::T* buf, const typename C2<R>::T* __restrict__ tw, LoadA lda,
                                      StoreB stb) {
  typedef typename C2<R>::T V;
  constexpr int RP = row_pitch4<M, M1>();
  constexpr bool a_buf = std::is_same<LoadA, Fft4InBuf>::value, b_buf = std::is_same<StoreB, Fft4InBuf>::value;
  // step A: thread (r, n1) -> M2-point DFT over n2 of x[n1 + M1 n2], twiddle, store in place
  for (int e = threadIdx.x; e < NR * M1; e += NT) {
    const int r = e / M1, n1 = e - r * M1;
    V* row = buf + r * RP;
    V x[M2], y[M2];
    if constexpr (a_buf) {
#pragma unroll
      for (int n2 = 0; n2 < M2; ++n2) x[n2] = row[n1 + (M1 + 1) * n2];  // pad_addr(n1 + M1 n2), n1 < M1
    } else {
      lda(r, n1, x);
    }
    reg_fft<R, M2, M, SIGN>(x, y);
#pragma unroll
    for (int k2 = 1; k2 < M2; ++k2) {
      if (n1 > 0) {
        V w = tw[n1 * k2];
        if (SIGN > 0) w.y = -w.y;
        x[k2] = cmul(x[k2], w);
      }
    }
#pragma unroll
    for (int k2 = 0; k2 < M2; ++k2) row[n1 + (M1 + 1) * k2] = x[k2];
  }
  __syncthreads();
  // step B: thread (r, k2) -> M1-point DFT over n1 of Y[n1 + M1 k2]; result X[k2 + M2 k1]
  static_assert(NR * M2 <= NT, "step B needs one task per thread");
  const int e = threadIdx.x;
  const int r = e / M2, k2 = e - r * M2;
  V x[M1], y[M1];
  if (e < NR * M2) {
    const V* row = buf + r * RP + (M1 + 1) * k2;  // pad_addr(n1 + M1 k2) = n1 + (M1 + 1) k2
#pragma unroll
    for (int n1 = 0; n1 < M1; ++n1) x[n1] = row[n1];
    reg_fft<R, M1, M, SIGN>(x, y);
  }
  if constexpr (b_buf) {
    __syncthreads();
    if (e < NR * M2) {
      V* row = buf + r * RP;
#pragma unroll
      for (int k1 = 0; k1 < M1; ++k1) row[pad_addr<M, M1>(k2 + M2 * k1)] = x[k1];
    }
    __syncthreads();
  } else {
    if (e < NR * M2) stb(r, k2, x);
  }
}
template <typename R, int M, int M1, int M2, int NR, int NT, int SIGN>
__device__ __forceinline__ void fft4(typename C2<R>::T* buf, const typename C2<R>::T* __restrict__ tw) {
  fft4x<R, M, M1, M2, NR, NT, SIGN>(buf, tw, Fft4InBuf{}, Fft4InBuf{});
}

// Minimum resident CTAs per SM: these kernels are latency-bound and run
// best at the occupancy their shared memory allows (measured: c2r with 5,
// r2c with 4 CTAs of 8 FP32 rows of 576 points; without a bound the
// compiler takes more registers and fewer CTAs fit).
constexpr int C2R4_MINB = 5, R2C4_MINB = 4;
// G (the grid type) differs from R in the eddy form of the FP64-state mode:
// the FFT of orders m >= 1 runs in R = float from FP32 Fourier rows, order 0
// (the zonal mean alpha Re F_0) is read in FP64 from FP0/FH0 (same pitches)
// and added in FP64 to every FP64 grid value of its row.
template <typename R, int M, int M1, int M2, typename G = R>
__global__ void __launch_bounds__(((nr4_of<R>() * (M1 > M2 ? M1 : M2) + 31) / 32) * 32, C2R4_MINB)
    k_c2r_4(const int2* __restrict__ jobs, const SynthDesc* __restrict__ descs, ShtDev<R> d,
            const R* __restrict__ FP, long ldP, const R* __restrict__ FH, long ldH, G* __restrict__ grid,
            const double* __restrict__ FP0, const double* __restrict__ FH0) {
  typedef typename C2<R>::T V;
  typedef typename C4<R>::T V4;
  constexpr bool kEddy = !std::is_same<G, R>::value;
  constexpr int NR = nr4_of<R>(), NT = ((NR * (M1 > M2 ? M1 : M2) + 31) / 32) * 32, RP = row_pitch4<M, M1>();
  constexpr int KS = NT / NR;  // order stride of one thread in the gather
  static_assert(NT % NR == 0 && M1 % 2 == 0, "thread maps of the four-step kernels");
  __shared__ V buf[NR * RP];
  __shared__ double mean_s[kEddy ? NR : 1];
  const int T = d.T, nlat = d.nlat, nlon = d.nlon;
  const int2 jb = jobs[blockIdx.x];
  const SynthDesc ds = descs[jb.x];
  const int j = blockIdx.y, r0 = jb.y;
  const int nr = min(NR, ds.count - r0);
  const R rc = d.rcos[j], alpha = (R)ds.alpha, beta = (R)ds.beta;
  // gather: the thread's row r is fixed, its orders are kq, kq + KS, ...
  const int r = threadIdx.x % NR, kq = threadIdx.x / NR;
  const bool live = r < nr;
  const R* pa = nullptr;
  const R* pb = nullptr;
  long sa = 0, sb = 0;  // distance between consecutive orders
  if (live && ds.srcA >= 0) {
    const long ld = ds.srcA == 0 ? ldP : ldH;
    pa = (ds.srcA == 0 ? FP : FH) + (long)j * ld + 2 * (ds.colA + r0 + r);
    sa = (long)nlat * ld;
  }
  if (live && ds.srcB >= 0) {
    const long ld = ds.srcB == 0 ? ldP : ldH;
    pb = (ds.srcB == 0 ? FP : FH) + (long)j * ld + 2 * (ds.colB + r0 + r);
    sb = (long)nlat * ld;
  }
  V* brow = buf + r * RP;
  if constexpr (kEddy) {
    if (kq == 0) {  // one thread per row: the FP64 zonal mean of the row
      double mv = 0.0;
      if (live && ds.srcA >= 0) {
        const long ld = ds.srcA == 0 ? ldP : ldH;
        mv = ds.alpha * (ds.srcA == 0 ? FP0 : FH0)[(long)j * ld + 2 * (ds.colA + r0 + r)];
      }
      mean_s[r] = mv;
    }
  }
  // the gather issues the loads of CB consecutive orders of the thread
  // before using any of them: the loads are latency-bound, not issue-bound
  constexpr int CB = 4;
  for (int kb = kq; kb <= M / 2; kb += CB * KS) {
    const V zz = mk2<R>(R(0), R(0));
    V la1[CB], la2[CB], lb1[CB], lb2[CB];
#pragma unroll
    for (int c = 0; c < CB; ++c) {
      const int kk = kb + c * KS, k2 = M - kk;
      la1[c] = la2[c] = lb1[c] = lb2[c] = zz;
      if (kk <= M / 2 && live && kk <= T) {
        if (pa) {
          la1[c] = *reinterpret_cast<const V*>(pa + kk * sa);
          if (kk > 0 && k2 <= T) la2[c] = *reinterpret_cast<const V*>(pa + k2 * sa);
        }
        if (pb) {
          lb1[c] = *reinterpret_cast<const V*>(pb + kk * sb);
          if (kk > 0 && k2 <= T) lb2[c] = *reinterpret_cast<const V*>(pb + k2 * sb);
        }
      }
    }
#pragma unroll
    for (int c = 0; c < CB; ++c) {
    const int kk = kb + c * KS;
    if (kk > M / 2) break;
    const int k2 = M - kk;
    V z1 = mk2<R>(R(0), R(0)), z2 = z1;
    if (live && kk <= T) {  // kk > T: both orders above the truncation, z = 0
      // x_k = alpha A_k + beta (i k / cos) B_k, zero above the truncation
      V x1 = z1, x2 = z1;
      if (pa) {
        const V v1 = la1[c];
        x1.x = alpha * v1.x;
        x1.y = alpha * v1.y;
        if (kk > 0 && k2 <= T) {
          const V v2 = la2[c];
          x2.x = alpha * v2.x;
          x2.y = alpha * v2.y;
        }
      }
      if (pb) {
        const V v1 = lb1[c];
        const R f1 = beta * (R)kk * rc;
        x1.x -= f1 * v1.y;
        x1.y += f1 * v1.x;
        if (kk > 0 && k2 <= T) {
          const V v2 = lb2[c];
          const R f2 = beta * (R)k2 * rc;
          x2.x -= f2 * v2.y;
          x2.y += f2 * v2.x;
        }
      }
      if (kk == 0) x1.y = R(0);
      if constexpr (kEddy) {
        if (kk == 0) x1.x = R(0);  // order 0 is added in FP64 at the store
      }
      V A = cadd(x1, cconj(x2)), B = csub(x1, cconj(x2));
      V Bw = cmul(B, cconj(d.twN[kk]));
      z1.x = A.x - Bw.y;
      z1.y = A.y + Bw.x;
      if (kk > 0 && k2 != kk) {
        V A2 = cadd(x2, cconj(x1)), B2 = csub(x2, cconj(x1));
        V Bw2 = cmul(B2, cconj(d.twN[k2]));
        z2.x = A2.x - Bw2.y;
        z2.y = A2.y + Bw2.x;
      }
    }
    brow[pad_addr<M, M1>(kk)] = z1;
    if (kk > 0 && k2 != kk) brow[pad_addr<M, M1>(k2)] = z2;
    }
  }
  __syncthreads();
  // step B stores its outputs straight to the grid row: z[n] is the real
  // pair (x[2n], x[2n+1]); a warp's lanes hold consecutive n of a row
  G* const gout = grid + ((long)(ds.dst + r0) * nlat + j) * nlon;
  const long rstride = (long)nlat * nlon;
  fft4x<R, M, M1, M2, NR, NT, +1>(buf, d.twM, Fft4InBuf{}, [&](int rr, int k2, const V* x) {
    if (rr < nr) {
      if constexpr (kEddy) {
        const double mv = mean_s[rr];
        double2* o = reinterpret_cast<double2*>(gout + rr * rstride) + k2;
#pragma unroll
        for (int k1 = 0; k1 < M1; ++k1) o[M2 * k1] = make_double2((double)x[k1].x + mv, (double)x[k1].y + mv);
      } else {
        V* o = reinterpret_cast<V*>(gout + rr * rstride) + k2;
#pragma unroll
        for (int k1 = 0; k1 < M1; ++k1) o[M2 * k1] = x[k1];
      }
    }
  });
}

// Eddy form (G = double, R = float): the row's FP64 zonal mean rmean (from
// k_rowmean) is subtracted in FP64 before the values are rounded to FP32, the
// FFT of the remainder gives orders m >= 1 in FP32 (GP, GH), and order 0 is
// written in FP64 to GP0 / GH0 (same pitches): 2 pi w_j times the mean.
template <typename R, int M, int M1, int M2, typename G = R>
__global__ void __launch_bounds__(((nr4_of<R>() * (M1 > M2 ? M1 : M2) + 31) / 32) * 32, R2C4_MINB)
    k_r2c_4(const int2* __restrict__ jobs, const AnalDesc* __restrict__ descs, ShtDev<R> d,
            const G* __restrict__ grid, R* __restrict__ GP, long ldP, R* __restrict__ GH, long ldH,
            const double* __restrict__ rmean, const double* __restrict__ wn64, double* __restrict__ GP0,
            double* __restrict__ GH0) {
  typedef typename C2<R>::T V;
  typedef typename C4<R>::T V4;
  constexpr bool kEddy = !std::is_same<G, R>::value;
  constexpr int NR = nr4_of<R>(), NT = ((NR * (M1 > M2 ? M1 : M2) + 31) / 32) * 32, RP = row_pitch4<M, M1>();
  constexpr int KS = NT / NR;
  static_assert(NT % NR == 0 && M1 % 2 == 0, "thread maps of the four-step kernels");
  __shared__ V buf[NR * RP];
  const int T = d.T, nlat = d.nlat, nlon = d.nlon;
  const int2 jb = jobs[blockIdx.x];
  const AnalDesc ds = descs[jb.x];
  const int j = blockIdx.y, r0 = jb.y;
  const int nr = min(NR, ds.count - r0);
  // step A loads its inputs straight from the grid row: x[n] is the real
  // pair (g[2n], g[2n+1]); rows past nr are zero
  const G* const gin = grid + ((long)(ds.src + r0) * nlat + j) * nlon;
  const long rstride = (long)nlat * nlon;
  fft4x<R, M, M1, M2, NR, NT, -1>(buf, d.twM, [&](int rr, int n1, V* x) {
    if (rr < nr) {
      if constexpr (kEddy) {
        const double mv = rmean[(long)(ds.src + r0 + rr) * nlat + j];
        const double2* g = reinterpret_cast<const double2*>(gin + rr * rstride) + n1;
#pragma unroll
        for (int n2 = 0; n2 < M2; ++n2) {
          const double2 t = g[M1 * n2];
          x[n2] = mk2<R>((R)(t.x - mv), (R)(t.y - mv));
        }
      } else {
        const V* g = reinterpret_cast<const V*>(gin + rr * rstride) + n1;
#pragma unroll
        for (int n2 = 0; n2 < M2; ++n2) x[n2] = g[M1 * n2];
      }
    } else {
#pragma unroll
      for (int n2 = 0; n2 < M2; ++n2) x[n2] = mk2<R>(R(0), R(0));
    }
  }, Fft4InBuf{});
  const R wn = d.wn[j] * R(0.5), rc = d.rcos[j];
  const int r = threadIdx.x % NR, kq = threadIdx.x / NR;
  if (r >= nr) return;
  const int col = r0 + r;
  R* pP = ds.dstP >= 0 ? GP + (long)j * ldP + 2 * (ds.dstP + col) : nullptr;
  R* pH = ds.dstH >= 0 ? GH + (long)j * ldH + 2 * (ds.dstH + col) : nullptr;
  const long sP = (long)nlat * ldP, sH = (long)nlat * ldH;
  const R scP = (R)ds.scaleP, scH = (R)ds.scaleH;
  const V* brow = buf + r * RP;
  for (int kk = kq; kk <= M / 2; kk += KS) {
    const V Z1 = brow[pad_addr<M, M1>(kk)], Z2 = brow[pad_addr<M, M1>((M - kk) % M)];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = h ? M - kk : kk;
      if (k > T || (h && (kk == 0 || M - kk == kk))) continue;
      if constexpr (kEddy) {
        if (k == 0) {  // order 0 in FP64 from the row mean; zeros in the FP32 rows
          const double x0 = wn64[j] * (double)nlon * rmean[(long)(ds.src + col) * nlat + j];
          if (pP) {
            *reinterpret_cast<V*>(pP) = mk2<R>(R(0), R(0));
            double* q = GP0 + (long)j * ldP + 2 * (ds.dstP + col);
            q[0] = ds.imcosP ? 0.0 : x0 * ds.scaleP;
            q[1] = 0.0;
          }
          if (pH) {
            *reinterpret_cast<V*>(pH) = mk2<R>(R(0), R(0));
            double* q = GH0 + (long)j * ldH + 2 * (ds.dstH + col);
            q[0] = x0 * ds.scaleH;
            q[1] = 0.0;
          }
          continue;
        }
      }
      const V za = h ? Z2 : Z1, zb = h ? Z1 : Z2;
      V E = cadd(za, cconj(zb)), O = csub(za, cconj(zb));
      V Oi;
      Oi.x = O.y;
      Oi.y = -O.x;
      V X = cadd(E, cmul(d.twN[k], Oi));
      X.x *= wn;
      X.y *= wn;
      if (pP) {
        V y = X;
        if (ds.imcosP) {
          const R f = (R)k * rc;
          y.x = -f * X.y;
          y.y = f * X.x;
        }
        y.x *= scP;
        y.y *= scP;
        *reinterpret_cast<V*>(pP + k * sP) = y;
      }
      if (pH) {
        V y = X;
        y.x *= scH;
        y.y *= scH;
        *reinterpret_cast<V*>(pH + k * sH) = y;
      }
    }
  }
}

template <int M, int M1, int M2>
constexpr int nt4(int nr) {
  return ((nr * (M1 > M2 ? M1 : M2) + 31) / 32) * 32;
}

template <typename R>
static bool launch_c2r_fixed(const ShtDev<R>& d, const FftPlan& plan, const R* FP, long ldP, const R* FH, long ldH,
                             R* grid, cudaStream_t s) {
  dim3 grd(plan.njobs, d.nlat);
  const SynthDesc* ds = (const SynthDesc*)plan.descs;
#define GD_C2R(MM)                                                                               \
  case MM:                                                                                       \
    k_c2r_t<R, MM><<<grd, 128, 0, s>>>(plan.jobs, ds, d, FP, ldP, FH, ldH, grid);                \
    return true;
  if (!getenv("GD_FFT_STOCKHAM")) {
    constexpr int NR = nr4_of<R>();
    switch (d.M) {
#define GD_C2R4(MM, A, B)                                                                         \
  case MM:                                                                                        \
    k_c2r_4<R, MM, A, B><<<grd, nt4<MM, A, B>(NR), 0, s>>>(plan.jobs, ds, d, FP, ldP, FH, ldH, grid, nullptr, \
                                                            nullptr);                                        \
    return true;
      GD_C2R4(64, 8, 8)
      GD_C2R4(96, 8, 12)
      GD_C2R4(192, 12, 16)
      GD_C2R4(384, 16, 24)
      GD_C2R4(576, 24, 24)
#undef GD_C2R4
      default:
        break;
    }
  }
  switch (d.M) {
    GD_C2R(32)
    GD_C2R(48)
    GD_C2R(64)
    GD_C2R(96)
    GD_C2R(128)
    GD_C2R(192)
    GD_C2R(256)
    GD_C2R(384)
    GD_C2R(576)
    GD_C2R(768)
    default:
      return false;
  }
#undef GD_C2R
}
template <typename R>
static bool launch_r2c_fixed(const ShtDev<R>& d, const FftPlan& plan, const R* grid, R* GP, long ldP, R* GH,
                             long ldH, cudaStream_t s) {
  dim3 grd(plan.njobs, d.nlat);
  const AnalDesc* ds = (const AnalDesc*)plan.descs;
#define GD_R2C(MM)                                                                               \
  case MM:                                                                                       \
    k_r2c_t<R, MM><<<grd, 128, 0, s>>>(plan.jobs, ds, d, grid, GP, ldP, GH, ldH);                \
    return true;
  if (!getenv("GD_FFT_STOCKHAM")) {
    constexpr int NR = nr4_of<R>();
    switch (d.M) {
#define GD_R2C4(MM, A, B)                                                                         \
  case MM:                                                                                        \
    k_r2c_4<R, MM, A, B><<<grd, nt4<MM, A, B>(NR), 0, s>>>(plan.jobs, ds, d, grid, GP, ldP, GH, ldH, nullptr, \
                                                            nullptr, nullptr, nullptr);                      \
    return true;
      GD_R2C4(64, 8, 8)
      GD_R2C4(96, 8, 12)
      GD_R2C4(192, 12, 16)
      GD_R2C4(384, 16, 24)
      GD_R2C4(576, 24, 24)
#undef GD_R2C4
      default:
        break;
    }
  }
  switch (d.M) {
    GD_R2C(32)
    GD_R2C(48)
    GD_R2C(64)
    GD_R2C(96)
    GD_R2C(128)
    GD_R2C(192)
    GD_R2C(256)
    GD_R2C(384)
    GD_R2C(576)
    GD_R2C(768)
    default:
      return false;
  }
#undef GD_R2C
}

template <typename R, typename D>
static FftPlan make_plan(const D* descs, int ndesc, cudaStream_t s, int M) {
  const int NR = fft_rows_per_cta<R>(M);
  std::vector<int2> jobs;
  for (int i = 0; i < ndesc; ++i)
    for (int r = 0; r < descs[i].count; r += NR) jobs.push_back(make_int2(i, r));
  FftPlan p;
  p.njobs = (int)jobs.size();
  if (p.njobs == 0) return p;
  GD_CUDA(cudaMalloc(&p.jobs, sizeof(int2) * jobs.size()));
  GD_CUDA(cudaMalloc(&p.descs, sizeof(D) * ndesc));
  GD_CUDA(cudaMemcpyAsync(p.jobs, jobs.data(), sizeof(int2) * jobs.size(), cudaMemcpyHostToDevice, s));
  GD_CUDA(cudaMemcpyAsync(p.descs, descs, sizeof(D) * ndesc, cudaMemcpyHostToDevice, s));
  GD_CUDA(cudaStreamSynchronize(s));
  return p;
}
template <typename R>
FftPlan make_c2r_plan(const SynthDesc* descs, int ndesc, cudaStream_t s, int M) {
  return make_plan<R>(descs, ndesc, s, M);
}
template <typename R>
FftPlan make_r2c_plan(const AnalDesc* descs, int ndesc, cudaStream_t s, int M) {
  return make_plan<R>(descs, ndesc, s, M);
}
template FftPlan make_c2r_plan<double>(const SynthDesc*, int, cudaStream_t, int);
template FftPlan make_c2r_plan<float>(const SynthDesc*, int, cudaStream_t, int);
template FftPlan make_r2c_plan<double>(const AnalDesc*, int, cudaStream_t, int);
template FftPlan make_r2c_plan<float>(const AnalDesc*, int, cudaStream_t, int);

void free_fft_plan(FftPlan& p) {
  if (p.jobs) cudaFree(p.jobs);
  if (p.descs) cudaFree(p.descs);
  p.jobs = nullptr;
  p.descs = nullptr;
  p.njobs = 0;
}

template <typename R>
static size_t fft_smem(int M) {
  return 2 * (size_t)nr_of<R>() * M * sizeof(typename C2<R>::T);
}

template <typename R>
void launch_c2r(const ShtDev<R>& d, const FftPlan& plan, const R* FP, long ldP, const R* FH, long ldH, R* grid,
                cudaStream_t s) {
  if (plan.njobs == 0) return;
  if (launch_c2r_fixed<R>(d, plan, FP, ldP, FH, ldH, grid, s)) {
    count_launch();
    GD_LAUNCH_CHECK();
    return;
  }
  FftArgs fa;
  fa.nrad = d.nrad;
  for (int i = 0; i < 12; ++i) fa.rad[i] = d.rad[i];
  size_t sm = fft_smem<R>(d.M);
  static bool attr = false;
  if (!attr) {
    GD_CUDA(cudaFuncSetAttribute(k_c2r<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr = true;
  }
  dim3 grd(plan.njobs, d.nlat);
  k_c2r<R><<<grd, 256, sm, s>>>(plan.jobs, (const SynthDesc*)plan.descs, d, fa, FP, ldP, FH, ldH, grid);
  count_launch();
  GD_LAUNCH_CHECK();
}
template <typename R>
void launch_r2c(const ShtDev<R>& d, const FftPlan& plan, const R* grid, R* GP, long ldP, R* GH, long ldH,
                cudaStream_t s) {
  if (plan.njobs == 0) return;
  if (launch_r2c_fixed<R>(d, plan, grid, GP, ldP, GH, ldH, s)) {
    count_launch();
    GD_LAUNCH_CHECK();
    return;
  }
  FftArgs fa;
  fa.nrad = d.nrad;
  for (int i = 0; i < 12; ++i) fa.rad[i] = d.rad[i];
  size_t sm = fft_smem<R>(d.M);
  static bool attr = false;
  if (!attr) {
    GD_CUDA(cudaFuncSetAttribute(k_r2c<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr = true;
  }
  dim3 grd(plan.njobs, d.nlat);
  k_r2c<R><<<grd, 256, sm, s>>>(plan.jobs, (const AnalDesc*)plan.descs, d, fa, grid, GP, ldP, GH, ldH);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_c2r<double>(const ShtDev<double>&, const FftPlan&, const double*, long, const double*, long,
                                 double*, cudaStream_t);
template void launch_c2r<float>(const ShtDev<float>&, const FftPlan&, const float*, long, const float*, long,
                                float*, cudaStream_t);
template void launch_r2c<double>(const ShtDev<double>&, const FftPlan&, const double*, double*, long, double*,
                                 long, cudaStream_t);
template void launch_r2c<float>(const ShtDev<float>&, const FftPlan&, const float*, float*, long, float*, long,
                                cudaStream_t);

// ------------------------------------------------- eddy FFTs (FP64 state) --
// FP64 zonal mean of every (grid row, latitude) a r2c plan reads, one warp
// per row in a fixed summation order (lane-strided partial sums, then the
// xor butterfly; lane 0 writes), so the result does not depend on the launch.
// The job list is the FP32 four-step plan's: NR rows per job.
template <int NR>
__global__ void __launch_bounds__(32 * NR) k_rowmean(const int2* __restrict__ jobs, const AnalDesc* __restrict__ descs,
                                                     int nlat, int nlon, const double* __restrict__ grid,
                                                     double* __restrict__ rmean) {
  const int2 jb = jobs[blockIdx.x];
  const AnalDesc ds = descs[jb.x];
  const int j = blockIdx.y, rr = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (rr >= min(NR, ds.count - jb.y)) return;
  const long row = (long)ds.src + jb.y + rr;
  const double* g = grid + (row * nlat + j) * nlon;
  double sum = 0.0;
  for (int i = lane; i < nlon; i += 32) sum += g[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) rmean[row * nlat + j] = sum / (double)nlon;
}

bool fft_eddy_supported(int M) { return four_step_len(M) && !getenv("GD_FFT_STOCKHAM"); }

void launch_c2r_eddy(const ShtDev<float>& d, const FftPlan& plan, const float* FP, const double* FP0, long ldP,
                     const float* FH, const double* FH0, long ldH, double* grid, cudaStream_t s) {
  if (plan.njobs == 0) return;
  dim3 grd(plan.njobs, d.nlat);
  const SynthDesc* ds = (const SynthDesc*)plan.descs;
  constexpr int NR = nr4_of<float>();
  switch (d.M) {
#define GD_C2RE(MM, A, B)                                                                                    \
  case MM:                                                                                                   \
    k_c2r_4<float, MM, A, B, double><<<grd, nt4<MM, A, B>(NR), 0, s>>>(plan.jobs, ds, d, FP, ldP, FH, ldH, grid, \
                                                                       FP0, FH0);                            \
    break;
    GD_C2RE(64, 8, 8)
    GD_C2RE(96, 8, 12)
    GD_C2RE(192, 12, 16)
    GD_C2RE(384, 16, 24)
    GD_C2RE(576, 24, 24)
#undef GD_C2RE
    default:
      throw CudaError("eddy FFT: no four-step kernel for this longitude count");
  }
  count_launch();
  GD_LAUNCH_CHECK();
}

void launch_r2c_eddy(const ShtDev<float>& d, const FftPlan& plan, const double* grid, double* rmean,
                     const double* wn64, float* GP, double* GP0, long ldP, float* GH, double* GH0, long ldH,
                     cudaStream_t s) {
  if (plan.njobs == 0) return;
  dim3 grd(plan.njobs, d.nlat);
  const AnalDesc* ds = (const AnalDesc*)plan.descs;
  constexpr int NR = nr4_of<float>();
  k_rowmean<NR><<<grd, 32 * NR, 0, s>>>(plan.jobs, ds, d.nlat, d.nlon, grid, rmean);
  count_launch();
  GD_LAUNCH_CHECK();
  switch (d.M) {
#define GD_R2CE(MM, A, B)                                                                                     \
  case MM:                                                                                                    \
    k_r2c_4<float, MM, A, B, double><<<grd, nt4<MM, A, B>(NR), 0, s>>>(plan.jobs, ds, d, grid, GP, ldP, GH, ldH, \
                                                                       rmean, wn64, GP0, GH0);                \
    break;
    GD_R2CE(64, 8, 8)
    GD_R2CE(96, 8, 12)
    GD_R2CE(192, 12, 16)
    GD_R2CE(384, 16, 24)
    GD_R2CE(576, 24, 24)
#undef GD_R2CE
    default:
      throw CudaError("eddy FFT: no four-step kernel for this longitude count");
  }
  count_launch();
  GD_LAUNCH_CHECK();
}

}  // namespace gd

// gd_kernels.h -- host launchers of the dycore kernels (all on one stream).
#pragma once
#include <cuda_runtime.h>

#include "gd_common.cuh"

namespace gd {

// ---------------------------------------------------------------- grid / SHT
// Device description of the Gaussian grid and the transform tables.
template <typename R>
struct ShtDev {
  int T, nlon, nlat, nh, nlm, M;  // M = nlon / 2 (half-length complex FFT)
  const long* moff;               // [T+2] first spectral index of order m
  const long* toff;               // [T+2] first table element of order m
  const R* P;                     // [m][j<nh][n-m]  orthonormal P_n^m(mu_j)
  const R* H;                     // [m][j<nh][n-m]  dP_n^m/dphi
  const R* rcos;                  // [nlat] 1/cos(lat)
  const R* wn;                    // [nlat] 2 pi w_j / nlon
  const typename C2<R>::T* twM;   // [M]   exp(-2 pi i k / M)
  const typename C2<R>::T* twN;   // [M+1] exp(-2 pi i k / nlon)
  int nrad, rad[12];              // radix plan of M
};

// Stochastic-physics pattern (truncation pj <= T, FP32 coefficients) on the
// grid [nlat][nlon], logit-transformed as run.f90:281 does.
template <typename R>
void launch_pattern_grid(const ShtDev<R>& d, const float2* spec, int pj, R* out, cudaStream_t s);

// FP64 grid + table construction on the device.
void launch_gauss(int nlat, double* mu, double* w, cudaStream_t s);
void launch_legendre_tables(int T, int nh, const double* mu, const long* toff, double* P64, double* H64,
                            cudaStream_t s);
template <typename R>
void launch_convert(const double* src, R* dst, long n, cudaStream_t s);
// strided 2-D copy with a type change (rows x cols, row pitches lds / ldd)
template <typename S, typename D>
void launch_convert2d(const S* src, long lds, D* dst, long ldd, long rows, int cols, cudaStream_t s);
// dst[r][c] = sum_q src[q seg_stride + r lds + c] (q < nseg, FP64 sum in order q)
void launch_sumconvert(const float* src, long lds, long seg_stride, int nseg, double* dst, long ldd, long rows,
                       int cols, cudaStream_t s);

// Legendre stage, per-order SIMT GEMMs with the even/odd split.
// synthesis: F[m][j][c] = sum_{n} T[m][j][n-m] B[idx(n,m)][c]   (real columns)
// analysis : A[idx(n,m)][c] = sum_{j} T[m][j][n-m] G[m][j][c]    (N/S folded)
struct GemmPlan {
  int4* items = nullptr;  // device work list
  int nitems = 0;
};
// work lists over orders m in [m_lo, m_hi] (default: all orders)
GemmPlan make_synth_plan(int T, int nh, int ncols_real, cudaStream_t s, int m_lo = 0, int m_hi = -1);
GemmPlan make_anal_plan(int T, int ncols_real, cudaStream_t s, int m_lo = 0, int m_hi = -1);
void free_plan(GemmPlan& p);
template <typename R>
void launch_synth(const ShtDev<R>& d, bool useH, const GemmPlan& plan, const R* B, long ldB, int ncols_real,
                  R* F, long ldF, cudaStream_t s);
template <typename R>
void launch_anal(const ShtDev<R>& d, bool useH, const GemmPlan& plan, const R* G, long ldG, int ncols_real,
                 R* A, long ldA, cudaStream_t s);

// Longitude stage.
struct SynthDesc {  // a run of output grid rows
  int count;        // rows in the run
  int dst;          // first output grid row (grid[row][nlat][nlon])
  int srcA, colA;   // 0: P-Fourier, 1: H-Fourier, -1: none; first complex column
  int srcB, colB;   // term multiplied by i m / cos(lat)
  double alpha, beta;
};
struct AnalDesc {  // a run of input grid rows
  int count;
  int src;             // first input grid row
  int dstP, imcosP;    // complex column in GP (-1 none); multiply by i m/cos
  int dstH;            // complex column in GH (-1 none)
  double scaleP, scaleH;
};
struct FftPlan {
  int2* jobs = nullptr;
  void* descs = nullptr;
  int njobs = 0;
};
template <typename R>
int fft_rows_per_cta(int M);
template <typename R>
FftPlan make_c2r_plan(const SynthDesc* descs, int ndesc, cudaStream_t s, int M);
template <typename R>
FftPlan make_r2c_plan(const AnalDesc* descs, int ndesc, cudaStream_t s, int M);
void free_fft_plan(FftPlan& p);
template <typename R>
void launch_c2r(const ShtDev<R>& d, const FftPlan& plan, const R* FP, long ldP, const R* FH, long ldH, R* grid,
                cudaStream_t s);
template <typename R>
void launch_r2c(const ShtDev<R>& d, const FftPlan& plan, const R* grid, R* GP, long ldP, R* GH, long ldH,
                cudaStream_t s);
template <typename R>
void fft_init_tables(int nlon, typename C2<R>::T* twM, typename C2<R>::T* twN, cudaStream_t s);
// Eddy FFTs of the FP64-state mode (four-step lengths only, see
// fft_eddy_supported): orders m >= 1 in FP32 from / to the FP32 Fourier rows
// FP, FH (or GP, GH); order 0 in FP64 from / to FP0, FH0 (GP0, GH0), same
// pitches; FP64 grid.  Plans come from make_c2r_plan<float> /
// make_r2c_plan<float>.  rmean holds one double per (grid row, latitude)
// the r2c plan reads.
bool fft_eddy_supported(int M);
void launch_c2r_eddy(const ShtDev<float>& d, const FftPlan& plan, const float* FP, const double* FP0, long ldP,
                     const float* FH, const double* FH0, long ldH, double* grid, cudaStream_t s);
void launch_r2c_eddy(const ShtDev<float>& d, const FftPlan& plan, const double* grid, double* rmean,
                     const double* wn64, float* GP, double* GP0, long ldP, float* GH, double* GH0, long ldH,
                     cudaStream_t s);
void fft_radix_plan(int M, int* nrad, int* rad);

}  // namespace gd

// gd_tc.cuh -- split-precision (TF32x3 / BF16x3) Legendre GEMMs on the
// sm_103a tensor cores (tcgen05 + TMEM + TMA).  Declarations.
#pragma once
#include <cuda.h>

#include <array>

#include "gd_kernels.h"

namespace gd {

enum TcKind { TC_TF32 = 0, TC_BF16 = 1 };

// Tables and staging buffers of the tensor-core Legendre path for one grid.
struct TcPlan {
  int kind = TC_TF32;
  int T = 0, nh = 0, nlat = 0;
  int esize = 4;    // bytes per operand element (4 tf32, 2 bf16)
  int kc = 32;      // K elements per 128-byte swizzle row
  int kepad = 0;    // padded even/odd K extent of the synthesis tables
  int nhpad = 0;    // padded latitude extent of the analysis operands
  int nsyn = 0;     // N tile (latitudes) of the synthesis GEMM
  int nana = 0;     // N tile (degrees per parity) of the analysis GEMM
  int kirows = 0;   // rows per parity of the analysis tables
  int ncap = 0;     // real-column capacity of the staging buffers
  bool persistent = true;  // persistent warp-specialised GEMM (N <= 128)
  // fused TF32x3 GEMM: the hi*lo and lo*hi products in their own accumulator
  // (a third of the truncating accumulation steps in the main one); set by
  // the FP64-state modes (and GD_TC_SEPX) before tc_init (it bounds the N
  // tile)
  bool sepx = false;
  // fused TF32x3 GEMM: K segments of cps chunks per parity, accumulated afresh
  // and folded in FP32 (round to nearest) by the epilogue; 0 = none; set
  // before tc_init (it bounds the N tile)
  int cps = 0;
  // fused TF32x3 GEMM: A-operand slots in tensor memory requested (2..4; a
  // launch gets as many as fit beside its accumulators)
  int aslots = 2;
  // widest N tile tc_init chooses for the fused TF32x3 GEMM (tiles above 96
  // are single-buffered in TMEM); the autotuner may widen the synthesis tile
  int tile_cap = 96;
  // fused TF32x3 analysis: the latitude sum in aseg segments, each written as
  // FP32 partial sums to its own copy of the output (nlm x ldA floats apart),
  // to be added in the caller's precision; set by the FP64-state modes
  int aseg = 1;
  int nsm = 0;             // SMs of the device (persistent grid size)
  long xlen = 0;    // padded spectral length of the synthesis operand
  std::vector<long> xbase;  // [T+1] start of order m in the padded layout
  long* d_xbase = nullptr;
  // tables: synthesis [m][j][2*kepad], analysis [m][2*kirows][nhpad]; hi/lo
  void* tsyn[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [P/H][hi/lo]
  void* tana[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  // staging: X [ncap][xlen] hi/lo; G+- [T+1][ncap][nhpad] hi/lo
  void* x[2] = {nullptr, nullptr};
  void* gp[2] = {nullptr, nullptr};
  void* gm[2] = {nullptr, nullptr};
  CUtensorMap m_tsyn[2][2], m_tana[2][2], m_x[2], m_gp[2], m_gm[2];
  std::vector<std::pair<long, int4*>> item_cache;  // work lists by (ncols, direction)
  std::vector<std::pair<std::array<uint64_t, 9>, CUtensorMap>> raw_maps;  // fused-path maps by geometry
  int* d_xmap = nullptr;  // padded synthesis position -> spectral index (or -1)
  int* d_err = nullptr;   // device error flag (bounded waits)
  std::vector<void*> allocs;
};

// Builds tables (from the FP64 tables), staging buffers and tensor maps.
void tc_init(TcPlan& p, int kind, int T, int nh, int nlat, int ncap, const long* d_toff, const double* P64,
             const double* H64, cudaStream_t s);
void tc_free(TcPlan& p);
// the balanced tile at most cap wide over n rows (a multiple of 16)
int tc_tile_n(int n, int cap);
// largest N tile the plan's GEMM kernel takes (TMEM budget)
int tc_max_n(const TcPlan& p);
// A slots a fused launch at N tile n gets (the request, as far as TMEM holds)
int tc_slots(const TcPlan& p, int n);
// switches the synthesis GEMM to latitude tile nsyn (autotuning)
void tc_set_nsyn(TcPlan& p, int nsyn);

// F[m][j][c] (real columns c0.. of the GEMM) = Legendre synthesis of the
// real columns [0, ncols) of B[idx][.] (row pitch ldB, nrowsB rows
// allocated), tensor-core path.  The fused path reads B in pairs of rows,
// so it needs 2 floor(nrowsB / 2) >= nlm; otherwise the split path runs.
void tc_synth(TcPlan& p, const long* d_moff, bool useH, const float* B, long ldB, long nrowsB, int ncols, float* F,
              long ldF, cudaStream_t s);
// A[idx][c] = Legendre analysis of G[m][j][c] (real columns [0, ncols)).
void tc_anal(TcPlan& p, const long* d_moff, bool useH, const float* G, long ldG, int ncols, float* A, long ldA,
             cudaStream_t s);
// the K segments tc_anal uses (the plan's aseg, at most one per latitude chunk)
int tc_anal_segments(const TcPlan& p);
// returns and clears the device error flag (nonzero: a bounded wait gave up)
int tc_check(TcPlan& p, cudaStream_t s);

// One dense layer of the closure network on the tensor cores: for m < M,
// n < N, acc[m][n] = sum_k (Ah[m][k] + Al[m][k]) W[n][k], A split to TF32 hi +
// lo (row pitch Kp, a multiple of 32 with zeros past the layer's inputs), W
// exact in TF32 ([Np][Kp], Np = N rounded up to 16, zero rows past N), FP32
// accumulation in TMEM.  The epilogue adds the bias, then either applies GELU
// and writes the next layer's split operands (oh, ol, row pitch ldo) or
// writes FP32 outputs y (row pitch ldy).  N <= 256.
struct TcMlpLayer {
  CUtensorMap ah, al, w;
  int M = 0, N = 0, Np = 0, Kp = 0;
  const float* wbase = nullptr;  // the weights the map w covers ([Np][Kp])
  int wbox = 0;                  // N rows of the map's box (the N tile it was made for)
  const float* bias = nullptr;
  int gelu = 0;
  uint32_t* oh = nullptr;
  uint32_t* ol = nullptr;
  int ldo = 0;
  float* y = nullptr;
  int ldy = 0;
  int* err = nullptr;  // device flag: nonzero when a bounded wait gave up
  // training: mode 2, a hidden layer of the forward pass that also stores its
  // pre-activation z = A W^T + b and activation gelu(z) in FP32 ([M][ldz]);
  // mode 3, the backward product dZ_prev = (dZ W) * gelu'(zin) (no bias),
  // stored in FP32 to y and split hi + lo to oh / ol.  Mode 0: inference
  // (gelu selects a hidden layer or the output).
  int mode = 0;
  float* z = nullptr;
  float* act = nullptr;
  const float* zin = nullptr;
  int ldz = 0;
};
// tensor maps of a layer over its operand buffers (rows M of A)
void tc_mlp_maps(TcMlpLayer& L, const uint32_t* ah, const uint32_t* al, const float* w);
void tc_mlp_layer(const TcMlpLayer& L, cudaStream_t s);

// Weight gradient of a closure layer: part[s][m][n] = sum over the K chunks
// of slice s of A(m, k) B(n, k), both operands TF32 hi + lo rows with the
// batch (K) contiguous: A = dZ^T (Mp rows, a multiple of 128), B = the
// layer's input transposed (Np <= 256 rows).  Three products per K step
// (hi hi, hi lo, lo hi), FP32 accumulation in TMEM; the slices' partial
// tiles are summed afterwards in a fixed order.
struct TcWgrad {
  CUtensorMap ah, al, bh, bl;
  int Mp = 0, Np = 0;
  float* part = nullptr;  // [nsplit][Mp][Np]
  int* err = nullptr;
};
// maps over the transposed operands; kpitch = their row length (batch
// capacity, a multiple of 32)
void tc_wgrad_maps(TcWgrad& W, const uint32_t* ah, const uint32_t* al, const uint32_t* bh, const uint32_t* bl,
                   int kpitch);
// nk = K chunks of 32 in use, split over nsplit slices of cps chunks each
// (every slice non-empty)
void tc_wgrad(const TcWgrad& W, int nk, int cps, int nsplit, cudaStream_t s);

}  // namespace gd

// gd_dycore.cu -- host orchestration of the GB300 spectral dycore step and
// the C ABI of include/gd_api.h.
//
// Mirrors the reference's dynamics interface: init_dyn
// (src/dyn_init.f90:37-91), getdyntend (src/dyn_run.f90:33-305), advance
// (src/run.f90:194-565), getphytend for Held-Suarez (src/phy_run_hs.f90:22),
// finalize_dyn (src/dyn_finalize.f90:19-28), and the transform facade of
// src/shtns.f90.  All state lives on one GPU; one context owns one stream,
// and every step is one CUDA graph replay.
#include <algorithm>
#include <atomic>
#include <functional>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/gd_api.h"
#include "gd_grid.cuh"
#include "gd_kernels.h"
#include "gd_pattern.cuh"
#include "gd_dcmip.h"
#include "gd_physics.cuh"
#include "gd_mlp.cuh"
#include "gd_spec.cuh"
#include "gd_tc.cuh"
#include <type_traits>

namespace gd {

// Lorenz 3-cycle + trapezoidal IMEX tableau (src/semimp_data.f90:74-88),
// single-precision literals as in the reference.
struct Tableau {
  double a21 = GD_FLIT(1.f / 3.f), a31 = GD_FLIT(1.f / 6.f), a32 = GD_FLIT(1.f / 2.f);
  double aa21 = GD_FLIT(1.f / 6.f), aa22 = GD_FLIT(1.f / 6.f), aa31 = GD_FLIT(1.f / 3.f), aa32 = 0.0,
         aa33 = GD_FLIT(1.f / 3.f);
  double b1 = GD_FLIT(1.f / 2.f), b2 = GD_FLIT(-1.f / 2.f), b3 = 1.0;
  double bb1 = GD_FLIT(3.f / 8.f), bb2 = 0.0, bb3 = GD_FLIT(3.f / 8.f), bb4 = GD_FLIT(1.f / 4.f);
};

class DycoreBase {
 public:
  virtual ~DycoreBase() {}
  virtual void set_state(const double*, const double*, const double*, const double*, const double*,
                         const double*) = 0;
  virtual void get_state(double*, double*, double*, double*, double*) = 0;
  // single-precision host arrays (the reference's default complex(4) / real(4))
  virtual void set_state(const float*, const float*, const float*, const float*, const float*, const float*) = 0;
  virtual void get_state(float*, float*, float*, float*, float*) = 0;
  virtual void getdyntend(int, int, double*, double*, double*, double*, double*) = 0;
  virtual void getphytend(double*, double*, double*, double*, double*) = 0;
  virtual void advance(int nsteps) = 0;
  virtual void set_iau(int nf, const double* fhrs, double delthrs, const double* vrt, const double* div,
                       const double* tv, const double* trc, const double* lnps) = 0;
  virtual void dfi(double t, int ntdfi) = 0;
  double t_cur = 0.0;  // model time (s) of the next step, for the IAU forcing
  virtual void spectogrd(int, const double*, double*) = 0;
  virtual void grdtospec(int, const double*, double*) = 0;
  virtual void getuv(int, const double*, const double*, double*, double*) = 0;
  virtual void getvrtdivspec(int, const double*, const double*, double*, double*) = 0;
  virtual void getgrad(int, const double*, double*, double*) = 0;
  virtual void spectogrd(int, const float*, float*) = 0;
  virtual void grdtospec(int, const float*, float*) = 0;
  virtual void getuv(int, const float*, const float*, float*, float*) = 0;
  virtual void getvrtdivspec(int, const float*, const float*, float*, float*) = 0;
  virtual void getgrad(int, const float*, float*, float*) = 0;
  virtual void grid_info(double*, double*, double*, int*, int*, double*, double*) = 0;
  virtual int get_grid(const char*, double*) = 0;
  virtual void diag(double*) = 0;
  virtual void profile_step(double*, int) = 0;
  virtual void check() = 0;
  virtual void set_sppt(gd_pattern*, double, double) = 0;
  virtual void set_closure(gd_mlp*) = 0;
  virtual void autotune(int*) = 0;
  // For gd_ensemble_advance's one launch over all members: the captured step
  // graph and its capture epoch, when this context can take part (a step has
  // been captured, no per-step host work such as the IAU forcing); and the
  // host bookkeeping of one step taken inside the ensemble graph.
  virtual bool ensemble_step_graph(cudaGraph_t* g, unsigned long long* epoch) = 0;
  virtual void ensemble_step_done() = 0;
  const unsigned long long uid = next_uid();  // unique over the process (addresses are reused)
  static unsigned long long next_uid() {
    static std::atomic<unsigned long long> n{0};
    return ++n;
  }
  virtual void closure_features(float*) = 0;
  virtual double get_pdryini() = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = true;
  std::string err;
};

// set_dfi_wts (run.f90:567-588): Lanczos-windowed sinc weights over 2 n + 1
// steps, normalised to sum 1.  The angles are single precision, as
// acos(-1.) * (k - n) / n is for a literal without a kind suffix.
void dfi_weights(int n, double* w) {
  const float pif = 3.14159265358979323846f;
  double tot = 0.0;
  for (int k = 0; k <= 2 * n; ++k) {
    const double sx = (double)(pif * (float)(k - n) / (float)n);
    const double wx = (double)(pif * (float)(k - n) / (float)(n + 1));
    w[k] = (k != n) ? sin(wx) / wx * sin(sx) / sx : 1.0;
    tot += w[k];
  }
  for (int k = 0; k <= 2 * n; ++k) w[k] = w[k] / tot;
}

template <typename R>
class Dycore : public DycoreBase {
 public:
  typedef typename C2<R>::T V;
  gd_config c;
  int T, nlon, nlat, nh, L, nt, nlm, M;
  long ng;
  std::vector<void*> allocs;
  // grid and tables
  double *mu = nullptr, *w = nullptr;
  long *moff = nullptr, *toff = nullptr;
  R *P = nullptr, *H = nullptr, *rcos = nullptr, *wn = nullptr, *sinlat = nullptr, *coslat = nullptr;
  V *twM = nullptr, *twN = nullptr;
  ShtDev<R> sd;
  std::vector<double> h_mu, h_w, h_lat;
  std::vector<int> h_deg, h_ord;
  std::vector<double> h_lap;
  // vertical coordinate, damping, semi-implicit matrices
  R *ak = nullptr, *bk = nullptr, *dbk = nullptr, *ck = nullptr;
  R *lapv = nullptr, *disspec = nullptr, *diff_prof = nullptr, *dmp_prof = nullptr;
  R *amhyb = nullptr, *bmhyb = nullptr, *svhyb = nullptr, *tor = nullptr, *dhyb = nullptr;
  // state and work buffers
  R *S = nullptr, *S0 = nullptr, *TD[3] = {nullptr, nullptr, nullptr}, *AP = nullptr, *AH = nullptr;
  R *FPb = nullptr, *FHb = nullptr, *gS = nullptr, *gA = nullptr;
  R *psg = nullptr, *dlnpsdt = nullptr, *dlnpdtg = nullptr, *etadot = nullptr, *prs = nullptr;
  R *dphisdx = nullptr, *dphisdy = nullptr;
  // DCMIP simple physics (phy_data.f90): latitude, precipitation rate,
  // precipitable water, accumulated precipitation
  R *latr = nullptr, *precip = nullptr, *pwat = nullptr, *apcp = nullptr;
  double *pmoist = nullptr, *pwatg = nullptr;
  bool simple() const { return c.dcmip >= 0 && !c.dry; }
  double *pdryini = nullptr, *pmean = nullptr, *rowsum = nullptr, *diagbuf = nullptr, *diagout = nullptr;
  int4* stage_items = nullptr;
  int nstage_items = 0;
  SpecCols sc;
  TendCols tc;
  APCols ap;
  AHCols ah;
  SynthRows sr;
  AnalRows ar;
  long ldS, ldTD, ldAP, ldAH, ldFP, ldFH, ldGP, ldGH;
  long nlm_rows = 0;  // allocated rows of the synthesis sources: nlm rounded up to even
  GemmPlan synP, synH, anaP, anaH, anaPhys, anaSimple;
  FftPlan c2rFull, c2rInv, r2cDyn, r2cPhys, r2cSimple, r2cClos;
  Tableau tb;
  // per-phase CUDA-event profiling of one eager step (gd_profile_step)
  enum { PH_LSYN, PH_FSYN, PH_COL, PH_FANA, PH_LANA, PH_SEMI, PH_PHYS, PH_OTHER, PH_CPHYS, PH_N };
  bool profiling = false;
  std::vector<std::pair<int, cudaEvent_t>> marks;
  std::vector<cudaEvent_t> evpool;
  void mark(int ph) {
    if (!profiling) return;
    if (marks.size() >= evpool.size()) {
      cudaEvent_t e;
      GD_CUDA(cudaEventCreate(&e));
      evpool.push_back(e);
    }
    cudaEvent_t e = evpool[marks.size()];
    GD_CUDA(cudaEventRecord(e, stream));
    marks.push_back({ph, e});
  }
  bool state_set = false;
  cudaGraphExec_t gexec = nullptr;
  cudaGraph_t gstep = nullptr;  // the captured step (kept for gd_ensemble_advance's ensemble graph)
  unsigned long long graph_epoch = 0;  // counts captures: an ensemble graph built on an older one is stale
  void drop_graph() {
    if (gexec) {
      GD_CUDA(cudaStreamSynchronize(stream));
      GD_CUDA(cudaGraphExecDestroy(gexec));
      gexec = nullptr;
    }
    if (gstep) {
      GD_CUDA(cudaGraphDestroy(gstep));
      gstep = nullptr;
    }
    ++graph_epoch;
  }
  int steps_done = 0;
  long long launches_per_step = 0;
  std::map<int, GemmPlan> synth_cache, anal_cache;
  // tensor-core split-precision Legendre path: FP32 state (TF32x3, BF16x3)
  // or FP64 state with FP32 staging copies around the GEMM (F64_TF32X3)
  std::unique_ptr<TcPlan> tcp;
  double *P64keep = nullptr, *H64keep = nullptr;
  bool split_mode() const {
    return c.precision == GD_PREC_TF32X3 || c.precision == GD_PREC_BF16X3 || c.precision == GD_PREC_F64_TF32X3 ||
           c.precision == GD_PREC_F64_EDDY;
  }
  // K segments of the tensor-core GEMMs in the FP64-state modes (the
  // truncating FP32 accumulation in tensor memory over all 288 degrees or
  // latitudes of T574 was the modes' largest error): segments of
  // kFoldChunks K chunks, each accumulated afresh and folded in FP32 (round
  // to nearest) by the GEMM's epilogue.  Without folding (GD_TC_FOLD_CHUNKS=0)
  // the analysis' latitude sum goes in kAnalSegments segments to global
  // memory, added in FP64.  Both are read from the environment at init.
  static constexpr int kFoldChunks = 1;
  static constexpr int kAnalSegments = 4;
  static int env_int(const char* name, int dflt) {
    const char* e = getenv(name);
    return (e && *e) ? atoi(e) : dflt;
  }
  // FP32 staging of the FP64-state split modes: spectral side (GEMM operand
  // of the synthesis, result of the analysis) and the Fourier side of the P
  // and H buffers (FPb, FHb)
  float *stSpec = nullptr, *stFourP = nullptr, *stFourH = nullptr;
  float* stFour(const R* F) const { return (const void*)F == (const void*)FHb ? stFourH : stFourP; }
  // eddy FFTs (GD_PREC_F64_EDDY on a four-step grid): FP32 tables of the
  // longitude stage and the FP64 row means of the analysis
  bool eddy_ = false;
  ShtDev<float> sdf;
  double* rmean = nullptr;
  template <typename D>
  FftPlan mk_c2r(const D* descs, int n) {
    return eddy_ ? make_c2r_plan<float>(descs, n, stream, M) : make_c2r_plan<R>(descs, n, stream, M);
  }
  template <typename D>
  FftPlan mk_r2c(const D* descs, int n) {
    return eddy_ ? make_r2c_plan<float>(descs, n, stream, M) : make_r2c_plan<R>(descs, n, stream, M);
  }
  void c2r(const FftPlan& plan, const R* FP, long ldP, const R* FH, long ldH, R* grid) {
    if constexpr (std::is_same<R, double>::value) {
      if (eddy_) {
        launch_c2r_eddy(sdf, plan, stFour(FP), FP, ldP, stFour(FH), FH, ldH, grid, stream);
        return;
      }
    }
    launch_c2r<R>(sd, plan, FP, ldP, FH, ldH, grid, stream);
  }
  void r2c(const FftPlan& plan, const R* grid, R* GP, long ldP, R* GH, long ldH) {
    if constexpr (std::is_same<R, double>::value) {
      if (eddy_) {
        launch_r2c_eddy(sdf, plan, grid, rmean, wn, stFour(GP), GP, ldP, stFour(GH), GH, ldH, stream);
        return;
      }
    }
    launch_r2c<R>(sd, plan, grid, GP, ldP, GH, ldH, stream);
  }
  std::map<int, GemmPlan> synth0_cache, anal0_cache;  // order-0-only SIMT work lists
  // Side stream of the split modes: order 0 runs on the SIMT path beside the
  // tensor-core GEMM of orders m >= 1 (disjoint output rows; the small SIMT
  // CTAs fit in the SM resources the persistent GEMM leaves free).  Forked
  // and joined with events on the context's stream, so a graph captured on
  // that stream captures both branches.
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  void fork() {
    GD_CUDA(cudaEventRecord(ev_fork, stream));
    GD_CUDA(cudaStreamWaitEvent(side, ev_fork, 0));
  }
  void join() {
    GD_CUDA(cudaEventRecord(ev_join, side));
    GD_CUDA(cudaStreamWaitEvent(stream, ev_join, 0));
  }
  void do_synth(bool useH, const GemmPlan& plan, const R* B, long ldB, int ncr, R* F, long ldF) {
    if (tcp) {
      auto it = synth0_cache.find(ncr);
      if (it == synth0_cache.end()) it = synth0_cache.emplace(ncr, make_synth_plan(T, nh, ncr, stream, 0, 0)).first;
      if constexpr (std::is_same<R, float>::value) {
        fork();
        tc_synth(*tcp, moff, useH, B, ldB, nlm_rows, ncr, F, ldF, stream);
        launch_synth<R>(sd, useH, it->second, B, ldB, ncr, F, ldF, side);
        join();
      } else {
        // FP64 state: the GEMM of orders m >= 1 reads an FP32 copy of the
        // spectral columns and writes FP32 Fourier rows, widened after it;
        // order 0 runs on the FP64 SIMT path straight into F
        // (the eddy FFT reads the FP32 rows where the GEMM left them)
        launch_convert2d<double, float>(B, ldB, stSpec, ldB, nlm_rows, ncr, stream);
        fork();
        tc_synth(*tcp, moff, useH, stSpec, ldB, nlm_rows, ncr, stFour(F), ldF, stream);
        launch_synth<R>(sd, useH, it->second, B, ldB, ncr, F, ldF, side);
        join();
        if (!eddy_)
          launch_convert2d<float, double>(stFour(F) + (long)nlat * ldF, ldF, F + (long)nlat * ldF, ldF,
                                          (long)T * nlat, ncr, stream);
      }
      return;
    }
    launch_synth<R>(sd, useH, plan, B, ldB, ncr, F, ldF, stream);
  }
  void do_anal(bool useH, const GemmPlan& plan, const R* G, long ldG, int ncr, R* A, long ldA) {
    if (tcp) {
      auto it = anal0_cache.find(ncr);
      if (it == anal0_cache.end()) it = anal0_cache.emplace(ncr, make_anal_plan(T, ncr, stream, 0, 0)).first;
      if constexpr (std::is_same<R, float>::value) {
        fork();
        tc_anal(*tcp, moff, useH, G, ldG, ncr, A, ldA, stream);
        launch_anal<R>(sd, useH, it->second, G, ldG, ncr, A, ldA, side);
        join();
      } else {
        // FP64 state: FP32 copy of every Fourier row (order 0 included, so the
        // GEMM reads no stale staging), FP32 result rows of orders m >= 1
        // (spectral rows T+1.. in the m-major order) widened after it
        // (the eddy FFT already wrote the FP32 rows, with zeros for order 0)
        if (!eddy_) launch_convert2d<double, float>(G, ldG, stFour(G), ldG, (long)(T + 1) * nlat, ncr, stream);
        fork();
        tc_anal(*tcp, moff, useH, stFour(G), ldG, ncr, stSpec, ldA, stream);
        launch_anal<R>(sd, useH, it->second, G, ldG, ncr, A, ldA, side);
        join();
        // the analysis GEMM's K segments are added here in FP64
        launch_sumconvert(stSpec + (long)(T + 1) * ldA, ldA, (long)nlm * ldA, tc_anal_segments(*tcp),
                          A + (long)(T + 1) * ldA, ldA, (long)nlm - (T + 1), ncr, stream);
      }
      return;
    }
    launch_anal<R>(sd, useH, plan, G, ldG, ncr, A, ldA, stream);
  }
  void check() override {
    tc_status();
    if (closure) mlp_check(closure, stream);
  }
  void tc_status() {
    if (tcp && tc_check(*tcp, stream))
      throw CudaError("tensor-core Legendre pipeline: a bounded wait gave up (results invalid)");
  }

  template <typename X>
  X* dalloc(size_t n) {
    X* p = nullptr;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(X));
    if (e != cudaSuccess) throw CudaError(std::string("cudaMalloc: ") + cudaGetErrorString(e));
    allocs.push_back(p);
    return p;
  }
  template <typename X>
  X* upload(const std::vector<X>& h) {
    X* p = dalloc<X>(h.size());
    GD_CUDA(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(X), cudaMemcpyHostToDevice, stream));
    return p;
  }
  std::vector<R> toR(const std::vector<double>& v) {
    std::vector<R> r(v.size());
    for (size_t i = 0; i < v.size(); ++i) r[i] = (R)v[i];
    return r;
  }
  static long pad2(long ncol) { return 2 * ((ncol + 1) / 2 * 2); }  // reals, even complex count

  Dycore(const gd_config& cfg, const double* ak_, const double* bk_) : c(cfg) {
    T = c.ntrunc;
    nlon = c.nlon;
    nlat = c.nlat;
    nh = nlat / 2;
    L = c.nlev;
    nt = c.ntrac;
    nlm = (T + 1) * (T + 2) / 2;
    M = nlon / 2;
    ng = (long)nlon * nlat;
    GD_CUDA(cudaSetDevice(c.device));
    GD_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    eddy_ = sizeof(R) == 8 && c.precision == GD_PREC_F64_EDDY && fft_eddy_supported(M);
    init_grid();
    init_vertical(ak_, bk_);
    init_buffers();
    init_plans();
    if (split_mode()) {
      GD_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
      GD_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
      GD_CUDA(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
      tcp.reset(new TcPlan());
      // widest N tile at init (GD_TC_TILE_CAP: a tuning and measurement knob)
      tcp->tile_cap = std::max(16, env_int("GD_TC_TILE_CAP", tcp->tile_cap) / 16 * 16);
      const int ncap = 2 * std::max(sc.ncol, ap.ncol);
      if constexpr (std::is_same<R, float>::value) {
        // GD_TC_SEPX=1: the cross products in their own accumulator here too
        // (a tuning and measurement knob; the FP64-state modes always do it)
        tcp->sepx = c.precision == GD_PREC_TF32X3 && env_int("GD_TC_SEPX", 0) != 0;
        tc_init(*tcp, c.precision == GD_PREC_TF32X3 ? TC_TF32 : TC_BF16, T, nh, nlat, ncap, toff, P64keep, H64keep,
                stream);
      } else {
        // the FP64 tables are the state precision's own; the staging copies
        // take the widest row pitch any synthesis or analysis call uses
        tcp->sepx = true;  // these choose the N tiles: set before tc_init
        tcp->cps = std::max(0, env_int("GD_TC_FOLD_CHUNKS", kFoldChunks));
        tcp->aseg = std::max(1, env_int("GD_TC_ANAL_SEGMENTS", tcp->cps > 0 ? 1 : kAnalSegments));
        tc_init(*tcp, TC_TF32, T, nh, nlat, ncap, toff, P, H, stream);
        const long ldmax = std::max(std::max(std::max(ldS, ldAP), std::max(ldAH, ldFP)), std::max(ldGP, ldGH));
        const size_t nfour = (size_t)(T + 1) * nlat * ldmax;
        stSpec = dalloc<float>((size_t)tc_anal_segments(*tcp) * nlm_rows * ldmax);
        stFourP = dalloc<float>(nfour);
        stFourH = dalloc<float>(nfour);
        GD_CUDA(cudaMemsetAsync(stSpec, 0, sizeof(float) * tc_anal_segments(*tcp) * nlm_rows * ldmax, stream));
        GD_CUDA(cudaMemsetAsync(stFourP, 0, sizeof(float) * nfour, stream));
        GD_CUDA(cudaMemsetAsync(stFourH, 0, sizeof(float) * nfour, stream));
      }
      release(P64keep);
      release(H64keep);
      P64keep = H64keep = nullptr;
    }
    GD_CUDA(cudaStreamSynchronize(stream));
  }
  ~Dycore() override {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (gstep) cudaGraphDestroy(gstep);
    if (tcp) tc_free(*tcp);
    for (auto e : evpool) cudaEventDestroy(e);
    free_plan(synP);
    free_plan(synH);
    free_plan(anaP);
    free_plan(anaH);
    free_plan(anaPhys);
    for (auto& kv : synth_cache) free_plan(kv.second);
    for (auto& kv : anal_cache) free_plan(kv.second);
    for (auto& kv : synth0_cache) free_plan(kv.second);
    for (auto& kv : anal0_cache) free_plan(kv.second);
    free_fft_plan(c2rFull);
    free_fft_plan(c2rInv);
    free_fft_plan(r2cDyn);
    free_fft_plan(r2cPhys);
    free_plan(anaSimple);
    free_fft_plan(r2cSimple);
    free_fft_plan(r2cClos);
    if (stream) cudaStreamSynchronize(stream);
    if (side) cudaStreamSynchronize(side);
    for (void* p : allocs) cudaFree(p);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (side) cudaStreamDestroy(side);
    if (stream && own_stream) cudaStreamDestroy(stream);
  }

  // --- shtns_init (shtns.f90:90-156): nodes, weights, tables, all FP64 ---
  void init_grid() {
    std::vector<long> hm(T + 2), ht(T + 2);
    hm[0] = ht[0] = 0;
    for (int m = 0; m <= T; ++m) {
      hm[m + 1] = hm[m] + (T - m + 1);
      ht[m + 1] = ht[m] + (long)(T - m + 1) * nh;
    }
    moff = upload(hm);
    toff = upload(ht);
    mu = dalloc<double>(nlat);
    w = dalloc<double>(nlat);
    launch_gauss(nlat, mu, w, stream);
    double* P64 = dalloc<double>(ht[T + 1]);
    double* H64 = dalloc<double>(ht[T + 1]);
    launch_legendre_tables(T, nh, mu, toff, P64, H64, stream);
    if (sizeof(R) == 8) {
      P = reinterpret_cast<R*>(P64);
      H = reinterpret_cast<R*>(H64);
    } else {
      P = dalloc<R>(ht[T + 1]);
      H = dalloc<R>(ht[T + 1]);
      launch_convert<R>(P64, P, ht[T + 1], stream);
      launch_convert<R>(H64, H, ht[T + 1], stream);
    }
    h_mu.resize(nlat);
    h_w.resize(nlat);
    GD_CUDA(cudaMemcpyAsync(h_mu.data(), mu, nlat * sizeof(double), cudaMemcpyDeviceToHost, stream));
    GD_CUDA(cudaMemcpyAsync(h_w.data(), w, nlat * sizeof(double), cudaMemcpyDeviceToHost, stream));
    GD_CUDA(cudaStreamSynchronize(stream));
    if (sizeof(R) != 8) {  // FP64 copies: kept only to split for the tensor-core path
      if (split_mode()) {
        P64keep = P64;
        H64keep = H64;
      } else {
        release(P64);
        release(H64);
      }
    }
    std::vector<double> rc(nlat), wnv(nlat), sl(nlat), cl(nlat);
    h_lat.resize(nlat);
    for (int j = 0; j < nlat; ++j) {
      h_lat[j] = asin(h_mu[j]);
      rc[j] = 1.0 / sqrt((1.0 - h_mu[j]) * (1.0 + h_mu[j]));
      wnv[j] = 2.0 * M_PI * h_w[j] / nlon;
      sl[j] = sin(h_lat[j]);
      cl[j] = cos(h_lat[j]);
    }
    rcos = upload(toR(rc));
    wn = upload(toR(wnv));
    sinlat = upload(toR(sl));
    coslat = upload(toR(cl));
    latr = upload(toR(h_lat));
    twM = dalloc<V>(M);
    twN = dalloc<V>(M + 1);
    fft_init_tables<R>(nlon, twM, twN, stream);
    h_deg.resize(nlm);
    h_ord.resize(nlm);
    h_lap.resize(nlm);
    for (int m = 0, k = 0; m <= T; ++m)
      for (int n = m; n <= T; ++n, ++k) {
        h_deg[k] = n;
        h_ord[k] = m;
        h_lap[k] = -(double)n * (n + 1.0);
      }
    lapv = upload(toR(h_lap));
    sd.T = T;
    sd.nlon = nlon;
    sd.nlat = nlat;
    sd.nh = nh;
    sd.nlm = nlm;
    sd.M = M;
    sd.moff = moff;
    sd.toff = toff;
    sd.P = P;
    sd.H = H;
    sd.rcos = rcos;
    sd.wn = wn;
    sd.twM = twM;
    sd.twN = twN;
    fft_radix_plan(M, &sd.nrad, sd.rad);
    if (eddy_) {
      std::vector<float> rcf(nlat), wnf(nlat);
      for (int j = 0; j < nlat; ++j) rcf[j] = (float)rc[j], wnf[j] = (float)wnv[j];
      sdf.T = T, sdf.nlon = nlon, sdf.nlat = nlat, sdf.nh = nh, sdf.nlm = nlm, sdf.M = M;
      sdf.moff = moff, sdf.toff = toff, sdf.P = nullptr, sdf.H = nullptr;
      sdf.rcos = upload(rcf);
      sdf.wn = upload(wnf);
      float2* tmf = dalloc<float2>(M);
      float2* tnf = dalloc<float2>(M + 1);
      fft_init_tables<float>(nlon, tmf, tnf, stream);
      sdf.twM = tmf, sdf.twN = tnf;
      sdf.nrad = sd.nrad;
      for (int i = 0; i < 12; ++i) sdf.rad[i] = sd.rad[i];
    }
  }

  // --- pressure_data / setdampspec / init_semimpdata ---
  void init_vertical(const double* ak_, const double* bk_) {
    std::vector<double> a(ak_, ak_ + L + 1), b(bk_, bk_ + L + 1), db(L), ckv(L), si(L + 1), slv(L);
    for (int k = 0; k < L; ++k) {  // dyn_init.f90:57-61
      db[k] = b[k + 1] - b[k];
      ckv[k] = a[k + 1] * b[k] - a[k] * b[k + 1];
    }
    ak = upload(toR(a));
    bk = upload(toR(b));
    dbk = upload(toR(db));
    ck = upload(toR(ckv));
    for (int k = 0; k <= L; ++k) si[L - k] = a[k] / 101300.0 + b[k];  // pressure_data.f90:65-67
    for (int k = 0; k < L; ++k) slv[k] = 0.5 * (si[k] + si[k + 1]);
    sl_levels = slv;
    // setdampspec (dyn_init.f90:450-494)
    int ndiss = c.ndiss == 0 ? 8 : c.ndiss;
    double efold = c.efold, fshk = c.fshk;
    const double RE = Phys::rerth;
    if (efold <= 0) {
      if (T > 170) {
        float x = (float)T / 170.f;
        float x4 = (x * x) * (x * x);
        efold = 3600. / (c.hdif_fac2 * (double)x4 * GD_FLIT(1.1f));
      } else if (T == 126 || T == 170) {
        efold = 1. / (c.hdif_fac2 * GD_FLIT(12.E15f) / pow(RE, 4) * 41990400.0);
      } else {
        efold = 1. / (c.hdif_fac2 * GD_FLIT(3.E15f) / pow(RE, 4) * 41990400.0);
      }
      efold = 2. * efold;
    }
    if (fshk <= 0) {
      fshk = 1.0 * c.hdif_fac;
      if (T > 170) fshk = GD_FLIT(2.2f) * c.hdif_fac;
      if (T == 126) fshk = GD_FLIT(1.5f) * c.hdif_fac;
    }
    const double slrd0 = GD_FLIT(0.002f), dmp1 = 1. / c.taustratdamp;
    std::vector<double> dp(L), mp(L, 0.0), dis(nlm);
    for (int k = 0; k < L; ++k) {
      dp[k] = pow(slv[k], log(1. / fshk));
      if (slv[k] < slrd0) mp[k] = dmp1 * log(slrd0 / slv[k]);
    }
    double minlap = *std::min_element(h_lap.begin(), h_lap.end());
    for (int k = 0; k < nlm; ++k) {
      double r = h_lap[k] / minlap, rp = 1.0;
      for (int q = 0; q < ndiss / 2; ++q) rp *= r;
      dis[k] = -(1. / efold) * rp;
    }
    diff_prof = upload(toR(dp));
    dmp_prof = upload(toR(mp));
    disspec = upload(toR(dis));
    // semi-implicit reference-state operators (semimp_data.f90:174-234)
    const double RD = Phys::rd, KAPPA = Phys::rd / Phys::cp, TREF = 300.0, PREF = 800.e2;
    std::vector<double> pkref(L + 1), dpkref(L), alfaref(L), yecm((long)L * L, 0), tecm((long)L * L, 0), vecm(L);
    for (int k = 0; k <= L; ++k) pkref[k] = a[k] + b[k] * PREF;
    for (int k = 0; k < L; ++k) dpkref[k] = pkref[k + 1] - pkref[k];
    alfaref[0] = GD_FLIT(logf(2.f));
    for (int k = 1; k < L; ++k) alfaref[k] = 1. - (pkref[k] / dpkref[k]) * log(pkref[k + 1] / pkref[k]);
    for (int i = 0; i < L; ++i) {
      yecm[(long)i * L + i] = alfaref[i] * RD;
      for (int j = i + 1; j < L; ++j) yecm[(long)i * L + j] = RD * log(pkref[j + 1] / pkref[j]);
      tecm[(long)i * L + i] = KAPPA * TREF * alfaref[i];
      for (int j = 0; j < i; ++j)
        tecm[(long)i * L + j] = (KAPPA * TREF * dpkref[j] / dpkref[i]) * log(pkref[i + 1] / pkref[i]);
    }
    for (int k = 0; k < L; ++k) vecm[k] = dpkref[k] / PREF;
    std::vector<double> am((long)L * L), bm((long)L * L), sv(L), to(L);
    for (int j = 0; j < L; ++j) {
      sv[j] = vecm[L - 1 - j];
      for (int k = 0; k < L; ++k) {
        am[(long)k * L + j] = yecm[(long)(L - 1 - k) * L + (L - 1 - j)];
        bm[(long)k * L + j] = tecm[(long)(L - 1 - k) * L + (L - 1 - j)];
      }
    }
    for (auto& x : am) x /= RE * RE;
    for (int k = 0; k < L; ++k) to[k] = RD * TREF / (RE * RE);
    // the state arithmetic uses these in r_kind; ym is formed in FP64 from
    // the r_kind values (semimp_data.f90:130,216-234)
    for (auto* v : {&am, &bm, &sv, &to})
      for (auto& x : *v) x = (double)(R)x;
    // the stage kernel reads the L x L operators transposed (coalesced over
    // the output level): upload A^T, B^T, and invert Y^T = (inv Y)^T below
    std::vector<double> amT((long)L * L), bmT((long)L * L);
    for (int i = 0; i < L; ++i)
      for (int j = 0; j < L; ++j) {
        amT[(long)j * L + i] = am[(long)i * L + j];
        bmT[(long)j * L + i] = bm[(long)i * L + j];
      }
    amhyb = upload(toR(amT));
    bmhyb = upload(toR(bmT));
    svhyb = upload(toR(sv));
    tor = upload(toR(to));
    std::vector<double> ym((long)L * L);
    for (int i = 0; i < L; ++i) {
      for (int j = 0; j < L; ++j) ym[(long)i * L + j] = to[i] * sv[j];
      for (int k = 0; k < L; ++k)
        for (int j = 0; j < L; ++j) ym[(long)i * L + j] += am[(long)i * L + k] * bm[(long)k * L + j];
    }
    const double consts[3] = {tb.aa22, tb.aa33, tb.bb4};
    std::vector<double> Y((long)3 * (T + 1) * L * L);
    for (int s = 0; s < 3; ++s)
      for (int n = 0; n <= T; ++n) {
        double f = (consts[s] * c.dt) * (consts[s] * c.dt) * ((double)n * (n + 1));
        double* y = &Y[((long)s * (T + 1) + n) * L * L];
        for (int i = 0; i < L; ++i)
          for (int j = 0; j < L; ++j) y[(long)i * L + j] = (i == j ? 1.0 : 0.0) + f * ym[(long)j * L + i];
      }
    double* dY = dalloc<double>(Y.size());
    GD_CUDA(cudaMemcpyAsync(dY, Y.data(), Y.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
    launch_batched_inverse(dY, 3 * (T + 1), L, stream);  // FP64 on the GPU
    if (sizeof(R) == 8) {
      dhyb = reinterpret_cast<R*>(dY);
    } else {
      dhyb = dalloc<R>(Y.size());
      launch_convert<R>(dY, dhyb, (long)Y.size(), stream);
    }
    GD_CUDA(cudaStreamSynchronize(stream));
  }

  void init_buffers() {
    sc.vrt = 0;
    sc.div = L;
    sc.tv = 2 * L;
    sc.trc = 3 * L;
    sc.s = (3 + nt) * L;
    sc.c = (4 + nt) * L;
    sc.lnps = (5 + nt) * L;
    sc.ncol = (5 + nt) * L + 1;
    tc.dvrt = 0;
    tc.ddiv = L;
    tc.dtv = 2 * L;
    tc.dtrc = 3 * L;
    tc.dlnps = (3 + nt) * L;
    tc.ddl = (3 + nt) * L + 1;
    tc.dtl = (4 + nt) * L + 1;
    tc.dpl = (5 + nt) * L + 1;
    tc.ncol = (5 + nt) * L + 2;
    ap.ttend = 0;
    ap.ke = L;
    ap.qtend = 2 * L;
    ap.dlnps = (2 + nt) * L;
    ap.imfv = (2 + nt) * L + 1;
    ap.imfu = (3 + nt) * L + 1;
    ap.ncol = (4 + nt) * L + 1;
    ah.fu = 0;
    ah.mfv = L;
    ah.ncol = 2 * L;
    sr.vrt = 0;
    sr.div = L;
    sr.tv = 2 * L;
    sr.trc = 3 * L;
    sr.u = (3 + nt) * L;
    sr.v = (4 + nt) * L;
    sr.dtvdx = (5 + nt) * L;
    sr.dtvdy = (6 + nt) * L;
    sr.dqdx = (7 + nt) * L;
    sr.dqdy = (7 + 2 * nt) * L;
    sr.lnps = (7 + 3 * nt) * L;
    sr.dlnpsdx = sr.lnps + 1;
    sr.dlnpsdy = sr.lnps + 2;
    sr.total = sr.lnps + 3;
    ar.ttend = 0;
    ar.ke = L;
    ar.qtend = 2 * L;
    ar.dlnps = (2 + nt) * L;
    ar.fu = (2 + nt) * L + 1;
    ar.fv = (3 + nt) * L + 1;
    ar.total = (4 + nt) * L + 1;
    ldS = pad2(sc.ncol);
    ldTD = pad2(tc.ncol);
    ldAP = pad2(ap.ncol);
    ldAH = pad2(ah.ncol);
    ldFP = pad2(sc.ncol);
    ldFH = pad2(sc.ncol - 2 * L);
    ldGP = pad2(ap.ncol);
    ldGH = pad2(ah.ncol);
    nlm_rows = nlm + (nlm & 1);  // the tensor-core synthesis reads rows in pairs
    S = dalloc<R>((size_t)nlm_rows * ldS);
    S0 = dalloc<R>((size_t)nlm * ldS);
    GD_CUDA(cudaMemsetAsync(S, 0, sizeof(R) * nlm_rows * ldS, stream));
    for (int i = 0; i < 3; ++i) TD[i] = dalloc<R>((size_t)nlm * ldTD);
    AP = dalloc<R>((size_t)nlm * ldAP);
    AH = dalloc<R>((size_t)nlm * ldAH);
    const long nf = (long)(T + 1) * nlat;
    FPb = dalloc<R>((size_t)nf * std::max(std::max(ldFP, ldGP), ldS));
    // the transform API writes both Fourier buffers with the S row pitch
    FHb = dalloc<R>((size_t)nf * std::max(std::max(ldFH, ldGH), ldS));
    gS = dalloc<R>((size_t)sr.total * ng);
    gA = dalloc<R>((size_t)ar.total * ng);
    if (eddy_) rmean = dalloc<double>((size_t)ar.total * nlat);  // one mean per analysed (row, latitude)
    psg = dalloc<R>(ng);
    dlnpsdt = dalloc<R>(ng);
    dlnpdtg = dalloc<R>((size_t)L * ng);
    etadot = dalloc<R>((size_t)(L + 1) * ng);
    prs = dalloc<R>((size_t)L * ng);
    dphisdx = dalloc<R>(ng);
    dphisdy = dalloc<R>(ng);
    GD_CUDA(cudaMemsetAsync(dphisdx, 0, sizeof(R) * ng, stream));
    GD_CUDA(cudaMemsetAsync(dphisdy, 0, sizeof(R) * ng, stream));
    pdryini = dalloc<double>(1);
    pmean = dalloc<double>(1);
    pmoist = dalloc<double>(1);
    pwatg = dalloc<double>(1);
    precip = dalloc<R>(ng);
    pwat = dalloc<R>(ng);
    apcp = dalloc<R>(ng);
    for (R* z : {precip, pwat, apcp}) GD_CUDA(cudaMemsetAsync(z, 0, sizeof(R) * ng, stream));
    rowsum = dalloc<double>(nlat);
    diagbuf = dalloc<double>(4 * nlat);
    diagout = dalloc<double>(8);
    GD_CUDA(cudaMemcpyAsync(pdryini, &c.pdryini, sizeof(double), cudaMemcpyHostToDevice, stream));
    auto items = make_stage_items(T, GD_STAGE_QC);
    nstage_items = (int)items.size();
    stage_items = upload(items);
  }

  void init_plans() {
    synP = make_synth_plan(T, nh, 2 * sc.ncol, stream);
    synH = make_synth_plan(T, nh, 2 * (sc.ncol - 2 * L), stream);
    anaP = make_anal_plan(T, 2 * ap.ncol, stream);
    anaH = make_anal_plan(T, 2 * ah.ncol, stream);
    anaPhys = make_anal_plan(T, 2 * (3 * L + 1), stream);
    const double ai = 1.0 / Phys::rerth;
    const int h0 = 2 * L;  // FH column = S column - 2L
    std::vector<SynthDesc> full = {
        {L, sr.vrt, 0, sc.vrt, -1, 0, 1.0, 0.0},
        {L, sr.div, 0, sc.div, -1, 0, 1.0, 0.0},
        {L, sr.tv, 0, sc.tv, -1, 0, 1.0, 0.0},
        {L, sr.u, 1, sc.s - h0, 0, sc.c, -1.0, 1.0},
        {L, sr.v, 1, sc.c - h0, 0, sc.s, 1.0, 1.0},
        {L, sr.dtvdx, -1, 0, 0, sc.tv, 0.0, ai},
        {L, sr.dtvdy, 1, sc.tv - h0, -1, 0, ai, 0.0},
        {1, sr.lnps, 0, sc.lnps, -1, 0, 1.0, 0.0},
        {1, sr.dlnpsdx, -1, 0, 0, sc.lnps, 0.0, ai},
        {1, sr.dlnpsdy, 1, sc.lnps - h0, -1, 0, ai, 0.0},
    };
    if (nt > 0) {
      full.push_back({nt * L, sr.trc, 0, sc.trc, -1, 0, 1.0, 0.0});
      full.push_back({nt * L, sr.dqdx, -1, 0, 0, sc.trc, 0.0, ai});
      full.push_back({nt * L, sr.dqdy, 1, sc.trc - h0, -1, 0, ai, 0.0});
    }
    c2rFull = mk_c2r(full.data(), (int)full.size());
    std::vector<SynthDesc> inv = {
        full[0], full[1], full[2], full[3], full[4], full[7], full[8], full[9],
    };
    if (nt > 0) inv.push_back(full[10]);
    c2rInv = mk_c2r(inv.data(), (int)inv.size());
    std::vector<AnalDesc> an = {
        {L, ar.ttend, ap.ttend, 0, -1, 1.0, 0.0},
        {L, ar.ke, ap.ke, 0, -1, 1.0, 0.0},
        {1, ar.dlnps, ap.dlnps, 0, -1, 1.0, 0.0},
        {L, ar.fu, ap.imfu, 1, ah.fu, 1.0, 1.0},
        {L, ar.fv, ap.imfv, 1, ah.mfv, 1.0, -1.0},
    };
    if (nt > 0) an.push_back({nt * L, ar.qtend, ap.qtend, 0, -1, 1.0, 0.0});
    r2cDyn = mk_r2c(an.data(), (int)an.size());
    AnalDesc ph = {3 * L + 1, 0, 0, 0, -1, 1.0, 0.0};
    r2cPhys = mk_r2c(&ph, 1);
    if (simple()) {
      // grid rows: Tv [0,L), q [L,2L), u [2L,3L), v [3L,4L), fixer 4L.  As in
      // getvrtdivspec: GP gets i m/cos V (vorticity) and i m/cos U
      // (divergence), GH gets U and -V.
      std::vector<AnalDesc> sd_ = {
          {L, 0, 0, 0, -1, 1.0, 0.0},
          {L, L, L, 0, -1, 1.0, 0.0},
          {L, 2 * L, 3 * L + 1, 1, 0, 1.0, 1.0},
          {L, 3 * L, 2 * L + 1, 1, L, 1.0, -1.0},
      };
      if (c.massfix) sd_.push_back({1, 4 * L, 2 * L, 0, -1, 1.0, 0.0});
      r2cSimple = mk_r2c(sd_.data(), (int)sd_.size());
      anaSimple = make_anal_plan(T, 2 * (4 * L + 1), stream);
    }
  }

  // ------------------------------------------------------------ passes --
  void synthesis(const FftPlan& plan) {
    do_synth(false, synP, S, ldS, 2 * sc.ncol, FPb, ldFP);
    do_synth(true, synH, S + 2 * (2 * L), ldS, 2 * (sc.ncol - 2 * L), FHb, ldFH);
    mark(PH_LSYN);
    c2r(plan, FPb, ldFP, FHb, ldFH, gS);
    mark(PH_FSYN);
  }
  ColumnArgs<R> column_args(bool want_extra) {
    ColumnArgs<R> a;
    a.L = L;
    a.nt = nt;
    a.nlon = nlon;
    a.nlat = nlat;
    a.dry = c.dry;
    a.ak = ak;
    a.bk = bk;
    a.dbk = dbk;
    a.ck = ck;
    a.sinlat = sinlat;
    a.coslat = coslat;
    a.gS = gS;
    a.s = sr;
    a.dphisdx = dphisdx;
    a.dphisdy = dphisdy;
    a.gA = gA;
    a.a = ar;
    a.psg = psg;
    a.dlnpsdt = dlnpsdt;
    a.dlnpdtg = want_extra ? dlnpdtg : nullptr;
    a.etadot = want_extra ? etadot : nullptr;
    a.prs = want_extra ? prs : nullptr;
    a.kappa = (R)(Phys::rd / Phys::cp);
    a.rd = (R)Phys::rd;
    a.cvap_cp = (R)(Phys::cvap / Phys::cp - 1.0);
    a.omega2 = (R)(2.0 * Phys::omega);
    a.log2sp = (R)GD_FLIT(logf(2.f));
    a.rlnp_top = (R)GD_FLIT(99999.99f);
    return a;
  }
  // getdyntend: transforms to the grid, column physics, transforms back
  void dyn_pass(int stage, bool want_extra) {
    synthesis(c2rFull);
    launch_dyn_columns<R>(column_args(want_extra), false, stream, col_lb);
    if (stage == 0) {  // pdry on stage 1 (dyn_run.f90:135-153)
      launch_area_mean_ps<R>(psg, w, nlat, nlon, rowsum, pmean, stream);
      const bool moist = !c.dry && nt > 0;
      if (moist)
        launch_area_pmoist<R>(gS + (long)sr.trc * ng, c.dcmip > 0 ? 1 : nt, L, psg, ak, bk, w, nlat, nlon, rowsum,
                              pmoist, stream);
      launch_pdry_init(pmean, moist ? pmoist : nullptr, pdryini, stream);
    }
    mark(PH_COL);
    r2c(r2cDyn, gA, FPb, ldGP, FHb, ldGH);
    mark(PH_FANA);
    do_anal(false, anaP, FPb, ldGP, 2 * ap.ncol, AP, ldAP);
    do_anal(true, anaH, FHb, ldGH, 2 * ah.ncol, AH, ldAH);
    mark(PH_LANA);
  }
  void inverse_pass(bool want_extra) {
    synthesis(c2rInv);
    launch_dyn_columns<R>(column_args(want_extra), true, stream, col_lb);
    mark(PH_COL);
  }
  StageArgs<R> stage_args(int s) {
    StageArgs<R> a;
    a.L = L;
    a.nt = nt;
    a.T = T;
    a.stage = s;
    a.explicit_ = c.explicit_;
    a.final_ = (s == 2);
    a.items = stage_items;
    a.nitems = nstage_items;
    a.moff = moff;
    a.S = S;
    a.S0 = S0;
    a.ldS = ldS;
    a.AP = AP;
    a.ldAP = ldAP;
    a.AH = AH;
    a.ldAH = ldAH;
    a.TD0 = TD[0];
    a.TD1 = TD[1];
    a.TD2 = TD[2];
    a.ldTD = ldTD;
    a.amhyb = amhyb;
    a.bmhyb = bmhyb;
    a.svhyb = svhyb;
    a.tor = tor;
    a.dhyb = dhyb;
    a.disspec = disspec;
    a.diff_prof = diff_prof;
    a.dmp_prof = dmp_prof;
    a.dt = (R)c.dt;
    a.ainv = (R)(1.0 / Phys::rerth);
    a.ainv2 = (R)(1.0 / (Phys::rerth * Phys::rerth));
    a.rerth = (R)Phys::rerth;
    double ce[3][3] = {{tb.a21, 0, 0}, {tb.a31, tb.a32, 0}, {tb.b1, tb.b2, tb.b3}};
    double ci[3][3] = {{tb.aa21, 0, 0}, {tb.aa31, tb.aa32, 0}, {tb.bb1, tb.bb2, tb.bb3}};
    double cimp[3] = {tb.aa22, tb.aa33, fabs(tb.bb4) > 1.e-5 ? tb.bb4 : 0.0};
    for (int r = 0; r < 3; ++r) {
      a.ce[r] = (R)ce[s][r];
      a.ci[r] = c.explicit_ ? R(0) : (R)ci[s][r];
    }
    a.cimp = c.explicit_ ? R(0) : (R)cimp[s];
    a.F = iau_nf ? iau_F : nullptr;
    a.sc = sc;
    a.tc = tc;
    a.ap = ap;
    a.ah = ah;
    return a;
  }
  HsArgs<R> hs_args() {
    HsArgs<R> h;
    h.L = L;
    h.nlon = nlon;
    h.nlat = nlat;
    h.ak = ak;
    h.bk = bk;
    h.sinlat = sinlat;
    h.coslat = coslat;
    h.gS = gS;
    h.s = sr;
    h.gA = gA;
    h.kappa = (R)(Phys::rd / Phys::cp);
    h.sigbot = (R)GD_FLIT(0.7f);  // phy_run_hs.f90:42-49
    h.kdrag = (R)GD_FLIT(1.f / (1.f * 86400.f));
    h.krada = (R)GD_FLIT(1.f / (40.f * 86400.f));
    h.kradb = (R)GD_FLIT(1.f / (4.f * 86400.f));
    h.expo = (R)GD_FLIT(2.f / 7.f);
    h.sppt = sppt ? spptg : nullptr;
    h.vfact = vfact_d;
    return h;
  }
  SimpleArgs<R> simple_args() {
    SimpleArgs<R> a;
    a.L = L;
    a.nlon = nlon;
    a.nlat = nlat;
    a.ak = ak;
    a.bk = bk;
    a.dbk = dbk;
    a.lat = latr;
    a.gS = gS;
    a.s = sr;
    a.psg = psg;
    a.gA = gA;
    a.precip = precip;
    a.pwat = pwat;
    a.apcp = apcp;
    a.dt = (R)c.dt;
    a.test = (c.dcmip / 10 == 4) ? 1 : 0;
    a.turbflux = (c.dcmip == 43 || c.dcmip / 10 == 5) ? 1 : 0;
    a.fvirt = (R)(Phys::rv / Phys::rd - 1.0);
    a.qmin = (R)GD_FLIT(1.e-10f);
    a.grav = (R)Phys::grav;
    a.kappa = (R)(Phys::rd / Phys::cp);
    return a;
  }
  // DCMIP simple physics on the grid, its increments analysed (scalar Tv and
  // q, vector u, v) with the dry-mass fixer row
  void simple_pass() {
    launch_simple_physics<R>(simple_args(), stream);
    mark(PH_CPHYS);
    if (c.massfix) {
      launch_area_mean_ps<R>(psg, w, nlat, nlon, rowsum, pmean, stream);
      launch_area_mean_ps<R>(pwat, w, nlat, nlon, rowsum, pwatg, stream);
      launch_massfix_grid<R>(psg, pdryini, pmean, pwatg, Phys::grav, (int)ng, gA + (long)4 * L * ng, stream);
    }
    mark(PH_PHYS);
    r2c(r2cSimple, gA, FPb, ldGP, FHb, ldGH);
    mark(PH_FANA);
    do_anal(false, anaSimple, FPb, ldGP, 2 * (4 * L + 1), AP, ldAP);
    do_anal(true, anaH, FHb, ldGH, 2 * ah.ncol, AH, ldAH);
    mark(PH_LANA);
  }
  void phys_pass() {
    inverse_pass(false);
    if (simple()) {
      simple_pass();
      launch_simple_update<R>(S, ldS, sc, L, nlm, AP, ldAP, AH, ldAH, c.massfix, 1, (R)c.dt, (R)(1.0 / Phys::rerth),
                              lapv, (R)Phys::rerth, stream);
      mark(PH_PHYS);
      return;
    }
    if (c.heldsuarez) launch_hs_forcing<R>(hs_args(), stream);
    if (c.massfix) {
      launch_area_mean_ps<R>(psg, w, nlat, nlon, rowsum, pmean, stream);
      launch_massfix_grid<R>(psg, pdryini, pmean, nullptr, Phys::grav, (int)ng, gA + (long)3 * L * ng, stream);
    }
    mark(PH_PHYS);
    if (c.heldsuarez || c.massfix) {
      r2c(r2cPhys, gA, FPb, ldGP, FHb, ldGH);
      mark(PH_FANA);
      do_anal(false, anaPhys, FPb, ldGP, 2 * (3 * L + 1), AP, ldAP);
      mark(PH_LANA);
      launch_phys_update<R>(S, ldS, sc, L, nt, nlm, AP, ldAP, c.massfix, c.heldsuarez, (R)c.dt, lapv,
                            (R)Phys::rerth, stream);
      mark(PH_PHYS);
    }
    if (closure) closure_pass();
  }
  // Autotuning: the column kernel's levels per warp, and (split modes) the
  // synthesis GEMM's latitude tile together with the tensor-memory A slots of
  // both GEMMs, each chosen by timing its candidates on this context's own
  // buffers (the transform rows of the current state; a tile and slot count
  // by one synthesis and one analysis of the step).  The choices hold for the
  // context's later steps.  GD_AUTOTUNE_VERBOSE=1 prints every candidate's
  // time to stderr.
  int col_lb = 0;
  void autotune(int* out) override {
    if (!state_set) throw std::runtime_error("state not set (gd_set_state)");
    GD_CUDA(cudaStreamSynchronize(stream));
    cudaEvent_t e0, e1;
    GD_CUDA(cudaEventCreate(&e0));
    GD_CUDA(cudaEventCreate(&e1));
    auto timed = [&](const std::function<void()>& f) {
      f();  // warm-up
      GD_CUDA(cudaEventRecord(e0, stream));
      for (int r = 0; r < 3; ++r) f();
      GD_CUDA(cudaEventRecord(e1, stream));
      GD_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      GD_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      return ms;
    };
    synthesis(c2rFull);  // the grid rows the column kernel reads
    float best = 1e30f;
    int blb = 4;
    for (int lb : {4, 8}) {
      if (lb == 4 && L > 64) continue;
      const float ms = timed([&] { launch_dyn_columns<R>(column_args(false), false, stream, lb); });
      if (ms < best) best = ms, blb = lb;
    }
    col_lb = blb;
    if (tcp) {
      std::vector<int> tiles;
      for (int cap : {48, 64, 80, 96, 128, 144, 192}) {
        if (cap > tc_max_n(*tcp)) continue;  // beyond the GEMM kernel's TMEM budget
        const int n = tc_tile_n(nh, cap);
        if (std::find(tiles.begin(), tiles.end(), n) == tiles.end()) tiles.push_back(n);
      }
      const bool verbose = env_int("GD_AUTOTUNE_VERBOSE", 0) != 0;
      best = 1e30f;
      int bn = tcp->nsyn, bs = tcp->aslots;
      for (int na : {2, 3, 4}) {
        tcp->aslots = na;
        for (int n : tiles) {
          // a count that fits neither GEMM's tile is a candidate already timed
          if (na > 2 && tc_slots(*tcp, n) < na && tc_slots(*tcp, tcp->nana) < na) continue;
          tc_set_nsyn(*tcp, n);
          const float ms = timed([&] {
            do_synth(false, synP, S, ldS, 2 * sc.ncol, FPb, ldFP);
            do_synth(true, synH, S + 2 * (2 * L), ldS, 2 * (sc.ncol - 2 * L), FHb, ldFH);
            do_anal(false, anaP, FPb, ldGP, 2 * ap.ncol, AP, ldAP);
            do_anal(true, anaH, FHb, ldGH, 2 * ah.ncol, AH, ldAH);
          });
          if (verbose)
            fprintf(stderr, "autotune: synthesis tile %d, A slots %d/%d (synthesis/analysis): %.3f ms\n", n,
                    tc_slots(*tcp, n), tc_slots(*tcp, tcp->nana), ms / 3);
          if (ms < best) best = ms, bn = n, bs = na;
        }
      }
      tcp->aslots = bs;
      tc_set_nsyn(*tcp, bn);
      tc_status();
    }
    GD_CUDA(cudaEventDestroy(e0));
    GD_CUDA(cudaEventDestroy(e1));
    out[0] = tcp ? tcp->nsyn : 0;
    out[1] = col_lb;
    out[2] = tcp ? tcp->aslots : 0;
    drop_graph();  // the captured step changes
    steps_done = 0;  // the next step runs eagerly (new work lists), the one after is captured
  }
  // Learned closure: the attached net's tendencies from the grid columns of
  // the step's inverse transform (the state before the forcing, as the
  // forcing sees it), times dt, analysed as in the column-physics update (Tv
  // scalar, u and v through the vector analysis) and added to the state.
  gd_mlp* closure = nullptr;
  float *clos_x = nullptr, *clos_y = nullptr;
  void closure_pass() {
    const float *imu, *isd, *omu, *osd;
    mlp_norm(closure, &imu, &isd, &omu, &osd);
    launch_closure_in<R>(gS, sr, L, ng, imu, isd, clos_x, stream);
    mlp_forward_on(closure, clos_x, (int)ng, clos_y, stream);
    launch_closure_out<R>(clos_y, L, ng, omu, osd, (R)c.dt, gA, stream);
    mark(PH_PHYS);
    r2c(r2cClos, gA, FPb, ldGP, FHb, ldGH);
    mark(PH_FANA);
    do_anal(false, anaSimple, FPb, ldGP, 2 * (4 * L + 1), AP, ldAP);
    do_anal(true, anaH, FHb, ldGH, 2 * ah.ncol, AH, ldAH);
    mark(PH_LANA);
    launch_simple_update<R>(S, ldS, sc, L, nlm, AP, ldAP, AH, ldAH, 0, 0, (R)c.dt, (R)(1.0 / Phys::rerth), lapv,
                            (R)Phys::rerth, stream);
    mark(PH_PHYS);
  }
  void closure_buffers() {
    if (!clos_x) clos_x = dalloc<float>((size_t)ng * (3 * L + 1));
    if (!clos_y) clos_y = dalloc<float>((size_t)ng * 3 * L);
  }
  void set_closure(gd_mlp* net) override {
    if (net) {
      if (mlp_device(net) != c.device) throw std::invalid_argument("gd_set_closure: net on another device");
      if (mlp_nin(net) != 3 * L + 1 || mlp_nout(net) != 3 * L)
        throw std::invalid_argument("gd_set_closure: need nin = 3 nlev + 1 and nout = 3 nlev");
      const float *a, *b, *d, *e;
      if (!mlp_norm(net, &a, &b, &d, &e)) throw std::invalid_argument("gd_set_closure: net has no normalisation");
      if (simple()) throw std::invalid_argument("gd_set_closure: not with the DCMIP simple physics");
      GD_CUDA(cudaStreamSynchronize(stream));
      closure_buffers();
      mlp_reserve(net, (int)ng);
      if (!r2cClos.jobs) {  // grid rows Tv [0,L), u [2L,3L), v [3L,4L) as in the column-physics update
        std::vector<AnalDesc> cd = {
            {L, 0, 0, 0, -1, 1.0, 0.0},
            {L, 2 * L, 3 * L + 1, 1, 0, 1.0, 1.0},
            {L, 3 * L, 2 * L + 1, 1, L, 1.0, -1.0},
        };
        r2cClos = mk_r2c(cd.data(), (int)cd.size());
      }
      if (!anaSimple.items) anaSimple = make_anal_plan(T, 2 * (4 * L + 1), stream);
      GD_CUDA(cudaStreamSynchronize(stream));
    }
    closure = net;
    drop_graph();  // the captured step changes
    steps_done = 0;  // the next step runs eagerly (the net's kernels set their attributes), then is captured
  }
  void closure_features(float* x) override {
    if (!state_set) throw std::runtime_error("state not set (gd_set_state)");
    closure_buffers();
    inverse_pass(false);
    launch_closure_in<R>(gS, sr, L, ng, nullptr, nullptr, clos_x, stream);
    GD_CUDA(cudaMemcpyAsync(x, clos_x, sizeof(float) * (size_t)ng * (3 * L + 1), cudaMemcpyDeviceToHost, stream));
    GD_CUDA(cudaStreamSynchronize(stream));
  }
  // Stochastically perturbed physics: an attached pattern (gd_pattern) is
  // advanced one step at the start of every step and put on the grid with the
  // logit transform (run.f90:277-281); the physics tendencies are scaled by
  // 1 + vfact(k) * pattern (phy_run_gfs.f90:617-620), vfact tapering to 0
  // between sigma sigbot and sigtop (stoch_data.f90:86-94).
  gd_pattern* sppt = nullptr;
  R* spptg = nullptr;
  R* vfact_d = nullptr;
  std::vector<double> sl_levels;
  void set_sppt(gd_pattern* p, double sigtop, double sigbot) override {
    if (p) {
      if (pattern_device(p) != c.device) throw std::invalid_argument("gd_set_sppt: pattern on another device");
      if (pattern_jcap(p) > T) throw std::invalid_argument("gd_set_sppt: pattern truncation above the model's");
      if (!(sigbot > sigtop)) throw std::invalid_argument("gd_set_sppt: need sigbot > sigtop");
      std::vector<double> vf(L);
      for (int k = 0; k < L; ++k) {
        const double s = sl_levels[k];
        vf[k] = 1.0;
        if (s < sigbot && s > sigtop)
          vf[k] = (s - sigtop) / (sigbot - sigtop);
        else if (s <= sigtop)
          vf[k] = 0.0;
      }
      if (!spptg) spptg = dalloc<R>(ng);
      if (!vfact_d) vfact_d = dalloc<R>(L);
      std::vector<R> vr(vf.begin(), vf.end());
      GD_CUDA(cudaMemcpyAsync(vfact_d, vr.data(), sizeof(R) * L, cudaMemcpyHostToDevice, stream));
      GD_CUDA(cudaStreamSynchronize(stream));
    }
    sppt = p;
    drop_graph();  // the captured step changes
  }
  // IAU (iau_module.f90): increments analysis - first guess at nf times,
  // a forcing interpolated in time, constant over the RK stages of a step
  R *iau_inc = nullptr, *iau_F = nullptr;
  int iau_nf = 0;
  std::vector<double> iau_fh;
  double iau_delthrs = 6.0;
  void set_iau(int nf, const double* fhrs, double delthrs, const double* vrt, const double* div, const double* tv,
               const double* trc, const double* lnps) override {
    if (nf == 0) {
      iau_nf = 0;
    } else {
      if (nf < 2) throw std::invalid_argument("IAU needs at least two times");
      for (int n = 1; n < nf; ++n)
        if (fhrs[n] - fhrs[n - 1] != fhrs[1] - fhrs[0])
          throw std::invalid_argument("IAU times must be equally spaced (iau_module.f90:41-46)");
      if (!(delthrs > 0)) throw std::invalid_argument("IAU interval must be positive");
      if (!vrt || !div || !tv || !lnps || (nt > 0 && !trc)) throw std::invalid_argument("IAU increments missing");
      const long per = (long)nlm * ldS;
      if (iau_inc) release(iau_inc);
      iau_inc = dalloc<R>((size_t)nf * per);
      GD_CUDA(cudaMemsetAsync(iau_inc, 0, sizeof(R) * nf * per, stream));
      if (!iau_F) iau_F = dalloc<R>((size_t)per);
      GD_CUDA(cudaMemsetAsync(iau_F, 0, sizeof(R) * per, stream));
      double* st = staging();
      const long nS = 2L * nlm * L, nT = 2L * nlm * L * nt, nP = 2L * nlm;
      for (int n = 0; n < nf; ++n) {
        R* dst = iau_inc + n * per;
        auto put = [&](const double* h, int nb, int col) {
          GD_CUDA(cudaMemcpyAsync(st, h, sizeof(double) * 2 * (long)nb * nlm, cudaMemcpyHostToDevice, stream));
          launch_ref2int<R>(st, nb, nlm, dst, ldS, col, stream);
          GD_CUDA(cudaStreamSynchronize(stream));
        };
        put(vrt + n * nS, L, sc.vrt);
        put(div + n * nS, L, sc.div);
        put(tv + n * nS, L, sc.tv);
        if (nt > 0) put(trc + n * nT, nt * L, sc.trc);
        put(lnps + n * nP, 1, sc.lnps);
      }
      iau_fh.assign(fhrs, fhrs + nf);
      iau_delthrs = delthrs;
      iau_nf = nf;
    }
    drop_graph();  // the captured step changes
  }
  // getiauforcing (iau_module.f90:88-135) at time t into iau_F
  void iau_forcing(double t) {
    const int nf = iau_nf;
    const double dtiau = iau_delthrs * 3600.;
    int ia = 0, ib = 0;
    double ca = 0.0, cb = 0.0;
    if (t < iau_fh[0] * 3600. || t > iau_fh[nf - 1] * 3600.) {
      // outside the window: no forcing
    } else if (t == 3600. * iau_fh[nf - 1]) {
      ia = nf - 1, ca = 1.0;
    } else if (t == 3600. * iau_fh[0]) {
      ia = 0, ca = 1.0;
    } else {
      int n = 0;
      while (n < nf && !(iau_fh[n] * 3600. > t)) ++n;
      const double delt = (iau_fh[n] - (t / 3600.)) / (iau_fh[n] - iau_fh[n - 1]);
      ia = n, ca = 1. - delt;
      ib = n - 1, cb = delt;
    }
    launch_iau_forcing<R>(iau_F, iau_inc, ldS, sc, (3 + nt) * L, nlm, ia, ca, ib, cb, dtiau, stream);
  }
  // Digital filter initialisation (run.f90:58-145): 2 ntdfi steps from t,
  // the Lanczos-weighted average of the states (FP64 accumulator) becomes
  // the state, valid at t + ntdfi dt; accumulated precipitation restarts
  // (init_phydata).
  void dfi(double t, int ntdfi) override {
    if (!state_set) throw std::runtime_error("state not set (gd_set_state)");
    std::vector<double> wts(2 * ntdfi + 1);
    dfi_weights(ntdfi, wts.data());
    const int ncs = (3 + nt) * L;
    double* acc = dalloc<double>(2L * nlm * (ncs + 1));
    t_cur = t;
    launch_dfi_acc<R>(acc, S, ldS, sc, ncs, nlm, wts[0], 1, stream);
    for (int k = 1; k <= 2 * ntdfi; ++k) {
      advance(1);
      launch_dfi_acc<R>(acc, S, ldS, sc, ncs, nlm, wts[k], 0, stream);
    }
    launch_dfi_set<R>(S, ldS, sc, ncs, nlm, acc, stream);
    launch_sc<R>(S, ldS, sc, L, nlm, lapv, (R)Phys::rerth, stream);
    GD_CUDA(cudaMemsetAsync(apcp, 0, sizeof(R) * ng, stream));
    GD_CUDA(cudaStreamSynchronize(stream));
    release(acc);
    t_cur = t + ntdfi * c.dt;
  }
  // advance (run.f90:194-565)
  void step() {
    mark(-1);
    if (sppt) {
      pattern_advance_on(sppt, 1, stream);
      launch_pattern_grid<R>(sd, pattern_spec(sppt), pattern_jcap(sppt), spptg, stream);
    }
    GD_CUDA(cudaMemcpyAsync(S0, S, sizeof(R) * nlm * ldS, cudaMemcpyDeviceToDevice, stream));
    mark(PH_OTHER);
    for (int s = 0; s < 3; ++s) {
      dyn_pass(s, false);
      launch_stage<R>(stage_args(s), stream);
      mark(PH_SEMI);
    }
    if (!c.adiabatic) phys_pass();
  }
  // one eager step with CUDA events between phases; ms[ph] accumulates
  void profile_step(double* ms, int n) override {
    if (!state_set) throw std::runtime_error("state not set (gd_set_state)");
    for (int i = 0; i < n; ++i) ms[i] = 0;
    if (iau_nf) iau_forcing(t_cur);
    t_cur += c.dt;
    marks.clear();
    profiling = true;
    step();
    profiling = false;
    GD_CUDA(cudaStreamSynchronize(stream));
    for (size_t i = 1; i < marks.size(); ++i) {
      float t = 0;
      GD_CUDA(cudaEventElapsedTime(&t, marks[i - 1].second, marks[i].second));
      int ph = marks[i].first;
      if (ph == PH_CPHYS && n <= PH_CPHYS) ph = PH_PHYS;  // callers with 8 phases: within physics
      if (ph >= 0 && ph < n) ms[ph] += t;
    }
    ++steps_done;
  }
  bool ensemble_step_graph(cudaGraph_t* g, unsigned long long* epoch) override {
    const bool capturable = stream != nullptr && stream != cudaStreamLegacy && stream != cudaStreamPerThread;
    if (!state_set || !capturable || !gexec || !gstep || steps_done == 0 || iau_nf) return false;
    *g = gstep;
    *epoch = graph_epoch;
    return true;
  }
  void ensemble_step_done() override {
    t_cur += c.dt;
    g_launches += launches_per_step;
    ++steps_done;
  }
  void advance(int nsteps) override {
    if (!state_set) throw std::runtime_error("state not set (gd_set_state)");
    for (int i = 0; i < nsteps; ++i) {
      if (iau_nf) iau_forcing(t_cur);  // outside the captured step: its coefficients change with time
      t_cur += c.dt;
      // the legacy default stream cannot be captured: launch eagerly there
      const bool capturable = stream != nullptr && stream != cudaStreamLegacy && stream != cudaStreamPerThread;
      if (!capturable) {
        step();
      } else if (steps_done == 0 || gexec == nullptr) {
        if (steps_done == 0) {  // first step eagerly (sets kernel attributes)
          long long l0 = g_launches;
          step();
          launches_per_step = g_launches - l0;
        } else {
          cudaGraph_t g;
          GD_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
          step();
          GD_CUDA(cudaStreamEndCapture(stream, &g));
          GD_CUDA(cudaGraphInstantiate(&gexec, g, 0));
          if (gstep) GD_CUDA(cudaGraphDestroy(gstep));
          gstep = g;
          ++graph_epoch;
          g_launches -= launches_per_step;  // counted once per replay below
          GD_CUDA(cudaGraphLaunch(gexec, stream));
          g_launches += launches_per_step;
        }
      } else {
        GD_CUDA(cudaGraphLaunch(gexec, stream));
        g_launches += launches_per_step;
      }
      ++steps_done;
    }
  }

  // ------------------------------------------------------------ state --
  // Persistent FP64 staging area in the reference layout: one region per
  // field, so host copies of all fields are in flight together.
  double* staging_ = nullptr;
  double* staging() {
    if (!staging_) staging_ = dalloc<double>(2L * nlm * ((3 + nt) * (long)L + 1));
    return staging_;
  }
  void set_state(const double* vrt, const double* div, const double* tv, const double* trc, const double* lnps,
                 const double* topo) override {
    set_state_t(vrt, div, tv, trc, lnps, topo);
  }
  void set_state(const float* vrt, const float* div, const float* tv, const float* trc, const float* lnps,
                 const float* topo) override {
    std::vector<double> t64;
    if (topo) t64.assign(topo, topo + 2 * (size_t)nlm);
    set_state_t(vrt, div, tv, trc, lnps, topo ? t64.data() : nullptr);
  }
  void get_state(double* vrt, double* div, double* tv, double* trc, double* lnps) override {
    get_state_t(vrt, div, tv, trc, lnps);
  }
  void get_state(float* vrt, float* div, float* tv, float* trc, float* lnps) override {
    get_state_t(vrt, div, tv, trc, lnps);
  }
  // H: the host element type (double, or float for the single-precision
  // entry points); host arrays are copied as they are and converted on the
  // device, so a float caller moves half the bytes
  template <typename H>
  void set_state_t(const H* vrt, const H* div, const H* tv, const H* trc, const H* lnps, const double* topo) {
    if (nt > 0 && !trc) throw std::invalid_argument("trc is NULL but ntrac > 0");
    H* st = reinterpret_cast<H*>(staging());
    long off = 0;
    auto put = [&](const H* h, int nb, int col) {
      H* d = st + off;
      GD_CUDA(cudaMemcpyAsync(d, h, sizeof(H) * 2 * (long)nb * nlm, cudaMemcpyHostToDevice, stream));
      launch_ref2int<R>(d, nb, nlm, S, ldS, col, stream);
      off += 2L * nb * nlm;
    };
    put(vrt, L, sc.vrt);
    put(div, L, sc.div);
    put(tv, L, sc.tv);
    if (nt > 0) put(trc, nt * L, sc.trc);
    put(lnps, 1, sc.lnps);
    launch_sc<R>(S, ldS, sc, L, nlm, lapv, (R)Phys::rerth, stream);
    if (topo != topo_seen_ || topo) {  // grad(grav*topo) (dyn_init.f90:84)
      if (topo) {
        std::vector<double> gt(2 * (size_t)nlm);
        for (long q = 0; q < 2L * nlm; ++q) gt[q] = Phys::grav * topo[q];
        std::vector<double> gx(ng), gy(ng);
        getgrad(1, gt.data(), gx.data(), gy.data());
        std::vector<R> rx(gx.begin(), gx.end()), ry(gy.begin(), gy.end());
        GD_CUDA(cudaMemcpyAsync(dphisdx, rx.data(), sizeof(R) * ng, cudaMemcpyHostToDevice, stream));
        GD_CUDA(cudaMemcpyAsync(dphisdy, ry.data(), sizeof(R) * ng, cudaMemcpyHostToDevice, stream));
      } else {
        GD_CUDA(cudaMemsetAsync(dphisdx, 0, sizeof(R) * ng, stream));
        GD_CUDA(cudaMemsetAsync(dphisdy, 0, sizeof(R) * ng, stream));
      }
      topo_seen_ = topo;
    }
    GD_CUDA(cudaStreamSynchronize(stream));
    state_set = true;
  }
  const double* topo_seen_ = reinterpret_cast<const double*>(1);
  void release(void* p) {
    cudaFree(p);
    allocs.erase(std::remove(allocs.begin(), allocs.end(), p), allocs.end());
  }
  template <typename H>
  void get_state_t(H* vrt, H* div, H* tv, H* trc, H* lnps) {
    H* st = reinterpret_cast<H*>(staging());
    long off = 0;
    auto get = [&](H* h, int nb, int col) {
      H* d = st + off;
      off += 2L * nb * nlm;
      if (!h) return;
      launch_int2ref<R>(S, ldS, col, nb, nlm, d, stream);
      GD_CUDA(cudaMemcpyAsync(h, d, sizeof(H) * 2 * (long)nb * nlm, cudaMemcpyDeviceToHost, stream));
    };
    get(vrt, L, sc.vrt);
    get(div, L, sc.div);
    get(tv, L, sc.tv);
    if (nt > 0) get(trc, nt * L, sc.trc);
    get(lnps, 1, sc.lnps);
    GD_CUDA(cudaStreamSynchronize(stream));
    tc_status();
  }
  void spec_out(const R* src, long ld, int col, int nb, double* h, double* tmp) {
    if (!h) return;
    launch_int2ref<R>(src, ld, col, nb, nlm, tmp, stream);
    GD_CUDA(cudaMemcpyAsync(h, tmp, sizeof(double) * 2 * (long)nb * nlm, cudaMemcpyDeviceToHost, stream));
    GD_CUDA(cudaStreamSynchronize(stream));
  }
  void getdyntend(int rkstage, int inverse_only, double* dvrt, double* ddiv, double* dtv, double* dtrc,
                  double* dlnps) override {
    if (!state_set) throw std::runtime_error("state not set (gd_set_state)");
    if (inverse_only) {
      inverse_pass(true);
      GD_CUDA(cudaStreamSynchronize(stream));
      return;
    }
    dyn_pass(rkstage == 1 ? 0 : 1, true);
    StageArgs<R> a = stage_args(0);
    launch_assemble<R>(a, TD[0], stream);
    double* tmp = dalloc<double>(2L * nlm * L * std::max(1, nt));
    spec_out(TD[0], ldTD, tc.dvrt, L, dvrt, tmp);
    spec_out(TD[0], ldTD, tc.ddiv, L, ddiv, tmp);
    spec_out(TD[0], ldTD, tc.dtv, L, dtv, tmp);
    if (nt > 0) spec_out(TD[0], ldTD, tc.dtrc, nt * L, dtrc, tmp);
    spec_out(TD[0], ldTD, tc.dlnps, 1, dlnps, tmp);
    release(tmp);
  }
  void getphytend(double* dvrt, double* ddiv, double* dtv, double* dtrc, double* dlnps) override {
    if (!state_set) throw std::runtime_error("state not set (gd_set_state)");
    if (simple()) {  // phy_run_simple.f90:145-160 on the grid of the last getdyntend
      launch_simple_physics<R>(simple_args(), stream);
      r2c(r2cSimple, gA, FPb, ldGP, FHb, ldGH);
      do_anal(false, anaSimple, FPb, ldGP, 2 * (4 * L + 1), AP, ldAP);
      do_anal(true, anaH, FHb, ldGH, 2 * ah.ncol, AH, ldAH);
      const R ai = (R)(1.0 / Phys::rerth);
      // vorticity and divergence to AP columns [2L+1, 4L+1)
      launch_combine<R>(AP, ldAP, 2 * L + 1, AH, ldAH, 0, AP, ldAP, 2 * L + 1, 2 * L, nlm, ai, stream);
      double* tmp = dalloc<double>(2L * nlm * L);
      const size_t n1 = 2 * (size_t)L * nlm;
      auto out = [&](int col, double* h) {
        if (!h) return;
        spec_out(AP, ldAP, col, L, h, tmp);
        for (size_t i = 0; i < n1; ++i) h[i] = h[i] / c.dt;
      };
      out(0, dtv);
      out(2 * L + 1, dvrt);
      out(3 * L + 1, ddiv);
      if (dtrc) {
        memset(dtrc, 0, sizeof(double) * 2 * (size_t)nt * L * nlm);
        out(L, dtrc);
      }
      release(tmp);
      if (dlnps) memset(dlnps, 0, sizeof(double) * 2 * (size_t)nlm);
      return;
    }
    if (c.dcmip >= 0 || !c.heldsuarez) {  // dry DCMIP or no physics: zero tendencies
      for (double* h : {dvrt, ddiv, dtv})
        if (h) memset(h, 0, sizeof(double) * 2 * (size_t)L * nlm);
      if (dtrc) memset(dtrc, 0, sizeof(double) * 2 * (size_t)nt * L * nlm);
      if (dlnps) memset(dlnps, 0, sizeof(double) * 2 * (size_t)nlm);
      return;
    }
    launch_hs_forcing<R>(hs_args(), stream);
    r2c(r2cPhys, gA, FPb, ldGP, FHb, ldGH);
    do_anal(false, anaPhys, FPb, ldGP, 2 * (3 * L + 1), AP, ldAP);
    double* tmp = dalloc<double>(2L * nlm * L);
    spec_out(AP, ldAP, 0, L, dtv, tmp);
    spec_out(AP, ldAP, L, L, dvrt, tmp);
    spec_out(AP, ldAP, 2 * L, L, ddiv, tmp);
    release(tmp);
    if (dtrc) memset(dtrc, 0, sizeof(double) * 2 * (size_t)nt * L * nlm);
    if (dlnps) memset(dlnps, 0, sizeof(double) * 2 * (size_t)nlm);
  }

  // ------------------------------------------------------ transform API --
  const GemmPlan& synth_plan(int ncr) {
    auto it = synth_cache.find(ncr);
    if (it != synth_cache.end()) return it->second;
    return synth_cache[ncr] = make_synth_plan(T, nh, ncr, stream);
  }
  const GemmPlan& anal_plan(int ncr) {
    auto it = anal_cache.find(ncr);
    if (it != anal_cache.end()) return it->second;
    return anal_cache[ncr] = make_anal_plan(T, ncr, stream);
  }
  int chunk_cols() const { return std::max(1, std::min(sc.ncol / 2, ar.total / 2)); }
  // synthesis of ncs complex columns X[nlm][ldS] with descriptors -> host grids
  template <typename H>
  void api_synth(const R* X, int ncs, bool needH, const std::vector<SynthDesc>& ds, int nrows, H* out) {
    do_synth(false, synth_plan(2 * ncs), X, ldS, 2 * ncs, FPb, ldS);
    if (needH) do_synth(true, synth_plan(2 * ncs), X, ldS, 2 * ncs, FHb, ldS);
    FftPlan p = mk_c2r(ds.data(), (int)ds.size());
    c2r(p, FPb, ldS, FHb, ldS, gS);
    grid_out(gS, nrows, out);
    free_fft_plan(p);
  }
  // device grid rows (R) -> host (H), converted on the device when the types differ
  template <typename H>
  void grid_out(const R* g, int nrows, H* out) {
    long n = (long)nrows * ng;
    if constexpr (std::is_same<R, H>::value) {
      GD_CUDA(cudaMemcpyAsync(out, g, sizeof(H) * n, cudaMemcpyDeviceToHost, stream));
    } else {
      H* tmp = dalloc<H>(n);
      launch_convert2d<R, H>(g, ng, tmp, ng, nrows, (int)ng, stream);
      GD_CUDA(cudaMemcpyAsync(out, tmp, sizeof(H) * n, cudaMemcpyDeviceToHost, stream));
      GD_CUDA(cudaStreamSynchronize(stream));
      release(tmp);
    }
    GD_CUDA(cudaStreamSynchronize(stream));
  }
  template <typename H>
  void grid_in(const H* in, int nrows, R* g) {
    long n = (long)nrows * ng;
    if constexpr (std::is_same<R, H>::value) {
      GD_CUDA(cudaMemcpyAsync(g, in, sizeof(H) * n, cudaMemcpyHostToDevice, stream));
      GD_CUDA(cudaStreamSynchronize(stream));
    } else {
      H* tmp = dalloc<H>(n);
      GD_CUDA(cudaMemcpyAsync(tmp, in, sizeof(H) * n, cudaMemcpyHostToDevice, stream));
      launch_convert2d<H, R>(tmp, ng, g, ng, nrows, (int)ng, stream);
      GD_CUDA(cudaStreamSynchronize(stream));
      release(tmp);
    }
  }
  R* X_ = nullptr;
  R* scratchX() {
    if (!X_) {
      X_ = dalloc<R>((size_t)nlm_rows * ldS);
      GD_CUDA(cudaMemsetAsync(X_, 0, sizeof(R) * nlm_rows * ldS, stream));
    }
    return X_;
  }
  template <typename H>
  void spec_in(const H* h, int nb, R* X, int col) {
    H* tmp = dalloc<H>(2L * nb * nlm);
    GD_CUDA(cudaMemcpyAsync(tmp, h, sizeof(H) * 2 * (long)nb * nlm, cudaMemcpyHostToDevice, stream));
    launch_ref2int<R>(tmp, nb, nlm, X, ldS, col, stream);
    GD_CUDA(cudaStreamSynchronize(stream));
    release(tmp);
  }
  void spectogrd(int nb, const double* spec, double* grid) override { spectogrd_t(nb, spec, grid); }
  void spectogrd(int nb, const float* spec, float* grid) override { spectogrd_t(nb, spec, grid); }
  void getuv(int nb, const double* vrt, const double* div, double* u, double* v) override { getuv_t(nb, vrt, div, u, v); }
  void getuv(int nb, const float* vrt, const float* div, float* u, float* v) override { getuv_t(nb, vrt, div, u, v); }
  void getgrad(int nb, const double* spec, double* gx, double* gy) override { getgrad_t(nb, spec, gx, gy); }
  void getgrad(int nb, const float* spec, float* gx, float* gy) override { getgrad_t(nb, spec, gx, gy); }
  void grdtospec(int nb, const double* grid, double* spec) override { grdtospec_t(nb, grid, spec); }
  void grdtospec(int nb, const float* grid, float* spec) override { grdtospec_t(nb, grid, spec); }
  void getvrtdivspec(int nb, const double* u, const double* v, double* vrt, double* div) override {
    getvrtdivspec_t(nb, u, v, vrt, div);
  }
  void getvrtdivspec(int nb, const float* u, const float* v, float* vrt, float* div) override {
    getvrtdivspec_t(nb, u, v, vrt, div);
  }
  template <typename H>
  void spectogrd_t(int nb, const H* spec, H* grid) {
    R* X = scratchX();
    for (int b0 = 0; b0 < nb; b0 += chunk_cols()) {
      int k = std::min(chunk_cols(), nb - b0);
      spec_in(spec + 2L * b0 * nlm, k, X, 0);
      std::vector<SynthDesc> ds = {{k, 0, 0, 0, -1, 0, 1.0, 0.0}};
      api_synth(X, k, false, ds, k, grid + (long)b0 * ng);
    }
  }
  template <typename H>
  void getuv_t(int nb, const H* vrt, const H* div, H* u, H* v) {
    R* X = scratchX();
    const int ch = chunk_cols();
    for (int b0 = 0; b0 < nb; b0 += ch) {
      int k = std::min(ch, nb - b0);
      spec_in(vrt + 2L * b0 * nlm, k, X, 0);
      spec_in(div + 2L * b0 * nlm, k, X, k);
      // s = a invlap vrt, c = a invlap div (shtns.f90:259-260)
      launch_scale_cols<R>(X, ldS, 0, 2 * k, nlm, invlap_a(), R(1), stream);
      std::vector<SynthDesc> ds = {{k, 0, 1, 0, 0, k, -1.0, 1.0}, {k, k, 1, k, 0, 0, 1.0, 1.0}};
      std::vector<H> out(2L * k * ng);
      api_synth(X, 2 * k, true, ds, 2 * k, out.data());
      memcpy(u + (long)b0 * ng, out.data(), sizeof(H) * k * ng);
      memcpy(v + (long)b0 * ng, out.data() + (long)k * ng, sizeof(H) * k * ng);
    }
  }
  R* invlap_ = nullptr;
  const R* invlap_a() {  // rerth * invlap, 0 for n = 0
    if (!invlap_) {
      std::vector<double> il(nlm);
      for (int q = 0; q < nlm; ++q) il[q] = (q == 0) ? 0.0 : Phys::rerth / h_lap[q];
      invlap_ = upload(toR(il));
    }
    return invlap_;
  }
  template <typename H>
  void getgrad_t(int nb, const H* spec, H* gx, H* gy) {
    R* X = scratchX();
    const double ai = 1.0 / Phys::rerth;
    const int ch = chunk_cols();
    for (int b0 = 0; b0 < nb; b0 += ch) {
      int k = std::min(ch, nb - b0);
      spec_in(spec + 2L * b0 * nlm, k, X, 0);
      std::vector<SynthDesc> ds = {{k, 0, -1, 0, 0, 0, 0.0, ai}, {k, k, 1, 0, -1, 0, ai, 0.0}};
      std::vector<H> out(2L * k * ng);
      api_synth(X, k, true, ds, 2 * k, out.data());
      memcpy(gx + (long)b0 * ng, out.data(), sizeof(H) * k * ng);
      memcpy(gy + (long)b0 * ng, out.data() + (long)k * ng, sizeof(H) * k * ng);
    }
  }
  void api_anal(const std::vector<AnalDesc>& ds, int ncP, int ncH) {
    FftPlan p = mk_r2c(ds.data(), (int)ds.size());
    r2c(p, gA, FPb, ldS, FHb, ldS);
    do_anal(false, anal_plan(2 * ncP), FPb, ldS, 2 * ncP, AP, ldAP);
    if (ncH > 0) do_anal(true, anal_plan(2 * ncH), FHb, ldS, 2 * ncH, AH, ldAH);
    free_fft_plan(p);
  }
  int achunk() const { return std::max(1, std::min(ap.ncol / 2, ar.total / 2)); }
  template <typename H>
  void grdtospec_t(int nb, const H* grid, H* spec) {
    const int ch = achunk();
    H* tmp = dalloc<H>(2L * ch * nlm);
    for (int b0 = 0; b0 < nb; b0 += ch) {
      int k = std::min(ch, nb - b0);
      grid_in(grid + (long)b0 * ng, k, gA);
      api_anal({{k, 0, 0, 0, -1, 1.0, 0.0}}, k, 0);
      launch_int2ref<R>(AP, ldAP, 0, k, nlm, tmp, stream);
      GD_CUDA(cudaMemcpyAsync(spec + 2L * b0 * nlm, tmp, sizeof(H) * 2 * (long)k * nlm, cudaMemcpyDeviceToHost,
                              stream));
      GD_CUDA(cudaStreamSynchronize(stream));
    }
    release(tmp);
  }
  template <typename H>
  void getvrtdivspec_t(int nb, const H* u, const H* v, H* vrt, H* div) {
    const int ch = std::max(1, std::min(ah.ncol / 2, achunk()));
    H* tmp = dalloc<H>(2L * ch * nlm);
    const R ai = (R)(1.0 / Phys::rerth);
    for (int b0 = 0; b0 < nb; b0 += ch) {
      int k = std::min(ch, nb - b0);
      grid_in(u + (long)b0 * ng, k, gA);
      grid_in(v + (long)b0 * ng, k, gA + (long)k * ng);
      // GP: [i m/cos V | i m/cos U], GH: [U | -V]
      std::vector<AnalDesc> ds = {{k, 0, k, 1, 0, 1.0, 1.0}, {k, k, 0, 1, k, 1.0, -1.0}};
      api_anal(ds, 2 * k, 2 * k);
      // vrt = (AP[0:k] + AH[0:k]) / a, div = (AP[k:2k] + AH[k:2k]) / a
      launch_combine<R>(AP, ldAP, 0, AH, ldAH, 0, AP, ldAP, 0, 2 * k, nlm, ai, stream);
      launch_int2ref<R>(AP, ldAP, 0, k, nlm, tmp, stream);
      GD_CUDA(cudaMemcpyAsync(vrt + 2L * b0 * nlm, tmp, sizeof(H) * 2 * (long)k * nlm, cudaMemcpyDeviceToHost,
                              stream));
      GD_CUDA(cudaStreamSynchronize(stream));
      launch_int2ref<R>(AP, ldAP, k, k, nlm, tmp, stream);
      GD_CUDA(cudaMemcpyAsync(div + 2L * b0 * nlm, tmp, sizeof(H) * 2 * (long)k * nlm, cudaMemcpyDeviceToHost,
                              stream));
      GD_CUDA(cudaStreamSynchronize(stream));
    }
    release(tmp);
  }

  void grid_info(double* lats, double* gauwts, double* areawts, int* degree, int* order, double* lap,
                 double* invlap) override {
    for (int j = 0; j < nlat; ++j) {
      if (lats) lats[j] = h_lat[j];
      if (gauwts) gauwts[j] = h_w[j];
      if (areawts) areawts[j] = h_w[j] / (2.0 * nlon);
    }
    for (int q = 0; q < nlm; ++q) {
      if (degree) degree[q] = h_deg[q];
      if (order) order[q] = h_ord[q];
      if (lap) lap[q] = h_lap[q];
      if (invlap) invlap[q] = q == 0 ? 0.0 : 1.0 / h_lap[q];
    }
  }
  int get_grid(const char* name, double* out) override {
    std::string n(name);
    const R* src = nullptr;
    int rows = 0;
    if (n == "ug") src = gS + (long)sr.u * ng, rows = L;
    else if (n == "vg") src = gS + (long)sr.v * ng, rows = L;
    else if (n == "vrtg") src = gS + (long)sr.vrt * ng, rows = L;
    else if (n == "divg") src = gS + (long)sr.div * ng, rows = L;
    else if (n == "tvg") src = gS + (long)sr.tv * ng, rows = L;
    else if (n == "trcg") src = gS + (long)sr.trc * ng, rows = nt * L;
    else if (n == "lnpsg") src = gS + (long)sr.lnps * ng, rows = 1;
    else if (n == "dlnpdtg") src = dlnpdtg, rows = L;
    else if (n == "etadot") src = etadot, rows = L + 1;
    else if (n == "psg") src = psg, rows = 1;
    else if (n == "dlnpsdt") src = dlnpsdt, rows = 1;
    else if (n == "prs") src = prs, rows = L;
    else if (n == "dphisdx") src = dphisdx, rows = 1;
    else if (n == "dphisdy") src = dphisdy, rows = 1;
    else if (n == "sppt" && sppt) src = spptg, rows = 1;
    else if (n == "precip") src = precip, rows = 1;
    else if (n == "apcp") src = apcp, rows = 1;
    else if (n == "pwat") src = pwat, rows = 1;
    if (!src || rows == 0) return GD_ERR_ARG;
    grid_out(src, rows, out);
    return GD_OK;
  }
  double get_pdryini() override {
    double h = 0.0;
    GD_CUDA(cudaMemcpyAsync(&h, pdryini, sizeof(double), cudaMemcpyDeviceToHost, stream));
    GD_CUDA(cudaStreamSynchronize(stream));
    return h;
  }
  void diag(double* out) override {
    launch_diag<R>(gS + (long)sr.u * ng, gS + (long)sr.v * ng, L, psg, dlnpsdt, w, nlat, nlon, diagbuf, diagout,
                   stream);
    double h[5];
    GD_CUDA(cudaMemcpyAsync(h, diagout, 4 * sizeof(double), cudaMemcpyDeviceToHost, stream));
    GD_CUDA(cudaMemcpyAsync(h + 4, pdryini, sizeof(double), cudaMemcpyDeviceToHost, stream));
    GD_CUDA(cudaStreamSynchronize(stream));
    memcpy(out, h, sizeof(h));
  }
};

}  // namespace gd

// ====================================================================== ABI
struct gd_ctx {
  std::unique_ptr<gd::DycoreBase> d;
  gd_config cfg;
  std::string err;
  std::vector<double> topo;  // orography of the last gd_set_state (complex [nlm]), for gd_write_sig
  std::vector<double> ak, bk;  // the vertical coordinate gd_init was given
};

static std::string g_init_error;

template <typename F>
static int guarded(gd_ctx* ctx, F f) {
  if (!ctx || !ctx->d) return GD_ERR_ARG;
  try {
    f();
    return GD_OK;
  } catch (const gd::CudaError& e) {
    ctx->err = e.what();
    return GD_ERR_CUDA;
  } catch (const std::invalid_argument& e) {
    ctx->err = e.what();
    return GD_ERR_ARG;
  } catch (const std::runtime_error& e) {
    ctx->err = e.what();
    return GD_ERR_STATE;
  } catch (const std::exception& e) {
    ctx->err = e.what();
    return GD_ERR_CUDA;
  }
}

static bool is_2a3b(int n) {
  if (n <= 0) return false;
  while (n % 2 == 0) n /= 2;
  while (n % 3 == 0) n /= 3;
  return n == 1;
}

extern "C" {

int gd_default_config(gd_config* c) {
  if (!c) return GD_ERR_ARG;
  memset(c, 0, sizeof(*c));
  c->ntrunc = 42;
  c->nlon = 128;
  c->nlat = 64;
  c->nlev = 20;
  c->ntrac = 0;
  c->dt = 1200.0;
  c->precision = GD_PREC_FP64;
  c->explicit_ = 0;
  c->adiabatic = 0;
  c->heldsuarez = 1;
  c->massfix = 1;
  c->dry = 1;
  c->ndiss = 0;
  c->efold = 0.0;
  c->hdif_fac = 1.0;
  c->hdif_fac2 = 1.0;
  c->fshk = 0.0;
  c->taustratdamp = 5.0 * 86400.0;
  c->pdryini = 0.0;
  c->device = 0;
  c->dcmip = -1;
  return GD_OK;
}

int gd_init(const gd_config* cfg, const double* ak, const double* bk, gd_ctx** out) {
  if (!cfg || !ak || !bk || !out) {
    g_init_error = "gd_init: null argument";
    return GD_ERR_ARG;
  }
  *out = nullptr;
  const gd_config& c = *cfg;
  std::string why;
  if (!is_2a3b(c.nlon) || c.nlon % 2) why = "nlon must be an even 2^a 3^b";
  else if (c.nlat < 4 || c.nlat % 2) why = "nlat must be even and >= 4";
  else if (c.ntrunc < 1 || c.ntrunc >= c.nlon / 2 || c.ntrunc >= c.nlat) why = "ntrunc must satisfy 1 <= T < nlon/2 and T < nlat";
  else if (c.nlev < 3 || c.nlev > 126) why = "nlev must be in [3, 126]";
  else if (c.ntrac < 0) why = "ntrac must be >= 0";
  else if (!(c.dt > 0)) why = "dt must be positive";
  else if (c.precision < GD_PREC_FP64 || c.precision > GD_PREC_F64_EDDY) why = "unknown precision";
  else if (c.dcmip >= 0 && c.heldsuarez) why = "heldsuarez and dcmip cannot both be set";
  else if (c.dcmip >= 0 && c.dcmip / 10 != 4 && c.dcmip / 10 != 5) why = "dcmip must be 4x or 5x (or -1)";
  else if (c.dcmip >= 0 && !c.dry && c.ntrac < 1) why = "moist DCMIP physics needs ntrac >= 1 (humidity)";
  else if (c.dcmip >= 0 && !c.dry && c.nlev > 128) why = "DCMIP physics supports at most 128 levels";
  if (!why.empty()) {
    g_init_error = "gd_init: " + why;
    return (why.find("not supported") != std::string::npos) ? GD_ERR_UNSUPPORTED : GD_ERR_ARG;
  }
  gd_ctx* ctx = new gd_ctx();
  ctx->cfg = c;
  ctx->ak.assign(ak, ak + c.nlev + 1);
  ctx->bk.assign(bk, bk + c.nlev + 1);
  try {
    if (c.precision == GD_PREC_FP64 || c.precision == GD_PREC_F64_TF32X3 || c.precision == GD_PREC_F64_EDDY)
      ctx->d.reset(new gd::Dycore<double>(c, ak, bk));
    else
      ctx->d.reset(new gd::Dycore<float>(c, ak, bk));
  } catch (const gd::CudaError& e) {
    g_init_error = e.what();
    delete ctx;
    return std::string(e.what()).find("cudaMalloc") != std::string::npos ? GD_ERR_NOMEM : GD_ERR_CUDA;
  } catch (const std::exception& e) {
    g_init_error = e.what();
    delete ctx;
    return GD_ERR_CUDA;
  }
  *out = ctx;
  return GD_OK;
}

int gd_finalize(gd_ctx* ctx) {
  if (!ctx) return GD_ERR_ARG;
  delete ctx;
  return GD_OK;
}

int gd_set_state(gd_ctx* ctx, const double* vrt, const double* div, const double* tv, const double* trc,
                 const double* lnps, const double* topo) {
  if (!vrt || !div || !tv || !lnps) {
    if (ctx) ctx->err = "gd_set_state: null state array";
    return GD_ERR_ARG;
  }
  return guarded(ctx, [&] {
    ctx->d->set_state(vrt, div, tv, trc, lnps, topo);
    const long n2 = (long)(ctx->cfg.ntrunc + 1) * (ctx->cfg.ntrunc + 2);
    if (topo) ctx->topo.assign(topo, topo + n2);
    else ctx->topo.assign((size_t)n2, 0.0);
  });
}
int gd_get_state(gd_ctx* ctx, double* vrt, double* div, double* tv, double* trc, double* lnps) {
  return guarded(ctx, [&] { ctx->d->get_state(vrt, div, tv, trc, lnps); });
}
int gd_set_state_f(gd_ctx* ctx, const float* vrt, const float* div, const float* tv, const float* trc,
                   const float* lnps, const float* topo) {
  if (!vrt || !div || !tv || !lnps) {
    if (ctx) ctx->err = "gd_set_state_f: null state array";
    return GD_ERR_ARG;
  }
  return guarded(ctx, [&] {
    ctx->d->set_state(vrt, div, tv, trc, lnps, topo);
    const long n2 = (long)(ctx->cfg.ntrunc + 1) * (ctx->cfg.ntrunc + 2);
    if (topo) ctx->topo.assign(topo, topo + n2);
    else ctx->topo.assign((size_t)n2, 0.0);
  });
}
int gd_get_state_f(gd_ctx* ctx, float* vrt, float* div, float* tv, float* trc, float* lnps) {
  return guarded(ctx, [&] { ctx->d->get_state(vrt, div, tv, trc, lnps); });
}
int gd_get_topo(gd_ctx* ctx, double* topo) {
  if (!ctx || !ctx->d || !topo) return GD_ERR_ARG;
  const size_t n2 = 2 * (size_t)(ctx->cfg.ntrunc + 1) * (ctx->cfg.ntrunc + 2) / 2;
  if (ctx->topo.size() == n2) std::copy(ctx->topo.begin(), ctx->topo.end(), topo);
  else std::fill(topo, topo + n2, 0.0);
  return GD_OK;
}
int gd_getdyntend(gd_ctx* ctx, int rkstage, int inverse_only, double* dvrt, double* ddiv, double* dtv, double* dtrc,
                  double* dlnps) {
  if (rkstage < 1 || rkstage > 3) {
    if (ctx) ctx->err = "gd_getdyntend: rkstage must be 1, 2 or 3";
    return GD_ERR_ARG;
  }
  if (!inverse_only && (!dvrt || !ddiv || !dtv || !dlnps)) {
    if (ctx) ctx->err = "gd_getdyntend: null tendency array";
    return GD_ERR_ARG;
  }
  return guarded(ctx, [&] { ctx->d->getdyntend(rkstage, inverse_only, dvrt, ddiv, dtv, dtrc, dlnps); });
}
int gd_getphytend(gd_ctx* ctx, double* dvrt, double* ddiv, double* dtv, double* dtrc, double* dlnps) {
  return guarded(ctx, [&] { ctx->d->getphytend(dvrt, ddiv, dtv, dtrc, dlnps); });
}
int gd_advance(gd_ctx* ctx, double t, int nsteps) {
  if (nsteps < 0) {
    if (ctx) ctx->err = "gd_advance: nsteps < 0";
    return GD_ERR_ARG;
  }
  return guarded(ctx, [&] {
    ctx->d->t_cur = t;
    ctx->d->advance(nsteps);
  });
}
int gd_set_iau(gd_ctx* ctx, int nfiles, const double* fhrs, double delthrs, const double* vrt, const double* div,
               const double* tv, const double* trc, const double* lnps) {
  if (nfiles < 0 || (nfiles > 0 && !fhrs)) {
    if (ctx) ctx->err = "gd_set_iau: bad nfiles or null times";
    return GD_ERR_ARG;
  }
  return guarded(ctx, [&] { ctx->d->set_iau(nfiles, fhrs, delthrs, vrt, div, tv, trc, lnps); });
}
int gd_set_iau_files(gd_ctx* ctx, int nfiles, const double* fhrs, double delthrs, const char* const* fg,
                     const char* const* anl) {
  if (!ctx || !ctx->d) return GD_ERR_ARG;
  if (nfiles < 2 || !fhrs || !fg || !anl) {
    ctx->err = "gd_set_iau_files: need at least two first-guess / analysis pairs";
    return GD_ERR_ARG;
  }
  const gd_config& c = ctx->cfg;
  const size_t n2 = (size_t)(c.ntrunc + 1) * (c.ntrunc + 2), L = (size_t)c.nlev, nt = (size_t)c.ntrac;
  std::vector<double> inc[5], tmp[5];
  const size_t sz[5] = {n2 * L, n2 * L, n2 * L, n2 * L * nt, n2};
  try {
    for (int f = 0; f < 5; ++f) {
      inc[f].assign(sz[f] * nfiles, 0.0);
      tmp[f].assign(sz[f], 0.0);
    }
  } catch (const std::bad_alloc&) {
    ctx->err = "gd_set_iau_files: host allocation failed";
    return GD_ERR_NOMEM;
  }
  for (int n = 0; n < nfiles; ++n) {  // init_iau (iau_module.f90:57-78): analysis - first guess
    gd_sighead h;
    int rc = gd_sigio_read(fg[n], c.ntrunc, c.nlev, c.ntrac, &h, tmp[0].data(), tmp[1].data(), tmp[2].data(),
                           nt ? tmp[3].data() : nullptr, tmp[4].data(), nullptr);
    double* o[5];
    for (int f = 0; f < 5; ++f) o[f] = inc[f].data() + n * sz[f];
    if (rc == GD_OK)
      rc = gd_sigio_read(anl[n], c.ntrunc, c.nlev, c.ntrac, &h, o[0], o[1], o[2], nt ? o[3] : nullptr, o[4], nullptr);
    if (rc != GD_OK) {
      ctx->err = gd_sigio_last_error();
      return rc;
    }
    for (int f = 0; f < 5; ++f)
      for (size_t i = 0; i < sz[f]; ++i) o[f][i] = o[f][i] - tmp[f][i];
  }
  return gd_set_iau(ctx, nfiles, fhrs, delthrs, inc[0].data(), inc[1].data(), inc[2].data(),
                    nt ? inc[3].data() : nullptr, inc[4].data());
}
int gd_dfi(gd_ctx* ctx, double t, int ntdfi) {
  if (ntdfi < 1) {
    if (ctx) ctx->err = "gd_dfi: ntdfi must be >= 1";
    return GD_ERR_ARG;
  }
  return guarded(ctx, [&] { ctx->d->dfi(t, ntdfi); });
}
int gd_dfi_weights(int ntdfi, double* w) {
  if (ntdfi < 1 || !w) return GD_ERR_ARG;
  gd::dfi_weights(ntdfi, w);
  return GD_OK;
}
int gd_spectogrd(gd_ctx* ctx, int nb, const double* spec, double* grid) {
  if (nb < 0 || (nb > 0 && (!spec || !grid))) return GD_ERR_ARG;
  return guarded(ctx, [&] { ctx->d->spectogrd(nb, spec, grid); });
}
int gd_grdtospec(gd_ctx* ctx, int nb, const double* grid, double* spec) {
  if (nb < 0 || (nb > 0 && (!spec || !grid))) return GD_ERR_ARG;
  return guarded(ctx, [&] { ctx->d->grdtospec(nb, grid, spec); });
}
int gd_getuv(gd_ctx* ctx, int nb, const double* vrt, const double* div, double* u, double* v) {
  if (nb < 0 || (nb > 0 && (!vrt || !div || !u || !v))) return GD_ERR_ARG;
  return guarded(ctx, [&] { ctx->d->getuv(nb, vrt, div, u, v); });
}
int gd_getvrtdivspec(gd_ctx* ctx, int nb, const double* u, const double* v, double* vrt, double* div) {
  if (nb < 0 || (nb > 0 && (!vrt || !div || !u || !v))) return GD_ERR_ARG;
  return guarded(ctx, [&] { ctx->d->getvrtdivspec(nb, u, v, vrt, div); });
}
int gd_getgrad(gd_ctx* ctx, int nb, const double* spec, double* gx, double* gy) {
  if (nb < 0 || (nb > 0 && (!spec || !gx || !gy))) return GD_ERR_ARG;
  return guarded(ctx, [&] { ctx->d->getgrad(nb, spec, gx, gy); });
}
int gd_spectogrd_f(gd_ctx* ctx, int nb, const float* spec, float* grid) {
  if (nb < 0 || (nb > 0 && (!spec || !grid))) return GD_ERR_ARG;
  return guarded(ctx, [&] { ctx->d->spectogrd(nb, spec, grid); });
}
int gd_grdtospec_f(gd_ctx* ctx, int nb, const float* grid, float* spec) {
  if (nb < 0 || (nb > 0 && (!spec || !grid))) return GD_ERR_ARG;
  return guarded(ctx, [&] { ctx->d->grdtospec(nb, grid, spec); });
}
int gd_getuv_f(gd_ctx* ctx, int nb, const float* vrt, const float* div, float* u, float* v) {
  if (nb < 0 || (nb > 0 && (!vrt || !div || !u || !v))) return GD_ERR_ARG;
  return guarded(ctx, [&] { ctx->d->getuv(nb, vrt, div, u, v); });
}
int gd_getvrtdivspec_f(gd_ctx* ctx, int nb, const float* u, const float* v, float* vrt, float* div) {
  if (nb < 0 || (nb > 0 && (!vrt || !div || !u || !v))) return GD_ERR_ARG;
  return guarded(ctx, [&] { ctx->d->getvrtdivspec(nb, u, v, vrt, div); });
}
int gd_getgrad_f(gd_ctx* ctx, int nb, const float* spec, float* gx, float* gy) {
  if (nb < 0 || (nb > 0 && (!spec || !gx || !gy))) return GD_ERR_ARG;
  return guarded(ctx, [&] { ctx->d->getgrad(nb, spec, gx, gy); });
}
int gd_grid_info(gd_ctx* ctx, double* lats, double* gauwts, double* areawts, int* degree, int* order, double* lap,
                 double* invlap) {
  return guarded(ctx, [&] { ctx->d->grid_info(lats, gauwts, areawts, degree, order, lap, invlap); });
}
int gd_get_grid(gd_ctx* ctx, const char* name, double* out) {
  if (!name || !out) return GD_ERR_ARG;
  int rc = GD_OK;
  int g = guarded(ctx, [&] { rc = ctx->d->get_grid(name, out); });
  return g != GD_OK ? g : rc;
}
int gd_diag(gd_ctx* ctx, double* out5) {
  if (!out5) return GD_ERR_ARG;
  return guarded(ctx, [&] { ctx->d->diag(out5); });
}
int gd_profile_step(gd_ctx* ctx, double* ms, int nphase) {
  if (!ms || nphase < 8) {
    if (ctx) ctx->err = "gd_profile_step: need room for 8 phases";
    return GD_ERR_ARG;
  }
  return guarded(ctx, [&] { ctx->d->profile_step(ms, nphase); });
}
int gd_set_sppt(gd_ctx* ctx, gd_pattern* pattern, double sigtop, double sigbot) {
  return guarded(ctx, [&] { ctx->d->set_sppt(pattern, sigtop, sigbot); });
}
int gd_autotune(gd_ctx* ctx, int* choices) {
  if (!choices) return GD_ERR_ARG;
  return guarded(ctx, [&] { ctx->d->autotune(choices); });
}
int gd_set_closure(gd_ctx* ctx, gd_mlp* net) {
  return guarded(ctx, [&] { ctx->d->set_closure(net); });
}
int gd_closure_features(gd_ctx* ctx, float* x) {
  if (!x) return GD_ERR_ARG;
  return guarded(ctx, [&] { ctx->d->closure_features(x); });
}
// The ensemble graph: one child node per member's captured step, no edges
// between them, so one launch runs every member's step and the graph
// executor overlaps them.  Cached for the last member set (by the members'
// unique ids and capture epochs); rebuilt when either changes.
struct EnsembleGraph {
  std::vector<unsigned long long> key;
  cudaGraphExec_t exec = nullptr;
};
static std::mutex g_ens_mutex;
static EnsembleGraph g_ens;

int gd_ensemble_advance(gd_ctx** ctxs, int n, double t, int nsteps) {
  if (!ctxs || n < 1 || nsteps < 0) return GD_ERR_ARG;
  for (int i = 0; i < n; ++i)
    if (!ctxs[i] || !ctxs[i]->d) return GD_ERR_ARG;
  for (int i = 0; i < n; ++i) ctxs[i]->d->t_cur = t;
  const int dev = ctxs[0]->cfg.device;
  bool one_device = true;  // and no member twice (its step would run twice at once)
  for (int i = 1; i < n; ++i) {
    one_device = one_device && ctxs[i]->cfg.device == dev;
    for (int j = 0; j < i; ++j) one_device = one_device && ctxs[j] != ctxs[i];
  }
  int s = 0;
  while (s < nsteps) {
    // one launch over all members once every member has a captured step
    std::vector<cudaGraph_t> gs(n);
    std::vector<unsigned long long> key;
    bool ready = one_device && n > 1;
    for (int i = 0; i < n && ready; ++i) {
      unsigned long long ep = 0;
      ready = ctxs[i]->d->ensemble_step_graph(&gs[i], &ep);
      key.push_back(ctxs[i]->d->uid);
      key.push_back(ep);
    }
    if (ready) {
      const int rest = nsteps - s;
      const int rc = guarded(ctxs[0], [&] {
        GD_CUDA(cudaSetDevice(dev));
        std::lock_guard<std::mutex> lk(g_ens_mutex);
        if (!g_ens.exec || g_ens.key != key) {
          if (g_ens.exec) GD_CUDA(cudaGraphExecDestroy(g_ens.exec));
          g_ens.exec = nullptr;
          cudaGraph_t parent;
          GD_CUDA(cudaGraphCreate(&parent, 0));
          for (int i = 0; i < n; ++i) {
            cudaGraphNode_t node;
            GD_CUDA(cudaGraphAddChildGraphNode(&node, parent, nullptr, 0, gs[i]));
          }
          GD_CUDA(cudaGraphInstantiate(&g_ens.exec, parent, 0));
          GD_CUDA(cudaGraphDestroy(parent));
          g_ens.key = key;
        }
        // order: every member's earlier work before the launch, the launch
        // before every member's later work
        cudaStream_t s0 = ctxs[0]->d->stream;
        cudaEvent_t ev;
        GD_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        for (int i = 1; i < n; ++i) {
          GD_CUDA(cudaEventRecord(ev, ctxs[i]->d->stream));
          GD_CUDA(cudaStreamWaitEvent(s0, ev, 0));
        }
        for (int k = 0; k < rest; ++k) {
          GD_CUDA(cudaGraphLaunch(g_ens.exec, s0));
          for (int i = 0; i < n; ++i) ctxs[i]->d->ensemble_step_done();
        }
        GD_CUDA(cudaEventRecord(ev, s0));
        for (int i = 1; i < n; ++i) GD_CUDA(cudaStreamWaitEvent(ctxs[i]->d->stream, ev, 0));
        GD_CUDA(cudaEventDestroy(ev));
      });
      if (rc != GD_OK) return rc;
      s = nsteps;
      break;
    }
    // otherwise one step per member, each on its own stream (the first steps
    // of a context run eagerly, then capture its step)
    for (int i = 0; i < n; ++i) {
      const int rc = guarded(ctxs[i], [&] {
        GD_CUDA(cudaSetDevice(ctxs[i]->cfg.device));
        ctxs[i]->d->advance(1);
      });
      if (rc != GD_OK) return rc;
    }
    ++s;
  }
  for (int i = 0; i < n; ++i) {
    const int rc = guarded(ctxs[i], [&] {
      GD_CUDA(cudaSetDevice(ctxs[i]->cfg.device));
      GD_CUDA(cudaStreamSynchronize(ctxs[i]->d->stream));
      ctxs[i]->d->check();
    });
    if (rc != GD_OK) return rc;
  }
  return GD_OK;
}
// ln(1000) on the (0,0) coefficient: the constant field c has coefficient
// c * sqrt(4 pi) with orthonormal harmonics.  dyn_init.f90:46-48 and :160-162
// make the same change on the grid (spectogrd, x1000 or /1000 of exp,
// log, grdtospec), which returns the band-limited field exactly.
static const double kLn1000Y00 = std::log(1000.0) * std::sqrt(4.0 * 3.14159265358979323846);

int gd_read_sig(gd_ctx* ctx, const char* path, gd_sighead* head) {
  if (!ctx || !ctx->d) return GD_ERR_ARG;
  if (!path || !head) {
    ctx->err = "gd_read_sig: null argument";
    return GD_ERR_ARG;
  }
  const gd_config& c = ctx->cfg;
  const size_t n2 = (size_t)(c.ntrunc + 1) * (c.ntrunc + 2), L = (size_t)c.nlev, nt = (size_t)c.ntrac;
  std::vector<double> vrt, div, tv, trc, lnps, topo;
  try {
    vrt.resize(n2 * L), div.resize(n2 * L), tv.resize(n2 * L), trc.resize(n2 * L * nt);
    lnps.resize(n2), topo.resize(n2);
  } catch (const std::bad_alloc&) {
    ctx->err = "gd_read_sig: host allocation failed";
    return GD_ERR_NOMEM;
  }
  const int rc = gd_sigio_read(path, c.ntrunc, c.nlev, c.ntrac, head, vrt.data(), div.data(), tv.data(),
                               nt ? trc.data() : nullptr, lnps.data(), topo.data());
  if (rc != GD_OK) {
    ctx->err = gd_sigio_last_error();
    return rc;
  }
  lnps[0] += kLn1000Y00;  // ln(ps in cb) -> ln(ps in Pa)
  return gd_set_state(ctx, vrt.data(), div.data(), tv.data(), nt ? trc.data() : nullptr, lnps.data(),
                      topo.data());
}

int gd_write_sig(gd_ctx* ctx, const char* path, double fhour, gd_sighead* head) {
  if (!ctx || !ctx->d) return GD_ERR_ARG;
  if (!path || !head) {
    ctx->err = "gd_write_sig: null argument";
    return GD_ERR_ARG;
  }
  const gd_config& c = ctx->cfg;
  if (head->jcap != c.ntrunc || head->levs != c.nlev || head->ntrac < c.ntrac) {
    ctx->err = "gd_write_sig: header jcap/levs/ntrac do not match the context";
    return GD_ERR_ARG;
  }
  const size_t n2 = (size_t)(c.ntrunc + 1) * (c.ntrunc + 2), L = (size_t)c.nlev, nt = (size_t)c.ntrac;
  std::vector<double> vrt, div, tv, trc, lnps;
  try {
    vrt.resize(n2 * L), div.resize(n2 * L), tv.resize(n2 * L), trc.resize(n2 * L * nt), lnps.resize(n2);
  } catch (const std::bad_alloc&) {
    ctx->err = "gd_write_sig: host allocation failed";
    return GD_ERR_NOMEM;
  }
  double pdry = 0.0;
  int rc = guarded(ctx, [&] {
    ctx->d->get_state(vrt.data(), div.data(), tv.data(), nt ? trc.data() : nullptr, lnps.data());
    pdry = ctx->d->get_pdryini();
  });
  if (rc != GD_OK) return rc;
  lnps[0] -= kLn1000Y00;  // ln(ps in Pa) -> ln(ps in cb)
  if (ctx->topo.size() != n2) ctx->topo.assign(n2, 0.0);
  head->fhour = (float)fhour;
  head->pdryini = (float)(pdry / 1000.0);
  rc = gd_sigio_write(path, head, c.ntrac, vrt.data(), div.data(), tv.data(), nt ? trc.data() : nullptr,
                      lnps.data(), ctx->topo.data());
  if (rc != GD_OK) ctx->err = gd_sigio_last_error();
  return rc;
}

int gd_dcmip_ics(gd_ctx* ctx, int testcase) {
  if (!ctx || !ctx->d) return GD_ERR_ARG;
  const gd_config& c = ctx->cfg;
  const int tc = testcase / 10;
  const int L = c.nlev, nt = c.ntrac, nlon = c.nlon, nlat = c.nlat;
  const bool moist = !c.dry;
  std::string why;
  if (testcase < 0 || (tc != 4 && tc != 5)) why = "testcase must be 4x or 5x";
  else if (tc == 5 && !moist) why = "the tropical cyclone case needs dry = 0";
  else if (tc == 4 && nt < 3) why = "the baroclinic wave case writes 3 tracers (ntrac >= 3)";
  else if (tc == 5 && nt < 1) why = "the tropical cyclone case writes humidity (ntrac >= 1)";
  if (!why.empty()) {
    ctx->err = "gd_dcmip_ics: " + why;
    return GD_ERR_ARG;
  }
  const long ng = (long)nlon * nlat, nlm = (long)(c.ntrunc + 1) * (c.ntrunc + 2) / 2;
  const double fv = gd::Phys::rv / gd::Phys::rd - 1.0, kap = gd::Phys::rd / gd::Phys::cp;
  std::vector<double> lats(nlat);
  int rc = gd_grid_info(ctx, lats.data(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
  if (rc != GD_OK) return rc;
  auto LON = [&](long p) { return 2.0 * 3.14159265358979323846 * (double)(p % nlon) / nlon; };
  auto LAT = [&](long p) { return lats[p / nlon]; };
  // calc_pressdata (pressure_data.f90:58-100) on the host: prs [L][ng] bottom to top
  std::vector<double> prs((size_t)L * ng);
  auto pressdata = [&](const std::vector<double>& lnpsg) {
    for (long p = 0; p < ng; ++p) {
      const double ps = std::exp(lnpsg[p]);
      for (int k = 0; k < L; ++k) {
        const double pu = ctx->ak[k] + ctx->bk[k] * ps, pl = ctx->ak[k + 1] + ctx->bk[k + 1] * ps;
        prs[(size_t)(L - 1 - k) * ng + p] =
            std::pow((std::pow(pl, kap) * pl - std::pow(pu, kap) * pu) / ((kap + 1.) * (pl - pu)), 1. / kap);
      }
    }
  };
  std::vector<double> psg(ng), lnpsg(ng);
  if (tc == 4) {
    std::fill(psg.begin(), psg.end(), 1.e5);
  } else {  // a first pass only for ps (dyn_init.f90:359-373)
    for (long p = 0; p < ng; ++p) lnpsg[p] = std::log(1.015e5);
    pressdata(lnpsg);
    for (long p = 0; p < ng; ++p) psg[p] = gd::dcmip::test5(LON(p), LAT(p), prs[p]).ps;
  }
  for (long p = 0; p < ng; ++p) lnpsg[p] = std::log(psg[p]);
  pressdata(lnpsg);
  std::vector<double> ug((size_t)L * ng), vg(ug.size()), tvg(ug.size()), trcg((size_t)nt * L * ng, 0.0), phis(ng);
  auto fill = [&](long p0, long p1) {  // the analytic state at columns [p0, p1)
    for (int k = 0; k < L; ++k)
      for (long p = p0; p < p1; ++p) {
        const size_t o = (size_t)k * ng + p;
        double t, q;
        if (tc == 4) {
          const gd::dcmip::Point4 r = gd::dcmip::test4(moist, LON(p), LAT(p), prs[o]);
          ug[o] = r.u, vg[o] = r.v, t = r.t, q = r.q, phis[p] = r.phis;
          trcg[(size_t)(1 * L + k) * ng + p] = r.q1;
          trcg[(size_t)(2 * L + k) * ng + p] = r.q2;
        } else {
          const gd::dcmip::Point5 r = gd::dcmip::test5(LON(p), LAT(p), prs[o]);
          ug[o] = r.u, vg[o] = r.v, t = r.t, q = r.q, phis[p] = r.phis;
        }
        tvg[o] = moist ? t * (1. + fv * q) : t;
        trcg[o] = moist ? q : 0.0;  // tracer 1
      }
  };
  {  // host threads over disjoint column ranges
    const long nth = std::max(1L, std::min<long>(std::thread::hardware_concurrency(), ng / 4096 + 1));
    std::vector<std::thread> pool;
    for (long i = 0; i < nth; ++i) pool.emplace_back(fill, ng * i / nth, ng * (i + 1) / nth);
    for (auto& th : pool) th.join();
  }
  std::vector<double> vrt(2 * (size_t)L * nlm), div(vrt.size()), tv(vrt.size()), trc(2 * (size_t)nt * L * nlm),
      lnps(2 * (size_t)nlm), topo(2 * (size_t)nlm);
  for (long p = 0; p < ng; ++p) phis[p] = phis[p] / gd::Phys::grav;
  if ((rc = gd_getvrtdivspec(ctx, L, ug.data(), vg.data(), vrt.data(), div.data())) != GD_OK) return rc;
  if ((rc = gd_grdtospec(ctx, L, tvg.data(), tv.data())) != GD_OK) return rc;
  if (nt > 0 && (rc = gd_grdtospec(ctx, nt * L, trcg.data(), trc.data())) != GD_OK) return rc;
  if ((rc = gd_grdtospec(ctx, 1, lnpsg.data(), lnps.data())) != GD_OK) return rc;
  if ((rc = gd_grdtospec(ctx, 1, phis.data(), topo.data())) != GD_OK) return rc;
  return gd_set_state(ctx, vrt.data(), div.data(), tv.data(), nt ? trc.data() : nullptr, lnps.data(), topo.data());
}

int gd_dcmip_point(int testcase, int moist, double lon, double lat, double p, double* out) {
  if (!out || testcase < 0 || (testcase / 10 != 4 && testcase / 10 != 5)) return GD_ERR_ARG;
  if (testcase / 10 == 4) {
    const gd::dcmip::Point4 r = gd::dcmip::test4(moist != 0, lon, lat, p);
    const double v[8] = {r.u, r.v, r.t, r.phis, r.ps, r.q, r.q1, r.q2};
    memcpy(out, v, sizeof(v));
  } else {
    const gd::dcmip::Point5 r = gd::dcmip::test5(lon, lat, p);
    const double v[8] = {r.u, r.v, r.t, r.phis, r.ps, r.q, 0.0, 0.0};
    memcpy(out, v, sizeof(v));
  }
  return GD_OK;
}

int gd_set_stream(gd_ctx* ctx, void* stream) {
  return guarded(ctx, [&] {
    GD_CUDA(cudaStreamSynchronize(ctx->d->stream));
    if (ctx->d->own_stream) cudaStreamDestroy(ctx->d->stream);
    ctx->d->stream = (cudaStream_t)stream;
    ctx->d->own_stream = false;
  });
}
int gd_sync(gd_ctx* ctx) {
  return guarded(ctx, [&] {
    GD_CUDA(cudaStreamSynchronize(ctx->d->stream));
    ctx->d->check();
  });
}
long long gd_launch_count(gd_ctx* ctx) {
  (void)ctx;
  return gd::g_launches;
}
const char* gd_last_error(gd_ctx* ctx) {
  if (!ctx) return g_init_error.c_str();
  return ctx->err.c_str();
}

}  // extern "C"

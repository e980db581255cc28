// gd_pattern.cu -- the stochastic pattern generator of src/patterngenerator.f90
// (AR(1) random patterns in spherical-harmonic space with a Gaussian
// covariance) and the w3lib Mersenne twister it draws from
// (src/w3lib/mersenne_twister.f), on the GPU behind the C ABI.
//
// Arithmetic follows the reference's default build: IEEE single precision
// (kinds.f90:100 default_real = 1; w3lib's `real` is single).  Device
// expressions whose order matters use explicit round-to-nearest intrinsics
// so that nvcc does not fuse them; host set-up is compiled without FMA
// contraction.
//
// The Mersenne twister is one sequential stream per pattern, so one CTA owns
// it: the 624-word state lives in shared memory, each twist runs as the three
// dependency phases of the in-place recurrence (words [0,227) read only old
// words; [227,454) read [0,227); [454,624) read [227,397) and word 0), every
// thread then tempers one pair of words, applies the polar test and the
// accepted pairs are compacted with a block scan.  The stream stops exactly
// after the pair the reference's random_gauss would stop at.  The spectral
// work (getnoise scaling, the AR(1) steps) is elementwise over coefficients,
// with all requested steps of one coefficient in registers.
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "gd_api.h"
#include "gd_common.cuh"
#include "gd_pattern.cuh"

namespace gd {
namespace {

constexpr int MT_N = 624, MT_M = 397, MT_A = MT_N - MT_M;  // 227
constexpr int GT = 320;  // threads of the stream kernel: >= 312 pairs per twist

__device__ __forceinline__ uint32_t mt_mix(uint32_t hi, uint32_t lo, uint32_t far) {
  const uint32_t y = (hi & 0x80000000u) | (lo & 0x7fffffffu);
  return far ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}
__device__ __forceinline__ uint32_t mt_temper(uint32_t y) {
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}
// the word as w3lib's default real: the signed word (shifted by 2^32 if
// negative) over 2^32 - 1, a divisor that rounds to 2^32 in single precision
__device__ __forceinline__ float mt_unit(uint32_t y) {
  const int s = (int)y;
  const float two32 = 4294967296.0f;
  const float f = __int2float_rn(s);
  return s < 0 ? __fdiv_rn(__fadd_rn(f, two32), two32) : __fdiv_rn(f, two32);
}

// Draws `need` accepted pairs (2 need Gaussians, in stream order) from the
// stream whose state is mtg[624] and st[0] (the index of the next word).
__global__ void __launch_bounds__(GT) k_mt_gauss(uint32_t* __restrict__ mtg, int* __restrict__ st,
                                                 float* __restrict__ out, long need) {
  __shared__ uint32_t mt[MT_N];
  __shared__ int wsum[GT / 32];
  __shared__ int s_last;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < MT_N; i += GT) mt[i] = mtg[i];
  int mti = st[0];
  __syncthreads();
  long done = 0;
  while (done < need) {
    if (mti >= MT_N) {  // the twist (mersenne_twister.f:337-351), in three phases
      uint32_t v = 0;
      if (tid < MT_A) v = mt_mix(mt[tid], mt[tid + 1], mt[tid + MT_M]);
      __syncthreads();
      if (tid < MT_A) mt[tid] = v;
      __syncthreads();
      int kk = tid + MT_A;
      if (tid < MT_A) v = mt_mix(mt[kk], mt[kk + 1], mt[kk - MT_A]);
      __syncthreads();
      if (tid < MT_A) mt[kk] = v;
      __syncthreads();
      kk = tid + 2 * MT_A;
      if (kk < MT_N - 1)
        v = mt_mix(mt[kk], mt[kk + 1], mt[kk - MT_A]);
      else if (kk == MT_N - 1)
        v = mt_mix(mt[MT_N - 1], mt[0], mt[MT_M - 1]);
      __syncthreads();
      if (kk < MT_N) mt[kk] = v;
      __syncthreads();
      mti = 0;
    }
    // polar test of the uniform pairs left in this block (mti is even)
    const int npair = (MT_N - mti) >> 1;
    bool acc = false;
    float v1 = 0.f, v2 = 0.f, r = 1.f;
    if (tid < npair) {
      const float u1 = mt_unit(mt_temper(mt[mti + 2 * tid])), u2 = mt_unit(mt_temper(mt[mti + 2 * tid + 1]));
      v1 = __fsub_rn(__fmul_rn(2.f, u1), 1.f);
      v2 = __fsub_rn(__fmul_rn(2.f, u2), 1.f);
      r = __fadd_rn(__fmul_rn(v1, v1), __fmul_rn(v2, v2));
      acc = r < 1.f;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, acc);
    if (lane == 0) wsum[warp] = __popc(bal);
    __syncthreads();
    int base = 0, total = 0;
    for (int w = 0; w < GT / 32; ++w) {
      const int c = wsum[w];
      if (w < warp) base += c;
      total += c;
    }
    const int rank = base + __popc(bal & ((1u << lane) - 1u));
    const long left = need - done;
    if (acc && rank < left) {
      const float fac = __fsqrt_rn(__fdiv_rn(__fmul_rn(-2.f, logf(r)), r));
      out[2 * (done + rank)] = __fmul_rn(v1, fac);
      out[2 * (done + rank) + 1] = __fmul_rn(v2, fac);
      if (rank == left - 1) s_last = tid;
    }
    __syncthreads();
    if (total >= left) {  // stop right after the last pair needed
      mti += 2 * (s_last + 1);
      done = need;
    } else {
      done += total;
      mti = MT_N;
    }
  }
  __syncthreads();
  for (int i = tid; i < MT_N; i += GT) mtg[i] = mt[i];
  if (tid == 0) st[0] = mti;
}

// getnoise (patterngenerator.f90:115-132) for nsteps x nfields draws held in
// g ([step][field][2 nlm] Gaussians), then per mode:
//   0  the start of stoch_data.f90:58: x = (stdev * noise) * varspectrum
//   1  patterngenerator_advance (:134-143): x = phi x + (stdev sqrt(1-phi^2) vs) noise
//   2  the raw noise
__global__ void k_pattern_update(float2* __restrict__ x_io, const float* __restrict__ vs,
                                 const int2* __restrict__ dego, const float* __restrict__ g, int nlm, int nfields,
                                 int nsteps, int mode, float phi, float stdev, float nf) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)nfields * nlm) return;
  const int f = (int)(e / nlm), n = (int)(e - (long)f * nlm);
  const int2 d = dego[n];  // (degree, order)
  const float sq = __fsqrt_rn(__fadd_rn(__fmul_rn(2.f, (float)d.x), 1.f));
  const float s2 = __fsqrt_rn(2.f);
  const float vn = vs[n];
  const float av = __fmul_rn(__fmul_rn(stdev, __fsqrt_rn(__fsub_rn(1.f, __fmul_rn(phi, phi)))), vn);
  float2 x = mode == 1 ? x_io[e] : make_float2(0.f, 0.f);
  for (int s = 0; s < nsteps; ++s) {
    const float* gs = g + ((long)s * nfields + f) * 2 * nlm;
    float gr = gs[n], gi = gs[n + nlm];
    if (n == 0) gr = gi = 0.f;  // noiser(1) = noiser(ndimspec+1) = 0
    float2 z;
    if (d.y != 0) {
      z.x = __fdiv_rn(gr, sq);
      z.y = __fdiv_rn(gi, sq);
    } else {
      z.x = __fdiv_rn(__fmul_rn(s2, gr), sq);
      z.y = 0.f;
    }
    z.x = __fmul_rn(z.x, nf);
    z.y = __fmul_rn(z.y, nf);
    if (mode == 0) {
      x.x = __fmul_rn(__fmul_rn(stdev, z.x), vn);
      x.y = __fmul_rn(__fmul_rn(stdev, z.y), vn);
    } else if (mode == 1) {
      x.x = __fadd_rn(__fmul_rn(phi, x.x), __fmul_rn(av, z.x));
      x.y = __fadd_rn(__fmul_rn(phi, x.y), __fmul_rn(av, z.y));
    } else {
      x = z;
    }
  }
  x_io[e] = x;
}

}  // namespace
}  // namespace gd

// ------------------------------------------------------------------ C ABI --
struct gd_pattern {
  int device = 0, jcap = 0, nlm = 0, nfields = 1, nlon = 0, nlat = 0, seed = 0;
  float lengthscale = 0, tau = 0, dt = 0, phi = 0, stdev = 0, normfact = 0, nf = 0;
  std::vector<float> vs, vs1d;  // varspectrum [nlm], varspectrum1d [jcap+1]
  std::vector<int2> dego;       // (degree, order) per coefficient, m-major
  float2* d_spec = nullptr;     // [nfields][nlm] pattern coefficients
  float2* d_noise = nullptr;    // [nlm] raw noise of gd_pattern_getnoise
  float* d_vs = nullptr;
  int2* d_dego = nullptr;
  uint32_t* d_mt = nullptr;  // stream state: 624 words
  int* d_st = nullptr;       // index of the next word
  float* d_g = nullptr;      // Gaussians of up to gsteps draws of all fields
  int gsteps = 1;
  cudaStream_t stream = nullptr;
  long long launches = 0;
  std::string err;
  std::vector<void*> allocs;
  void* alloc(size_t bytes) {
    void* p = nullptr;
    GD_CUDA(cudaMalloc(&p, bytes));
    allocs.push_back(p);
    return p;
  }
  ~gd_pattern() {
    int cur = 0;
    if (cudaGetDevice(&cur) == cudaSuccess) {
      cudaSetDevice(device);
      for (void* p : allocs) cudaFree(p);
      cudaSetDevice(cur);
    }
  }
  // gaussian_spect (patterngenerator.f90:145-177) and computevarspec (:73-88),
  // single precision, sums in coefficient order
  void spectra() {
    const float rerth = 6.3712e+6f;  // physcons.f90:23
    vs1d.resize(jcap + 1);
    vs.resize(nlm);
    std::vector<float> lap(nlm);
    for (int i = 0; i < nlm; ++i) lap[i] = (float)(-dego[i].x) * ((float)dego[i].x + 1.0f);
    for (int n = 0; n <= jcap; ++n)
      vs1d[n] = std::exp(-(lengthscale * lengthscale * ((float)n * ((float)n + 1.f)) / (4.f * (rerth * rerth))));
    for (int i = 0; i < nlm; ++i)
      vs[i] = std::sqrt((float)jcap * std::exp(lengthscale * lengthscale * lap[i] / (4.f * (rerth * rerth))));
    // variance of the unit template pattern, scaled as getnoise scales white noise
    float var = 0.f;
    for (int i = 0; i < nlm; ++i) {
      const float s = std::sqrt(2.f * (float)dego[i].x + 1.f);
      float re, im;
      if (dego[i].y != 0) {
        re = 1.f / s;
        im = 1.f / s;
      } else {
        re = std::sqrt(2.f) / s;
        im = 0.f;
      }
      if (i == 0) re = im = 0.f;  // no global mean
      re = re * nf;
      im = im * nf;
      re = vs[i] * re;
      im = vs[i] * im;
      if (dego[i].y != 0) {
        var = var + (re * re - im * (-im));
      } else {
        const float hr = 0.5f * re, hi = 0.5f * im;
        var = var + (hr * re - hi * (-im));
      }
    }
    var = var / normfact;
    const float sv = std::sqrt(var);
    for (int i = 0; i < nlm; ++i) vs[i] = vs[i] / sv;
    for (int n = 0; n <= jcap; ++n) vs1d[n] = vs1d[n] / var;
  }
  void draw(long pairs, cudaStream_t s) {  // the next `pairs` accepted Gaussian pairs into d_g
    gd::k_mt_gauss<<<1, gd::GT, 0, s>>>(d_mt, d_st, d_g, pairs);
    ++launches;
    GD_LAUNCH_CHECK();
  }
  void update(float2* x, int nf_, int nsteps, int mode, cudaStream_t s) {
    const long n = (long)nf_ * nlm;
    gd::k_pattern_update<<<gd::ceil_div(n, 256), 256, 0, s>>>(x, d_vs, d_dego, d_g, nlm, nf_, nsteps, mode, phi,
                                                              stdev, nf);
    ++launches;
    GD_LAUNCH_CHECK();
  }
  void advance_on(int nsteps, cudaStream_t s) {
    for (int s0 = 0; s0 < nsteps; s0 += gsteps) {
      const int ns = std::min(gsteps, nsteps - s0);
      draw((long)ns * nfields * nlm, s);
      update(d_spec, nfields, ns, 1, s);
    }
  }
};

// internal interface for the dycore's stochastic physics (gd_pattern.cuh)
namespace gd {
void pattern_advance_on(gd_pattern* p, int nsteps, cudaStream_t s) {
  p->advance_on(nsteps, s);
  count_launch(2 * ((nsteps + p->gsteps - 1) / p->gsteps));
}
const float2* pattern_spec(const gd_pattern* p) { return p->d_spec; }
int pattern_jcap(const gd_pattern* p) { return p->jcap; }
int pattern_device(const gd_pattern* p) { return p->device; }
int pattern_nfields(const gd_pattern* p) { return p->nfields; }
}  // namespace gd

namespace {
template <typename F>
int pguard(gd_pattern* p, F f) {
  if (!p) return GD_ERR_ARG;
  try {
    int cur = 0;
    GD_CUDA(cudaGetDevice(&cur));
    if (cur != p->device) GD_CUDA(cudaSetDevice(p->device));
    f();
    if (cur != p->device) GD_CUDA(cudaSetDevice(cur));
    return GD_OK;
  } catch (const gd::CudaError& e) {
    p->err = e.what();
    return GD_ERR_CUDA;
  } catch (const std::invalid_argument& e) {
    p->err = e.what();
    return GD_ERR_ARG;
  } catch (const std::exception& e) {
    p->err = e.what();
    return GD_ERR_CUDA;
  }
}
std::string g_pattern_init_error;
}  // namespace

extern "C" {

int gd_pattern_init(double lscale, double delt, double tscale, double stdev, int iseed, int nlon, int nlat,
                    int jcap, double normalization, int nfields, int device, gd_pattern** out) {
  if (!out) return GD_ERR_ARG;
  *out = nullptr;
  if (jcap < 1 || nfields < 1 || !(delt > 0) || !(tscale > 0) || !(normalization > 0) || lscale < 0) {
    g_pattern_init_error = "gd_pattern_init: need jcap >= 1, nfields >= 1, delt > 0, tscale > 0, normalization > 0";
    return GD_ERR_ARG;
  }
  std::unique_ptr<gd_pattern> p(new gd_pattern());
  p->device = device;
  p->jcap = jcap;
  p->nlm = (jcap + 1) * (jcap + 2) / 2;
  p->nfields = nfields;
  p->nlon = nlon;
  p->nlat = nlat;
  p->lengthscale = (float)lscale;
  p->dt = (float)delt;
  p->tau = (float)tscale;
  p->stdev = (float)stdev;
  p->normfact = (float)normalization;
  p->phi = std::exp(-p->dt / p->tau);
  p->nf = std::sqrt(p->normfact / (float)jcap);
  // seed 0: a seed from the clock, as patterngenerator.f90:54-57 does
  p->seed = iseed != 0 ? iseed
                       : (int)(std::chrono::steady_clock::now().time_since_epoch().count() & 0x7fffffff) | 1;
  p->dego.resize(p->nlm);
  for (int m = 0, i = 0; m <= jcap; ++m)
    for (int n = m; n <= jcap; ++n, ++i) p->dego[i] = make_int2(n, m);
  p->spectra();
  const int rc = pguard(p.get(), [&] {
    const long nlm = p->nlm;
    p->gsteps = (int)std::max<long>(1, std::min<long>(64, (1L << 26) / (2 * nlm * nfields)));
    p->d_spec = (float2*)p->alloc(sizeof(float2) * nlm * nfields);
    p->d_noise = (float2*)p->alloc(sizeof(float2) * nlm);
    p->d_vs = (float*)p->alloc(sizeof(float) * nlm);
    p->d_dego = (int2*)p->alloc(sizeof(int2) * nlm);
    p->d_mt = (uint32_t*)p->alloc(sizeof(uint32_t) * gd::MT_N);
    p->d_st = (int*)p->alloc(sizeof(int));
    p->d_g = (float*)p->alloc(sizeof(float) * 2 * nlm * nfields * p->gsteps);
    // random_setseed_t (mersenne_twister.f:282-296): mt[i] = 69069 mt[i-1]
    uint32_t mt[gd::MT_N];
    mt[0] = (uint32_t)p->seed;
    for (int i = 1; i < gd::MT_N; ++i) mt[i] = 69069u * mt[i - 1];
    const int mti = gd::MT_N;
    GD_CUDA(cudaMemcpy(p->d_mt, mt, sizeof(mt), cudaMemcpyHostToDevice));
    GD_CUDA(cudaMemcpy(p->d_st, &mti, sizeof(int), cudaMemcpyHostToDevice));
    GD_CUDA(cudaMemcpy(p->d_vs, p->vs.data(), sizeof(float) * nlm, cudaMemcpyHostToDevice));
    GD_CUDA(cudaMemcpy(p->d_dego, p->dego.data(), sizeof(int2) * nlm, cudaMemcpyHostToDevice));
    GD_CUDA(cudaMemset(p->d_spec, 0, sizeof(float2) * nlm * nfields));
  });
  if (rc != GD_OK) {
    g_pattern_init_error = p->err;
    return rc;
  }
  *out = p.release();
  return GD_OK;
}

int gd_pattern_destroy(gd_pattern* p) {
  if (!p) return GD_ERR_ARG;
  delete p;
  return GD_OK;
}

int gd_pattern_set_stream(gd_pattern* p, void* stream) {
  if (!p) return GD_ERR_ARG;
  p->stream = (cudaStream_t)stream;
  return GD_OK;
}

int gd_pattern_start(gd_pattern* p) {
  return pguard(p, [&] {
    p->draw((long)p->nfields * p->nlm, p->stream);
    p->update(p->d_spec, p->nfields, 1, 0, p->stream);
  });
}

int gd_pattern_advance(gd_pattern* p, int nsteps) {
  if (p && nsteps < 0) return GD_ERR_ARG;
  return pguard(p, [&] { p->advance_on(nsteps, p->stream); });
}

int gd_pattern_getnoise(gd_pattern* p, double* noise) {
  if (p && !noise) return GD_ERR_ARG;
  return pguard(p, [&] {
    p->draw(p->nlm, p->stream);
    p->update(p->d_noise, 1, 1, 2, p->stream);
    std::vector<float2> h(p->nlm);
    GD_CUDA(cudaMemcpyAsync(h.data(), p->d_noise, sizeof(float2) * p->nlm, cudaMemcpyDeviceToHost, p->stream));
    GD_CUDA(cudaStreamSynchronize(p->stream));
    for (int i = 0; i < p->nlm; ++i) {
      noise[2 * i] = h[i].x;
      noise[2 * i + 1] = h[i].y;
    }
  });
}

int gd_pattern_get(gd_pattern* p, double* spec) {
  if (p && !spec) return GD_ERR_ARG;
  return pguard(p, [&] {
    const long n = (long)p->nfields * p->nlm;
    std::vector<float2> h(n);
    GD_CUDA(cudaMemcpyAsync(h.data(), p->d_spec, sizeof(float2) * n, cudaMemcpyDeviceToHost, p->stream));
    GD_CUDA(cudaStreamSynchronize(p->stream));
    for (long i = 0; i < n; ++i) {
      spec[2 * i] = h[i].x;
      spec[2 * i + 1] = h[i].y;
    }
  });
}

int gd_pattern_set(gd_pattern* p, const double* spec) {
  if (p && !spec) return GD_ERR_ARG;
  return pguard(p, [&] {
    const long n = (long)p->nfields * p->nlm;
    std::vector<float2> h(n);
    for (long i = 0; i < n; ++i) h[i] = make_float2((float)spec[2 * i], (float)spec[2 * i + 1]);
    GD_CUDA(cudaMemcpyAsync(p->d_spec, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice, p->stream));
    GD_CUDA(cudaStreamSynchronize(p->stream));
  });
}

int gd_pattern_spectra(gd_pattern* p, double* varspectrum, double* varspectrum1d, double* phi) {
  if (!p) return GD_ERR_ARG;
  if (varspectrum)
    for (int i = 0; i < p->nlm; ++i) varspectrum[i] = p->vs[i];
  if (varspectrum1d)
    for (int n = 0; n <= p->jcap; ++n) varspectrum1d[n] = p->vs1d[n];
  if (phi) *phi = p->phi;
  return GD_OK;
}

int gd_pattern_sync(gd_pattern* p) {
  return pguard(p, [&] { GD_CUDA(cudaStreamSynchronize(p->stream)); });
}

long long gd_pattern_launch_count(gd_pattern* p) { return p ? p->launches : -1; }

const char* gd_pattern_last_error(gd_pattern* p) {
  return p ? p->err.c_str() : g_pattern_init_error.c_str();
}

}  // extern "C"

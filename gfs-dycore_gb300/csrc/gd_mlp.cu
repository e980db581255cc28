// gd_mlp.cu -- the learned per-column closure's network: a fully connected
// net nin -> nh (GELU) -> ... -> nh (GELU) -> nout with BF16 weights and FP32
// accumulation.  Forward and backward passes, the mean-squared-error loss and
// Adam run as CUDA kernels on the net's stream; the dycore applies a trained
// net to its grid columns once per step (gd_set_closure, gd_dycore.cu).
//
// Parameters are one FP32 master array, layer after layer: W_l [fout][fin]
// row-major, then b_l [fout].  The forward and backward passes read the
// weights from a BF16 copy made after every update (biases stay FP32), so a
// trained net is exactly the BF16 net it is evaluated as.
//
// The products with the batch (the grid's columns) as rows, X W^T and dZ W,
// run on the tensor cores (k_tc_mlp in gd_tc.cu) when every layer is at most
// 256 wide: the weights are exact in TF32 and each activation or gradient is
// split into TF32 hi + lo, so two MMAs per K step give the FP32 products of
// the BF16 net.  That covers inference (gd_mlp_forward and the closure in
// the step), the training forward pass (which also stores each hidden
// layer's Z and A) and the backward product dZ_l W_l with the GELU
// derivative fused.  The weight gradient dZ^T A, a reduction over the batch,
// runs on the tensor cores too (k_tc_wgrad): both operands transposed with
// the batch contiguous and split hi + lo (k_tsplit), the batch in K slices
// whose partial tiles k_wsum adds in order.  Nets wider than 256 (and
// GD_MLP_TRAIN_TC=0) train on a tiled SIMT GEMM: 64 x 64 output tiles, K in
// steps of 16 through shared memory, 4 x 4 outputs per thread, operands
// addressed through (row, column) strides, split K for the weight gradient.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdlib>
#include <cstdint>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "gd_api.h"
#include "gd_common.cuh"
#include "gd_mlp.cuh"
#include "gd_tc.cuh"

struct gd_mlp {
  int device = 0;
  int nin = 0, nh = 0, nl = 0, nout = 0;  // nl hidden layers
  int nlayer = 0;                          // nl + 1 linear layers
  std::vector<int> fin, fout;
  std::vector<long> offw, offb;  // offsets of W_l and b_l in the parameter array
  long np = 0;
  float* p32 = nullptr;          // master parameters
  __nv_bfloat16* w16 = nullptr;  // BF16 copy (all np entries; the bias slots are unused)
  float* grad = nullptr;
  float* am = nullptr;  // Adam moments
  float* av = nullptr;
  long adam_t = 0;
  // normalisation of the closure's inputs and outputs (device, nin / nout)
  float *in_mu = nullptr, *in_sd = nullptr, *out_mu = nullptr, *out_sd = nullptr;
  bool has_norm = false;
  // activations: Z_l (pre-activation) and A_l (GELU) of each hidden layer,
  // the output and its gradient, two gradient buffers for the backward pass
  int bcap = 0;
  float *zb = nullptr, *ab = nullptr, *yb = nullptr, *gy = nullptr, *g0 = nullptr, *g1 = nullptr;
  float* partial = nullptr;  // loss partial sums
  float* kpart = nullptr;    // split-K partial weight gradients
  float* lossd = nullptr;
  // tensor-core inference (gd_tc.cu, k_tc_mlp): weights exact in TF32, padded
  // to [Np][Kp] per layer; the input and hidden activations split hi + lo
  bool tc = false;
  std::vector<int> kp, npd;
  std::vector<long> tcoff;
  float* wtc = nullptr;
  uint32_t *xh = nullptr, *xl = nullptr;
  uint32_t* hh[2] = {nullptr, nullptr};
  uint32_t* hl[2] = {nullptr, nullptr};
  std::vector<gd::TcMlpLayer> layers;
  // tensor-core training: the forward pass that keeps Z and A (tlayers) and
  // the backward products dZ_l W_l (blayers, l >= 1) against the weights
  // transposed to [npt][kpt] (wtct); the output gradient and the hidden
  // gradients split hi + lo (gyh/gyl, dzh/dzl ping-pong)
  bool tcb = false;
  std::vector<int> kpt, npt;
  std::vector<long> tctoff;
  float* wtct = nullptr;
  uint32_t *gyh = nullptr, *gyl = nullptr;
  uint32_t* dzh[2] = {nullptr, nullptr};
  uint32_t* dzl[2] = {nullptr, nullptr};
  std::vector<gd::TcMlpLayer> tlayers, blayers;
  // the weight gradients dZ_l^T A_{l-1}: dZ and the layer inputs transposed
  // (batch contiguous) and split, the slices' partial tiles
  std::vector<gd::TcWgrad> wgl;
  uint32_t *zth = nullptr, *ztl = nullptr, *ath = nullptr, *atl = nullptr;
  float* wpart = nullptr;
  int tcap = 0;        // batch capacity of the training buffers
  int tbcap = 0;       // bcap the training layers were built over
  int wsplit_max = 0;  // slices the partial buffer holds
  int* terr = nullptr;
  cudaStream_t stream = nullptr;  // the stream the net's work runs on
  cudaStream_t own = nullptr;     // the net's own stream (destroyed with it)
  std::string err;
  std::vector<void*> allocs;
  void* alloc(size_t bytes) {
    void* p = nullptr;
    GD_CUDA(cudaMalloc(&p, std::max<size_t>(bytes, 16)));
    allocs.push_back(p);
    return p;
  }
  ~gd_mlp() {
    int cur = 0;
    if (cudaGetDevice(&cur) == cudaSuccess && cur != device) cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    for (void* p : allocs)
      if (p) cudaFree(p);
    if (own) cudaStreamDestroy(own);
    if (cur != device) cudaSetDevice(cur);
  }
};

namespace gd {
namespace {

constexpr int GM = 64, GN = 64, GK = 16;
constexpr int KPART = 256;  // loss partial sums

__device__ __forceinline__ float tofloat(float x) { return x; }
__device__ __forceinline__ float tofloat(__nv_bfloat16 x) { return __bfloat162float(x); }

// GELU with the exact normal CDF, and its derivative
__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float z) {
  return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// C(m, n) = sum_k A(m, k) B(k, n) with A(m, k) = A[m sam + k sak], B(k, n) =
// B[k sbk + n sbn]; epi(m, n, c) takes each output
template <typename TA, typename TB, typename Epi>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, int kchunk, const TA* __restrict__ A, long sam,
                                              long sak, const TB* __restrict__ B, long sbk, long sbn, Epi epi) {
  __shared__ float As[GK][GM + 4];
  __shared__ float Bs[GK][GN + 4];
  const int tid = threadIdx.x;
  const int m0 = blockIdx.y * GM, n0 = blockIdx.x * GN;
  const int tm = (tid >> 4) * 4, tn = (tid & 15) * 4;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
  const bool a_kfast = sak == 1, b_nfast = sbn == 1;
  // split K: this CTA sums k in [kb, ke) (blockIdx.z-th chunk)
  const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
  for (int k0 = kb; k0 < ke; k0 += GK) {
    for (int e = tid; e < GM * GK; e += 256) {  // the unit-stride index fastest over the threads
      const int mm = a_kfast ? e / GK : e % GM, kk = a_kfast ? e % GK : e / GM;
      const int m = m0 + mm, k = k0 + kk;
      As[kk][mm] = (m < M && k < ke) ? tofloat(A[(long)m * sam + (long)k * sak]) : 0.f;
    }
    for (int e = tid; e < GK * GN; e += 256) {
      const int nn = b_nfast ? e % GN : e / GK, kk = b_nfast ? e / GN : e % GK;
      const int n = n0 + nn, k = k0 + kk;
      Bs[kk][nn] = (n < N && k < ke) ? tofloat(B[(long)k * sbk + (long)n * sbn]) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        a[i] = As[kk][tm + i];
        b[i] = Bs[kk][tn + i];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int m = m0 + tm + i, n = n0 + tn + j;
      if (m < M && n < N) epi(m + blockIdx.z * M, n, acc[i][j]);  // split K: partial z at rows zM..
    }
}

struct EpiHidden {  // Z = acc + b, A = GELU(Z)
  const float* b;
  float* Z;
  float* Aout;
  int N;
  __device__ void operator()(int m, int n, float c) const {
    const float z = c + b[n];
    Z[(long)m * N + n] = z;
    Aout[(long)m * N + n] = gelu(z);
  }
};
struct EpiLinear {  // Y = acc + b
  const float* b;
  float* Y;
  int N;
  __device__ void operator()(int m, int n, float c) const { Y[(long)m * N + n] = c + b[n]; }
};
struct EpiStore {  // G = acc
  float* G;
  int N;
  __device__ void operator()(int m, int n, float c) const { G[(long)m * N + n] = c; }
};
struct EpiGeluD {  // dZ = acc * GELU'(Z)
  const float* Z;
  float* G;
  int N;
  __device__ void operator()(int m, int n, float c) const {
    const long i = (long)m * N + n;
    G[i] = c * gelu_d(Z[i]);
  }
};

template <typename TA, typename TB, typename Epi>
void gemm(int M, int N, int K, const TA* A, long sam, long sak, const TB* B, long sbk, long sbn, Epi epi,
          cudaStream_t s) {
  if (M <= 0 || N <= 0) return;
  dim3 grid((unsigned)ceil_div(N, GN), (unsigned)ceil_div(M, GM));
  k_gemm<TA, TB, Epi><<<grid, 256, 0, s>>>(M, N, K, K, A, sam, sak, B, sbk, sbn, epi);
  count_launch();
  GD_LAUNCH_CHECK();
}
// C = A B with K split into nsplit chunks: partial z goes to part[z][M][N],
// then the partials are summed in order (deterministic) into out [M][N]
constexpr int KSPLIT = 16;
__global__ void k_sum_parts(const float* __restrict__ part, int nsplit, long count, float* __restrict__ out) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (long)gridDim.x * blockDim.x) {
    float t = 0.f;
    for (int z = 0; z < nsplit; ++z) t += part[z * count + i];
    out[i] = t;
  }
}
template <typename TA, typename TB>
void gemm_splitk(int M, int N, int K, const TA* A, long sam, long sak, const TB* B, long sbk, long sbn, float* part,
                 float* out, cudaStream_t s) {
  if (M <= 0 || N <= 0) return;
  const int nsplit = std::max(1, std::min(KSPLIT, K / 256));
  const int kchunk = (ceil_div(K, nsplit) + GK - 1) / GK * GK;
  const int ns = ceil_div(K, kchunk);
  dim3 grid((unsigned)ceil_div(N, GN), (unsigned)ceil_div(M, GM), (unsigned)ns);
  k_gemm<TA, TB, EpiStore><<<grid, 256, 0, s>>>(M, N, K, kchunk, A, sam, sak, B, sbk, sbn, EpiStore{part, N});
  const long cnt = (long)M * N;
  k_sum_parts<<<std::min(ceil_div(cnt, 256), 1024), 256, 0, s>>>(part, ns, cnt, out);
  count_launch(2);
  GD_LAUNCH_CHECK();
}

// db[n] = sum_m G[m][n] (fixed order: 8 strided partial sums, then a tree)
__global__ void k_colsum(const float* __restrict__ G, int M, int N, float* db) {
  __shared__ float red[8][33];
  const int n = blockIdx.x * 32 + threadIdx.x;
  float s = 0.f;
  if (n < N)
    for (int m = threadIdx.y; m < M; m += 8) s += G[(long)m * N + n];
  red[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && n < N) {
    float t = 0.f;
#pragma unroll
    for (int y = 0; y < 8; ++y) t += red[y][threadIdx.x];
    db[n] = t;
  }
}

// squared error: gy = 2 (y - t) / count, partial[block] = sum (y - t)^2
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ t, long count, float* gy,
                      float* partial) {
  __shared__ float red[256];
  float s = 0.f;
  const float sc = 2.f / (float)count;
  for (long i = (long)blockIdx.x * 256 + threadIdx.x; i < count; i += (long)gridDim.x * 256) {
    const float d = y[i] - t[i];
    s += d * d;
    if (gy) gy[i] = sc * d;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}
__global__ void k_mse_final(const float* partial, int n, long count, float* loss) {
  __shared__ float red[KPART];
  red[threadIdx.x] = threadIdx.x < n ? partial[threadIdx.x] : 0.f;
  __syncthreads();
  for (int o = KPART / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = red[0] / (float)count;
}

__global__ void k_adam(float* p, const float* g, float* m, float* v, __nv_bfloat16* w16, long n, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    w16[i] = __float2bfloat16_rn(pi);
  }
}
__global__ void k_to_bf16(const float* p, __nv_bfloat16* w16, long n) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    w16[i] = __float2bfloat16_rn(p[i]);
}

// a layer's BF16 weights as FP32 (exact in TF32), padded to [Np][Kp] with zeros
__global__ void k_w_tc(const __nv_bfloat16* __restrict__ w, int fo, int fi, int Np, int Kp, float* __restrict__ o) {
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < (long)Np * Kp; e += (long)gridDim.x * blockDim.x) {
    const int n = (int)(e / Kp), k = (int)(e % Kp);
    o[e] = (n < fo && k < fi) ? __bfloat162float(w[(long)n * fi + k]) : 0.f;
  }
}
// the same weights transposed, [Np][Kp] with Np >= fi and Kp >= fo: the B
// operand of the backward product dZ W
__global__ void k_w_tc_t(const __nv_bfloat16* __restrict__ w, int fo, int fi, int Np, int Kp, float* __restrict__ o) {
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < (long)Np * Kp; e += (long)gridDim.x * blockDim.x) {
    const int n = (int)(e / Kp), k = (int)(e % Kp);
    o[e] = (n < fi && k < fo) ? __bfloat162float(w[(long)k * fi + n]) : 0.f;
  }
}
// rows r < nbc of src [n][w] (rows r >= n read as zero) transposed and
// split to TF32 hi + lo: dh / dl [c][r], row pitch kp -- the operands of a
// weight gradient, with the batch contiguous
__global__ void k_tsplit(const float* __restrict__ src, int n, int w, int nbc, int kp, uint32_t* __restrict__ dh,
                         uint32_t* __restrict__ dl) {
  __shared__ float t[32][33];
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int r = r0 + i, c = c0 + threadIdx.x;
    t[i][threadIdx.x] = (r < n && c < w) ? src[(long)r * w + c] : 0.f;
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int c = c0 + i, r = r0 + threadIdx.x;
    if (c < w && r < nbc) {
      const float v = t[threadIdx.x][i];
      const uint32_t h = (__float_as_uint(v) + 0x1000u) & 0xFFFFE000u;  // nearest TF32, ties away
      dh[(long)c * kp + r] = h;
      dl[(long)c * kp + r] = __float_as_uint(v - __uint_as_float(h));
    }
  }
}
// dW [fo][fi] = the sum of the slices' partial tiles [Mp][Np], in slice order
__global__ void k_wsum(const float* __restrict__ part, int nsplit, int Mp, int Np, int fo, int fi,
                       float* __restrict__ dw) {
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < (long)fo * fi; e += (long)gridDim.x * blockDim.x) {
    const int m = (int)(e / fi), c = (int)(e % fi);
    float s = 0.f;
    for (int q = 0; q < nsplit; ++q) s += part[((long)q * Mp + m) * Np + c];
    dw[e] = s;
  }
}
// inputs x [n][nin] split to TF32 hi + lo rows of pitch Kp (the padding
// columns stay zero from allocation)
__global__ void k_split_in(const float* __restrict__ x, long n, int nin, int Kp, uint32_t* __restrict__ xh,
                           uint32_t* __restrict__ xl) {
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n * nin; e += (long)gridDim.x * blockDim.x) {
    const long m = e / nin;
    const int k = (int)(e % nin);
    const float v = x[e];
    const uint32_t h = (__float_as_uint(v) + 0x1000u) & 0xFFFFE000u;  // nearest TF32, ties away
    xh[m * Kp + k] = h;
    xl[m * Kp + k] = __float_as_uint(v - __uint_as_float(h));
  }
}

template <typename F>
int mguard(gd_mlp* p, F f) {
  if (!p) return GD_ERR_ARG;
  try {
    int cur = 0;
    GD_CUDA(cudaGetDevice(&cur));
    if (cur != p->device) GD_CUDA(cudaSetDevice(p->device));
    f();
    if (cur != p->device) GD_CUDA(cudaSetDevice(cur));
    return GD_OK;
  } catch (const CudaError& e) {
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
std::string g_mlp_init_error;

// x, t and y of the batch entry points must be device memory of the net's
// device (a host pointer would fault the kernels)
void need_device(const gd_mlp* p, const void* ptr, const char* what) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
    cudaGetLastError();
    throw std::invalid_argument(std::string("gd_mlp: ") + what + " is not a device pointer");
  }
  if ((a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) || a.device != p->device)
    throw std::invalid_argument(std::string("gd_mlp: ") + what + " is not device memory of the net's device");
}

void to_bf16(gd_mlp* p) {
  k_to_bf16<<<std::min(ceil_div(p->np, 256), 4096), 256, 0, p->stream>>>(p->p32, p->w16, p->np);
  count_launch();
  GD_LAUNCH_CHECK();
}

}  // namespace

// --------------------------------------------------- shared with the dycore
// Grows the activation buffers to ncols columns.  The old buffers are kept
// until the net is destroyed: a context's captured step may still address
// them (a step graph holds the buffers and tensor maps of its capture).
void mlp_reserve(gd_mlp* p, int ncols) {
  if (ncols <= p->bcap) return;
  GD_CUDA(cudaStreamSynchronize(p->stream));
  const long w = std::max(p->nh, std::max(p->nin, p->nout));
  p->zb = (float*)p->alloc(sizeof(float) * (size_t)p->nl * ncols * p->nh);
  p->ab = (float*)p->alloc(sizeof(float) * (size_t)p->nl * ncols * p->nh);
  p->yb = (float*)p->alloc(sizeof(float) * (size_t)ncols * p->nout);
  p->gy = (float*)p->alloc(sizeof(float) * (size_t)ncols * p->nout);
  p->g0 = (float*)p->alloc(sizeof(float) * (size_t)ncols * w);
  p->g1 = (float*)p->alloc(sizeof(float) * (size_t)ncols * w);
  p->bcap = ncols;
  if (p->tc) {  // tensor-core operands (zero padding) and the layers' tensor maps
    const int ldh = p->kp.size() > 1 ? p->kp[1] : p->kp[0];
    auto z = [&](size_t words) {
      uint32_t* b = (uint32_t*)p->alloc(sizeof(uint32_t) * words);
      GD_CUDA(cudaMemsetAsync(b, 0, sizeof(uint32_t) * words, p->stream));
      return b;
    };
    p->xh = z((size_t)ncols * p->kp[0]);
    p->xl = z((size_t)ncols * p->kp[0]);
    for (int i = 0; i < 2; ++i) {
      p->hh[i] = z((size_t)ncols * ldh);
      p->hl[i] = z((size_t)ncols * ldh);
    }
    GD_CUDA(cudaStreamSynchronize(p->stream));
    p->layers.assign(p->nlayer, TcMlpLayer{});
    for (int l = 0; l < p->nlayer; ++l) {
      TcMlpLayer& L = p->layers[l];
      L.M = ncols;
      L.N = p->fout[l];
      L.Np = p->npd[l];
      L.Kp = p->kp[l];
      L.bias = p->p32 + p->offb[l];
      L.gelu = l < p->nl;
      L.err = p->terr;
      const uint32_t* ah = l == 0 ? p->xh : p->hh[(l - 1) & 1];
      const uint32_t* al = l == 0 ? p->xl : p->hl[(l - 1) & 1];
      if (L.gelu) {
        L.oh = p->hh[l & 1];
        L.ol = p->hl[l & 1];
        L.ldo = ldh;
      }
      tc_mlp_maps(L, ah, al, p->wtc + p->tcoff[l]);
    }
  }
}

namespace {
void forward_simt(gd_mlp* p, const float* x, int n, float* y, cudaStream_t s);
// the tensor-core forward: weights refreshed from the BF16 copy, inputs
// split, one k_tc_mlp launch per layer
void forward_tc(gd_mlp* p, const float* x, int n, float* y, cudaStream_t s) {
  for (int l = 0; l < p->nlayer; ++l) {
    const long cnt = (long)p->npd[l] * p->kp[l];
    k_w_tc<<<std::min(ceil_div(cnt, 256), 1024), 256, 0, s>>>(p->w16 + p->offw[l], p->fout[l], p->fin[l], p->npd[l],
                                                              p->kp[l], p->wtc + p->tcoff[l]);
  }
  k_split_in<<<std::min(ceil_div((long)n * p->nin, 256), 8192), 256, 0, s>>>(x, n, p->nin, p->kp[0], p->xh, p->xl);
  count_launch(p->nlayer + 1);
  GD_LAUNCH_CHECK();
  for (int l = 0; l < p->nlayer; ++l) {
    TcMlpLayer L = p->layers[l];
    L.M = n;  // rows past n are neither needed nor stored
    if (!L.gelu) {
      L.y = y;
      L.ldy = p->nout;
    }
    tc_mlp_layer(L, s);
  }
}
}  // namespace

// Training buffers (tensor-core path): the split gradients, the transposed
// operands of the weight gradients and the slices' partial tiles for
// batches of up to ncols, and the training layers over them and over the
// activation buffers of mlp_reserve (rebuilt when those move).
void train_reserve(gd_mlp* p, int ncols) {
  if (!p->tcb || (ncols <= p->tcap && p->tbcap == p->bcap)) return;
  GD_CUDA(cudaStreamSynchronize(p->stream));
  auto z = [&](size_t words) {
    uint32_t* b = (uint32_t*)p->alloc(sizeof(uint32_t) * words);
    GD_CUDA(cudaMemsetAsync(b, 0, sizeof(uint32_t) * words, p->stream));
    return b;
  };
  const int L1 = p->nlayer - 1;
  const int ldd = (p->nh + 31) / 32 * 32;  // pitch of a hidden gradient's split (= kpt of a hidden layer)
  if (ncols > p->tcap) {
    const int cap = (ncols + 31) / 32 * 32;
    int mp = 0, np = 0;
    for (int l = 0; l < p->nlayer; ++l) {
      mp = std::max(mp, (p->fout[l] + 127) / 128 * 128);
      np = std::max(np, (p->fin[l] + 15) / 16 * 16);
    }
    int nsm = 0;
    GD_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, p->device));
    p->wsplit_max = std::max(1, 2 * nsm);
    p->gyh = z((size_t)cap * p->kpt[L1]);
    p->gyl = z((size_t)cap * p->kpt[L1]);
    for (int i = 0; i < 2; ++i) {
      p->dzh[i] = z((size_t)cap * ldd);
      p->dzl[i] = z((size_t)cap * ldd);
    }
    p->zth = z((size_t)mp * cap);
    p->ztl = z((size_t)mp * cap);
    p->ath = z((size_t)np * cap);
    p->atl = z((size_t)np * cap);
    p->wpart = (float*)p->alloc(sizeof(float) * (size_t)p->wsplit_max * mp * np);
    p->tcap = cap;
  }
  GD_CUDA(cudaStreamSynchronize(p->stream));
  const int ncb = p->bcap;
  p->tlayers = p->layers;
  for (int l = 0; l < p->nl; ++l) {
    TcMlpLayer& T = p->tlayers[l];
    T.mode = 2;
    T.z = p->zb + (size_t)l * ncb * p->nh;
    T.act = p->ab + (size_t)l * ncb * p->nh;
    T.ldz = p->nh;
  }
  p->tlayers[L1].y = p->yb;
  p->tlayers[L1].ldy = p->nout;
  // backward product of layer l: A = split dZ_l (the output gradient, or
  // what layer l + 1 wrote), writes dZ_{l-1} to g0 / g1 and its split
  p->blayers.assign(p->nlayer, TcMlpLayer{});
  for (int l = 1; l < p->nlayer; ++l) {
    TcMlpLayer& B = p->blayers[l];
    const int out = (L1 - l) & 1;
    B.M = p->tcap;  // the A operand's rows: the split gradients hold tcap
    B.N = p->fin[l];
    B.Np = p->npt[l];
    B.Kp = p->kpt[l];
    B.mode = 3;
    B.err = p->terr;
    B.zin = p->zb + (size_t)(l - 1) * ncb * p->nh;
    B.ldz = p->nh;
    B.y = out ? p->g1 : p->g0;
    B.ldy = p->fin[l];
    B.oh = p->dzh[out];
    B.ol = p->dzl[out];
    B.ldo = ldd;
    const uint32_t* ah = l == L1 ? p->gyh : p->dzh[out ^ 1];
    const uint32_t* al = l == L1 ? p->gyl : p->dzl[out ^ 1];
    tc_mlp_maps(B, ah, al, p->wtct + p->tctoff[l]);
  }
  // weight gradients: A = dZ_l transposed (fout rows), B = the layer's input transposed (fin rows)
  p->wgl.assign(p->nlayer, TcWgrad{});
  for (int l = 0; l < p->nlayer; ++l) {
    TcWgrad& W = p->wgl[l];
    W.Mp = (p->fout[l] + 127) / 128 * 128;
    W.Np = (p->fin[l] + 15) / 16 * 16;
    W.part = p->wpart;
    W.err = p->terr;
    tc_wgrad_maps(W, p->zth, p->ztl, p->ath, p->atl, p->tcap);
  }
  p->tbcap = p->bcap;
}

namespace {
// the tensor-core forward of a training step: the hidden layers also keep
// their pre-activations and activations (FP32) for the backward pass; the
// transposed weights of the backward products are refreshed with the others
void forward_tc_train(gd_mlp* p, const float* x, int n) {
  cudaStream_t s = p->stream;
  for (int l = 0; l < p->nlayer; ++l) {
    const long cnt = (long)p->npd[l] * p->kp[l];
    k_w_tc<<<std::min(ceil_div(cnt, 256), 1024), 256, 0, s>>>(p->w16 + p->offw[l], p->fout[l], p->fin[l], p->npd[l],
                                                              p->kp[l], p->wtc + p->tcoff[l]);
    if (l >= 1) {
      const long ct = (long)p->npt[l] * p->kpt[l];
      k_w_tc_t<<<std::min(ceil_div(ct, 256), 1024), 256, 0, s>>>(p->w16 + p->offw[l], p->fout[l], p->fin[l],
                                                                  p->npt[l], p->kpt[l], p->wtct + p->tctoff[l]);
    }
  }
  k_split_in<<<std::min(ceil_div((long)n * p->nin, 256), 8192), 256, 0, s>>>(x, n, p->nin, p->kp[0], p->xh, p->xl);
  count_launch(2 * p->nlayer);
  GD_LAUNCH_CHECK();
  for (int l = 0; l < p->nlayer; ++l) {
    TcMlpLayer L = p->tlayers[l];
    L.M = n;
    tc_mlp_layer(L, s);
  }
}
}  // namespace

// y [n][nout] = net(x [n][nin]) on stream s, on the tensor cores when the
// shape allows (every layer at most 256 wide).  No allocation when n <= bcap.
void mlp_forward_on(gd_mlp* p, const float* x, int n, float* y, cudaStream_t s) {
  if (n > p->bcap) throw std::invalid_argument("gd_mlp: batch above the reserved capacity");
  if (n <= 0) return;
  if (p->tc)
    forward_tc(p, x, n, y, s);
  else
    forward_simt(p, x, n, y, s);
}

namespace {
// the SIMT forward; the hidden pre-activations and activations stay in the
// net's buffers for a backward pass
void forward_simt(gd_mlp* p, const float* x, int n, float* y, cudaStream_t s) {
  const float* in = x;
  for (int l = 0; l < p->nlayer; ++l) {
    const int fi = p->fin[l], fo = p->fout[l];
    const __nv_bfloat16* W = p->w16 + p->offw[l];
    const float* b = p->p32 + p->offb[l];
    if (l < p->nl) {
      float* Z = p->zb + (size_t)l * p->bcap * p->nh;
      float* A = p->ab + (size_t)l * p->bcap * p->nh;
      gemm(n, fo, fi, in, (long)fi, 1L, W, 1L, (long)fi, EpiHidden{b, Z, A, fo}, s);
      in = A;
    } else {
      gemm(n, fo, fi, in, (long)fi, 1L, W, 1L, (long)fi, EpiLinear{b, y, fo}, s);
    }
  }
}
}  // namespace

// raises (and clears) a bounded wait's timeout in the tensor-core forward
void mlp_check(gd_mlp* p, cudaStream_t s) {
  if (!p->terr) return;
  int e = 0;
  GD_CUDA(cudaMemcpyAsync(&e, p->terr, sizeof(int), cudaMemcpyDeviceToHost, s));
  GD_CUDA(cudaStreamSynchronize(s));
  if (e) {
    GD_CUDA(cudaMemsetAsync(p->terr, 0, sizeof(int), s));
    GD_CUDA(cudaStreamSynchronize(s));
    throw CudaError("closure net: a tensor-core wait timed out (code " + std::to_string(e) + ")");
  }
}

int mlp_nin(const gd_mlp* p) { return p->nin; }
int mlp_nout(const gd_mlp* p) { return p->nout; }
int mlp_device(const gd_mlp* p) { return p->device; }
bool mlp_norm(const gd_mlp* p, const float** in_mu, const float** in_sd, const float** out_mu,
              const float** out_sd) {
  *in_mu = p->in_mu;
  *in_sd = p->in_sd;
  *out_mu = p->out_mu;
  *out_sd = p->out_sd;
  return p->has_norm;
}

namespace {
// loss and gradient of a batch into p->grad; the loss lands in p->lossd
void loss_grad(gd_mlp* p, const float* x, const float* t, int n) {
  cudaStream_t s = p->stream;
  if (p->tcb)
    forward_tc_train(p, x, n);
  else
    forward_simt(p, x, n, p->yb, s);
  const long cnt = (long)n * p->nout;
  const int nb = std::min(KPART, ceil_div(cnt, 256));
  k_mse<<<nb, 256, 0, s>>>(p->yb, t, cnt, p->gy, p->partial);
  k_mse_final<<<1, KPART, 0, s>>>(p->partial, nb, cnt, p->lossd);
  count_launch(2);
  GD_LAUNCH_CHECK();
  if (p->tcb) {  // the output gradient split, the A operand of the last layer's backward product
    k_split_in<<<std::min(ceil_div(cnt, 256), 8192), 256, 0, s>>>(p->gy, n, p->nout, p->kpt[p->nlayer - 1], p->gyh,
                                                                    p->gyl);
    count_launch();
    GD_LAUNCH_CHECK();
  }
  // backward: dZ of layer l in cur; dW_l = dZ^T A_{l-1}, db_l = colsum dZ,
  // dZ_{l-1} = (dZ W_l) * GELU'(Z_{l-1})
  const float* cur = p->gy;
  for (int l = p->nlayer - 1; l >= 0; --l) {
    const int fi = p->fin[l], fo = p->fout[l];
    const float* Ain = l == 0 ? x : p->ab + (size_t)(l - 1) * p->bcap * p->nh;
    if (p->tcb) {  // dW_l on the tensor cores: dZ and the input transposed and split, K = the batch in slices
      const int nbc = (n + 31) / 32 * 32, nk = nbc / 32;
      const TcWgrad& W = p->wgl[l];
      int ns = std::max(1, std::min(nk / 4, std::max(1, p->wsplit_max / (W.Mp / 128))));  // >= 4 chunks per slice
      const int cps = (nk + ns - 1) / ns;
      ns = (nk + cps - 1) / cps;  // every slice non-empty
      k_tsplit<<<dim3(nbc / 32, ceil_div(fo, 32)), dim3(32, 8), 0, s>>>(cur, n, fo, nbc, p->tcap, p->zth, p->ztl);
      k_tsplit<<<dim3(nbc / 32, ceil_div(fi, 32)), dim3(32, 8), 0, s>>>(Ain, n, fi, nbc, p->tcap, p->ath, p->atl);
      count_launch(2);
      GD_LAUNCH_CHECK();
      tc_wgrad(W, nk, cps, ns, s);
      k_wsum<<<std::min(ceil_div((long)fo * fi, 256), 1024), 256, 0, s>>>(p->wpart, ns, W.Mp, W.Np, fo, fi,
                                                                        p->grad + p->offw[l]);
      count_launch();
      GD_LAUNCH_CHECK();
    } else {
      gemm_splitk(fo, fi, n, cur, 1L, (long)fo, Ain, (long)fi, 1L, p->kpart, p->grad + p->offw[l], s);
    }
    k_colsum<<<ceil_div(fo, 32), dim3(32, 8), 0, s>>>(cur, n, fo, p->grad + p->offb[l]);
    count_launch();
    GD_LAUNCH_CHECK();
    if (l > 0 && p->tcb) {  // dZ_{l-1} on the tensor cores, stored and split for layer l - 1
      TcMlpLayer B = p->blayers[l];
      B.M = n;
      tc_mlp_layer(B, s);
      cur = B.y;
    } else if (l > 0) {
      float* nxt = (cur == p->g0) ? p->g1 : p->g0;
      const float* Zp = p->zb + (size_t)(l - 1) * p->bcap * p->nh;
      gemm(n, fi, fo, cur, (long)fo, 1L, p->w16 + p->offw[l], (long)fi, 1L, EpiGeluD{Zp, nxt, fi}, s);
      cur = nxt;
    }
  }
}
}  // namespace

}  // namespace gd

using namespace gd;

extern "C" {

int gd_mlp_init(int nin, int nhidden, int nlayers, int nout, unsigned long long seed, int device, gd_mlp** out) {
  if (!out) return GD_ERR_ARG;
  *out = nullptr;
  if (nin < 1 || nhidden < 1 || nlayers < 1 || nout < 1) {
    g_mlp_init_error = "gd_mlp_init: need nin, nhidden, nlayers, nout >= 1";
    return GD_ERR_ARG;
  }
  std::unique_ptr<gd_mlp> p(new gd_mlp());
  p->device = device;
  p->nin = nin;
  p->nh = nhidden;
  p->nl = nlayers;
  p->nout = nout;
  p->nlayer = nlayers + 1;
  long off = 0;
  for (int l = 0; l < p->nlayer; ++l) {
    const int fi = l == 0 ? nin : nhidden, fo = l == nlayers ? nout : nhidden;
    p->fin.push_back(fi);
    p->fout.push_back(fo);
    p->offw.push_back(off);
    off += (long)fi * fo;
    p->offb.push_back(off);
    off += fo;
  }
  p->np = off;
  // tensor-core inference when every layer is at most 256 wide
  p->tc = true;
  long toff = 0;
  for (int l = 0; l < p->nlayer; ++l) {
    p->kp.push_back((p->fin[l] + 31) / 32 * 32);
    p->npd.push_back((p->fout[l] + 15) / 16 * 16);
    if (p->npd[l] > 256) p->tc = false;
    p->tcoff.push_back(toff);
    toff += (long)p->npd[l] * p->kp[l];
  }
  // tensor-core training when the backward products dZ_l W_l fit as well
  // (every layer's input at most 256 wide); GD_MLP_TRAIN_TC=0 keeps it on
  // the SIMT kernels (a comparison knob)
  {
    const char* e = getenv("GD_MLP_TRAIN_TC");
    p->tcb = p->tc && !(e && e[0] == '0');
  }
  long ttoff = 0;
  for (int l = 0; l < p->nlayer; ++l) {
    p->kpt.push_back((p->fout[l] + 31) / 32 * 32);
    p->npt.push_back((p->fin[l] + 15) / 16 * 16);
    p->tctoff.push_back(ttoff);
    if (l >= 1) {
      if (p->npt[l] > 256) p->tcb = false;
      ttoff += (long)p->npt[l] * p->kpt[l];
    }
  }
  // He-normal hidden weights, the output layer scaled by 0.1 (the net starts
  // close to no correction), zero biases
  std::vector<float> h(off, 0.f);
  std::mt19937_64 rng(seed);
  std::normal_distribution<double> nd(0.0, 1.0);
  for (int l = 0; l < p->nlayer; ++l) {
    const double sd = std::sqrt(2.0 / p->fin[l]) * (l == nlayers ? 0.1 : 1.0);
    for (long i = 0; i < (long)p->fin[l] * p->fout[l]; ++i) h[p->offw[l] + i] = (float)(sd * nd(rng));
  }
  const int rc = mguard(p.get(), [&] {
    GD_CUDA(cudaStreamCreateWithFlags(&p->own, cudaStreamNonBlocking));
    p->stream = p->own;
    p->p32 = (float*)p->alloc(sizeof(float) * off);
    p->w16 = (__nv_bfloat16*)p->alloc(sizeof(__nv_bfloat16) * off);
    p->grad = (float*)p->alloc(sizeof(float) * off);
    p->am = (float*)p->alloc(sizeof(float) * off);
    p->av = (float*)p->alloc(sizeof(float) * off);
    p->partial = (float*)p->alloc(sizeof(float) * KPART);
    long wmax = 0;
    for (int l = 0; l < p->nlayer; ++l) wmax = std::max(wmax, (long)p->fin[l] * p->fout[l]);
    p->kpart = (float*)p->alloc(sizeof(float) * KSPLIT * wmax);
    p->lossd = (float*)p->alloc(sizeof(float));
    p->in_mu = (float*)p->alloc(sizeof(float) * nin);
    p->in_sd = (float*)p->alloc(sizeof(float) * nin);
    p->out_mu = (float*)p->alloc(sizeof(float) * nout);
    p->out_sd = (float*)p->alloc(sizeof(float) * nout);
    if (p->tcb) p->wtct = (float*)p->alloc(sizeof(float) * std::max(ttoff, 1L));
    if (p->tc) {
      p->wtc = (float*)p->alloc(sizeof(float) * toff);
      p->terr = (int*)p->alloc(sizeof(int));
      GD_CUDA(cudaMemset(p->terr, 0, sizeof(int)));
    }
    GD_CUDA(cudaMemcpy(p->p32, h.data(), sizeof(float) * off, cudaMemcpyHostToDevice));
    GD_CUDA(cudaMemset(p->am, 0, sizeof(float) * off));
    GD_CUDA(cudaMemset(p->av, 0, sizeof(float) * off));
    GD_CUDA(cudaMemset(p->grad, 0, sizeof(float) * off));
    to_bf16(p.get());
    GD_CUDA(cudaStreamSynchronize(p->stream));
  });
  if (rc != GD_OK) {
    g_mlp_init_error = p->err;
    return rc;
  }
  *out = p.release();
  return GD_OK;
}

int gd_mlp_destroy(gd_mlp* p) {
  if (!p) return GD_ERR_ARG;
  delete p;
  return GD_OK;
}

int gd_mlp_nparams(gd_mlp* p, long long* n) {
  if (!p || !n) return GD_ERR_ARG;
  *n = p->np;
  return GD_OK;
}

int gd_mlp_get_params(gd_mlp* p, float* params) {
  if (!params) return GD_ERR_ARG;
  return mguard(p, [&] {
    GD_CUDA(cudaStreamSynchronize(p->stream));
    GD_CUDA(cudaMemcpy(params, p->p32, sizeof(float) * p->np, cudaMemcpyDeviceToHost));
  });
}

int gd_mlp_set_params(gd_mlp* p, const float* params) {
  if (!params) return GD_ERR_ARG;
  return mguard(p, [&] {
    GD_CUDA(cudaStreamSynchronize(p->stream));
    GD_CUDA(cudaMemcpy(p->p32, params, sizeof(float) * p->np, cudaMemcpyHostToDevice));
    to_bf16(p);
    GD_CUDA(cudaStreamSynchronize(p->stream));
  });
}

int gd_mlp_set_norm(gd_mlp* p, const float* in_mu, const float* in_sd, const float* out_mu, const float* out_sd) {
  if (!in_mu || !in_sd || !out_mu || !out_sd) return GD_ERR_ARG;
  return mguard(p, [&] {
    for (int i = 0; i < p->nin; ++i)
      if (!(in_sd[i] > 0)) throw std::invalid_argument("gd_mlp_set_norm: input scales must be > 0");
    GD_CUDA(cudaStreamSynchronize(p->stream));
    GD_CUDA(cudaMemcpy(p->in_mu, in_mu, sizeof(float) * p->nin, cudaMemcpyHostToDevice));
    GD_CUDA(cudaMemcpy(p->in_sd, in_sd, sizeof(float) * p->nin, cudaMemcpyHostToDevice));
    GD_CUDA(cudaMemcpy(p->out_mu, out_mu, sizeof(float) * p->nout, cudaMemcpyHostToDevice));
    GD_CUDA(cudaMemcpy(p->out_sd, out_sd, sizeof(float) * p->nout, cudaMemcpyHostToDevice));
    p->has_norm = true;
  });
}

int gd_mlp_forward(gd_mlp* p, const float* x, int ncols, float* y) {
  if (!x || !y || ncols < 0) return GD_ERR_ARG;
  return mguard(p, [&] {
    if (ncols == 0) return;
    need_device(p, x, "x");
    need_device(p, y, "y");
    mlp_reserve(p, ncols);
    mlp_forward_on(p, x, ncols, y, p->stream);
    mlp_check(p, p->stream);
  });
}

int gd_mlp_loss_grad(gd_mlp* p, const float* x, const float* t, int ncols, float* loss, float* grad) {
  if (!x || !t || ncols < 1) return GD_ERR_ARG;
  return mguard(p, [&] {
    need_device(p, x, "x");
    need_device(p, t, "t");
    mlp_reserve(p, ncols);
    train_reserve(p, ncols);
    loss_grad(p, x, t, ncols);
    mlp_check(p, p->stream);
    if (loss) GD_CUDA(cudaMemcpy(loss, p->lossd, sizeof(float), cudaMemcpyDeviceToHost));
    if (grad) GD_CUDA(cudaMemcpy(grad, p->grad, sizeof(float) * p->np, cudaMemcpyDeviceToHost));
  });
}

int gd_mlp_train_step(gd_mlp* p, const float* x, const float* t, int ncols, float lr, float* loss) {
  if (!x || !t || ncols < 1 || !(lr > 0)) return GD_ERR_ARG;
  return mguard(p, [&] {
    need_device(p, x, "x");
    need_device(p, t, "t");
    mlp_reserve(p, ncols);
    train_reserve(p, ncols);
    loss_grad(p, x, t, ncols);
    ++p->adam_t;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)p->adam_t), c2 = 1.f - std::pow(b2, (float)p->adam_t);
    k_adam<<<std::min(ceil_div(p->np, 256), 4096), 256, 0, p->stream>>>(p->p32, p->grad, p->am, p->av, p->w16, p->np,
                                                                         lr, b1, b2, 1e-8f, c1, c2);
    count_launch();
    GD_LAUNCH_CHECK();
    if (loss) {
      GD_CUDA(cudaMemcpyAsync(loss, p->lossd, sizeof(float), cudaMemcpyDeviceToHost, p->stream));
      mlp_check(p, p->stream);  // synchronises; raises a tensor-core wait that gave up
    }
  });
}

int gd_mlp_set_stream(gd_mlp* p, void* stream) {
  return mguard(p, [&] {
    GD_CUDA(cudaStreamSynchronize(p->stream));
    p->stream = stream ? (cudaStream_t)stream : p->own;
  });
}

int gd_mlp_sync(gd_mlp* p) {
  return mguard(p, [&] {
    mlp_check(p, p->stream);
  });
}

const char* gd_mlp_last_error(gd_mlp* p) { return p ? p->err.c_str() : g_mlp_init_error.c_str(); }

}  // extern "C"

// ------------------------------------------------------ closure columns --
namespace gd {
namespace {
constexpr int CT = 32;  // grid columns per CTA of the transposes
}

// rows of gS (column index fastest) -> x [column][feature] through a shared
// tile: the reads and the writes both run along contiguous memory
template <typename R>
__global__ void k_closure_in(const R* __restrict__ gS, SynthRows s, int L, long ng, const float* __restrict__ mu,
                             const float* __restrict__ sd, float* __restrict__ x) {
  extern __shared__ float tile[];  // [nf][CT + 1]
  const int nf = 3 * L + 1;
  const long p0 = (long)blockIdx.x * CT;
  for (int e = threadIdx.x; e < nf * CT; e += blockDim.x) {
    const int f = e / CT, c = e % CT;
    const long p = p0 + c;
    float v = 0.f;
    if (p < ng) {
      if (f < L)
        v = (float)gS[(long)(s.u + f) * ng + p];
      else if (f < 2 * L)
        v = (float)gS[(long)(s.v + f - L) * ng + p];
      else if (f < 3 * L)
        v = (float)gS[(long)(s.tv + f - 2 * L) * ng + p];
      else
        v = (float)exp(gS[(long)s.lnps * ng + p]);
      if (mu) v = (v - mu[f]) / sd[f];
    }
    tile[f * (CT + 1) + c] = v;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nf * CT; e += blockDim.x) {
    const int c = e / nf, f = e % nf;
    const long p = p0 + c;
    if (p < ng) x[p * nf + f] = tile[f * (CT + 1) + c];
  }
}

template <typename R>
__global__ void k_closure_out(const float* __restrict__ y, int L, long ng, const float* __restrict__ mu,
                              const float* __restrict__ sd, R dt, R* __restrict__ gA) {
  extern __shared__ float tile[];  // [3L][CT + 1]
  const int no = 3 * L;
  const long p0 = (long)blockIdx.x * CT;
  for (int e = threadIdx.x; e < no * CT; e += blockDim.x) {
    const int c = e / no, f = e % no;
    const long p = p0 + c;
    tile[f * (CT + 1) + c] = p < ng ? y[p * no + f] * sd[f] + mu[f] : 0.f;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 4 * L * CT; e += blockDim.x) {
    const int r = e / CT, c = e % CT;
    const long p = p0 + c;
    if (p >= ng) continue;
    // grid row r: Tv [0,L) <- y[2L, 3L); q [L,2L) <- 0; u [2L,3L) <- y[0,L); v [3L,4L) <- y[L,2L)
    const int f = r < L ? 2 * L + r : r < 2 * L ? -1 : r - 2 * L;
    gA[(long)r * ng + p] = f < 0 ? R(0) : dt * (R)tile[f * (CT + 1) + c];
  }
}

template <typename R>
void launch_closure_in(const R* gS, const SynthRows& s, int L, long ng, const float* mu, const float* sd, float* x,
                       cudaStream_t st) {
  const size_t sm = sizeof(float) * (size_t)(3 * L + 1) * (CT + 1);
  if (sm > 48 * 1024) GD_CUDA(cudaFuncSetAttribute(k_closure_in<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  k_closure_in<R><<<ceil_div(ng, CT), 256, sm, st>>>(gS, s, L, ng, mu, sd, x);
  count_launch();
  GD_LAUNCH_CHECK();
}
template <typename R>
void launch_closure_out(const float* y, int L, long ng, const float* mu, const float* sd, R dt, R* gA,
                        cudaStream_t st) {
  const size_t sm = sizeof(float) * (size_t)(3 * L) * (CT + 1);
  if (sm > 48 * 1024)
    GD_CUDA(cudaFuncSetAttribute(k_closure_out<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  k_closure_out<R><<<ceil_div(ng, CT), 256, sm, st>>>(y, L, ng, mu, sd, dt, gA);
  count_launch();
  GD_LAUNCH_CHECK();
}
template void launch_closure_in<double>(const double*, const SynthRows&, int, long, const float*, const float*,
                                        float*, cudaStream_t);
template void launch_closure_in<float>(const float*, const SynthRows&, int, long, const float*, const float*, float*,
                                       cudaStream_t);
template void launch_closure_out<double>(const float*, int, long, const float*, const float*, double, double*,
                                         cudaStream_t);
template void launch_closure_out<float>(const float*, int, long, const float*, const float*, float, float*,
                                        cudaStream_t);

}  // namespace gd

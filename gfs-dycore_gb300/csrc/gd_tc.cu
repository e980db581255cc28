// gd_tc.cu -- split-precision Legendre GEMMs on the sm_103a tensor cores.
//
// The per-order Legendre contractions of the transforms (the work SHTns
// does inside shtns_sh_to_spat / shtns_spat_to_sh and the vector forms
// behind src/shtns.f90) as tcgen05 MMAs with FP32 accumulators in TMEM.
// Orders m >= 1 only: the tensor-core FP32 accumulation is not IEEE
// round-to-nearest, and fields with a large global mean (ln ps, T) carry
// it in order 0, so order 0 runs on the SIMT FMA path.
// Each FP32 operand x is carried as hi + lo, hi = round(x) and
// lo = round(x - hi) to TF32 (kind::tf32) or BF16 (kind::f16), and the
// product is hi*hi + hi*lo + lo*hi ("x3").  The Legendre tables are split
// from their FP64 values once at init; the data operands are split by
// transpose kernels on the way in.
//
// GEMM orientation (both directions): D[c][n] with M = 128 real batch
// columns c on the TMEM lanes (so every epilogue store of a warp is 128
// contiguous bytes), N = latitudes (synthesis) or degrees of one parity
// (analysis), K = degrees (synthesis) or latitudes (analysis).  Both
// operands are K-major, staged by TMA with 128-byte swizzle.  The even/odd
// hemispheric split is two TMEM accumulators over de-interleaved K ranges.
// One CTA per (order m, column tile, N tile); a 3-stage TMA -> MMA
// mbarrier ring; one elected thread issues TMA, one issues MMA; every wait
// is bounded and reports through a device error flag.
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <array>
#include <cstring>
#include <vector>

#include "gd_tc.cuh"

namespace gd {

constexpr int TC_NS = 3;          // pipeline stages
constexpr int TC_M = 128;         // MMA M (batch columns per CTA)
constexpr int TC_THREADS = 128;   // 4 warps
constexpr unsigned long long TC_WAIT_NS = 2000000000ull;  // bounded waits: 2 s

// ------------------------------------------------------------ PTX helpers --
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: false (and the error flag set) if the phase does not
// complete within TC_WAIT_NS
__device__ __noinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err, int code) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = globaltimer();
  for (;;) {
    for (int i = 0; i < 64; ++i)
      if (mbar_try(bar, parity)) return true;
    if (globaltimer() - t0 > TC_WAIT_NS) {
      atomicCAS(err, 0, code);
      return false;
    }
    __nanosleep(64);
  }
}
__device__ __forceinline__ void tma_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tma_3d(uint32_t dst, const CUtensorMap* map, int x, int y, int z, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(dst),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row
// groups 1024 bytes apart (SBO), descriptor version 1 (sm_100 family)
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;              // LBO (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;    // SBO
  d |= (uint64_t)1 << 46;              // version
  d |= (uint64_t)2 << 61;              // SWIZZLE_128B
  return d;
}
template <int KIND>
__device__ __forceinline__ void mma(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  if (KIND == TC_TF32)
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
  else
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ------------------------------------------------------------ splitting --
template <int KIND>
struct Elem;
template <>
struct Elem<TC_TF32> {
  typedef uint32_t T;  // tf32 bit pattern in a 32-bit word
  __device__ static void split(double x, T& hi, T& lo) {
    float f = (float)x;
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(f));
    float r = (float)(x - (double)__uint_as_float(h));
    uint32_t l;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(r));
    hi = h;
    lo = l;
  }
  // Round to nearest TF32, ties away from zero, on the bit pattern: adding
  // half a TF32 unit (bit 12) to the sign-magnitude encoding and clearing the
  // 13 low bits (the same result as cvt.rna.tf32.f32 for finite inputs, in two
  // full-rate integer operations).
  __device__ static uint32_t rna(float f) { return (__float_as_uint(f) + 0x1000u) & 0xFFFFE000u; }
  // lo = f - hi is exact in FP32 (at most 13 significant bits); the tensor
  // core reads its leading TF32 bits
  __device__ static void splitf(float f, T& hi, T& lo) {
    const uint32_t h = rna(f);
    hi = h;
    lo = __float_as_uint(f - __uint_as_float(h));
  }
};
template <>
struct Elem<TC_BF16> {
  typedef __nv_bfloat16 T;
  __device__ static void split(double x, T& hi, T& lo) {
    float f = (float)x;
    hi = __float2bfloat16_rn(f);
    lo = __float2bfloat16_rn((float)(x - (double)__bfloat162float(hi)));
  }
  __device__ static void splitf(float f, T& hi, T& lo) {
    hi = __float2bfloat16_rn(f);
    lo = __float2bfloat16_rn(f - __bfloat162float(hi));
  }
};

// synthesis tables: [m][j][par*kepad + i] = tab[m][j][2i+par]
template <int KIND>
__global__ void k_tc_tab_syn(int T, int nh, int kepad, const long* toff, const double* tab,
                             typename Elem<KIND>::T* hi, typename Elem<KIND>::T* lo) {
  const long tot = (long)(T + 1) * nh * 2 * kepad;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (long)gridDim.x * blockDim.x) {
    const int k = (int)(e % (2 * kepad));
    const long mj = e / (2 * kepad);
    const int j = (int)(mj % nh), m = (int)(mj / nh);
    const int par = k / kepad, i = k - par * kepad, q = 2 * i + par, K = T - m + 1;
    const double v = (q < K) ? tab[toff[m] + (long)j * K + q] : 0.0;
    Elem<KIND>::split(v, hi[e], lo[e]);
  }
}
// analysis tables: [m][par*kirows + i][j] = tab[m][j][2i+par]
template <int KIND>
__global__ void k_tc_tab_ana(int T, int nh, int kirows, int nhpad, const long* toff, const double* tab,
                             typename Elem<KIND>::T* hi, typename Elem<KIND>::T* lo) {
  const long tot = (long)(T + 1) * 2 * kirows * nhpad;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (long)gridDim.x * blockDim.x) {
    const int j = (int)(e % nhpad);
    const long mr = e / nhpad;
    const int r = (int)(mr % (2 * kirows)), m = (int)(mr / (2 * kirows));
    const int par = r / kirows, i = r - par * kirows, q = 2 * i + par, K = T - m + 1;
    const double v = (q < K && j < nh) ? tab[toff[m] + (long)j * K + q] : 0.0;
    Elem<KIND>::split(v, hi[e], lo[e]);
  }
}

// X[c][x] = B[xmap[x]][c] split, x in [0, xlen), c in [0, ncols)
template <int KIND>
__global__ void __launch_bounds__(256) k_tc_split_x(const float* __restrict__ B, long ldB, int ncols,
                                                    const int* __restrict__ xmap, long xlen,
                                                    typename Elem<KIND>::T* __restrict__ hi,
                                                    typename Elem<KIND>::T* __restrict__ lo) {
  __shared__ float t[32][33];
  const long x0 = (long)blockIdx.x * 32;
  const int c0 = blockIdx.y * 32;
  for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
    const long x = x0 + yy;
    const int c = c0 + threadIdx.x;
    float v = 0.f;
    if (x < xlen && c < ncols) {
      const int idx = xmap[x];
      if (idx >= 0) v = B[(long)idx * ldB + c];
    }
    t[yy][threadIdx.x] = v;
  }
  __syncthreads();
  for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
    const int c = c0 + yy;
    const long x = x0 + threadIdx.x;
    if (c < ncols && x < xlen) {
      typename Elem<KIND>::T h, l;
      Elem<KIND>::splitf(t[threadIdx.x][yy], h, l);
      hi[(long)c * xlen + x] = h;
      lo[(long)c * xlen + x] = l;
    }
  }
}

// G+-[m][c][j] = G[m][j][c] +- G[m][nlat-1-j][c] split, j < nhpad (0 >= nh)
template <int KIND>
__global__ void __launch_bounds__(256) k_tc_split_g(const float* __restrict__ G, long ldG, int ncols, int nh,
                                                    int nlat, int nhpad, int ncap, typename Elem<KIND>::T* __restrict__ ph,
                                                    typename Elem<KIND>::T* __restrict__ pl,
                                                    typename Elem<KIND>::T* __restrict__ mh,
                                                    typename Elem<KIND>::T* __restrict__ ml) {
  __shared__ float tp[32][33], tm[32][33];
  const int j0 = blockIdx.x * 32, c0 = blockIdx.y * 32, m = blockIdx.z;
  for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
    const int j = j0 + yy, c = c0 + threadIdx.x;
    float a = 0.f, b = 0.f;
    if (j < nh && c < ncols) {
      a = G[((long)m * nlat + j) * ldG + c];
      b = G[((long)m * nlat + (nlat - 1 - j)) * ldG + c];
    }
    tp[yy][threadIdx.x] = a + b;
    tm[yy][threadIdx.x] = a - b;
  }
  __syncthreads();
  for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
    const int c = c0 + yy, j = j0 + threadIdx.x;
    if (c < ncols && j < nhpad) {
      const long o = ((long)m * ncap + c) * nhpad + j;
      typename Elem<KIND>::T h, l;
      Elem<KIND>::splitf(tp[threadIdx.x][yy], h, l);
      ph[o] = h;
      pl[o] = l;
      Elem<KIND>::splitf(tm[threadIdx.x][yy], h, l);
      mh[o] = h;
      ml[o] = l;
    }
  }
}

// ------------------------------------------------------------- the GEMM --
struct TcArgs {
  const int4* items;
  int mode;  // 0 synthesis, 1 analysis
  int T, nh, nlat, N, kc, kepad, kirows;
  const long* xbase;
  const long* moff;
  int parityH;
  int ncols;  // real columns of this GEMM
  int coff;   // row offset of the first column in the synthesis staging
  float* out;
  long ldout;
  int* err;
  uint32_t idesc;
  uint32_t tmem_cols;
  // fused kernel only: accumulate the hi*lo and lo*hi products in their own
  // TMEM accumulator beside the main one, so the main accumulator takes a
  // third of the truncating FP32 accumulation steps
  int sepx;
  // fused kernel only: K segments of cps chunks per parity, each accumulated
  // afresh and folded by the epilogue into running FP32 sums in TMEM (round
  // to nearest); 0: one accumulation per parity
  int cps;
  // fused kernel only: A slots in tensor memory (the converters run up to na
  // chunks ahead of the MMAs)
  int na;
  // fused kernel only: accumulator buffers in tensor memory, 2 (an item's
  // epilogue overlaps the next item's MMAs) or 1 (wide N tiles)
  int nbuf;
  // analysis only: the latitude (K) range split into nseg segments, item.w
  // the segment; segment q writes its FP32 partial sums at out + q * seg_stride
  int nseg;
  long seg_stride;
};

template <int KIND>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap mA0h, const __grid_constant__ CUtensorMap mA0l,
              const __grid_constant__ CUtensorMap mA1h, const __grid_constant__ CUtensorMap mA1l,
              const __grid_constant__ CUtensorMap mBh, const __grid_constant__ CUtensorMap mBl, TcArgs a) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~(uintptr_t)1023);
  const int N = a.N;
  const uint32_t bytesA = TC_M * 128, bytesB = (uint32_t)N * 128;
  const uint32_t stage_bytes = 2 * bytesA + 2 * bytesB;
  unsigned char* bar_area = sm + TC_NS * stage_bytes;
  uint64_t* full = reinterpret_cast<uint64_t*>(bar_area);
  uint64_t* empty = full + TC_NS;
  uint64_t* done = empty + TC_NS;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  const int4 it = a.items[blockIdx.x];
  const int m = it.x, c0 = it.y * TC_M, n0 = it.z * N;
  const int K = a.T - m + 1;
  int nk0, nk1;
  long xb = 0;
  int kp = 0;
  if (a.mode == 0) {
    const int ke = (K + 1) / 2, ko = K / 2;
    kp = (ke + a.kc - 1) / a.kc * a.kc;
    nk0 = (ke + a.kc - 1) / a.kc;
    nk1 = (ko + a.kc - 1) / a.kc;
    xb = a.xbase[m];
  } else {
    nk0 = nk1 = (a.nh + a.kc - 1) / a.kc;
  }
  const int total = nk0 + nk1;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(a.tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < TC_NS; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&empty[s]), 1);
    }
    mbar_init(smem_u32(done), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;

  if (tid == 0) {  // ---- TMA producer
    int fills[TC_NS] = {0, 0, 0};
    for (int i = 0; i < total; ++i) {
      const int s = i % TC_NS, u = i / TC_NS;
      if (u >= 1 && !mbar_wait(smem_u32(&empty[s]), (u - 1) & 1, a.err, 1)) break;
      const int acc = (i < nk0) ? 0 : 1, kk = acc ? i - nk0 : i;
      unsigned char* st = sm + s * stage_bytes;
      const uint32_t fb = smem_u32(&full[s]);
      mbar_expect_tx(fb, stage_bytes);
      const CUtensorMap* ah = acc ? &mA1h : &mA0h;
      const CUtensorMap* al = acc ? &mA1l : &mA0l;
      if (a.mode == 0) {
        const int x = (int)(xb + (long)acc * kp + (long)kk * a.kc);
        tma_2d(smem_u32(st), ah, x, a.coff + c0, fb);
        tma_2d(smem_u32(st + bytesA), al, x, a.coff + c0, fb);
        const int xt = acc * a.kepad + kk * a.kc;
        tma_3d(smem_u32(st + 2 * bytesA), &mBh, xt, n0, m, fb);
        tma_3d(smem_u32(st + 2 * bytesA + bytesB), &mBl, xt, n0, m, fb);
      } else {
        const int x = kk * a.kc;
        tma_3d(smem_u32(st), ah, x, c0, m, fb);
        tma_3d(smem_u32(st + bytesA), al, x, c0, m, fb);
        const int yt = acc * a.kirows + n0;
        tma_3d(smem_u32(st + 2 * bytesA), &mBh, x, yt, m, fb);
        tma_3d(smem_u32(st + 2 * bytesA + bytesB), &mBl, x, yt, m, fb);
      }
      ++fills[s];
    }
    // never leave with copies in flight into this CTA's shared memory
    for (int s = 0; s < TC_NS; ++s)
      if (fills[s] > 0) mbar_wait(smem_u32(&full[s]), (fills[s] - 1) & 1, a.err, 2);
  } else if (tid == 32) {  // ---- MMA issuer
    for (int i = 0; i < total; ++i) {
      const int s = i % TC_NS, u = i / TC_NS;
      if (!mbar_wait(smem_u32(&full[s]), u & 1, a.err, 3)) break;
      tc_fence_after();
      const int acc = (i < nk0) ? 0 : 1, kk = acc ? i - nk0 : i;
      unsigned char* st = sm + s * stage_bytes;
      const uint64_t dah = smem_desc(smem_u32(st)), dal = smem_desc(smem_u32(st + bytesA));
      const uint64_t dbh = smem_desc(smem_u32(st + 2 * bytesA)), dbl = smem_desc(smem_u32(st + 2 * bytesA + bytesB));
      const uint32_t d = tbase + (uint32_t)(acc * N);
#pragma unroll
      for (int k4 = 0; k4 < 4; ++k4) {  // 4 MMAs of K = 32 bytes per 128-byte row
        const uint64_t o = (uint64_t)(2 * k4);
        mma<KIND>(d, dah + o, dbh + o, a.idesc, (kk > 0 || k4 > 0) ? 1u : 0u);
        mma<KIND>(d, dah + o, dbl + o, a.idesc, 1u);
        mma<KIND>(d, dal + o, dbh + o, a.idesc, 1u);
      }
      mma_commit(smem_u32(&empty[s]));
    }
    mma_commit(smem_u32(done));  // all issued MMAs complete -> done
  }
  __syncwarp();
  // ---- epilogue: warp w holds TMEM lanes 32w..32w+31 = columns c0+32w+lane
  const bool ok = mbar_wait(smem_u32(done), 0, a.err, 4);
  tc_fence_after();
  // warp-uniform decision: tcgen05.ld is a .sync.aligned warp instruction
  const bool go = __all_sync(0xffffffffu, ok && *(volatile int*)a.err == 0);
  if (go) {
    const int c = c0 + warp * 32 + lane;
    const uint32_t tw = tbase + ((uint32_t)(warp * 32) << 16);
    for (int g = 0; g < N; g += 16) {
      float e[16], o[16];
      tmem_ld16(tw + g, e);
      if (nk1 > 0)
        tmem_ld16(tw + N + g, o);
      else
#pragma unroll
        for (int q = 0; q < 16; ++q) o[q] = 0.f;
      if (c < a.ncols) {
        if (a.mode == 0) {
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const int j = n0 + g + q;
            if (j < a.nh) {
              a.out[((long)m * a.nlat + j) * a.ldout + c] = e[q] + o[q];
              a.out[((long)m * a.nlat + (a.nlat - 1 - j)) * a.ldout + c] = a.parityH ? o[q] - e[q] : e[q] - o[q];
            }
          }
        } else {
          const long base = a.moff[m];
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const int qe = 2 * (n0 + g + q), qo = qe + 1;
            if (qe < K) a.out[(base + qe) * a.ldout + c] = e[q];
            if (qo < K) a.out[(base + qo) * a.ldout + c] = o[q];
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(a.tmem_cols));
}

// ---------------------------------------------- persistent variant --
// One CTA per SM walks its items round-robin.  Warp 0: TMA producer;
// warp 1: TMEM owner and MMA issuer; warps 2-5: epilogue (warp w reads TMEM
// lane quadrant w % 4).  Two TMEM accumulator buffers (each E|O, 2N
// columns) let the epilogue of one item overlap the loads and MMAs of the
// next.  Every wait is bounded; on a timeout all roles fall through to the
// common exit, which waits for outstanding copies and MMAs and frees TMEM.
constexpr int TCP_THREADS = 192;

struct TcItem {
  int m, c0, n0, nk0, nk1, kp, K;
  long xb;
  int kb, seg;  // first K chunk of both parities, K segment (analysis with nseg > 1)
};
__device__ __forceinline__ TcItem tc_item(const TcArgs& a, int idx) {
  const int4 it = a.items[idx];
  TcItem t;
  t.m = it.x;
  t.c0 = it.y * TC_M;
  t.n0 = it.z * a.N;
  t.K = a.T - t.m + 1;
  if (a.mode == 0) {
    const int ke = (t.K + 1) / 2, ko = t.K / 2;
    t.kp = (ke + a.kc - 1) / a.kc * a.kc;
    t.nk0 = (ke + a.kc - 1) / a.kc;
    t.nk1 = (ko + a.kc - 1) / a.kc;
    t.xb = a.xbase[t.m];
  } else {
    t.kp = 0;
    t.nk0 = t.nk1 = (a.nh + a.kc - 1) / a.kc;
    t.xb = 0;
  }
  t.kb = 0;
  t.seg = 0;
  if (a.mode == 1 && a.nseg > 1) {  // segment it.w of the latitude chunks (nseg <= chunks)
    const int nk = t.nk0;
    t.seg = it.w;
    t.kb = t.seg * nk / a.nseg;
    t.nk0 = t.nk1 = (t.seg + 1) * nk / a.nseg - t.kb;
  }
  return t;
}

template <int KIND>
__global__ void __launch_bounds__(TCP_THREADS, 1)
    k_tc_gemm_p(const __grid_constant__ CUtensorMap mA0h, const __grid_constant__ CUtensorMap mA0l,
                const __grid_constant__ CUtensorMap mA1h, const __grid_constant__ CUtensorMap mA1l,
                const __grid_constant__ CUtensorMap mBh, const __grid_constant__ CUtensorMap mBl, TcArgs a,
                int nitems) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~(uintptr_t)1023);
  const int N = a.N;
  const uint32_t bytesA = TC_M * 128, bytesB = (uint32_t)N * 128;
  const uint32_t stage_bytes = 2 * bytesA + 2 * bytesB;
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + TC_NS * stage_bytes);
  uint64_t* empty = full + TC_NS;
  uint64_t* tfull = empty + TC_NS;  // [2] accumulator buffer ready
  uint64_t* tempty = tfull + 2;     // [2] accumulator buffer drained
  uint64_t* done = tempty + 2;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(a.tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < TC_NS; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&empty[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&tfull[b]), 1);
      mbar_init(smem_u32(&tempty[b]), 4);  // one arrive per epilogue warp
    }
    mbar_init(smem_u32(done), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;

  if (tid == 0) {  // ------------------------------------------- producer
    int fills[TC_NS] = {0, 0, 0};
    long g = 0;
    bool bad = false;
    for (int idx = blockIdx.x; idx < nitems && !bad; idx += gridDim.x) {
      const TcItem t = tc_item(a, idx);
      const int total = t.nk0 + t.nk1;
      for (int i = 0; i < total; ++i, ++g) {
        const int s = (int)(g % TC_NS);
        const long u = g / TC_NS;
        if (u >= 1 && !mbar_wait(smem_u32(&empty[s]), (uint32_t)((u - 1) & 1), a.err, 11)) {
          bad = true;
          break;
        }
        const int acc = (i < t.nk0) ? 0 : 1, kk = acc ? i - t.nk0 : i;
        unsigned char* st = sm + s * stage_bytes;
        const uint32_t fb = smem_u32(&full[s]);
        mbar_expect_tx(fb, stage_bytes);
        const CUtensorMap* ah = acc ? &mA1h : &mA0h;
        const CUtensorMap* al = acc ? &mA1l : &mA0l;
        if (a.mode == 0) {
          const int x = (int)(t.xb + (long)acc * t.kp + (long)kk * a.kc);
          tma_2d(smem_u32(st), ah, x, a.coff + t.c0, fb);
          tma_2d(smem_u32(st + bytesA), al, x, a.coff + t.c0, fb);
          const int xt = acc * a.kepad + kk * a.kc;
          tma_3d(smem_u32(st + 2 * bytesA), &mBh, xt, t.n0, t.m, fb);
          tma_3d(smem_u32(st + 2 * bytesA + bytesB), &mBl, xt, t.n0, t.m, fb);
        } else {
          const int x = kk * a.kc;
          tma_3d(smem_u32(st), ah, x, t.c0, t.m, fb);
          tma_3d(smem_u32(st + bytesA), al, x, t.c0, t.m, fb);
          const int yt = acc * a.kirows + t.n0;
          tma_3d(smem_u32(st + 2 * bytesA), &mBh, x, yt, t.m, fb);
          tma_3d(smem_u32(st + 2 * bytesA + bytesB), &mBl, x, yt, t.m, fb);
        }
        ++fills[s];
      }
    }
    for (int s = 0; s < TC_NS; ++s)  // no copies left in flight at exit
      if (fills[s] > 0) mbar_wait(smem_u32(&full[s]), (fills[s] - 1) & 1, a.err, 12);
  } else if (tid == 32) {  // ------------------------------------ MMA issuer
    long g = 0;
    int titem = 0;
    bool bad = false;
    for (int idx = blockIdx.x; idx < nitems && !bad; idx += gridDim.x, ++titem) {
      const TcItem t = tc_item(a, idx);
      const int b = titem & 1, u = titem >> 1;
      if (u >= 1 && !mbar_wait(smem_u32(&tempty[b]), (uint32_t)((u - 1) & 1), a.err, 13)) break;
      tc_fence_after();
      const int total = t.nk0 + t.nk1;
      for (int i = 0; i < total; ++i, ++g) {
        const int s = (int)(g % TC_NS);
        const long uu = g / TC_NS;
        if (!mbar_wait(smem_u32(&full[s]), (uint32_t)(uu & 1), a.err, 14)) {
          bad = true;
          break;
        }
        tc_fence_after();
        const int acc = (i < t.nk0) ? 0 : 1, kk = acc ? i - t.nk0 : i;
        unsigned char* st = sm + s * stage_bytes;
        const uint64_t dah = smem_desc(smem_u32(st)), dal = smem_desc(smem_u32(st + bytesA));
        const uint64_t dbh = smem_desc(smem_u32(st + 2 * bytesA)),
                       dbl = smem_desc(smem_u32(st + 2 * bytesA + bytesB));
        const uint32_t d = tbase + (uint32_t)(b * 2 * N + acc * N);
#pragma unroll
        for (int k4 = 0; k4 < 4; ++k4) {
          const uint64_t o = (uint64_t)(2 * k4);
          mma<KIND>(d, dah + o, dbh + o, a.idesc, (kk > 0 || k4 > 0) ? 1u : 0u);
          mma<KIND>(d, dah + o, dbl + o, a.idesc, 1u);
          mma<KIND>(d, dal + o, dbh + o, a.idesc, 1u);
        }
        mma_commit(smem_u32(&empty[s]));
      }
      if (!bad) mma_commit(smem_u32(&tfull[b]));
    }
    mma_commit(smem_u32(done));  // every issued MMA has completed at `done`
  } else if (warp >= 2) {  // ------------------------------------- epilogue
    const int q4 = warp & 3;  // TMEM lane quadrant of this warp
    int titem = 0;
    for (int idx = blockIdx.x; idx < nitems; idx += gridDim.x, ++titem) {
      const TcItem t = tc_item(a, idx);
      const int b = titem & 1, u = titem >> 1;
      const bool ok = mbar_wait(smem_u32(&tfull[b]), (uint32_t)(u & 1), a.err, 15);
      if (!__all_sync(0xffffffffu, ok)) break;
      tc_fence_after();
      const int c = t.c0 + q4 * 32 + lane;
      const uint32_t tw = tbase + ((uint32_t)(q4 * 32) << 16) + (uint32_t)(b * 2 * N);
      for (int g = 0; g < N; g += 16) {
        float e[16], o[16];
        tmem_ld16(tw + g, e);
        if (t.nk1 > 0)
          tmem_ld16(tw + N + g, o);
        else
#pragma unroll
          for (int q = 0; q < 16; ++q) o[q] = 0.f;
        if (c < a.ncols) {
          if (a.mode == 0) {
#pragma unroll
            for (int q = 0; q < 16; ++q) {
              const int j = t.n0 + g + q;
              if (j < a.nh) {
                a.out[((long)t.m * a.nlat + j) * a.ldout + c] = e[q] + o[q];
                a.out[((long)t.m * a.nlat + (a.nlat - 1 - j)) * a.ldout + c] = a.parityH ? o[q] - e[q] : e[q] - o[q];
              }
            }
          } else {
            const long base = a.moff[t.m];
#pragma unroll
            for (int q = 0; q < 16; ++q) {
              const int qe = 2 * (t.n0 + g + q), qo = qe + 1;
              if (qe < t.K) a.out[(base + qe) * a.ldout + c] = e[q];
              if (qo < t.K) a.out[(base + qo) * a.ldout + c] = o[q];
            }
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[b])) : "memory");
    }
  }
  __syncwarp();
  mbar_wait(smem_u32(done), 0, a.err, 16);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(a.tmem_cols));
}

// ------------------------------------------- fused-split variant (TF32) --
// The persistent kernel above reads operands that split kernels have
// already transposed into K-major hi/lo arrays.  This variant reads the raw
// FP32 data instead.  Warp 0 loads, per K chunk, the raw tile in its natural
// column-contiguous layout (synthesis: 32 degrees of one parity of the
// spectral array; analysis: 32 northern latitude rows of the Fourier array
// and their 32 mirrored southern rows) together with the table tiles.  Eight
// converter warps (6-13) turn the raw tile into the A operand directly in
// tensor memory: two threads on TMEM lane c (one per half of the chunk's 32
// K entries, in warps w and w + 4) own batch column c, mask
// degrees beyond the truncation and latitudes beyond the equator, forms
// G_N +- G_S for the analysis, split to hi + lo and write their 16 columns of
// each with one tcgen05.st.  The MMAs read A from TMEM (a ring of 2-4 slots
// beside one or two accumulator buffers, and in the FP64-state modes the
// cross products' accumulators and the running sums of folded K segments),
// so shared memory holds only the TMA ring, 2-6 stages deep.  The split is
// the same as in k_tc_split_x/g, so results match the unfused path bit for
// bit.
constexpr int TCF_THREADS = 448;  // producer, MMA, 4 epilogue, 8 converter warps
constexpr int TCF_MAXNS = 6;
constexpr int TCF_MAXA = 4;  // A slots in tensor memory at most (64 columns each)
constexpr int TCF_MAXN = 192;  // widest N tile (single-buffered E|O, 2N + 128 TMEM columns)

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t* v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16};" ::"r"(taddr), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15]) : "memory");
}
__device__ __forceinline__ void mma_tf32_ta(uint32_t dtmem, uint32_t atmem, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(dtmem),
      "r"(atmem), "l"(b), "r"(idesc), "r"(acc));
}

// Position of K chunk g in a ring of n slots, advanced once per chunk: the
// slot g mod n and the parity (g / n) & 1 of its use count, without the
// 64-bit division per chunk on the single-thread issue paths.
struct TcRing {
  int slot = 0;
  uint32_t ph = 0;
  __device__ __forceinline__ void next(int n) {
    if (++slot == n) {
      slot = 0;
      ph ^= 1u;
    }
  }
};

__global__ void __launch_bounds__(TCF_THREADS, 1)
    k_tc_gemm_f(const __grid_constant__ CUtensorMap mRaw, const __grid_constant__ CUtensorMap mBh,
                const __grid_constant__ CUtensorMap mBl, TcArgs a, int nitems, int ns, uint32_t raw_bytes) {
  const int na = a.na;  // A slots (2 <= na <= min(ns, TCF_MAXA))
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~(uintptr_t)1023);
  const int N = a.N, kc = a.kc;
  const uint32_t tab_bytes = (uint32_t)N * 128;
  const uint32_t raw_off = 2 * tab_bytes;
  const uint32_t stage_bytes = (raw_off + raw_bytes + 1023) & ~1023u;
  // full[s]: the TMA copies of a chunk landed; used[s]: the MMAs of the chunk
  // in stage s completed (frees the stage for the producer and, two chunks
  // na chunks later, the A slot for the converters); afull[na]: an A slot is
  // written
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + (size_t)ns * stage_bytes);
  uint64_t* used = full + ns;
  uint64_t* afull = used + ns;
  uint64_t* tfull = afull + TCF_MAXA;  // [2] accumulator buffer ready
  uint64_t* tempty = tfull + 2;  // [2] accumulator buffer drained
  uint64_t* done = tempty + 2;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // TMEM: nbuf accumulator buffers of bw columns, the running sums' E|O when
  // K segments are folded, then the na A slots (hi 32, lo 32 columns each).
  // A buffer holds E|O of an item, or one parity's K segment when folding,
  // and with sepx the cross products' accumulator beside each
  const bool fold = a.cps > 0;
  const bool dbuf = a.nbuf == 2;
  const uint32_t bw = (fold ? 1u : 2u) * (a.sepx ? 2u : 1u) * (uint32_t)N;
  const uint32_t rcol = (dbuf ? 2u : 1u) * bw;
  const uint32_t acol = rcol + (fold ? 2u * (uint32_t)N : 0u);

  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(a.tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < ns; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&used[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&tfull[b]), 1);
      mbar_init(smem_u32(&tempty[b]), 4);
    }
    for (int q = 0; q < na; ++q) mbar_init(smem_u32(&afull[q]), 8);  // one arrive per converter warp
    mbar_init(smem_u32(done), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;

  if (tid == 0) {  // ------------------------------------------- producer
    int fills[TCF_MAXNS] = {0, 0, 0, 0, 0, 0};
    long g = 0;
    TcRing rs;  // chunk g's stage
    bool bad = false;
    for (int idx = blockIdx.x; idx < nitems && !bad; idx += gridDim.x) {
      const TcItem t = tc_item(a, idx);
      const int total = t.nk0 + t.nk1;
      for (int i = 0; i < total; ++i, ++g) {
        const int s = rs.slot;
        // the stage's previous chunk, g - ns, must have been consumed
        if (g >= ns && !mbar_wait(smem_u32(&used[s]), rs.ph ^ 1u, a.err, 21)) {
          bad = true;
          break;
        }
        const int acc = (i < t.nk0) ? 0 : 1, kk = t.kb + (acc ? i - t.nk0 : i);
        unsigned char* st = sm + (size_t)s * stage_bytes;
        const uint32_t fb = smem_u32(&full[s]);
        mbar_expect_tx(fb, 2 * tab_bytes + raw_bytes);
        if (a.mode == 0) {
          const int xt = acc * a.kepad + kk * kc;
          tma_3d(smem_u32(st), &mBh, xt, t.n0, t.m, fb);
          tma_3d(smem_u32(st + tab_bytes), &mBl, xt, t.n0, t.m, fb);
          // degrees q = acc + 2 (kk kc + i) of order m: spectral rows moff[m] + q,
          // addressed as (row pair, parity slot)
          const long r0 = a.moff[t.m] + acc + 2L * kk * kc;
          tma_3d(smem_u32(st + raw_off), &mRaw, t.c0, (int)(r0 & 1), (int)(r0 >> 1), fb);
        } else {
          const int x = kk * kc;
          const int yt = acc * a.kirows + t.n0;
          tma_3d(smem_u32(st), &mBh, x, yt, t.m, fb);
          tma_3d(smem_u32(st + tab_bytes), &mBl, x, yt, t.m, fb);
          tma_3d(smem_u32(st + raw_off), &mRaw, t.c0, x, t.m, fb);
          tma_3d(smem_u32(st + raw_off + raw_bytes / 2), &mRaw, t.c0, a.nlat - x - kc, t.m, fb);
        }
        ++fills[s];
        rs.next(ns);
      }
    }
    for (int s = 0; s < ns; ++s)  // no copies left in flight at exit
      if (fills[s] > 0) mbar_wait(smem_u32(&full[s]), (fills[s] - 1) & 1, a.err, 22);
  } else if (tid == 32) {  // ------------------------------------ MMA issuer
    long g = 0;
    int titem = 0;  // accumulator hand-offs so far: items, or K segments when folding
    bool bad = false;
    const int cps = fold ? a.cps : (1 << 30);
    TcRing rs, ra;  // chunk g's stage and A slot
    for (int idx = blockIdx.x; idx < nitems && !bad; idx += gridDim.x) {
      const TcItem t = tc_item(a, idx);
      const int total = t.nk0 + t.nk1;
      int b = 0;   // accumulator buffer of the current hand-off
      int sc = 0;  // chunk of the current K segment (segments restart with each parity)
      for (int i = 0; i < total; ++i, ++g) {
        const int acc = (i < t.nk0) ? 0 : 1, ip = acc ? i - t.nk0 : i;  // chunk ip of parity acc
        const bool sfirst = sc == 0;  // a K segment starts: its accumulators start afresh
        const bool slast = sc == cps - 1 || ip == (acc ? t.nk1 : t.nk0) - 1;
        sc = slast ? 0 : sc + 1;
        if (fold ? sfirst : i == 0) {  // wait until the epilogue drained the buffer
          b = dbuf ? (titem & 1) : 0;
          const int u = dbuf ? (titem >> 1) : titem;
          if (u >= 1 && !mbar_wait(smem_u32(&tempty[b]), (uint32_t)((u - 1) & 1), a.err, 23)) {
            bad = true;
            break;
          }
          tc_fence_after();
        }
        const int s = rs.slot, cs = ra.slot;
        if (!mbar_wait(smem_u32(&full[s]), rs.ph, a.err, 24) || !mbar_wait(smem_u32(&afull[cs]), ra.ph, a.err, 25)) {
          bad = true;
          break;
        }
        tc_fence_after();
        unsigned char* st = sm + (size_t)s * stage_bytes;
        const uint32_t ah = tbase + acol + 64u * (uint32_t)cs, al = ah + 32u;
        const uint64_t dbh = smem_desc(smem_u32(st)), dbl = smem_desc(smem_u32(st + tab_bytes));
        const uint32_t d = tbase + (uint32_t)b * bw + (fold ? 0u : (uint32_t)(acc * N));
        if (a.sepx) {  // the cross products into their own accumulator, beside the E|O (or segment) one
          const uint32_t dx = d + (fold ? 1u : 2u) * (uint32_t)N;
#pragma unroll
          for (int k4 = 0; k4 < 4; ++k4) {
            const uint64_t o = (uint64_t)(2 * k4);
            const uint32_t ka = 8u * (uint32_t)k4;
            const uint32_t first = (!sfirst || k4 > 0) ? 1u : 0u;
            mma_tf32_ta(d, ah + ka, dbh + o, a.idesc, first);
            mma_tf32_ta(dx, ah + ka, dbl + o, a.idesc, first);
            mma_tf32_ta(dx, al + ka, dbh + o, a.idesc, 1u);
          }
        } else {
#pragma unroll
          for (int k4 = 0; k4 < 4; ++k4) {  // K = 8 TF32 per MMA: 8 TMEM columns of A, 32 bytes of B
            const uint64_t o = (uint64_t)(2 * k4);
            const uint32_t ka = 8u * (uint32_t)k4;
            mma_tf32_ta(d, ah + ka, dbh + o, a.idesc, (!sfirst || k4 > 0) ? 1u : 0u);
            mma_tf32_ta(d, ah + ka, dbl + o, a.idesc, 1u);
            mma_tf32_ta(d, al + ka, dbh + o, a.idesc, 1u);
          }
        }
        mma_commit(smem_u32(&used[s]));
        rs.next(ns);
        ra.next(na);
        if (fold ? slast : i == total - 1) {  // hand the buffer to the epilogue
          mma_commit(smem_u32(&tfull[b]));
          ++titem;
        }
      }
    }
    mma_commit(smem_u32(done));
  } else if (warp >= 6) {  // ----------------------------------- converters
    const int q4 = warp & 3;                // TMEM lane quadrant of this warp
    const int c = q4 * 32 + lane;           // batch column = row of A = TMEM lane
    const int k0 = ((warp - 6) >> 2) * 16;  // this thread's half of the chunk's K entries
    const uint32_t arow = tbase + ((uint32_t)(q4 * 32) << 16) + acol + (uint32_t)k0;
    long g = 0;
    TcRing rs, ra, rp;  // chunk g's stage and A slot; chunk g - na's stage
    bool bad = false;
    for (int idx = blockIdx.x; idx < nitems && !bad; idx += gridDim.x) {
      const TcItem t = tc_item(a, idx);
      const int total = t.nk0 + t.nk1;
      for (int i = 0; i < total; ++i, ++g) {
        const int s = rs.slot, cs = ra.slot;
        const bool okf = mbar_wait(smem_u32(&full[s]), rs.ph, a.err, 26);
        if (!__all_sync(0xffffffffu, okf)) {
          bad = true;
          break;
        }
        const int acc = (i < t.nk0) ? 0 : 1, kk = t.kb + (acc ? i - t.nk0 : i);
        const float* raw = reinterpret_cast<const float*>(sm + (size_t)s * stage_bytes + raw_off);
        int nv;  // valid K entries of this chunk: ii < nv
        bool plus = true;
        if (a.mode == 0) {
          const int q0 = acc + 2 * kk * kc;  // degree offset of entry 0
          nv = q0 < t.K ? (t.K - q0 + 1) / 2 : 0;
        } else {
          nv = a.nh - kk * kc;
          plus = (acc == 0) != (a.parityH != 0);
        }
        // convert before waiting for the A slot: the loads and the split
        // overlap the MMAs still reading it
        uint32_t h[16], l[16];
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          const int ii = k0 + e;
          float v = raw[ii * TC_M + c];
          if (a.mode == 1) {
            const float w = raw[(2 * kc - 1 - ii) * TC_M + c];  // mirrored row nlat-1-j
            v = plus ? v + w : v - w;
          }
          if (ii >= nv) v = 0.f;
          Elem<TC_TF32>::splitf(v, h[e], l[e]);
        }
        // the slot's previous contents fed chunk g - na
        if (g >= na) {
          const bool oku = mbar_wait(smem_u32(&used[rp.slot]), rp.ph, a.err, 27);
          if (!__all_sync(0xffffffffu, oku)) {
            bad = true;
            break;
          }
          rp.next(ns);
        }
        tc_fence_after();
        tmem_st16(arow + 64u * (uint32_t)cs, h);
        tmem_st16(arow + 64u * (uint32_t)cs + 32u, l);
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        tc_fence_before();
        __syncwarp();
        if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&afull[cs])) : "memory");
        rs.next(ns);
        ra.next(na);
      }
    }
  } else if (warp >= 2) {  // ------------------------------------- epilogue
    const int q4 = warp & 3;
    const uint32_t lw = tbase + ((uint32_t)(q4 * 32) << 16);  // this warp's TMEM lane quadrant
    int titem = 0;
    bool bad = false;
    for (int idx = blockIdx.x; idx < nitems && !bad; idx += gridDim.x) {
      const TcItem t = tc_item(a, idx);
      int bt = -1;       // the buffer holding the item's sums (without folding)
      uint32_t tw = lw;  // TMEM columns of the item's E|O sums
      if (fold) {
        // each K segment, main + cross products, folded into the running sums
        // of its parity (FP32, round to nearest)
        const int nsE = (t.nk0 + a.cps - 1) / a.cps, nsub = nsE + (t.nk1 + a.cps - 1) / a.cps;
        for (int j = 0; j < nsub; ++j, ++titem) {
          const int b = dbuf ? (titem & 1) : 0, u = dbuf ? (titem >> 1) : titem;
          const bool ok = mbar_wait(smem_u32(&tfull[b]), (uint32_t)(u & 1), a.err, 28);
          if (!__all_sync(0xffffffffu, ok)) {
            bad = true;
            break;
          }
          tc_fence_after();
          const uint32_t ts = lw + (uint32_t)b * bw, tr = lw + rcol + (j < nsE ? 0u : (uint32_t)N);
          const bool first = j == 0 || j == nsE;
          for (int g = 0; g < N; g += 16) {
            float v[16];
            uint32_t w[16];
            tmem_ld16(ts + g, v);
            if (a.sepx) {
              float x[16];
              tmem_ld16(ts + N + g, x);
#pragma unroll
              for (int q = 0; q < 16; ++q) v[q] += x[q];
            }
            if (!first) {
              float r[16];
              tmem_ld16(tr + g, r);
#pragma unroll
              for (int q = 0; q < 16; ++q) v[q] = r[q] + v[q];
            }
#pragma unroll
            for (int q = 0; q < 16; ++q) w[q] = __float_as_uint(v[q]);
            tmem_st16(tr + g, w);
          }
          asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
          tc_fence_before();
          __syncwarp();
          if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[b])) : "memory");
        }
        if (bad) break;
        tw = lw + rcol;
      } else {
        bt = dbuf ? (titem & 1) : 0;
        const bool ok = mbar_wait(smem_u32(&tfull[bt]), (uint32_t)((dbuf ? (titem >> 1) : titem) & 1), a.err, 28);
        if (!__all_sync(0xffffffffu, ok)) break;
        tc_fence_after();
        tw = lw + (uint32_t)bt * bw;
        ++titem;
      }
      const int c = t.c0 + q4 * 32 + lane;
      for (int g = 0; g < N; g += 16) {
        float e[16], o[16];
        tmem_ld16(tw + g, e);
        if (t.nk1 > 0)
          tmem_ld16(tw + N + g, o);
        else
#pragma unroll
          for (int q = 0; q < 16; ++q) o[q] = 0.f;
        if (a.sepx && !fold) {  // add the cross products' accumulator (round to nearest)
          float xe[16], xo[16];
          tmem_ld16(tw + 2 * N + g, xe);
          if (t.nk1 > 0)
            tmem_ld16(tw + 3 * N + g, xo);
          else
#pragma unroll
            for (int q = 0; q < 16; ++q) xo[q] = 0.f;
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            e[q] += xe[q];
            o[q] += xo[q];
          }
        }
        if (c < a.ncols) {
          if (a.mode == 0) {
#pragma unroll
            for (int q = 0; q < 16; ++q) {
              const int j = t.n0 + g + q;
              if (j < a.nh) {
                a.out[((long)t.m * a.nlat + j) * a.ldout + c] = e[q] + o[q];
                a.out[((long)t.m * a.nlat + (a.nlat - 1 - j)) * a.ldout + c] = a.parityH ? o[q] - e[q] : e[q] - o[q];
              }
            }
          } else {
            const long base = a.moff[t.m];
            float* const out = a.out + (long)t.seg * a.seg_stride;
#pragma unroll
            for (int q = 0; q < 16; ++q) {
              const int qe = 2 * (t.n0 + g + q), qo = qe + 1;
              if (qe < t.K) out[(base + qe) * a.ldout + c] = e[q];
              if (qo < t.K) out[(base + qo) * a.ldout + c] = o[q];
            }
          }
        }
      }
      if (bt >= 0) {
        tc_fence_before();
        __syncwarp();
        if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[bt])) : "memory");
      }
    }
  }
  __syncwarp();
  mbar_wait(smem_u32(done), 0, a.err, 29);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(a.tmem_cols));
}

// ------------------------------------------------------------ host side --
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    GD_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p) throw CudaError("cuTensorMapEncodeTiled unavailable");
    fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

static void make_map(CUtensorMap* m, void* base, int kind, int rank, const uint64_t* dims, int box_inner,
                     int box_rows) {
  const size_t es = kind == TC_TF32 ? 4 : 2;
  cuuint64_t gd[3], gs[2];
  cuuint32_t bx[3], estr[3] = {1, 1, 1};
  for (int i = 0; i < rank; ++i) gd[i] = dims[i];
  gs[0] = dims[0] * es;
  if (rank == 3) gs[1] = dims[0] * dims[1] * es;
  bx[0] = box_inner;
  bx[1] = box_rows;
  bx[2] = 1;
  CUresult r = encode_fn()(m, kind == TC_TF32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
                           rank, base, gd, gs, bx, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw CudaError("cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
}

// untiled-swizzle FP32 map over raw data (the fused path's loads)
static void make_raw_map(CUtensorMap* m, const void* base, const uint64_t* dims, const uint64_t* strides,
                         const uint32_t* box) {
  cuuint64_t gd[3] = {dims[0], dims[1], dims[2]}, gs[2] = {strides[0], strides[1]};
  cuuint32_t bx[3] = {box[0], box[1], box[2]}, estr[3] = {1, 1, 1};
  CUresult r = encode_fn()(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(base), gd, gs, bx, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw CudaError("cuTensorMapEncodeTiled (raw) failed: " + std::to_string((int)r));
}
static const CUtensorMap& cached_raw_map(TcPlan& p, const void* base, const uint64_t* dims, const uint64_t* strides,
                                         const uint32_t* box) {
  const std::array<uint64_t, 9> key = {(uint64_t)(uintptr_t)base, dims[0], dims[1], dims[2], strides[0],
                                       strides[1], box[0], box[1], box[2]};
  for (auto& kv : p.raw_maps)
    if (kv.first == key) return kv.second;
  p.raw_maps.emplace_back(key, CUtensorMap{});
  make_raw_map(&p.raw_maps.back().second, base, dims, strides, box);
  return p.raw_maps.back().second;
}

static int round_up(int x, int a) { return (x + a - 1) / a * a; }
// N tile: multiple of 16, at most 160 so that three stages of
// (2 x 128 + 2 x N) rows of 128 bytes fit in 227 KB of shared memory
static int tile_n(int n, int cap) {
  int nt = (n + cap - 1) / cap;
  return round_up((n + nt - 1) / nt, 16);
}

static void* tc_alloc(TcPlan& p, size_t bytes) {
  void* d = nullptr;
  cudaError_t e = cudaMalloc(&d, std::max<size_t>(bytes, 16));
  if (e != cudaSuccess) throw CudaError(std::string("cudaMalloc: ") + cudaGetErrorString(e));
  p.allocs.push_back(d);
  return d;
}

// TMEM columns of the fused kernel at N tile n: nbuf accumulator buffers
// (E|O of an item, or one parity's K segment when folding; doubled by the
// cross products' accumulator), the running E|O sums when folding, na A slots
static int tcf_tmem_cols(int n, bool sepx, bool fold, int na, int nbuf) {
  const int bw = (fold ? 1 : 2) * (sepx ? 2 : 1) * n;
  return nbuf * bw + (fold ? 2 * n : 0) + 64 * na;
}
// accumulator buffers of the fused kernel at N tile n: two where they fit
// beside two A slots, else one (wide tiles: the epilogue no longer overlaps
// the next item's MMAs, each chunk's MMAs cover more latitudes or degrees)
static int tcf_nbuf(const TcPlan& p, int n) { return tcf_tmem_cols(n, p.sepx, p.cps > 0, 2, 2) <= 512 ? 2 : 1; }
// A slots the fused kernel gets at N tile n: the plan's request, as far as
// tensor memory holds them (at least two)
static int tcf_slots(const TcPlan& p, int n) {
  const int nb = tcf_nbuf(p, n);
  int na = std::max(2, std::min(p.aslots, TCF_MAXA));
  while (na > 2 && tcf_tmem_cols(n, p.sepx, p.cps > 0, na, nb) > 512) --na;
  return na;
}

int tc_slots(const TcPlan& p, int n) { return tcf_slots(p, n); }

int tc_max_n(const TcPlan& p) {
  if (!p.persistent) return 160;
  if (p.kind != TC_TF32) return 128;
  int n = TCF_MAXN;
  while (n > 16 && tcf_tmem_cols(n, p.sepx, p.cps > 0, 2, 1) > 512) n -= 16;
  return n;
}

void tc_init(TcPlan& p, int kind, int T, int nh, int nlat, int ncap, const long* d_toff, const double* P64,
             const double* H64, cudaStream_t s) {
  p.kind = kind;
  p.T = T;
  p.nh = nh;
  p.nlat = nlat;
  p.esize = kind == TC_TF32 ? 4 : 2;
  p.kc = 128 / p.esize;
  const int kemax = (T + 2) / 2;  // even-degree count of m = 0
  p.kepad = round_up(kemax, p.kc);
  p.nhpad = round_up(nh, p.kc);
  {
    const char* env = getenv("GD_TC_PERSISTENT");
    p.persistent = !(env && env[0] == '0');
    int dev = 0;
    GD_CUDA(cudaGetDevice(&dev));
    GD_CUDA(cudaDeviceGetAttribute(&p.nsm, cudaDevAttrMultiProcessorCount, dev));
  }
  // persistent: two E|O accumulator buffers (4N TMEM columns) -> N <= 128;
  // the fused TF32 path also keeps two A slots in TMEM and, as configured,
  // cross-product accumulators and running sums (wider tiles, single-
  // buffered, by the plan's tile cap or the autotuner)
  const int ncap_n = !p.persistent ? 160 : kind == TC_TF32 ? std::min(tc_max_n(p), p.tile_cap) : 128;
  p.nsyn = tile_n(nh, ncap_n);
  p.nana = tile_n(kemax, ncap_n);
  p.kirows = round_up(kemax, p.nana);
  p.ncap = round_up(ncap, 32);
  p.xbase.assign(T + 1, 0);
  long x = 0;
  std::vector<int> xmap;
  for (int m = 0; m <= T; ++m) {
    const int K = T - m + 1, ke = (K + 1) / 2, kp = round_up(ke, p.kc);
    p.xbase[m] = x;
    x += 2L * kp;
  }
  p.xlen = x;
  const size_t es = p.esize;
  // tables
  const long nsyn = (long)(T + 1) * nh * 2 * p.kepad, nana = (long)(T + 1) * 2 * p.kirows * p.nhpad;
  for (int t = 0; t < 2; ++t)
    for (int h = 0; h < 2; ++h) {
      p.tsyn[t][h] = tc_alloc(p, nsyn * es);
      p.tana[t][h] = tc_alloc(p, nana * es);
    }
  for (int t = 0; t < 2; ++t) {
    const double* tab = t ? H64 : P64;
    if (kind == TC_TF32) {
      k_tc_tab_syn<TC_TF32><<<2048, 256, 0, s>>>(T, nh, p.kepad, d_toff, tab, (uint32_t*)p.tsyn[t][0],
                                                 (uint32_t*)p.tsyn[t][1]);
      k_tc_tab_ana<TC_TF32><<<2048, 256, 0, s>>>(T, nh, p.kirows, p.nhpad, d_toff, tab, (uint32_t*)p.tana[t][0],
                                                 (uint32_t*)p.tana[t][1]);
    } else {
      k_tc_tab_syn<TC_BF16><<<2048, 256, 0, s>>>(T, nh, p.kepad, d_toff, tab, (__nv_bfloat16*)p.tsyn[t][0],
                                                 (__nv_bfloat16*)p.tsyn[t][1]);
      k_tc_tab_ana<TC_BF16><<<2048, 256, 0, s>>>(T, nh, p.kirows, p.nhpad, d_toff, tab,
                                                 (__nv_bfloat16*)p.tana[t][0], (__nv_bfloat16*)p.tana[t][1]);
    }
    count_launch(2);
    GD_LAUNCH_CHECK();
  }
  // staging
  for (int h = 0; h < 2; ++h) {
    p.x[h] = tc_alloc(p, (size_t)p.ncap * p.xlen * es);
    p.gp[h] = tc_alloc(p, (size_t)(T + 1) * p.ncap * p.nhpad * es);
    p.gm[h] = tc_alloc(p, (size_t)(T + 1) * p.ncap * p.nhpad * es);
    GD_CUDA(cudaMemsetAsync(p.x[h], 0, (size_t)p.ncap * p.xlen * es, s));
  }
  p.d_xbase = (long*)tc_alloc(p, sizeof(long) * (T + 1));
  GD_CUDA(cudaMemcpyAsync(p.d_xbase, p.xbase.data(), sizeof(long) * (T + 1), cudaMemcpyHostToDevice, s));
  p.d_err = (int*)tc_alloc(p, sizeof(int));
  GD_CUDA(cudaMemsetAsync(p.d_err, 0, sizeof(int), s));
  // tensor maps
  for (int t = 0; t < 2; ++t)
    for (int h = 0; h < 2; ++h) {
      uint64_t ds[3] = {(uint64_t)2 * p.kepad, (uint64_t)nh, (uint64_t)T + 1};
      make_map(&p.m_tsyn[t][h], p.tsyn[t][h], kind, 3, ds, p.kc, p.nsyn);
      uint64_t da[3] = {(uint64_t)p.nhpad, (uint64_t)2 * p.kirows, (uint64_t)T + 1};
      make_map(&p.m_tana[t][h], p.tana[t][h], kind, 3, da, p.kc, p.nana);
    }
  for (int h = 0; h < 2; ++h) {
    uint64_t dx[2] = {(uint64_t)p.xlen, (uint64_t)p.ncap};
    make_map(&p.m_x[h], p.x[h], kind, 2, dx, p.kc, TC_M);
    uint64_t dg[3] = {(uint64_t)p.nhpad, (uint64_t)p.ncap, (uint64_t)T + 1};
    make_map(&p.m_gp[h], p.gp[h], kind, 3, dg, p.kc, TC_M);
    make_map(&p.m_gm[h], p.gm[h], kind, 3, dg, p.kc, TC_M);
  }
  GD_CUDA(cudaStreamSynchronize(s));
}

int tc_tile_n(int n, int cap) { return tile_n(n, cap); }

// a new latitude tile of the synthesis GEMM: the tables keep their layout,
// the tensor maps take the new box and the cached work lists are dropped
void tc_set_nsyn(TcPlan& p, int nsyn) {
  if (nsyn < 16 || nsyn % 16 || nsyn > (!p.persistent ? 160 : p.kind == TC_TF32 ? tc_max_n(p) : 128))
    throw std::invalid_argument("tc_set_nsyn: N tile must be a multiple of 16 within the TMEM budget");
  p.nsyn = nsyn;
  const int kind = p.kind;
  for (int t = 0; t < 2; ++t)
    for (int h = 0; h < 2; ++h) {
      uint64_t ds[3] = {(uint64_t)2 * p.kepad, (uint64_t)p.nh, (uint64_t)p.T + 1};
      make_map(&p.m_tsyn[t][h], p.tsyn[t][h], kind, 3, ds, p.kc, p.nsyn);
    }
  p.item_cache.clear();  // the lists depend on the tile; their device arrays are freed with the plan
}

void tc_free(TcPlan& p) {
  for (void* d : p.allocs) cudaFree(d);
  p.allocs.clear();
  p.item_cache.clear();
  p.raw_maps.clear();
  p.d_xmap = nullptr;
}

static uint32_t make_idesc(int kind, int N) {
  const uint32_t fmt = kind == TC_TF32 ? 2u : 1u;  // TF32 (kind::tf32) or BF16 (kind::f16)
  return (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
}

static uint32_t tmem_cols_for(int N) {
  uint32_t c = 32;
  while (c < (uint32_t)(2 * N)) c <<= 1;
  return c;
}

static size_t smem_for(int N) { return (size_t)TC_NS * (2 * TC_M * 128 + 2 * N * 128) + 1024 + 512; }

template <int KIND>
static void launch_gemm(const TcPlan& p, const CUtensorMap& a0h, const CUtensorMap& a0l, const CUtensorMap& a1h,
                        const CUtensorMap& a1l, const CUtensorMap& bh, const CUtensorMap& bl, TcArgs& args,
                        int nitems, cudaStream_t s) {
  const size_t sm = smem_for(args.N);
  if (sm > 227 * 1024 || args.N > (p.persistent ? 128 : 160) || args.N % 16)
    throw std::runtime_error("tc gemm: bad N tile");
  if (p.persistent) {
    args.tmem_cols = tmem_cols_for(2 * args.N);  // two E|O buffers
    static bool attr_p = false;
    if (!attr_p) {
      GD_CUDA(cudaFuncSetAttribute(k_tc_gemm_p<KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
      attr_p = true;
    }
    const int grid = std::min(nitems, p.nsm);
    k_tc_gemm_p<KIND><<<grid, TCP_THREADS, sm, s>>>(a0h, a0l, a1h, a1l, bh, bl, args, nitems);
  } else {
    static bool attr = false;
    if (!attr) {
      GD_CUDA(cudaFuncSetAttribute(k_tc_gemm<KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
      attr = true;
    }
    k_tc_gemm<KIND><<<nitems, TC_THREADS, sm, s>>>(a0h, a0l, a1h, a1l, bh, bl, args);
  }
  count_launch();
  GD_LAUNCH_CHECK();
}

static int4* cached_items(TcPlan& p, long key, const std::vector<int4>& it) {
  for (auto& kv : p.item_cache)
    if (kv.first == key) return kv.second;
  int4* d = nullptr;
  GD_CUDA(cudaMalloc(&d, sizeof(int4) * std::max<size_t>(it.size(), 1)));
  GD_CUDA(cudaMemcpy(d, it.data(), sizeof(int4) * it.size(), cudaMemcpyHostToDevice));
  p.item_cache.push_back({key, d});
  p.allocs.push_back(d);
  return d;
}

static bool fused_ok(const TcPlan& p, const void* base, long ld) {
  static const bool off = [] {
    const char* e = getenv("GD_TC_FUSED");
    return e && e[0] == '0';
  }();
  return !off && p.kind == TC_TF32 && p.persistent && p.nsyn <= tc_max_n(p) && p.nana <= tc_max_n(p) &&
         ((uintptr_t)base % 16) == 0 && ld % 4 == 0;
}

static void launch_fused(const TcPlan& p, const CUtensorMap& raw, const CUtensorMap& bh, const CUtensorMap& bl,
                         TcArgs& args, int nitems, uint32_t raw_bytes, cudaStream_t s) {
  const uint32_t stage = (uint32_t)round_up(2 * args.N * 128 + (int)raw_bytes, 1024);
  const size_t avail = 227 * 1024 - 1024 - 256;
  // TMA ring depth: as many stages as shared memory holds (at most
  // TCF_MAXNS; GD_TC_STAGES lowers the cap, a tuning and measurement knob)
  static const int cap = [] {
    const char* e = getenv("GD_TC_STAGES");
    const int v = (e && *e) ? atoi(e) : TCF_MAXNS;
    return std::max(2, std::min(v, TCF_MAXNS));
  }();
  const int ns = (int)std::min<size_t>((size_t)cap, avail / stage);
  args.nbuf = tcf_nbuf(p, args.N);
  args.na = tcf_slots(p, args.N);
  if (ns < args.na || args.N > TCF_MAXN || args.N % 16 ||
      tcf_tmem_cols(args.N, p.sepx, p.cps > 0, args.na, args.nbuf) > 512)
    throw std::runtime_error("tc fused gemm: bad tile");
  const size_t sm = (size_t)ns * stage + 1024 + 256;
  args.tmem_cols = 512;
  args.sepx = p.sepx ? 1 : 0;
  args.cps = p.cps;
  static bool attr = false;
  if (!attr) {
    GD_CUDA(cudaFuncSetAttribute(k_tc_gemm_f, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
    attr = true;
  }
  const int grid = std::min(nitems, p.nsm);
  k_tc_gemm_f<<<grid, TCF_THREADS, sm, s>>>(raw, bh, bl, args, nitems, ns, raw_bytes);
  count_launch();
  GD_LAUNCH_CHECK();
}

void tc_synth(TcPlan& p, const long* d_moff, bool useH, const float* B, long ldB, long nrowsB, int ncols, float* F,
              long ldF, cudaStream_t s) {
  if (ncols > p.ncap) throw std::runtime_error("tc_synth: too many columns");
  const long nlm = (long)(p.T + 1) * (p.T + 2) / 2;
  if (fused_ok(p, B, ldB) && 2 * (nrowsB / 2) >= nlm) {
    const int ct = (ncols + TC_M - 1) / TC_M, nt = (p.nh + p.nsyn - 1) / p.nsyn;
    std::vector<int4> it;
    for (int m = 1; m <= p.T; ++m)  // order 0 (zonal means) runs on the IEEE SIMT path
      for (int a = 0; a < ct; ++a)
        for (int b2 = 0; b2 < nt; ++b2) it.push_back(make_int4(m, a, b2, 0));
    if (it.empty()) return;
    TcArgs args{};
    args.items = cached_items(p, ((long)ncols << 2) | 0, it);
    args.mode = 0;
    args.T = p.T;
    args.nh = p.nh;
    args.nlat = p.nlat;
    args.N = p.nsyn;
    args.kc = p.kc;
    args.kepad = p.kepad;
    args.kirows = p.kirows;
    args.xbase = p.d_xbase;
    args.moff = d_moff;
    args.parityH = useH ? 1 : 0;
    args.ncols = ncols;
    args.coff = 0;
    args.out = F;
    args.ldout = ldF;
    args.err = p.d_err;
    args.idesc = make_idesc(p.kind, p.nsyn);
    // spectral rows viewed as (column, parity slot, row pair): a chunk is one
    // parity slot of kc consecutive pairs
    const uint64_t dims[3] = {(uint64_t)ncols, 2, (uint64_t)(nrowsB / 2)};
    const uint64_t strides[2] = {(uint64_t)ldB * 4, (uint64_t)ldB * 8};
    const uint32_t box[3] = {TC_M, 1, (uint32_t)p.kc};
    const CUtensorMap& raw = cached_raw_map(p, B, dims, strides, box);
    const int t = useH ? 1 : 0;
    launch_fused(p, raw, p.m_tsyn[t][0], p.m_tsyn[t][1], args, (int)it.size(), (uint32_t)(p.kc * TC_M * 4), s);
    return;
  }
  // 1) split the spectral columns into the padded K-major staging
  if (!p.d_xmap) {
    std::vector<long> hm(p.T + 2);
    hm[0] = 0;
    for (int m = 0; m <= p.T; ++m) hm[m + 1] = hm[m] + (p.T - m + 1);
    std::vector<int> xm(p.xlen, -1);
    for (int m = 0; m <= p.T; ++m) {
      const int K = p.T - m + 1, ke = (K + 1) / 2, kp = round_up(ke, p.kc);
      for (int par = 0; par < 2; ++par)
        for (int i = 0; i < kp; ++i) {
          const int q = 2 * i + par;
          if (q < K) xm[p.xbase[m] + (long)par * kp + i] = (int)(hm[m] + q);
        }
    }
    p.d_xmap = (int*)tc_alloc(p, sizeof(int) * p.xlen);
    GD_CUDA(cudaMemcpy(p.d_xmap, xm.data(), sizeof(int) * p.xlen, cudaMemcpyHostToDevice));
  }
  dim3 g((unsigned)((p.xlen + 31) / 32), (unsigned)((ncols + 31) / 32)), b(32, 8);
  if (p.kind == TC_TF32)
    k_tc_split_x<TC_TF32><<<g, b, 0, s>>>(B, ldB, ncols, p.d_xmap, p.xlen, (uint32_t*)p.x[0], (uint32_t*)p.x[1]);
  else
    k_tc_split_x<TC_BF16><<<g, b, 0, s>>>(B, ldB, ncols, p.d_xmap, p.xlen, (__nv_bfloat16*)p.x[0],
                                          (__nv_bfloat16*)p.x[1]);
  count_launch();
  GD_LAUNCH_CHECK();
  // 2) GEMM
  const int ct = (ncols + TC_M - 1) / TC_M, nt = (p.nh + p.nsyn - 1) / p.nsyn;
  std::vector<int4> it;
  for (int m = 1; m <= p.T; ++m)  // order 0 (zonal means) runs on the IEEE SIMT path
    for (int a = 0; a < ct; ++a)
      for (int b2 = 0; b2 < nt; ++b2) it.push_back(make_int4(m, a, b2, 0));
  if (it.empty()) return;
  int4* dit = cached_items(p, ((long)ncols << 2) | 0, it);
  TcArgs args{};
  args.items = dit;
  args.mode = 0;
  args.T = p.T;
  args.nh = p.nh;
  args.nlat = p.nlat;
  args.N = p.nsyn;
  args.kc = p.kc;
  args.kepad = p.kepad;
  args.kirows = p.kirows;
  args.xbase = p.d_xbase;
  args.moff = d_moff;
  args.parityH = useH ? 1 : 0;
  args.ncols = ncols;
  args.coff = 0;
  args.out = F;
  args.ldout = ldF;
  args.err = p.d_err;
  args.idesc = make_idesc(p.kind, p.nsyn);
  args.tmem_cols = tmem_cols_for(p.nsyn);
  const int t = useH ? 1 : 0;
  if (p.kind == TC_TF32)
    launch_gemm<TC_TF32>(p, p.m_x[0], p.m_x[1], p.m_x[0], p.m_x[1], p.m_tsyn[t][0], p.m_tsyn[t][1], args,
                         (int)it.size(), s);
  else
    launch_gemm<TC_BF16>(p, p.m_x[0], p.m_x[1], p.m_x[0], p.m_x[1], p.m_tsyn[t][0], p.m_tsyn[t][1], args,
                         (int)it.size(), s);
}

int tc_anal_segments(const TcPlan& p) {  // K segments of the latitude sum: at most one per chunk
  return std::max(1, std::min(p.aseg, (p.nh + p.kc - 1) / p.kc));
}

void tc_anal(TcPlan& p, const long* d_moff, bool useH, const float* G, long ldG, int ncols, float* A, long ldA,
             cudaStream_t s) {
  if (ncols > p.ncap) throw std::runtime_error("tc_anal: too many columns");
  if (fused_ok(p, G, ldG)) {
    const int ct = (ncols + TC_M - 1) / TC_M;
    std::vector<int4> it;
    const int nseg = tc_anal_segments(p);
    for (int m = 1; m <= p.T; ++m) {  // order 0 runs on the IEEE SIMT path
      const int ke = (p.T - m + 2) / 2;
      for (int a = 0; a < ct; ++a)
        for (int b2 = 0; b2 < (ke + p.nana - 1) / p.nana; ++b2)
          for (int q = 0; q < nseg; ++q) it.push_back(make_int4(m, a, b2, q));
    }
    if (it.empty()) return;
    TcArgs args{};
    args.items = cached_items(p, ((long)ncols << 8) | ((long)nseg << 2) | 1, it);
    args.nseg = nseg;
    args.seg_stride = (long)(p.T + 1) * (p.T + 2) / 2 * ldA;
    args.mode = 1;
    args.T = p.T;
    args.nh = p.nh;
    args.nlat = p.nlat;
    args.N = p.nana;
    args.kc = p.kc;
    args.kepad = p.kepad;
    args.kirows = p.kirows;
    args.xbase = p.d_xbase;
    args.moff = d_moff;
    args.parityH = useH ? 1 : 0;
    args.ncols = ncols;
    args.coff = 0;
    args.out = A;
    args.ldout = ldA;
    args.err = p.d_err;
    args.idesc = make_idesc(p.kind, p.nana);
    // Fourier rows [m][lat][column]: a chunk is kc northern latitudes plus
    // the kc mirrored southern ones
    const uint64_t dims[3] = {(uint64_t)ncols, (uint64_t)p.nlat, (uint64_t)p.T + 1};
    const uint64_t strides[2] = {(uint64_t)ldG * 4, (uint64_t)ldG * 4 * p.nlat};
    const uint32_t box[3] = {TC_M, (uint32_t)p.kc, 1};
    const CUtensorMap& raw = cached_raw_map(p, G, dims, strides, box);
    const int t = useH ? 1 : 0;
    launch_fused(p, raw, p.m_tana[t][0], p.m_tana[t][1], args, (int)it.size(), (uint32_t)(2 * p.kc * TC_M * 4), s);
    return;
  }
  dim3 g((unsigned)((p.nhpad + 31) / 32), (unsigned)((ncols + 31) / 32), (unsigned)(p.T + 1)), b(32, 8);
  if (p.kind == TC_TF32)
    k_tc_split_g<TC_TF32><<<g, b, 0, s>>>(G, ldG, ncols, p.nh, p.nlat, p.nhpad, p.ncap, (uint32_t*)p.gp[0],
                                          (uint32_t*)p.gp[1], (uint32_t*)p.gm[0], (uint32_t*)p.gm[1]);
  else
    k_tc_split_g<TC_BF16><<<g, b, 0, s>>>(G, ldG, ncols, p.nh, p.nlat, p.nhpad, p.ncap, (__nv_bfloat16*)p.gp[0],
                                          (__nv_bfloat16*)p.gp[1], (__nv_bfloat16*)p.gm[0],
                                          (__nv_bfloat16*)p.gm[1]);
  count_launch();
  GD_LAUNCH_CHECK();
  const int ct = (ncols + TC_M - 1) / TC_M;
  std::vector<int4> it;
  for (int m = 1; m <= p.T; ++m) {  // order 0 runs on the IEEE SIMT path
    const int ke = (p.T - m + 2) / 2;
    for (int a = 0; a < ct; ++a)
      for (int b2 = 0; b2 < (ke + p.nana - 1) / p.nana; ++b2) it.push_back(make_int4(m, a, b2, 0));
  }
  if (it.empty()) return;
  int4* dit = cached_items(p, ((long)ncols << 2) | 1, it);
  TcArgs args{};
  args.items = dit;
  args.mode = 1;
  args.T = p.T;
  args.nh = p.nh;
  args.nlat = p.nlat;
  args.N = p.nana;
  args.kc = p.kc;
  args.kepad = p.kepad;
  args.kirows = p.kirows;
  args.xbase = p.d_xbase;
  args.moff = d_moff;
  args.parityH = useH ? 1 : 0;
  args.ncols = ncols;
  args.coff = 0;
  args.out = A;
  args.ldout = ldA;
  args.err = p.d_err;
  args.idesc = make_idesc(p.kind, p.nana);
  args.tmem_cols = tmem_cols_for(p.nana);
  const int t = useH ? 1 : 0;
  // P: even degrees pair with G_N + G_S, odd with G_N - G_S; dP/dphi the reverse
  const CUtensorMap* e0 = useH ? p.m_gm : p.m_gp;
  const CUtensorMap* e1 = useH ? p.m_gp : p.m_gm;
  if (p.kind == TC_TF32)
    launch_gemm<TC_TF32>(p, e0[0], e0[1], e1[0], e1[1], p.m_tana[t][0], p.m_tana[t][1], args, (int)it.size(), s);
  else
    launch_gemm<TC_BF16>(p, e0[0], e0[1], e1[0], e1[1], p.m_tana[t][0], p.m_tana[t][1], args, (int)it.size(), s);
}

int tc_check(TcPlan& p, cudaStream_t s) {
  int h = 0;
  GD_CUDA(cudaMemcpyAsync(&h, p.d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  GD_CUDA(cudaStreamSynchronize(s));
  if (h) GD_CUDA(cudaMemsetAsync(p.d_err, 0, sizeof(int), s));
  return h;
}


// ------------------------------------------- closure network layers --
// One CTA per 128 rows (grid columns of the closure); warp 0's first thread
// issues the TMA copies of A hi, A lo and W per 32-wide K chunk into a
// 3-stage ring, warp 1's first thread issues two MMAs per K step (hi W and
// lo W; W is exact in TF32), all four warps drain the accumulator (warp w
// holds TMEM lanes 32w..32w+31 = rows).  Every wait is bounded.
struct TcMlpArgs {
  int M, N, Np, nk;  // Np: this launch's N tile (each CTA covers columns blockIdx.y * Np ...)
  const float* bias;
  int gelu;
  int mode;
  float* z;
  float* act;
  const float* zin;
  int ldz;
  uint32_t* oh;
  uint32_t* ol;
  int ldo;
  float* y;
  int ldy;
  int* err;
  uint32_t idesc, tmem_cols;
};

__device__ __forceinline__ float tc_gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float tc_gelu_d(float z) {
  return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    k_tc_mlp(const __grid_constant__ CUtensorMap mAh, const __grid_constant__ CUtensorMap mAl,
             const __grid_constant__ CUtensorMap mW, TcMlpArgs a) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~(uintptr_t)1023);
  const uint32_t bytesA = TC_M * 128, bytesW = (uint32_t)a.Np * 128;
  const uint32_t stage_bytes = 2 * bytesA + bytesW;
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + TC_NS * stage_bytes);
  uint64_t* empty = full + TC_NS;
  uint64_t* done = empty + TC_NS;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * TC_M, c0 = blockIdx.y * a.Np;  // rows, and the first of the CTA's Np columns

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(a.tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < TC_NS; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&empty[s]), 1);
    }
    mbar_init(smem_u32(done), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;

  if (tid == 0) {  // ---- TMA producer
    int fills[TC_NS] = {0, 0, 0};
    for (int i = 0; i < a.nk; ++i) {
      const int s = i % TC_NS, u = i / TC_NS;
      if (u >= 1 && !mbar_wait(smem_u32(&empty[s]), (u - 1) & 1, a.err, 31)) break;
      unsigned char* st = sm + s * stage_bytes;
      const uint32_t fb = smem_u32(&full[s]);
      mbar_expect_tx(fb, stage_bytes);
      tma_2d(smem_u32(st), &mAh, i * 32, m0, fb);
      tma_2d(smem_u32(st + bytesA), &mAl, i * 32, m0, fb);
      tma_2d(smem_u32(st + 2 * bytesA), &mW, i * 32, c0, fb);
      ++fills[s];
    }
    for (int s = 0; s < TC_NS; ++s)  // never leave with copies in flight
      if (fills[s] > 0) mbar_wait(smem_u32(&full[s]), (fills[s] - 1) & 1, a.err, 32);
  } else if (tid == 32) {  // ---- MMA issuer
    for (int i = 0; i < a.nk; ++i) {
      const int s = i % TC_NS, u = i / TC_NS;
      if (!mbar_wait(smem_u32(&full[s]), u & 1, a.err, 33)) break;
      tc_fence_after();
      unsigned char* st = sm + s * stage_bytes;
      const uint64_t dah = smem_desc(smem_u32(st)), dal = smem_desc(smem_u32(st + bytesA));
      const uint64_t dw = smem_desc(smem_u32(st + 2 * bytesA));
#pragma unroll
      for (int k4 = 0; k4 < 4; ++k4) {  // 4 MMAs of K = 8 per 128-byte row
        const uint64_t o = (uint64_t)(2 * k4);
        mma<TC_TF32>(tbase, dah + o, dw + o, a.idesc, (i > 0 || k4 > 0) ? 1u : 0u);
        mma<TC_TF32>(tbase, dal + o, dw + o, a.idesc, 1u);
      }
      mma_commit(smem_u32(&empty[s]));
    }
    mma_commit(smem_u32(done));  // every issued MMA has completed at done
  }
  __syncwarp();
  // ---- epilogue
  const bool ok = mbar_wait(smem_u32(done), 0, a.err, 34);
  tc_fence_after();
  const bool go = __all_sync(0xffffffffu, ok && *(volatile int*)a.err == 0);
  if (go && a.mode >= 2) {
    // training: each lane stages 64 accumulator columns of its row (plus the
    // bias in the forward), then the warp finishes row after row with
    // coalesced loads and stores: the forward stores z, gelu(z) and the split
    // of gelu(z); the backward reads z of the layer below and stores
    // dZ = acc * gelu'(z) and its split
    constexpr int TP = 65;
    uint32_t* th = reinterpret_cast<uint32_t*>(sm) + warp * (2 * 32 * TP);
    const uint32_t tw = tbase + ((uint32_t)(warp * 32) << 16);
    const int mw = m0 + warp * 32;
    for (int g0 = 0; g0 < a.Np; g0 += 64) {
      for (int g = g0; g < g0 + 64 && g < a.Np; g += 16) {
        float v[16];
        tmem_ld16(tw + g, v);
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int n = c0 + g + q;
          th[lane * TP + (g + q - g0)] = __float_as_uint(v[q] + (a.mode == 2 && n < a.N ? a.bias[n] : 0.f));
        }
      }
      __syncwarp();
      for (int r = 0; r < 32; ++r) {
        const int m = mw + r;
        if (m >= a.M) break;
#pragma unroll
        for (int c = 0; c < 64; c += 32) {
          const int n = c0 + g0 + c + lane;
          if (g0 + c + lane < a.Np && n < a.N) {
            const float v = __uint_as_float(th[r * TP + c + lane]);
            const long iz = (long)m * a.ldz + n;
            float o;  // the value the next product takes, split hi + lo
            if (a.mode == 2) {
              o = tc_gelu(v);
              a.z[iz] = v;
              a.act[iz] = o;
            } else {
              o = v * tc_gelu_d(a.zin[iz]);
              a.y[(long)m * a.ldy + n] = o;
            }
            uint32_t h, l;
            Elem<TC_TF32>::splitf(o, h, l);
            a.oh[(long)m * a.ldo + n] = h;
            a.ol[(long)m * a.ldo + n] = l;
          }
        }
      }
      __syncwarp();
    }
  } else if (go) {
    // each lane finishes 64 columns of its row into the warp's part of the
    // (now idle) ring, then the warp stores row after row: 128 contiguous
    // bytes per store instead of 32 rows' scattered words
    constexpr int TP = 65;  // tile pitch (words): conflict-free column writes
    uint32_t* th = reinterpret_cast<uint32_t*>(sm) + warp * (2 * 32 * TP);
    uint32_t* tl = th + 32 * TP;
    const uint32_t tw = tbase + ((uint32_t)(warp * 32) << 16);
    const int mw = m0 + warp * 32;
    for (int g0 = 0; g0 < a.Np; g0 += 64) {
      for (int g = g0; g < g0 + 64 && g < a.Np; g += 16) {
        float v[16];
        tmem_ld16(tw + g, v);
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int n = c0 + g + q;
          const float z = v[q] + (n < a.N ? a.bias[n] : 0.f);
          uint32_t h, l = 0;
          if (a.gelu)
            Elem<TC_TF32>::splitf(tc_gelu(z), h, l);
          else
            h = __float_as_uint(z);
          th[lane * TP + (g + q - g0)] = h;
          tl[lane * TP + (g + q - g0)] = l;
        }
      }
      __syncwarp();
      for (int r = 0; r < 32; ++r) {
        const int m = mw + r;
        if (m >= a.M) break;
#pragma unroll
        for (int c = 0; c < 64; c += 32) {
          const int n = c0 + g0 + c + lane;
          if (g0 + c + lane < a.Np && n < a.N) {
            if (a.gelu) {
              a.oh[(long)m * a.ldo + n] = th[r * TP + c + lane];
              a.ol[(long)m * a.ldo + n] = tl[r * TP + c + lane];
            } else {
              a.y[(long)m * a.ldy + n] = __uint_as_float(th[r * TP + c + lane]);
            }
          }
        }
      }
      __syncwarp();
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(a.tmem_cols));
}

// Weight gradient of a closure layer (see TcWgrad): one CTA per 128 rows of
// dZ^T and one slice of the batch; the producer loads A hi, A lo, B hi, B lo
// per 32-deep K chunk into a 2-stage ring, the MMA thread issues three
// products per K step into one accumulator, the four warps stage the
// accumulator through the idle ring and store the slice's partial tile row
// by row.  Every wait is bounded.
constexpr int TCW_NS = 2;
struct TcWgradArgs {
  int Np, cps, nkt;  // chunks per slice, chunks in all
  float* part;
  long pstride;  // floats per slice
  int* err;
  uint32_t idesc, tmem_cols;
};

__global__ void __launch_bounds__(TC_THREADS, 1)
    k_tc_wgrad(const __grid_constant__ CUtensorMap mAh, const __grid_constant__ CUtensorMap mAl,
               const __grid_constant__ CUtensorMap mBh, const __grid_constant__ CUtensorMap mBl, TcWgradArgs a) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~(uintptr_t)1023);
  const uint32_t bytesA = TC_M * 128, bytesB = (uint32_t)a.Np * 128;
  const uint32_t stage_bytes = 2 * bytesA + 2 * bytesB;
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + TCW_NS * stage_bytes);
  uint64_t* empty = full + TCW_NS;
  uint64_t* done = empty + TCW_NS;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * TC_M;
  const int ks = blockIdx.y * a.cps;           // this slice's first K chunk
  const int nk = max(0, min(a.cps, a.nkt - ks));  // its chunks (every slice has at least one)

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(a.tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < TCW_NS; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&empty[s]), 1);
    }
    mbar_init(smem_u32(done), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;

  if (tid == 0) {  // ---- TMA producer
    int fills[TCW_NS] = {0, 0};
    for (int i = 0; i < nk; ++i) {
      const int s = i % TCW_NS, u = i / TCW_NS;
      if (u >= 1 && !mbar_wait(smem_u32(&empty[s]), (u - 1) & 1, a.err, 41)) break;
      unsigned char* st = sm + s * stage_bytes;
      const uint32_t fb = smem_u32(&full[s]);
      const int x = (ks + i) * 32;
      mbar_expect_tx(fb, stage_bytes);
      tma_2d(smem_u32(st), &mAh, x, m0, fb);
      tma_2d(smem_u32(st + bytesA), &mAl, x, m0, fb);
      tma_2d(smem_u32(st + 2 * bytesA), &mBh, x, 0, fb);
      tma_2d(smem_u32(st + 2 * bytesA + bytesB), &mBl, x, 0, fb);
      ++fills[s];
    }
    for (int s = 0; s < TCW_NS; ++s)  // never leave with copies in flight
      if (fills[s] > 0) mbar_wait(smem_u32(&full[s]), (fills[s] - 1) & 1, a.err, 42);
  } else if (tid == 32) {  // ---- MMA issuer
    for (int i = 0; i < nk; ++i) {
      const int s = i % TCW_NS, u = i / TCW_NS;
      if (!mbar_wait(smem_u32(&full[s]), u & 1, a.err, 43)) break;
      tc_fence_after();
      unsigned char* st = sm + s * stage_bytes;
      const uint64_t dah = smem_desc(smem_u32(st)), dal = smem_desc(smem_u32(st + bytesA));
      const uint64_t dbh = smem_desc(smem_u32(st + 2 * bytesA)), dbl = smem_desc(smem_u32(st + 2 * bytesA + bytesB));
#pragma unroll
      for (int k4 = 0; k4 < 4; ++k4) {  // 4 K steps of 8 per 128-byte row
        const uint64_t o = (uint64_t)(2 * k4);
        mma<TC_TF32>(tbase, dah + o, dbh + o, a.idesc, (i > 0 || k4 > 0) ? 1u : 0u);
        mma<TC_TF32>(tbase, dah + o, dbl + o, a.idesc, 1u);
        mma<TC_TF32>(tbase, dal + o, dbh + o, a.idesc, 1u);
      }
      mma_commit(smem_u32(&empty[s]));
    }
    mma_commit(smem_u32(done));  // every issued MMA has completed at done
  }
  __syncwarp();
  // ---- epilogue: the slice's partial tile, rows m0 + 32 w + r
  const bool ok = mbar_wait(smem_u32(done), 0, a.err, 44);
  tc_fence_after();
  const bool go = __all_sync(0xffffffffu, ok && *(volatile int*)a.err == 0);
  if (go) {
    constexpr int TP = 65;
    uint32_t* th = reinterpret_cast<uint32_t*>(sm) + warp * (32 * TP);
    const uint32_t tw = tbase + ((uint32_t)(warp * 32) << 16);
    float* out = a.part + (long)blockIdx.y * a.pstride + (long)(m0 + warp * 32) * a.Np;
    for (int g0 = 0; g0 < a.Np; g0 += 64) {
      for (int g = g0; g < g0 + 64 && g < a.Np; g += 16) {
        float v[16];
        tmem_ld16(tw + g, v);
#pragma unroll
        for (int q = 0; q < 16; ++q) th[lane * TP + (g + q - g0)] = __float_as_uint(v[q]);
      }
      __syncwarp();
      for (int r = 0; r < 32; ++r)
#pragma unroll
        for (int c = 0; c < 64; c += 32) {
          const int n = g0 + c + lane;
          if (n < a.Np) out[(long)r * a.Np + n] = __uint_as_float(th[r * TP + c + lane]);
        }
      __syncwarp();
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(a.tmem_cols));
}

void tc_wgrad_maps(TcWgrad& W, const uint32_t* ah, const uint32_t* al, const uint32_t* bh, const uint32_t* bl,
                   int kpitch) {
  if (W.Mp < TC_M || W.Mp % TC_M || W.Np < 16 || W.Np > 256 || W.Np % 16 || kpitch < 32 || kpitch % 32)
    throw std::invalid_argument("tc_wgrad_maps: bad shape");
  const uint64_t da[2] = {(uint64_t)kpitch, (uint64_t)W.Mp}, db[2] = {(uint64_t)kpitch, (uint64_t)W.Np};
  make_map(&W.ah, const_cast<uint32_t*>(ah), TC_TF32, 2, da, 32, TC_M);
  make_map(&W.al, const_cast<uint32_t*>(al), TC_TF32, 2, da, 32, TC_M);
  make_map(&W.bh, const_cast<uint32_t*>(bh), TC_TF32, 2, db, 32, W.Np);
  make_map(&W.bl, const_cast<uint32_t*>(bl), TC_TF32, 2, db, 32, W.Np);
}

void tc_wgrad(const TcWgrad& W, int nk, int cps, int nsplit, cudaStream_t s) {
  if (nk < 1 || cps < 1 || nsplit < 1 || (long)(nsplit - 1) * cps >= nk || (long)nsplit * cps < nk || !W.part)
    throw std::invalid_argument("tc_wgrad: bad K split");
  TcWgradArgs a;
  a.Np = W.Np;
  a.cps = cps;
  a.nkt = nk;
  a.part = W.part;
  a.pstride = (long)W.Mp * W.Np;
  a.err = W.err;
  a.idesc = make_idesc(TC_TF32, W.Np);
  a.tmem_cols = tmem_cols_for(W.Np / 2);  // a power of two >= Np (and >= 32)
  const size_t sm = (size_t)TCW_NS * (2 * TC_M * 128 + 2 * (size_t)W.Np * 128) + 1024 + 256;
  static bool attr = false;
  if (!attr) {
    GD_CUDA(cudaFuncSetAttribute(k_tc_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
    attr = true;
  }
  k_tc_wgrad<<<dim3(W.Mp / TC_M, nsplit), TC_THREADS, sm, s>>>(W.ah, W.al, W.bh, W.bl, a);
  count_launch();
  GD_LAUNCH_CHECK();
}

void tc_mlp_maps(TcMlpLayer& L, const uint32_t* ah, const uint32_t* al, const float* w) {
  if (L.Kp % 32 || L.Np % 16 || L.Np < 16 || L.Np > 256 || L.N > L.Np || L.M < 1)
    throw std::invalid_argument("tc_mlp_maps: bad layer shape");
  const uint64_t da[2] = {(uint64_t)L.Kp, (uint64_t)L.M}, dw[2] = {(uint64_t)L.Kp, (uint64_t)L.Np};
  make_map(&L.ah, const_cast<uint32_t*>(ah), TC_TF32, 2, da, 32, TC_M);
  make_map(&L.al, const_cast<uint32_t*>(al), TC_TF32, 2, da, 32, TC_M);
  make_map(&L.w, const_cast<float*>(w), TC_TF32, 2, dw, 32, L.Np);
  L.wbase = w;
  L.wbox = L.Np;
}

void tc_mlp_layer(const TcMlpLayer& Lin, cudaStream_t s) {
  // N tile: the whole padded width, halved (down to 32 columns, a multiple
  // of 16) while the row tiles alone leave SMs idle; the weights' map is
  // made again for a narrower box
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    GD_CUDA(cudaGetDevice(&dev));
    GD_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  }
  const int mt = (Lin.M + TC_M - 1) / TC_M;
  int nt = Lin.Np;
  while (nt >= 64 && (nt / 2) % 16 == 0 && (long)mt * ((Lin.Np + nt - 1) / nt) < nsm) nt /= 2;
  TcMlpLayer L = Lin;
  if (nt != L.wbox) {
    if (!L.wbase) throw std::invalid_argument("tc_mlp_layer: layer without its weight map");
    const uint64_t dw[2] = {(uint64_t)L.Kp, (uint64_t)L.Np};
    make_map(&L.w, const_cast<float*>(L.wbase), TC_TF32, 2, dw, 32, nt);
    L.wbox = nt;
  }
  TcMlpArgs a;
  a.M = L.M;
  a.N = L.N;
  a.Np = nt;
  a.nk = L.Kp / 32;
  a.bias = L.bias;
  a.gelu = L.gelu;
  a.mode = L.mode;
  a.z = L.z;
  a.act = L.act;
  a.zin = L.zin;
  a.ldz = L.ldz;
  if (L.mode >= 2 && (!L.oh || !L.ol || L.ldz < L.N || (L.mode == 2 ? (!L.z || !L.act || !L.bias) : (!L.zin || !L.y))))
    throw std::invalid_argument("tc_mlp_layer: training layer without its buffers");
  a.oh = L.oh;
  a.ol = L.ol;
  a.ldo = L.ldo;
  a.y = L.y;
  a.ldy = L.ldy;
  a.err = L.err;
  a.idesc = make_idesc(TC_TF32, nt);
  a.tmem_cols = tmem_cols_for(nt / 2);  // a power of two >= nt (and >= 32)
  const size_t sm = (size_t)TC_NS * (2 * TC_M * 128 + (size_t)nt * 128) + 1024 + 256;
  static bool attr = false;
  if (!attr) {
    GD_CUDA(cudaFuncSetAttribute(k_tc_mlp, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
    attr = true;
  }
  k_tc_mlp<<<dim3(mt, (L.Np + nt - 1) / nt), TC_THREADS, sm, s>>>(L.ah, L.al, L.w, a);
  count_launch();
  GD_LAUNCH_CHECK();
}

}  // namespace gd

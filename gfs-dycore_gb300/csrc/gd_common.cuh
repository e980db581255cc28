// gd_common.cuh -- shared definitions of the GB300 spectral dycore kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>

namespace gd {

// Fortran literals without a kind suffix are single precision in the
// reference (no -fdefault-real-8, src/Makefile.conf.gfortran), so its
// constants carry float-rounded values in every build.
#define GD_FLIT(x) ((double)(float)(x))

// src/physcons.f90:17-56
struct Phys {
  static constexpr double rerth = GD_FLIT(6.3712e+6f);
  static constexpr double grav = GD_FLIT(9.80665e+0f);
  static constexpr double omega = GD_FLIT(7.2921e-5f);
  static constexpr double rd = GD_FLIT(2.8705e+2f);
  static constexpr double rv = GD_FLIT(4.6150e+2f);
  static constexpr double cp = GD_FLIT(1.0046e+3f);
  static constexpr double cvap = GD_FLIT(1.8460e+3f);
};

struct CudaError : std::runtime_error {
  explicit CudaError(const std::string& s) : std::runtime_error(s) {}
};

#define GD_CUDA(call)                                                                         \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      throw ::gd::CudaError(std::string(#call) + ": " + cudaGetErrorString(e_) + " @" +      \
                            __FILE__ + ":" + std::to_string(__LINE__));                      \
  } while (0)

#define GD_LAUNCH_CHECK() GD_CUDA(cudaGetLastError())

// 2-component vector of the real type (one complex number).
template <typename R>
struct C2;
template <>
struct C2<double> {
  typedef double2 T;
};
template <>
struct C2<float> {
  typedef float2 T;
};

// two complex values in one aligned load (16 bytes FP32, 32 bytes FP64)
struct __align__(32) GdDouble4 {
  double x, y, z, w;
};
template <typename R>
struct C4;
template <>
struct C4<double> {
  typedef GdDouble4 T;
};
template <>
struct C4<float> {
  typedef float4 T;
};

template <typename R>
__host__ __device__ inline typename C2<R>::T mk2(R x, R y) {
  typename C2<R>::T v;
  v.x = x;
  v.y = y;
  return v;
}

inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }

// Launch accounting (reported by gd_launch_count).
extern long long g_launches;
inline void count_launch(int n = 1) { g_launches += n; }

}  // namespace gd

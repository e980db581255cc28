// gd_noalloc.cu -- step diagnostics without any device allocation.
//
// Some callers of this library cannot call cudaMalloc: a host model whose
// device memory is owned by another runtime's pool allocator (a coupler or
// an ML framework that hands out pre-allocated buffers), or a process that
// runs under a hard device-memory budget with every byte already committed.
// gd_diag_static serves them: the caller passes device-accessible inputs
// and the output, and the per-latitude partial sums the reduction needs
// live in the fixed array below instead of in allocated scratch.
//
// The array is a module-scope device variable: every GPU that loads this
// library holds it (GD_DIAG_STATIC_MAX_NLAT * 4 doubles) until the process
// exits.  In host code its name is only a host-side stand-in; the device
// address is obtained once per device with cudaGetSymbolAddress, with that
// device current, on the first call made on it.  All calls share the
// array and it keeps the last call's contents; each call overwrites every
// entry it reads, so nothing needs clearing, but calls that overlap on the
// GPU (different streams or threads at once) race on it.
#include <mutex>

#include "../../include/gd_api.h"
#include "gd_grid.cuh"

namespace {

static __device__ __align__(256) double g_diag_scratch[4 * GD_DIAG_STATIC_MAX_NLAT];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {nullptr};

// device address of g_diag_scratch on the current device (set up once)
int scratch_for_current_device(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GD_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_diag_scratch) != cudaSuccess || !p) return GD_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return GD_OK;
}

}  // namespace

extern "C" int gd_diag_static(const double* ug, const double* vg, int nlev, const double* psg,
                              const double* dlnpsdt, const double* gauwts, int nlat, int nlon, double* out4,
                              void* stream) {
  if (!ug || !vg || !psg || !dlnpsdt || !gauwts || !out4) return GD_ERR_ARG;
  if (nlev < 1 || nlon < 1 || nlat < 1) return GD_ERR_ARG;
  if (nlat > GD_DIAG_STATIC_MAX_NLAT) return GD_ERR_ARG;
  double* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc != GD_OK) return rc;
  try {
    gd::launch_diag<double>(ug, vg, nlev, psg, dlnpsdt, gauwts, nlat, nlon, scratch, out4,
                            static_cast<cudaStream_t>(stream));
  } catch (const std::exception&) {
    return GD_ERR_CUDA;
  }
  return GD_OK;
}

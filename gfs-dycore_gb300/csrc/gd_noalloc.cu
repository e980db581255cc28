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
// device current, on the first call made on it.  The address belongs to the
// device's CUDA context: a cudaDeviceReset in the host process destroys that
// context, and the next context loads the module again, possibly elsewhere.
// So the cached address is stored with the unique id of the context it was
// looked up in (cuCtxGetId, never reused within a process), and a call made
// under a different context looks it up again.  All calls share the array
// and it keeps the last call's contents; each call overwrites every entry it
// reads, so nothing needs clearing, but calls that overlap on the GPU
// (different streams or threads at once) race on it.
#include <cudaTypedefs.h>

#include <mutex>

#include "../../include/gd_api.h"
#include "gd_grid.cuh"

namespace {

static __device__ __align__(256) double g_diag_scratch[4 * GD_DIAG_STATIC_MAX_NLAT];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {nullptr};
unsigned long long g_scratch_ctx[kMaxDevices] = {0};  // id of the context the address belongs to

// unique id of the context current on this thread (0 if none is current
// yet or the id cannot be read)
unsigned long long current_context_id() {
  static PFN_cuCtxGetCurrent_v4000 get_cur = nullptr;
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_cur = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(p);
  });
  if (!get_cur || !get_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_cur(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// device address of g_diag_scratch on the current device, looked up on the
// first call under each context of the device
int scratch_for_current_device(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GD_ERR_CUDA;
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev] || ctx == 0 || ctx != g_scratch_ctx[dev]) {
    // the lookup makes the runtime's context current if none was; the id is
    // read after it (an id of 0 means: look up again on the next call)
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_diag_scratch) != cudaSuccess || !p) return GD_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<double*>(p);
    g_scratch_ctx[dev] = current_context_id();
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

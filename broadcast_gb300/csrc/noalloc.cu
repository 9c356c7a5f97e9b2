// Allocation-free variant of the DNC5 residual (bcg_flux_num_dnc5_2d_noalloc).
//
// Some callers cannot let a library allocate device memory at call time: a
// host framework whose caching allocator has already reserved the GPU's
// memory, a solver that must run inside a fixed device-memory budget and may
// not fail with out-of-memory part-way through, or a latency-sensitive loop
// that cannot afford cudaMalloc's implicit device synchronisation.  This
// entry point serves them: it takes device arrays only (no host staging), and
// its working storage is the file-scope device array below, reserved when the
// library's module is loaded on a GPU and held by that GPU until the process
// exits.  Nothing here calls cudaMalloc, cudaFree or any allocating routine.
//
// Limits and sharing rules:
//  - the scratch holds kNoAllocScratchDoubles doubles (32 MiB); a grid needs
//    49*(im+2gh)*(jm+2gh) + 10*(im+1)*(jm+1) of them (e.g. 256 x 256 or
//    400 x 150 fit), larger grids are rejected with BCG_ERR_ARG;
//  - every call on a device uses the same array, which keeps the previous
//    call's contents.  The residual kernels write every scratch entry they
//    read earlier in the same call, so nothing needs clearing between calls;
//  - calls whose kernels overlap on the GPU (different streams, or host
//    threads sharing a device) race on the array: serialise them.
//  - the first call on a device looks up the array's device address for that
//    device (cudaGetSymbolAddress with the device current); make that first
//    call before any stream capture.
#include <cuda_runtime.h>
#include <mutex>
#include "residual.h"
#include "runtime.h"

namespace {

constexpr size_t kNoAllocScratchDoubles = (size_t)4 << 20;  // 4 Mi doubles = 32 MiB
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_addr[kMaxDevices] = {nullptr};

// device address of the scratch for the current device (looked up once)
int scratch_address(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return bcg::fail_cuda("flux_num_dnc5_2d_noalloc: cudaGetDevice", e);
  if (dev < 0 || dev >= kMaxDevices) return bcg::fail_arg("flux_num_dnc5_2d_noalloc: device index out of range");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return bcg::fail_cuda("flux_num_dnc5_2d_noalloc: cudaGetSymbolAddress", e);
    g_addr[dev] = (double*)p;
  }
  *out = g_addr[dev];
  return bcg::BCG_OK;
}

// the array is in device memory of the current device (managed memory is
// reachable from every device)
bool on_current_device(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
  if (a.type == cudaMemoryTypeManaged) return true;
  if (a.type != cudaMemoryTypeDevice) return false;
  int dev = -1;
  return cudaGetDevice(&dev) == cudaSuccess && a.device == dev;
}

}  // namespace

extern "C" {

// Same arguments and result as bcg_flux_num_dnc5_2d; every array must be a
// device pointer.  Queued on the library stream; returns without waiting.
int bcg_flux_num_dnc5_2d_noalloc(double* residu, const double* w, const double* x0, const double* y0,
                                 const double* nx, const double* ny, const double* xc, const double* yc,
                                 const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                                 double gam, double rgaz, double cs, double muref, double tref, double s_suth,
                                 double k2, double k4, int im, int jm) {
  using namespace bcg;
  (void)x0; (void)y0; (void)xc; (void)yc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail_arg("flux_num_dnc5_2d_noalloc: no CUDA device"), BCG_ERR_NODEV;
  }
  if (gh != 3 || im < 6 || jm < 6) return fail_arg("flux_num_dnc5_2d_noalloc: need gh == 3 and im, jm >= 6");
  const size_t need = residual_scratch_doubles(im, jm, gh, 0);
  if (need > kNoAllocScratchDoubles)
    return fail_arg("flux_num_dnc5_2d_noalloc: grid too large for the fixed 32 MiB scratch "
                    "(needs 49*(im+6)*(jm+6) + 10*(im+1)*(jm+1) <= 4194304 doubles)");
  const void* arrays[] = {residu, w, nx, ny, vol, volf};
  for (const void* a : arrays)
    if (!on_current_device(a))
      return fail_arg("flux_num_dnc5_2d_noalloc: every array must be a device pointer on the current device");
  double* scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc != BCG_OK) return rc;
  ResidualArgs a{};
  a.im = im; a.jm = jm; a.gh = gh; a.ndir = 0;
  a.phys = Phys{cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4};
  a.w = w; a.nx = nx; a.ny = ny; a.vol = vol; a.volf = volf;
  a.res = residu;
  a.dstride = (size_t)(im + 2 * gh) * (jm + 2 * gh) * 5;
  a.scratch = scratch;
  cudaError_t e = run_residual(a, current_stream());
  if (e != cudaSuccess) return fail_cuda("flux_num_dnc5_2d_noalloc", e);
  return BCG_OK;
}

}  // extern "C"

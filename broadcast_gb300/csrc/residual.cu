// DNC5 residual and fused residual + JVP kernels for sm_103a.
//
// Reference: srcfv/prepro/flux_num_dnc5.f90 (primal), the Tapenade tangent
// srcfv/tangent/flux_num_dnc5_d.f90 (S = DK<K> here).
//
// GB300 note: the stencil is bound by the FP64 pipe, not by HBM, so every
// cell primitive, cell gradient and face flux is computed exactly once and
// parked in HBM scratch (L2-resident for the grid sizes of interest); the
// memory traffic this costs is far below the bandwidth roof.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include "residual_impl.cuh"

namespace bcg {

namespace {
// count of nonzero i-face ny and j-face nx components (the planes ny(:,:,1)
// and nx(:,:,2) of the padded node set)
__global__ void k_rect_count(const double* __restrict__ nx, const double* __restrict__ ny, size_t nn,
                             unsigned* __restrict__ count) {
  unsigned bad = 0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += (size_t)gridDim.x * blockDim.x)
    bad |= (ny[k] != 0.0) | (nx[nn + k] != 0.0);
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicAdd(count, 1u);
}

__device__ unsigned g_rect_count;  // one per device
std::mutex g_rect_mu;
std::map<std::tuple<int, const double*, const double*, int, int, int>, bool> g_curvilinear;  // remembered false results
}  // namespace

bool face_rectilinear_host(const double* nx, const double* ny, int im, int jm, int gh) {
  const size_t nn = (size_t)(im + 2 * gh + 1) * (jm + 2 * gh + 1);
  for (size_t k = 0; k < nn; ++k)
    if (ny[k] != 0.0 || nx[nn + k] != 0.0) return false;
  return true;
}

bool face_rectilinear_device(const double* nx, const double* ny, int im, int jm, int gh, cudaStream_t st) {
  const size_t nn = (size_t)(im + 2 * gh + 1) * (jm + 2 * gh + 1);
  std::lock_guard<std::mutex> lk(g_rect_mu);
  unsigned* count = nullptr;
  if (cudaGetSymbolAddress((void**)&count, g_rect_count) != cudaSuccess) { cudaGetLastError(); return false; }
  unsigned h = 1;
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned), st);
  const unsigned nb = (unsigned)std::min<size_t>((nn + 255) / 256, 1024);
  if (e == cudaSuccess) {
    k_rect_count<<<nb, 256, 0, st>>>(nx, ny, nn, count);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, count, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { cudaGetLastError(); return false; }
  return h == 0;
}

bool face_rectilinear(const double* nx, const double* ny, int im, int jm, int gh, cudaStream_t st) {
  cudaPointerAttributes at;
  const bool dev = cudaPointerGetAttributes(&at, nx) == cudaSuccess &&
                   (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged);
  cudaGetLastError();
  if (!dev) return face_rectilinear_host(nx, ny, im, jm, gh);
  // a stream being captured into a graph cannot wait for the check: the general kernel
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) { cudaGetLastError(); return false; }
  if (cap != cudaStreamCaptureStatusNone) return false;
  int d = 0;
  cudaGetDevice(&d);
  const auto key = std::make_tuple(d, nx, ny, im, jm, gh);
  {
    std::lock_guard<std::mutex> lk(g_rect_mu);
    if (g_curvilinear.count(key)) return false;
  }
  const bool r = face_rectilinear_device(nx, ny, im, jm, gh, st);
  if (!r) {
    std::lock_guard<std::mutex> lk(g_rect_mu);
    if (g_curvilinear.size() > 4096) g_curvilinear.clear();
    g_curvilinear[key] = true;
  }
  return r;
}

void launch_primal_passes(const Ext& e, const Coef& c, const double* w, double* pr, double* gr, const double* nx,
                          const double* ny, const double* vol, cudaStream_t st) {
  const int B = 256;
  const GroupStride gs{0, 0};
  k_prim<double><<<(unsigned)((e.np + B - 1) / B), B, 0, st>>>(e, c, State<double>{w}, Scratch<double>{pr, e.np}, gs);
  if (c.k2 != 0.0)
    k_grad<double><<<(unsigned)((e.im * e.jm + B - 1) / B), B, 0, st>>>(e, c, Scratch<double>{pr, e.np},
                                                                        Scratch<double>{gr, e.np}, nx, ny, vol, gs);
}

size_t residual_scratch_doubles(int im, int jm, int gh, int ndir) {
  const Ext e = make_ext(im, jm, gh);
  const size_t nn = (size_t)(im + 1) * (jm + 1);
  return (size_t)(ndir + 1) * ((size_t)(F_NPRIM + S_NSENS + Q_NQ) * e.np + 10 * nn);
}

cudaError_t run_residual(const ResidualArgs& a, cudaStream_t st) {
  if (a.order != 0 && a.order != 5) return run_residual_scheme(a, st);
  switch (a.ndir) {
    case 0: return run_residual_t<double, 3>(a, st);
    case 1: return run_residual_t<DK<1>, 3>(a, st);
    case 2: return run_residual_t<DK<2>, 3>(a, st);
    case 4: return run_residual_t<DK<4>, 3>(a, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace bcg

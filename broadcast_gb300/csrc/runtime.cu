// Library runtime: stream selection, error recording, device pools, staging.
#include "runtime.h"
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

namespace bcg {

namespace {
std::mutex g_mu;
cudaStream_t g_stream = nullptr;
thread_local std::string g_err;
constexpr int kMaxDev = 64;
struct Pool { void* p = nullptr; size_t bytes = 0; };
Pool g_pool[kMaxDev][POOL_COUNT];
}  // namespace

cudaStream_t current_stream() { return g_stream; }
void set_stream(cudaStream_t s) { g_stream = s; }

int fail_cuda(const char* where, cudaError_t e) {
  char buf[256];
  std::snprintf(buf, sizeof buf, "%s: %s", where, cudaGetErrorString(e));
  g_err = buf;
  return BCG_ERR_CUDA;
}
int fail_arg(const char* msg) { g_err = msg; return BCG_ERR_ARG; }
const char* last_error() { return g_err.c_str(); }

void* pool_get(PoolKind k, size_t bytes) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  Pool& p = g_pool[dev][k];
  if (bytes == 0) bytes = 256;
  if (p.bytes >= bytes) return p.p;
  // the previous buffer may still be read by queued work on the stream
  if (p.p) { cudaStreamSynchronize(g_stream); cudaFree(p.p); p.p = nullptr; p.bytes = 0; }
  const size_t want = bytes + bytes / 4;
  if (cudaMalloc(&p.p, want) != cudaSuccess) {
    cudaGetLastError();
    if (cudaMalloc(&p.p, bytes) != cudaSuccess) { cudaGetLastError(); p.p = nullptr; return nullptr; }
    p.bytes = bytes;
    return p.p;
  }
  p.bytes = want;
  return p.p;
}

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int Stager::add(const void* p, size_t bytes, bool inp, bool outp) {
  Item it{p, bytes, 0, inp, outp, false};
  if (p && !is_device_ptr(p)) {
    it.staged = true;
    it.off = total_;
    total_ += (bytes + 255) & ~(size_t)255;
    ++nstaged_;
  }
  items_.push_back(it);
  ptrs_.push_back(const_cast<void*>(p));
  return (int)items_.size() - 1;
}

int Stager::out_interior(void* p, int ni, int nj, int nplanes, int gh, int im, int jm) {
  const int h = add(p, (size_t)ni * nj * nplanes * sizeof(double), false, true);
  Item& it = items_[h];
  it.ni = ni; it.nj = nj; it.nplanes = nplanes; it.gh = gh; it.im = im; it.jm = jm;
  return h;
}

int Stager::commit() {
  if (nstaged_ == 0) return BCG_OK;
  char* base = (char*)pool_get(POOL_STAGE, total_);
  if (!base) return fail_cuda("staging pool", cudaErrorMemoryAllocation), BCG_ERR_NOMEM;
  for (size_t k = 0; k < items_.size(); ++k) {
    Item& it = items_[k];
    if (!it.staged) continue;
    ptrs_[k] = base + it.off;
    if (it.inp) {
      cudaError_t e = cudaMemcpyAsync(ptrs_[k], it.host, it.bytes, cudaMemcpyHostToDevice, st_);
      if (e != cudaSuccess) return fail_cuda("host to device copy", e);
      h2d_ += it.bytes;
    }
  }
  return BCG_OK;
}

// the interiors of nplanes padded (ni, nj) planes, as one pitched 3D copy
// (rows of im doubles, jm rows per plane); the ghosts of dst stay untouched
cudaError_t copy_interior_planes(double* dst, const double* src, int ni, int nj, int nplanes, int gh, int im, int jm,
                                 cudaMemcpyKind kind, cudaStream_t st) {
  cudaMemcpy3DParms p = {};
  const size_t pitch = (size_t)ni * sizeof(double);
  p.srcPtr = make_cudaPitchedPtr(const_cast<double*>(src), pitch, (size_t)ni, (size_t)nj);
  p.dstPtr = make_cudaPitchedPtr(dst, pitch, (size_t)ni, (size_t)nj);
  p.srcPos = make_cudaPos((size_t)gh * sizeof(double), (size_t)gh, 0);
  p.dstPos = p.srcPos;
  p.extent = make_cudaExtent((size_t)im * sizeof(double), (size_t)jm, (size_t)nplanes);
  p.kind = kind;
  return cudaMemcpy3DAsync(&p, st);
}

int Stager::finish() {
  if (nstaged_ == 0) return BCG_OK;
  for (size_t k = 0; k < items_.size(); ++k) {
    Item& it = items_[k];
    if (!it.staged || !it.outp) continue;
    if (it.nplanes > 0) {
      cudaError_t e = copy_interior_planes((double*)const_cast<void*>(it.host), (const double*)ptrs_[k], it.ni, it.nj,
                                           it.nplanes, it.gh, it.im, it.jm, cudaMemcpyDeviceToHost, st_);
      if (e != cudaSuccess) return fail_cuda("device to host copy", e);
      d2h_ += (size_t)it.nplanes * it.im * it.jm * sizeof(double);
      continue;
    }
    cudaError_t e = cudaMemcpyAsync(const_cast<void*>(it.host), ptrs_[k], it.bytes, cudaMemcpyDeviceToHost, st_);
    if (e != cudaSuccess) return fail_cuda("device to host copy", e);
    d2h_ += it.bytes;
  }
  cudaError_t e = cudaStreamSynchronize(st_);
  if (e != cudaSuccess) return fail_cuda("stream synchronize", e);
  return BCG_OK;
}

}  // namespace bcg

// Library runtime: current stream, per-device scratch/staging pools and the
// host-or-device argument staging used by the C-ABI entry points.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <vector>

namespace bcg {

// Error codes returned by every bcg_* entry point.
enum {
  BCG_OK = 0,
  BCG_ERR_ARG = -1,     // bad extents, unknown loc string, unsupported size
  BCG_ERR_CUDA = -2,    // a CUDA call failed (see bcg_last_error_string)
  BCG_ERR_NOMEM = -3,   // device allocation failed
  BCG_ERR_NODEV = -4,   // no usable CUDA device
  BCG_ERR_SINGULAR = -5,  // the linear solve met a zero pivot
};

cudaStream_t current_stream();
// the interiors of nplanes padded (ni, nj) planes in one pitched 3D copy
cudaError_t copy_interior_planes(double* dst, const double* src, int ni, int nj, int nplanes, int gh, int im, int jm,
                                 cudaMemcpyKind kind, cudaStream_t st);
void set_stream(cudaStream_t s);
int fail_cuda(const char* where, cudaError_t e);   // records and returns BCG_ERR_CUDA
int fail_arg(const char* msg);                     // records and returns BCG_ERR_ARG
const char* last_error();

// Grow-only device buffer per device and purpose.  Calls are serialised on the
// library stream, so one buffer per purpose is reused across calls.
enum PoolKind { POOL_SCRATCH = 0, POOL_STAGE = 1, POOL_AUX = 2, POOL_STAGE_OUT = 3, POOL_COUNT = 4 };
void* pool_get(PoolKind k, size_t bytes);

bool is_device_ptr(const void* p);

// Staging of host arrays.  Device pointers pass through untouched; host arrays
// are copied into the staging pool before the kernels (inputs and in-out
// arrays) and back after them (outputs and in-out arrays).
class Stager {
 public:
  explicit Stager(cudaStream_t st) : st_(st) {}
  int in(const void* p, size_t bytes) { return add(p, bytes, true, false); }
  int inout(void* p, size_t bytes) { return add(p, bytes, true, true); }
  int out(void* p, size_t bytes) { return add(p, bytes, false, true); }
  // output whose kernels write only the interior of nplanes padded planes of
  // (ni, nj) doubles: nothing is copied in and only the interior
  // [gh, gh+im) x [gh, gh+jm) of each plane is copied back, so the caller's
  // ghost values stay untouched (the reference's intent(inout) semantics)
  int out_interior(void* p, int ni, int nj, int nplanes, int gh, int im, int jm);
  int commit();                           // BCG_OK or an error code
  template <class T> T* dev(int h) const { return (T*)ptrs_[h]; }
  int finish();                           // copy outputs back; sync if anything was staged
  bool staged() const { return nstaged_ > 0; }
  size_t h2d_bytes() const { return h2d_; }
  size_t d2h_bytes() const { return d2h_; }

 private:
  struct Item {
    const void* host; size_t bytes, off; bool inp, outp, staged;
    int ni = 0, nj = 0, nplanes = 0, gh = 0, im = 0, jm = 0;  // interior-only output when nplanes > 0
  };
  int add(const void* p, size_t bytes, bool inp, bool outp);
  cudaStream_t st_;
  std::vector<Item> items_;
  std::vector<void*> ptrs_;
  size_t total_ = 0, h2d_ = 0, d2h_ = 0;
  int nstaged_ = 0;
};

}  // namespace bcg

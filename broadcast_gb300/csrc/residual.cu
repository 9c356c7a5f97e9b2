// DNC5 residual and fused residual + JVP kernels for sm_103a.
//
// Reference: srcfv/prepro/flux_num_dnc5.f90 (primal), the Tapenade tangent
// srcfv/tangent/flux_num_dnc5_d.f90 (S = DK<K> here).
//
// GB300 note: the stencil is bound by the FP64 pipe, not by HBM, so every
// cell primitive, cell gradient and face flux is computed exactly once and
// parked in HBM scratch (L2-resident for the grid sizes of interest); the
// memory traffic this costs is far below the bandwidth roof.
#include "passes.cuh"
#include "residual.h"

namespace bcg {

// Direction groups: a launch may cover several groups of K directions, group
// g = blockIdx.y reading tangents g*K .. g*K+K-1 and owning its own scratch.
struct GroupStride {
  size_t tangent;  // doubles between the tangent planes of consecutive groups (K * dstride)
  size_t scratch;  // doubles between the scratch blocks of consecutive groups
};
BCG_HD void shift_state(State<double>&, size_t) {}
template <int K> BCG_HD void shift_state(State<DK<K>>& w, size_t off) { w.d += off; }
template <class S> BCG_HD void shift_scratch(Scratch<S>& s, size_t off) { s.p += off; }


// ---------------------------------------------------------------------------
// single-grid kernels: one thread per element, blockIdx.y = direction group
template <class S>
__global__ void __launch_bounds__(256) k_prim(Ext e, Coef c, State<S> w, Scratch<S> pr, GroupStride gs) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= e.np) return;
  shift_state(w, blockIdx.y * gs.tangent);
  shift_scratch(pr, blockIdx.y * gs.scratch);
  prim_cell<S>(e, c, w, pr, q);
}

template <class S>
__global__ void __launch_bounds__(256) k_qrows(Ext e, Scratch<S> pr, Scratch<S> qr, GroupStride gs) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= e.np) return;
  shift_scratch(pr, blockIdx.y * gs.scratch);
  shift_scratch(qr, blockIdx.y * gs.scratch);
  qrows_cell<S>(e, pr, qr, q);
}

template <class S>
__global__ void __launch_bounds__(256) k_vpts(Ext e, Scratch<S> qr, GroupStride gs) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= e.np) return;
  shift_scratch(qr, blockIdx.y * gs.scratch);
  vpts_cell<S>(e, qr, q);
}

template <class S>
__global__ void __launch_bounds__(256) k_grad(Ext e, Coef c, Scratch<S> pr, Scratch<S> gr, const double* __restrict__ nx,
                                              const double* __restrict__ ny, const double* __restrict__ vol,
                                              GroupStride gs) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= e.im * e.jm) return;
  shift_scratch(pr, blockIdx.y * gs.scratch);
  shift_scratch(gr, blockIdx.y * gs.scratch);
  grad_cell<S>(e, c, pr, gr, nx, ny, vol, t);
}

template <class S>
__global__ void __launch_bounds__(128) k_faces(FaceCtx<S> fc0, Scratch<S> hn, GroupStride gs) {
  const Ext& e = fc0.e;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (e.im + 1) * (e.jm + 1)) return;
  FaceCtx<S> fc = fc0;
  shift_state(fc.w, blockIdx.y * gs.tangent);
  shift_scratch(fc.pr, blockIdx.y * gs.scratch);
  shift_scratch(fc.gr, blockIdx.y * gs.scratch);
  shift_scratch(fc.qr, blockIdx.y * gs.scratch);
  shift_scratch(hn, blockIdx.y * gs.scratch);
  face_node<S>(fc, hn, t);
}

template <class S>
__global__ void __launch_bounds__(256) k_balance(Ext e, Scratch<S> hn, double* __restrict__ res, double* __restrict__ resd,
                                                 size_t dstride, GroupStride gs) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= e.im * e.jm) return;
  shift_scratch(hn, blockIdx.y * gs.scratch);
  if (blockIdx.y > 0) { res = nullptr; resd += blockIdx.y * gs.tangent; }
  balance_cell<S>(e, hn, res, resd, dstride, t);
}

// ---------------------------------------------------------------------------
template <class S>
static cudaError_t run_residual_t(const ResidualArgs& a, cudaStream_t st) {
  const Ext e = make_ext(a.im, a.jm, a.gh);
  Coef c = make_coef(a.phys);
  c.wall = a.nowall ? 0 : 1;
  constexpr int NP = NDir<S>::value + 1;
  const size_t nn = (size_t)(a.im + 1) * (a.jm + 1);
  Scratch<S> pr{a.scratch, e.np};
  Scratch<S> gr{a.scratch + (size_t)F_NPRIM * NP * e.np, e.np};
  Scratch<S> qr{a.scratch + (size_t)(F_NPRIM + G_NGRAD) * NP * e.np, e.np};
  Scratch<S> hn{a.scratch + (size_t)(F_NPRIM + G_NGRAD + Q_NQ) * NP * e.np, nn};
  State<S> w;
  if constexpr (NP == 1) w = State<S>{a.w};
  else w = State<S>{a.w, a.wd, a.dstride};
  const unsigned ng = a.ngroup > 1 ? (unsigned)a.ngroup : 1u;
  if (NP == 1 && ng > 1) return cudaErrorInvalidValue;
  const GroupStride gs{(size_t)NDir<S>::value * a.dstride, residual_scratch_doubles(a.im, a.jm, a.gh, NDir<S>::value)};
  const int B = 256;
  k_prim<S><<<dim3((unsigned)((e.np + B - 1) / B), ng), B, 0, st>>>(e, c, w, pr, gs);
  if (c.k2 != 0.0)
    k_grad<S><<<dim3((unsigned)((a.im * a.jm + B - 1) / B), ng), B, 0, st>>>(e, c, pr, gr, a.nx, a.ny, a.vol, gs);
  k_qrows<S><<<dim3((unsigned)((e.np + B - 1) / B), ng), B, 0, st>>>(e, pr, qr, gs);
  k_vpts<S><<<dim3((unsigned)((e.np + B - 1) / B), ng), B, 0, st>>>(e, qr, gs);
  FaceCtx<S> fc{e, c, w, pr, gr, qr, a.nx, a.ny, a.vol, a.volf};
  const int BF = 128;
  k_faces<S><<<dim3((unsigned)((nn + BF - 1) / BF), ng), BF, 0, st>>>(fc, hn, gs);
  k_balance<S><<<dim3((unsigned)((a.im * a.jm + B - 1) / B), ng), B, 0, st>>>(e, hn, a.res, a.resd, a.dstride, gs);
  return cudaGetLastError();
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
  return (size_t)(ndir + 1) * ((size_t)(F_NPRIM + G_NGRAD + Q_NQ) * e.np + 10 * nn);
}

cudaError_t run_residual(const ResidualArgs& a, cudaStream_t st) {
  switch (a.ndir) {
    case 0: return run_residual_t<double>(a, st);
    case 1: return run_residual_t<DK<1>>(a, st);
    case 2: return run_residual_t<DK<2>>(a, st);
    case 4: return run_residual_t<DK<4>>(a, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace bcg

// Kernels of the DNC residual and fused residual + JVP passes, templated on
// the scalar type S and the scheme's point pairs R; included by residual.cu
// (DNC5) and schemes.cu (DNC3, DNC7, DNC9), which instantiate them.
//
// Reference: srcfv/prepro/flux_num_dnc5.f90 (primal), the Tapenade tangent
// srcfv/tangent/flux_num_dnc5_d.f90 (S = DK<K> here), and the DNC3/7/9 forms
// srcfv/prepro/flux_num_dnc{3,7,9}.f90, srcfv/tangent/flux_num_dnc{3,7,9}_d.f90.
#pragma once
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

template <class S, int R = 3>
__global__ void __launch_bounds__(256) k_grad(Ext e, Coef c, Scratch<S> pr, Scratch<S> gr, const double* __restrict__ nx,
                                              const double* __restrict__ ny, const double* __restrict__ vol,
                                              GroupStride gs) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= e.im * e.jm) return;
  shift_scratch(pr, blockIdx.y * gs.scratch);
  shift_scratch(gr, blockIdx.y * gs.scratch);
  grad_cell<S, R>(e, c, pr, gr, nx, ny, vol, t);
}

template <class S, int R = 3>
__global__ void __launch_bounds__(256) k_sensor(Ext e, Coef c, Scratch<S> pr, Scratch<S> sg,
                                                const double* __restrict__ nx, const double* __restrict__ ny,
                                                const double* __restrict__ vol, GroupStride gs) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (e.im + 2) * (e.jm + 2)) return;
  shift_scratch(pr, blockIdx.y * gs.scratch);
  shift_scratch(sg, blockIdx.y * gs.scratch);
  sensor_cell<S, R>(e, c, pr, sg, nx, ny, vol, t);
}

template <class S, int R = 3, bool RECT = false>
__global__ void __launch_bounds__(128) k_faces(FaceCtx<S, R, RECT> fc0, Scratch<S> hn, GroupStride gs) {
  const Ext& e = fc0.e;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (e.im + 1) * (e.jm + 1)) return;
  FaceCtx<S, R, RECT> fc = fc0;
  shift_state(fc.w, blockIdx.y * gs.tangent);
  shift_scratch(fc.pr, blockIdx.y * gs.scratch);
  shift_scratch(fc.gr, blockIdx.y * gs.scratch);
  shift_scratch(fc.qr, blockIdx.y * gs.scratch);
  shift_scratch(hn, blockIdx.y * gs.scratch);
  face_node<S, R, RECT>(fc, hn, t);
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
// R: point pairs of the DNC scheme (3: DNC5; 2, 4, 5: DNC3, 7, 9)
template <class S, int R>
static cudaError_t run_residual_t(const ResidualArgs& a, cudaStream_t st) {
  const Ext e = make_ext(a.im, a.jm, a.gh);
  Coef c = make_coef(a.phys, 2 * R - 1);
  c.wall = a.nowall ? 0 : 1;
  constexpr int NP = NDir<S>::value + 1;
  const size_t nn = (size_t)(a.im + 1) * (a.jm + 1);
  Scratch<S> pr{a.scratch, e.np};
  Scratch<S> gr{a.scratch + (size_t)F_NPRIM * NP * e.np, e.np};
  Scratch<S> qr{a.scratch + (size_t)(F_NPRIM + S_NSENS) * NP * e.np, e.np};
  Scratch<S> hn{a.scratch + (size_t)(F_NPRIM + S_NSENS + Q_NQ) * NP * e.np, nn};
  State<S> w;
  if constexpr (NP == 1) w = State<S>{a.w};
  else w = State<S>{a.w, a.wd, a.dstride};
  const unsigned ng = a.ngroup > 1 ? (unsigned)a.ngroup : 1u;
  if (NP == 1 && ng > 1) return cudaErrorInvalidValue;
  const GroupStride gs{(size_t)NDir<S>::value * a.dstride, residual_scratch_doubles(a.im, a.jm, a.gh, NDir<S>::value)};
  const int B = 256;
  k_prim<S><<<dim3((unsigned)((e.np + B - 1) / B), ng), B, 0, st>>>(e, c, w, pr, gs);
  if (c.k2 != 0.0)
    k_sensor<S, R><<<dim3((unsigned)(((a.im + 2) * (a.jm + 2) + B - 1) / B), ng), B, 0, st>>>(e, c, pr, gr, a.nx,
                                                                                            a.ny, a.vol, gs);
  if (!FaceCtx<S, R>::ALL_O2) {  // the 4th-order viscous fluxes' interpolation rows
    k_qrows<S><<<dim3((unsigned)((e.np + B - 1) / B), ng), B, 0, st>>>(e, pr, qr, gs);
    k_vpts<S><<<dim3((unsigned)((e.np + B - 1) / B), ng), B, 0, st>>>(e, qr, gs);
  }
  const int BF = 128;
  const dim3 gf((unsigned)((nn + BF - 1) / BF), ng);
  if constexpr (R == 3) {  // DNC5 on a rectilinear grid: the face kernel without the zero metric products
    if (a.rect) {
      FaceCtx<S, R, true> fc{e, c, w, pr, gr, qr, a.nx, a.ny, a.vol, a.volf};
      k_faces<S, R, true><<<gf, BF, 0, st>>>(fc, hn, gs);
    } else {
      FaceCtx<S, R> fc{e, c, w, pr, gr, qr, a.nx, a.ny, a.vol, a.volf};
      k_faces<S, R><<<gf, BF, 0, st>>>(fc, hn, gs);
    }
  } else {
    FaceCtx<S, R> fc{e, c, w, pr, gr, qr, a.nx, a.ny, a.vol, a.volf};
    k_faces<S, R><<<gf, BF, 0, st>>>(fc, hn, gs);
  }
  k_balance<S><<<dim3((unsigned)((a.im * a.jm + B - 1) / B), ng), B, 0, st>>>(e, hn, a.res, a.resd, a.dstride, gs);
  return cudaGetLastError();
}

}  // namespace bcg

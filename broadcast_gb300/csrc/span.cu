// Spanwise operators of the DNC5 scheme for sm_103a: Dz (coefficient of i*beta)
// and Dzz (coefficient of -beta^2) of a perturbation exp(i beta z) about a 2-D
// base flow.
//
// Reference: srcfv/dz/coeffs_5p_dz.F90:10-174 and coeffs_5p_dz2.F90:10-147.
// Both evaluate  out(i,j,e) = sum_k coeffs(i,j,e,k) * (d func_k(i,j,e)/dw . wd)
// on the interior, with base-flow coefficients (dz/coeffs_dz.F:1-97,
// dz/coeffs_dz2.F) and auxiliary functions (matrix_dz/function_dz.F,
// matrix_dz2/function_dz2.F) whose tangents the reference takes from Tapenade
// (dz/function_5p_dz_d.f90, function_5p_dz2_d.f90).  Here a thread owns one
// interior cell and evaluates the functions on DK<K> numbers: the primitives
// (rhs/primvisc.F) of its 5-point cross stencil, the 4th-order gradients of
// u, v, w and mu (rhs/gradop_5pi.F, gradop_5pj.F, geom/dxdy.F, gradient.F),
// then the coefficient sums.  Only the interior of `out` is written.
#include "span.h"

namespace bcg {

namespace {

struct PrimK {
  template <int K>
  BCG_HD static void at(const Coef& c, const State<DK<K>>& w, size_t q, size_t n, DK<K>& u, DK<K>& v, DK<K>& ww,
                        DK<K>& t, DK<K>& p, DK<K>& mu) {
    const DK<K> ro = w(q), ru = w(q + n), rv = w(q + 2 * n), rw = w(q + 3 * n), re = w(q + 4 * n);
    const DK<K> rom1 = 1.0 / ro;
    u = ru * rom1; v = rv * rom1; ww = rw * rom1;
    const DK<K> ec = 0.5 * (u * u + v * v + ww * ww);
    const DK<K> eloc = (re - ec * ro) * rom1;
    t = eloc * c.cvm1;
    p = c.gam1 * ro * eloc;
    mu = c.betas / (t + c.s_suth) * sqrt_t(t) * t;
  }
};

template <int K>
__global__ void __launch_bounds__(128) k_dz(Ext e, Coef c, State<DK<K>> w, const double* __restrict__ nx,
                                            const double* __restrict__ ny, const double* __restrict__ vol,
                                            double* __restrict__ out, size_t dstride) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= e.im * e.jm) return;
  const int i = 1 + t % e.im, j = 1 + t / e.im;
  const size_t n = e.np;
  const size_t q = e.cidx(i, j);
  const int di = 1, dj = e.ni;
  // primitives of the cross stencil: index 0 = centre, 1..4 = i-2, i-1, i+1, i+2, 5..8 = same in j
  DK<K> u0, v0, w0, t0, p0, mu0;
  PrimK::at<K>(c, w, q, n, u0, v0, w0, t0, p0, mu0);
  const int off[8] = {-2 * di, -di, di, 2 * di, -2 * dj, -dj, dj, 2 * dj};
  DK<K> un[8], vn[8], wn[8];
  double mun[8];
#pragma unroll
  for (int s = 0; s < 8; ++s) {
    DK<K> tt, pp, mm;
    PrimK::at<K>(c, w, (size_t)((long long)q + off[s]), n, un[s], vn[s], wn[s], tt, pp, mm);
    mun[s] = mm.v;
  }
  const double b1 = 8.0 * (1.0 / 12.0), b2 = -(1.0 / 12.0);
  // gradop_5pi / gradop_5pj: b1 (f(+1) - f(-1)) + b2 (f(+2) - f(-2))
  const DK<K> gui = b1 * (un[2] - un[1]) + b2 * (un[3] - un[0]);
  const DK<K> gvi = b1 * (vn[2] - vn[1]) + b2 * (vn[3] - vn[0]);
  const DK<K> gwi = b1 * (wn[2] - wn[1]) + b2 * (wn[3] - wn[0]);
  const DK<K> guj = b1 * (un[6] - un[5]) + b2 * (un[7] - un[4]);
  const DK<K> gvj = b1 * (vn[6] - vn[5]) + b2 * (vn[7] - vn[4]);
  const DK<K> gwj = b1 * (wn[6] - wn[5]) + b2 * (wn[7] - wn[4]);
  const double gmui = b1 * (mun[2] - mun[1]) + b2 * (mun[3] - mun[0]);
  const double gmuj = b1 * (mun[6] - mun[5]) + b2 * (mun[7] - mun[4]);
  // geom/dxdy.F
  const size_t nn = e.nn();
  const double volm1 = 1.0 / __ldg(vol + q);
  const double dxm1 = 0.5 * (__ldg(nx + e.nidx(i, j)) + __ldg(nx + e.nidx(i + 1, j))) * volm1;
  const double dxm2 = 0.5 * (__ldg(nx + nn + e.nidx(i, j)) + __ldg(nx + nn + e.nidx(i, j + 1))) * volm1;
  const double dym1 = 0.5 * (__ldg(ny + e.nidx(i, j)) + __ldg(ny + e.nidx(i + 1, j))) * volm1;
  const double dym2 = 0.5 * (__ldg(ny + nn + e.nidx(i, j)) + __ldg(ny + nn + e.nidx(i, j + 1))) * volm1;
  const DK<K> gu1 = dxm1 * gui + dxm2 * guj;
  const DK<K> gv2 = dym1 * gvi + dym2 * gvj;
  const DK<K> gw1 = dxm1 * gwi + dxm2 * gwj;
  const DK<K> gw2 = dym1 * gwi + dym2 * gwj;
  const double gmu1 = dxm1 * gmui + dxm2 * gmuj, gmu2 = dym1 * gmui + dym2 * gmuj;
  // base-flow coefficients (coeffs_dz.F), non-zero entries only
  const double TWOTHIRD = 2.0 / 3.0;
  const double mu = mu0.v, vx = u0.v, vy = v0.v, vz = w0.v;
  const double c2_2 = TWOTHIRD * gmu1, c3_2 = TWOTHIRD * gmu2, c4_2 = -gmu1;
  const double c5_2 = TWOTHIRD * (gmu1 * vx + mu * gu1.v);
  const double c2_3 = TWOTHIRD * mu, c4_3 = -gmu2, c5_3 = TWOTHIRD * mu * vx;
  const double c4_4 = -mu, c5_4 = -(gmu1 * vz + mu * gw1.v);
  const double c5_5 = -(mu * vz);
  const double c5_6 = TWOTHIRD * (gmu2 * vy + mu * gv2.v);
  const double c5_7 = TWOTHIRD * mu * vy;
  const double c5_8 = -(gmu2 * vz + mu * gw2.v);
  const double c5_10 = -(mu * gw1.v), c5_11 = -vx, c5_12 = -(mu * gw2.v), c5_13 = -vy;
  const double c5_14 = TWOTHIRD * mu * (gu1.v + gv2.v);
  const double c5_15 = TWOTHIRD * vz * (gu1.v + gv2.v);
  const double c5_16 = TWOTHIRD * mu * vz;
  // auxiliary functions (function_dz.F) whose tangents enter the sums
  const DK<K> r2 = w(q + n), r3 = w(q + 2 * n), r4 = w(q + 3 * n), r5 = w(q + 4 * n);
  const DK<K> f0_2 = r2 * w0 - mu0 * gw1;
  const DK<K> f0_3 = r3 * w0 - mu0 * gw2;
  const DK<K> f0_4 = r4 * w0 + p0 + TWOTHIRD * mu0 * (gu1 + gv2);
  const DK<K> f0_5 = (r5 + p0) * w0;
  const DK<K> div = gu1 + gv2;
  const DK<K> f10 = mu0 * gw1, f12 = mu0 * gw2;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double* o = out + (size_t)k * dstride + q;
    o[0] = r4.d[k];
    o[n] = f0_2.d[k] + c2_2 * w0.d[k] + c2_3 * gw1.d[k];
    o[2 * n] = f0_3.d[k] + c3_2 * w0.d[k] + c2_3 * gw2.d[k];
    o[3 * n] = f0_4.d[k] + c4_2 * u0.d[k] + c4_3 * v0.d[k] + c4_4 * div.d[k];
    o[4 * n] = f0_5.d[k] + c5_2 * w0.d[k] + c5_3 * gw1.d[k] + c5_4 * u0.d[k] + c5_5 * gu1.d[k] + c5_6 * w0.d[k] +
               c5_7 * gw2.d[k] + c5_8 * v0.d[k] + c5_5 * gv2.d[k] + c5_10 * u0.d[k] + c5_11 * f10.d[k] +
               c5_12 * v0.d[k] + c5_13 * f12.d[k] + c5_14 * w0.d[k] + c5_15 * mu0.d[k] + c5_16 * div.d[k];
  }
}

template <int K>
__global__ void __launch_bounds__(128) k_dzz(Ext e, Coef c, double cpprandtl, State<DK<K>> w, double* __restrict__ out,
                                             size_t dstride) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= e.im * e.jm) return;
  const int i = 1 + t % e.im, j = 1 + t / e.im;
  const size_t n = e.np, q = e.cidx(i, j);
  DK<K> u, v, ww, tt, p, mu;
  PrimK::at<K>(c, w, q, n, u, v, ww, tt, p, mu);
  // coeffs_dz2.F: -mu (u, v, 4/3 w) and -mu cp/Pr T, -mu (u, v, 4/3 w) . (u, v, w)
  const double TWOTHIRD = 2.0 / 3.0;
  const double m = mu.v;
  const double c1 = -m, c4 = -(2.0 * TWOTHIRD * m), c5 = -(m * cpprandtl);
  const double c5u = -(m * u.v), c5v = -(m * v.v), c5w = -(2.0 * TWOTHIRD * m * ww.v);
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double* o = out + (size_t)k * dstride + q;
    o[0] = 0.0;
    o[n] = c1 * u.d[k];
    o[2 * n] = c1 * v.d[k];
    o[3 * n] = c4 * ww.d[k];
    o[4 * n] = c5 * tt.d[k] + c5u * u.d[k] + c5v * v.d[k] + c5w * ww.d[k];
  }
}

template <int K>
cudaError_t launch(const SpanArgs& a, cudaStream_t st) {
  const Ext e = make_ext(a.im, a.jm, a.gh);
  const Coef c = make_coef(a.phys);
  const State<DK<K>> w{a.w, a.wd, a.dstride};
  const int B = 128, nb = (a.im * a.jm + B - 1) / B;
  if (a.op == SPAN_DZ) k_dz<K><<<nb, B, 0, st>>>(e, c, w, a.nx, a.ny, a.vol, a.out, a.dstride);
  else k_dzz<K><<<nb, B, 0, st>>>(e, c, a.phys.cp / a.phys.prandtl, w, a.out, a.dstride);
  return cudaGetLastError();
}

}  // namespace

cudaError_t run_span(const SpanArgs& a, cudaStream_t st) {
  if (a.op != SPAN_DZ && a.op != SPAN_DZZ) return cudaErrorInvalidValue;
  switch (a.ndir) {
    case 1: return launch<1>(a, st);
    case 2: return launch<2>(a, st);
    case 4: return launch<4>(a, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace bcg

// C-ABI entry points of libbroadcast_gb300.so (declared in include/broadcast_gb300.h).
//
// Every array argument may be a host pointer (copied to and from the device
// around the call, which then completes before returning) or a device pointer
// (used in place; the call is queued on the library stream and returns at
// once).  Argument order and meaning follow the reference's f2py routines.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>
#include "bc.h"
#include "residual.h"
#include "runtime.h"
#include "assembly.h"
#include "adjoint.h"
#include "jacobian.h"
#include "span.h"
#include "batch.h"
#include "impli.h"
#include "bandlu.h"
#include "krylov.h"

using namespace bcg;

namespace {
inline bool dims_ok(int im, int jm, int gh) { return im >= 6 && jm >= 6 && gh == 3; }
inline size_t ncell(int im, int jm, int gh) { return (size_t)(im + 2 * gh) * (jm + 2 * gh); }
inline size_t nnode(int im, int jm, int gh) { return (size_t)(im + 2 * gh + 1) * (jm + 2 * gh + 1); }

int has_device() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) { cudaGetLastError(); return 0; }
  return 1;
}

// Streams of the pipelined host-array path (per device, created on first
// use, never destroyed): uploads, downloads, and two compute streams that
// alternate over the chunks.
struct CopyStreams { cudaStream_t in = nullptr, out = nullptr, comp[2] = {nullptr, nullptr}; };
int copy_streams(CopyStreams* cs) {
  static std::mutex mu;
  static std::map<int, CopyStreams> per_dev;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail_cuda("copy streams", e);
  std::lock_guard<std::mutex> lk(mu);
  CopyStreams& c = per_dev[dev];
  if (!c.in) {
    e = cudaStreamCreateWithFlags(&c.in, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c.out, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c.comp[0], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c.comp[1], cudaStreamNonBlocking);
    if (e != cudaSuccess) { c = CopyStreams{}; return fail_cuda("copy streams", e); }
  }
  *cs = c;
  return BCG_OK;
}

// device -> host copy of the interior of nplanes padded (ni, nj) planes
cudaError_t copy_interior_d2h(double* host, const double* dev, int ni, int nj, int nplanes, int gh, int im, int jm,
                              cudaStream_t st) {
  return copy_interior_planes(host, dev, ni, nj, nplanes, gh, im, jm, cudaMemcpyDeviceToHost, st);
}

// Host tangents and outputs of many directions: the directions run in up to
// eight chunks of whole 4-direction groups; chunk c's upload (copy stream in),
// its residual passes (compute stream c mod 2, with its own scratch) and its
// download (copy stream out) overlap the other chunks'.  Only the first
// chunk's upload and the last chunk's download are exposed, so more chunks
// shrink them; the two compute streams let a chunk's kernels fill the SMs the
// previous chunk's last partial waves leave idle.  Everything starts only after
// the library stream's earlier work, since the pool buffers may still be in
// use, and the library stream waits for the last download.
int residual_pipelined(ResidualArgs a, double* res, double* residud, const double* wd, int nd, cudaStream_t st) {
  const int im = a.im, jm = a.jm, gh = a.gh, ni = im + 2 * gh, nj = jm + 2 * gh;
  const size_t plane5 = (size_t)ni * nj * 5;
  CopyStreams cs;
  int rc = copy_streams(&cs);
  if (rc) return rc;
  constexpr int kMaxChunk = 8;
  const int ng = nd / 4;
  const int nch = std::max(1, std::min(kMaxChunk, ng));
  int bounds[kMaxChunk + 1];
  for (int c = 0; c < nch; ++c) bounds[c] = 4 * (int)((long long)ng * c / nch);
  bounds[nch] = nd;  // the last chunk also takes the 1-3 directions beyond the groups
  int gmax = 0;
  for (int c = 0; c < nch; ++c) gmax = std::max(gmax, (bounds[c + 1] - bounds[c]) / 4);
  double* wd_dev = (double*)pool_get(POOL_AUX, plane5 * nd * sizeof(double));
  double* rd_dev = (double*)pool_get(POOL_STAGE_OUT, plane5 * nd * sizeof(double));
  const size_t s4 = residual_scratch_doubles(im, jm, gh, 4);
  const size_t scr_each = s4 * (size_t)std::max(gmax, 1) + residual_scratch_doubles(im, jm, gh, 2);
  double* scr = (double*)pool_get(POOL_SCRATCH, 2 * scr_each * 8);
  if (!wd_dev || !rd_dev || !scr) return fail_arg("scratch allocation failed"), BCG_ERR_NOMEM;
  constexpr int kEv = 2 * kMaxChunk + 2;
  cudaEvent_t ev[kEv] = {};  // 0: start; 1 + c: chunk c uploaded; 1 + nch + c: chunk c computed; last: downloads done
  for (auto& x : ev)
    if (cudaEventCreateWithFlags(&x, cudaEventDisableTiming) != cudaSuccess) return fail_cuda("events", cudaGetLastError());
  struct Guard { cudaEvent_t* e; ~Guard() { for (int k = 0; k < kEv; ++k) if (e[k]) cudaEventDestroy(e[k]); } } guard{ev};
  cudaError_t e = cudaEventRecord(ev[0], st);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(cs.in, ev[0], 0);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(cs.comp[0], ev[0], 0);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(cs.comp[1], ev[0], 0);
  if (e != cudaSuccess) return fail_cuda("pipelined residual", e);
  for (int c = 0; c < nch; ++c) {
    const int d0 = bounds[c], d1 = bounds[c + 1];
    if (d1 <= d0) continue;
    cudaStream_t cst = cs.comp[c & 1];
    e = cudaMemcpyAsync(wd_dev + plane5 * d0, wd + plane5 * d0, plane5 * (d1 - d0) * sizeof(double),
                        cudaMemcpyHostToDevice, cs.in);
    if (e == cudaSuccess) e = cudaEventRecord(ev[1 + c], cs.in);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cst, ev[1 + c], 0);
    if (e != cudaSuccess) return fail_cuda("pipelined residual: upload", e);
    for (int k0 = d0; k0 < d1;) {
      const int left = d1 - k0;
      const int kk = left >= 4 ? 4 : (left >= 2 ? 2 : 1);
      a.ndir = kk; a.ngroup = left >= 4 ? left / 4 : 1;
      a.wd = wd_dev + plane5 * k0; a.resd = rd_dev + plane5 * k0;
      a.res = (k0 == 0) ? res : nullptr;
      a.scratch = scr + (size_t)(c & 1) * scr_each;
      e = run_residual(a, cst);
      if (e != cudaSuccess) return fail_cuda("flux_num_dnc5_2d_d", e);
      k0 += kk * a.ngroup;
    }
    e = cudaEventRecord(ev[1 + nch + c], cst);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cs.out, ev[1 + nch + c], 0);
    if (e == cudaSuccess)
      e = copy_interior_d2h(residud + plane5 * d0, rd_dev + plane5 * d0, ni, nj, 5 * (d1 - d0), gh, im, jm, cs.out);
    if (e != cudaSuccess) return fail_cuda("pipelined residual: download", e);
  }
  e = cudaEventRecord(ev[kEv - 1], cs.out);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev[kEv - 1], 0);
  return e == cudaSuccess ? BCG_OK : fail_cuda("pipelined residual", e);
}

// shared body of the residual / JVP entry points
int residual_call(double* residu, double* residud, const double* w, const double* wd, int nd, const double* nx,
                  const double* ny, const double* vol, const double* volf, int gh, double cp, double cv,
                  double prandtl, double gam, double rgaz, double cs, double muref, double tref, double s_suth,
                  double k2, double k4, int im, int jm, int nowall = 0, int order = 5) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (order == 5) {
    if (!dims_ok(im, jm, gh)) return fail_arg("flux_num_dnc5_2d: need gh == 3 and im, jm >= 6");
  } else {
    // DNC3/7/9: ghosts for the R-point stencils; the wall rows read the first nw cell rows
    const int R = dnc_pairs(order), nw = order == 3 ? 2 : (order == 7 ? 9 : 11);
    if (R == 0 || gh < R || im < std::max(6, nw) || jm < std::max(6, nw) || nd > 1)
      return fail_arg("flux_num_dnc_2d: need order 3, 7 or 9, gh >= (order+1)/2, im, jm >= max(6, wall rows)");
  }
  if (nd < 0) return fail_arg("flux_num_dnc5_2d_dn: negative direction count");
  const size_t np = ncell(im, jm, gh), nn = nnode(im, jm, gh);
  cudaStream_t st = current_stream();
  // DNC5 on a rectilinear grid takes the face kernel without the zero metric products
  const int rect = (order == 5 && nx && ny) ? (int)face_rectilinear(nx, ny, im, jm, gh, st) : 0;
  Stager sg(st);
  const int hw = sg.in(w, np * 5 * 8), hnx = sg.in(nx, nn * 2 * 8), hny = sg.in(ny, nn * 2 * 8);
  const int hvol = sg.in(vol, np * 8), hvolf = sg.in(volf, np * 2 * 8);
  const int ni = im + 2 * gh, nj = jm + 2 * gh;
  const int hres = residu ? sg.out_interior(residu, ni, nj, 5, gh, im, jm) : -1;
  // many directions in host memory: pipelined upload / compute / download
  const bool pipelined = nd >= 8 && wd && residud && !is_device_ptr(wd) && !is_device_ptr(residud);
  const int hwd = (nd && !pipelined) ? sg.in(wd, np * 5 * 8 * (size_t)nd) : -1;
  const int hresd = (nd && !pipelined) ? sg.out_interior(residud, ni, nj, 5 * nd, gh, im, jm) : -1;
  int rc = sg.commit();
  if (rc) return rc;
  ResidualArgs a{};
  a.im = im; a.jm = jm; a.gh = gh;
  a.phys = Phys{cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4};
  a.w = sg.dev<double>(hw); a.nx = sg.dev<double>(hnx); a.ny = sg.dev<double>(hny);
  a.vol = sg.dev<double>(hvol); a.volf = sg.dev<double>(hvolf);
  a.dstride = np * 5;
  a.nowall = nowall;
  a.order = order;
  a.rect = rect;
  double* res = hres >= 0 ? sg.dev<double>(hres) : nullptr;
  if (pipelined) {
    rc = residual_pipelined(a, res, residud, wd, nd, st);
    if (rc) return rc;
    rc = sg.finish();
    if (rc) return rc;
    const cudaError_t e = cudaStreamSynchronize(st);  // host outputs complete on return
    return e == cudaSuccess ? BCG_OK : fail_cuda("stream synchronize", e);
  }
  if (nd == 0) {
    a.ndir = 0; a.res = res;
    a.scratch = (double*)pool_get(POOL_SCRATCH, residual_scratch_doubles(im, jm, gh, 0) * 8);
    if (!a.scratch) return fail_arg("scratch allocation failed"), BCG_ERR_NOMEM;
    cudaError_t e = run_residual(a, st);
    if (e != cudaSuccess) return fail_cuda("flux_num_dnc5_2d", e);
  } else {
    const double* wdd = sg.dev<double>(hwd);
    double* rdd = sg.dev<double>(hresd);
    // full groups of 4 directions run as one launch per pass (blockIdx.y =
    // group), as many groups at a time as fit a 2 GiB scratch budget, split
    // in two halves on two streams (each with its own part of the scratch)
    // so that one half's kernels fill the SMs the other's last partial waves
    // leave idle; the remaining 1-3 directions run as 2 + 1
    const size_t s4 = residual_scratch_doubles(im, jm, gh, 4);
    const int gmax = (int)std::max<size_t>(1, ((size_t)2 << 30) / (s4 * 8));
    CopyStreams cs;
    rc = copy_streams(&cs);
    if (rc) return rc;
    cudaEvent_t ev[3] = {};
    struct Guard { cudaEvent_t* e; ~Guard() { for (int k = 0; k < 3; ++k) if (e[k]) cudaEventDestroy(e[k]); } } guard{ev};
    for (auto& x : ev)
      if (cudaEventCreateWithFlags(&x, cudaEventDisableTiming) != cudaSuccess) return fail_cuda("events", cudaGetLastError());
    int off = 0;
    while (off < nd) {
      const int left = nd - off;
      int kk, ng;
      if (left >= 4) { kk = 4; ng = std::min(left / 4, gmax); }
      else { kk = left >= 2 ? 2 : 1; ng = 1; }
      double* scr = (double*)pool_get(POOL_SCRATCH, residual_scratch_doubles(im, jm, gh, kk) * 8 * (size_t)ng);
      if (!scr) return fail_arg("scratch allocation failed"), BCG_ERR_NOMEM;
      a.ndir = kk;
      a.wd = wdd + (size_t)off * np * 5;
      a.resd = rdd + (size_t)off * np * 5;
      a.res = (off == 0) ? res : nullptr;
      cudaError_t e = cudaSuccess;
      if (kk == 4 && ng >= 2) {
        const int h0 = (ng + 1) / 2;
        e = cudaEventRecord(ev[0], st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(cs.comp[0], ev[0], 0);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(cs.comp[1], ev[0], 0);
        ResidualArgs b = a;
        a.ngroup = h0; a.scratch = scr;
        b.ngroup = ng - h0; b.scratch = scr + s4 * (size_t)h0; b.res = nullptr;
        b.wd = a.wd + (size_t)4 * h0 * np * 5; b.resd = a.resd + (size_t)4 * h0 * np * 5;
        if (e == cudaSuccess) e = run_residual(a, cs.comp[0]);
        if (e == cudaSuccess) e = run_residual(b, cs.comp[1]);
        if (e == cudaSuccess) e = cudaEventRecord(ev[1], cs.comp[0]);
        if (e == cudaSuccess) e = cudaEventRecord(ev[2], cs.comp[1]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev[1], 0);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev[2], 0);
      } else {
        a.ngroup = ng; a.scratch = scr;
        e = run_residual(a, st);
      }
      if (e != cudaSuccess) return fail_cuda("flux_num_dnc5_2d_d", e);
      off += kk * ng;
    }
  }
  return sg.finish();
}

int bc_call(int kind, double* w, double* wd, const double* aux, int lm, const char* loc, const int* interf,
            const double* nx, const double* ny, double gam, int gh, int im, int jm, int em) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (gh < 1 || im < 1 || jm < 1 || !interf || !loc) return fail_arg("boundary condition: bad extents");
  BcSide side;
  if (!make_side(loc, interf, &side)) return fail_arg("boundary condition: loc must be Ilo, Ihi, Jlo or Jhi");
  if (!side_in_bounds(side, im, jm, gh)) return fail_arg("boundary condition: interf outside the padded grid");
  const size_t np = ncell(im, jm, gh), nn = nnode(im, jm, gh);
  cudaStream_t st = current_stream();
  Stager sg(st);
  const int hw = sg.inout(w, np * em * 8);
  const int hwd = wd ? sg.inout(wd, np * em * 8) : -1;
  int haux = -1, hnx = -1, hny = -1;
  if (kind == BC_NOREF) haux = sg.in(aux, (size_t)lm * 5 * 8);
  if (kind == BC_INLET) haux = sg.in(aux, (size_t)lm * gh * 5 * 8);
  if (kind == BC_NOREF || kind == BC_INLET) { hnx = sg.in(nx, nn * 2 * 8); hny = sg.in(ny, nn * 2 * 8); }
  int rc = sg.commit();
  if (rc) return rc;
  BcArgs a{};
  a.kind = kind; a.ndir = wd ? 1 : 0; a.im = im; a.jm = jm; a.gh = gh; a.em = em; a.lm = lm; a.side = side;
  a.gam = gam; a.w = sg.dev<double>(hw); a.wd = wd ? sg.dev<double>(hwd) : nullptr; a.dstride = np * em;
  a.aux = haux >= 0 ? sg.dev<double>(haux) : nullptr;
  a.nx = hnx >= 0 ? sg.dev<double>(hnx) : nullptr;
  a.ny = hny >= 0 ? sg.dev<double>(hny) : nullptr;
  cudaError_t e = launch_bc(a, st);
  if (e != cudaSuccess) return fail_cuda("boundary condition", e);
  return sg.finish();
}

// index set-up of borders/jn_match.F90:3-66 shared by the copy and its adjoint
int jn_args(const int* prr, int gh1r, int gh2r, int gh3r, int gh4r, int imr, int jmr, const int* prd, int gh1d,
            int gh2d, int gh3d, int gh4d, int imd, int jmd, const int* tr, int em, JnArgs* out) {
  if (!prr || !prd || !tr) return fail_arg("jn_match_2d: null index array");
  auto P = [](const int* a, int r, int c) { return a[(r - 1) + (c - 1) * 2]; };
  JnArgs a{};
  a.em = em;
  a.istep = tr[0] >= 0 ? 1 : -1; a.jstep = tr[1] >= 0 ? 1 : -1;
  const int idir = tr[0] < 0 ? -tr[0] : tr[0], jdir = tr[1] < 0 ? -tr[1] : tr[1];
  if (idir < 1 || idir > 2 || jdir < 1 || jdir > 2) return fail_arg("jn_match_2d: tr must hold +-1 and +-2");
  const int ni = P(prd, 2, idir) - P(prd, 1, idir) + 1, nj = P(prd, 2, jdir) - P(prd, 1, jdir) + 1;
  a.i1 = a.istep == 1 ? 1 : ni; a.j1 = a.jstep == 1 ? 1 : nj;
  a.icount = ni; a.ncopy = ni * nj;
  a.prr11 = P(prr, 1, 1); a.prr12 = P(prr, 1, 2); a.prd1i = P(prd, 1, idir); a.prd1j = P(prd, 1, jdir);
  a.lor_i = 1 - gh1r; a.lor_j = 1 - gh3r; a.nir = imr + gh1r + gh2r; a.njr = jmr + gh3r + gh4r;
  a.lod_i = 1 - gh1d; a.lod_j = 1 - gh3d; a.nid = imd + gh1d + gh2d; a.njd = jmd + gh3d + gh4d;
  // bounds of the copied blocks
  const int ir_hi = a.prr11 + ni - 1, jr_hi = a.prr12 + nj - 1;
  if (a.prr11 < a.lor_i || a.prr12 < a.lor_j || ir_hi > a.lor_i + a.nir - 1 || jr_hi > a.lor_j + a.njr - 1)
    return fail_arg("jn_match_2d: receiver block outside the receiver array");
  const int id_lo = a.prd1i, jd_lo = a.prd1j, id_hi = a.prd1i + ni - 1, jd_hi = a.prd1j + nj - 1;
  if (id_lo < a.lod_i || jd_lo < a.lod_j || id_hi > a.lod_i + a.nid - 1 || jd_hi > a.lod_j + a.njd - 1)
    return fail_arg("jn_match_2d: donor block outside the donor array");
  *out = a;
  return BCG_OK;
}

int jn_call(double* wr, const int* prr, int gh1r, int gh2r, int gh3r, int gh4r, int imr, int jmr, const double* wdn,
            const int* prd, int gh1d, int gh2d, int gh3d, int gh4d, int imd, int jmd, const int* tr, int em) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  JnArgs a{};
  int rc0 = jn_args(prr, gh1r, gh2r, gh3r, gh4r, imr, jmr, prd, gh1d, gh2d, gh3d, gh4d, imd, jmd, tr, em, &a);
  if (rc0) return rc0;
  cudaStream_t st = current_stream();
  Stager sg(st);
  const size_t nr = (size_t)a.nir * a.njr * em, ndn = (size_t)a.nid * a.njd * em;
  int hr, hd;
  if ((const void*)wr == (const void*)wdn) { hr = sg.inout(wr, nr * 8); hd = hr; }
  else { hr = sg.inout(wr, nr * 8); hd = sg.in(wdn, ndn * 8); }
  int rc = sg.commit();
  if (rc) return rc;
  a.wr = sg.dev<double>(hr); a.wd = sg.dev<double>(hd);
  cudaError_t e = launch_jn_match(a, st);
  if (e != cudaSuccess) return fail_cuda("jn_match_2d", e);
  return sg.finish();
}

// adjoint of the join (adjoint/jn_match_2d_b.f90): wdb = 0, then
// wdb(donor) += wrb(receiver) and wrb(receiver) = 0; wr and wd are not used
int jn_b_call(double* wrb, const int* prr, int gh1r, int gh2r, int gh3r, int gh4r, int imr, int jmr, double* wdb,
              const int* prd, int gh1d, int gh2d, int gh3d, int gh4d, int imd, int jmd, const int* tr, int em) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (!wrb || !wdb) return fail_arg("jn_match_2d_b: null adjoint array");
  JnArgs a{};
  int rc = jn_args(prr, gh1r, gh2r, gh3r, gh4r, imr, jmr, prd, gh1d, gh2d, gh3d, gh4d, imd, jmd, tr, em, &a);
  if (rc) return rc;
  cudaStream_t st = current_stream();
  Stager sg(st);
  const size_t nr = (size_t)a.nir * a.njr * em, ndn = (size_t)a.nid * a.njd * em;
  int hr, hd;
  if ((const void*)wrb == (const void*)wdb) { hr = sg.inout(wrb, std::max(nr, ndn) * 8); hd = hr; }
  else { hr = sg.inout(wrb, nr * 8); hd = sg.out(wdb, ndn * 8); }
  rc = sg.commit();
  if (rc) return rc;
  cudaError_t e = launch_jn_match_adjoint(a, sg.dev<double>(hr), sg.dev<double>(hd), st);
  if (e != cudaSuccess) return fail_cuda("jn_match_2d_b", e);
  return sg.finish();
}

// adjoint of a ghost fill (srcfv/adjoint/bc_*_b.f90): w read, wb updated
int bc_b_call(int kind, const double* w, double* wb, const double* aux, int lm, const char* loc, const int* interf,
              const double* nx, const double* ny, double gam, int gh, int im, int jm, int em) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (gh != 3 || im < 1 || jm < 1 || !interf || !loc) return fail_arg("boundary condition adjoint: need gh == 3");
  if (em < 1 || em > 5) return fail_arg("boundary condition adjoint: em must be 1..5");
  BcSide side;
  if (!make_side(loc, interf, &side)) return fail_arg("boundary condition: loc must be Ilo, Ihi, Jlo or Jhi");
  if (!side_in_bounds(side, im, jm, gh)) return fail_arg("boundary condition: interf outside the padded grid");
  const size_t np = ncell(im, jm, gh), nn = nnode(im, jm, gh);
  cudaStream_t st = current_stream();
  Stager sg(st);
  const int hw = sg.in(w, np * em * 8);
  const int hwb = sg.inout(wb, np * em * 8);
  int haux = -1, hnx = -1, hny = -1;
  if (kind == BC_NOREF) haux = sg.in(aux, (size_t)lm * 5 * 8);
  if (kind == BC_INLET) haux = sg.in(aux, (size_t)lm * gh * 5 * 8);
  if (kind == BC_NOREF || kind == BC_INLET) { hnx = sg.in(nx, nn * 2 * 8); hny = sg.in(ny, nn * 2 * 8); }
  int rc = sg.commit();
  if (rc) return rc;
  BcArgs a{};
  a.kind = kind; a.im = im; a.jm = jm; a.gh = gh; a.em = em; a.lm = lm; a.side = side; a.gam = gam;
  a.w = const_cast<double*>(sg.dev<double>(hw));
  a.aux = haux >= 0 ? sg.dev<double>(haux) : nullptr;
  a.nx = hnx >= 0 ? sg.dev<double>(hnx) : nullptr;
  a.ny = hny >= 0 ? sg.dev<double>(hny) : nullptr;
  cudaError_t e = launch_bc_adjoint(a, sg.dev<double>(hwb), st);
  if (e != cudaSuccess) return fail_cuda("boundary condition adjoint", e);
  return sg.finish();
}
}  // namespace

extern "C" {

int bcg_abi_version(void) { return 1; }
int bcg_set_stream(void* stream) { set_stream((cudaStream_t)stream); return BCG_OK; }
void* bcg_get_stream(void) { return (void*)current_stream(); }
int bcg_synchronize(void) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  cudaError_t e = cudaStreamSynchronize(current_stream());
  return e == cudaSuccess ? BCG_OK : fail_cuda("bcg_synchronize", e);
}
const char* bcg_last_error_string(void) { return last_error(); }
size_t bcg_residual_scratch_bytes(int im, int jm, int gh, int ndir) {
  return residual_scratch_doubles(im, jm, gh, std::min(ndir, 4)) * 8;
}

// ---- residual and JVP (srcfv/rhs/flux_num_dnc5.F90:7-8,
//      srcfv/tangent/flux_num_dnc5_d.f90:15-17) -------------------------------
int bcg_flux_num_dnc5_2d(double* residu, const double* w, const double* x0, const double* y0, const double* nx,
                         const double* ny, const double* xc, const double* yc, const double* vol, const double* volf,
                         int gh, double cp, double cv, double prandtl, double gam, double rgaz, double cs,
                         double muref, double tref, double s_suth, double k2, double k4, int im, int jm) {
  (void)x0; (void)y0; (void)xc; (void)yc;
  return residual_call(residu, nullptr, w, nullptr, 0, nx, ny, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref,
                       tref, s_suth, k2, k4, im, jm);
}

// ---- residual without the wall rows (srcfv/rhs/flux_num_dnc5_nowall.F90:7) and
// its tangent (srcfv/tangent/flux_num_dnc5_nowall_d.f90) -----------------------
int bcg_flux_num_dnc5_nowall_2d(double* residu, const double* w, const double* x0, const double* y0,
                                const double* nx, const double* ny, const double* xc, const double* yc,
                                const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                                double gam, double rgaz, double cs, double muref, double tref, double s_suth,
                                double k2, double k4, int im, int jm) {
  (void)x0; (void)y0; (void)xc; (void)yc;
  return residual_call(residu, nullptr, w, nullptr, 0, nx, ny, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref,
                       tref, s_suth, k2, k4, im, jm, 1);
}
int bcg_flux_num_dnc5_nowall_2d_d(double* residu, double* residud, const double* w, const double* wd,
                                  const double* x0, const double* y0, const double* nx, const double* ny,
                                  const double* xc, const double* yc, const double* vol, const double* volf, int gh,
                                  double cp, double cv, double prandtl, double gam, double rgaz, double cs,
                                  double muref, double tref, double s_suth, double k2, double k4, int im, int jm) {
  (void)x0; (void)y0; (void)xc; (void)yc;
  return residual_call(residu, residud, w, wd, 1, nx, ny, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref,
                       s_suth, k2, k4, im, jm, 1);
}

// ---- the DNC schemes of order 3, 7 and 9 (srcfv/rhs/flux_num_dnc{3,7,9}.F90,
// flux_num_dnc{3,7,9}_nowall.F90) and their tangents (srcfv/tangent/
// flux_num_dnc{3,7,9}[_nowall]_d.f90); gh >= (order+1)/2 ------------------------
#define BCG_DNC_ENTRIES(ORD)                                                                                         \
  int bcg_flux_num_dnc##ORD##_2d(double* residu, const double* w, const double* x0, const double* y0,               \
                                 const double* nx, const double* ny, const double* xc, const double* yc,             \
                                 const double* vol, const double* volf, int gh, double cp, double cv,                \
                                 double prandtl, double gam, double rgaz, double cs, double muref, double tref,      \
                                 double s_suth, double k2, double k4, int im, int jm) {                              \
    (void)x0; (void)y0; (void)xc; (void)yc;                                                                         \
    return residual_call(residu, nullptr, w, nullptr, 0, nx, ny, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs,     \
                         muref, tref, s_suth, k2, k4, im, jm, 0, ORD);                                              \
  }                                                                                                                  \
  int bcg_flux_num_dnc##ORD##_2d_d(double* residu, double* residud, const double* w, const double* wd,              \
                                   const double* x0, const double* y0, const double* nx, const double* ny,           \
                                   const double* xc, const double* yc, const double* vol, const double* volf,        \
                                   int gh, double cp, double cv, double prandtl, double gam, double rgaz, double cs, \
                                   double muref, double tref, double s_suth, double k2, double k4, int im, int jm) { \
    (void)x0; (void)y0; (void)xc; (void)yc;                                                                         \
    return residual_call(residu, residud, w, wd, 1, nx, ny, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref,   \
                         tref, s_suth, k2, k4, im, jm, 0, ORD);                                                     \
  }                                                                                                                  \
  int bcg_flux_num_dnc##ORD##_nowall_2d(double* residu, const double* w, const double* x0, const double* y0,        \
                                        const double* nx, const double* ny, const double* xc, const double* yc,      \
                                        const double* vol, const double* volf, int gh, double cp, double cv,         \
                                        double prandtl, double gam, double rgaz, double cs, double muref,            \
                                        double tref, double s_suth, double k2, double k4, int im, int jm) {          \
    (void)x0; (void)y0; (void)xc; (void)yc;                                                                         \
    return residual_call(residu, nullptr, w, nullptr, 0, nx, ny, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs,     \
                         muref, tref, s_suth, k2, k4, im, jm, 1, ORD);                                              \
  }                                                                                                                  \
  int bcg_flux_num_dnc##ORD##_nowall_2d_d(double* residu, double* residud, const double* w, const double* wd,       \
                                          const double* x0, const double* y0, const double* nx, const double* ny,    \
                                          const double* xc, const double* yc, const double* vol,                     \
                                          const double* volf, int gh, double cp, double cv, double prandtl,          \
                                          double gam, double rgaz, double cs, double muref, double tref,             \
                                          double s_suth, double k2, double k4, int im, int jm) {                     \
    (void)x0; (void)y0; (void)xc; (void)yc;                                                                         \
    return residual_call(residu, residud, w, wd, 1, nx, ny, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref,   \
                         tref, s_suth, k2, k4, im, jm, 1, ORD);                                                     \
  }
BCG_DNC_ENTRIES(3)
BCG_DNC_ENTRIES(7)
BCG_DNC_ENTRIES(9)
#undef BCG_DNC_ENTRIES

// ---- Newton linear solve (BROADCAST_npz.py:1146-1158; MUMPS LU there) -----------
// x = A^-1 b for the n x n CSR matrix A (int32 indptr/indices, nnz entries,
// duplicates summed) by band LU with partial pivoting on the GPU; nb is the
// block size (0: 256).  Returns BCG_ERR_SINGULAR with *info = first zero pivot
// (1-based) for a singular matrix.
int bcg_csr_band_lu_solve(int n, const int* indptr, const int* indices, const double* data, long long nnz,
                          const int* perm, const double* b, double* x, int nb, int* info) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (n < 1 || nnz < 0 || !indptr || !indices || !data || !b || !x) return fail_arg("csr_band_lu_solve: bad arguments");
  cudaStream_t st = current_stream();
  if (perm) {  // the reordering indexes the band storage: check it is a permutation of 0..n-1
    std::vector<int> q((size_t)n);
    if (is_device_ptr(perm)) {
      const cudaError_t e = cudaMemcpy(q.data(), perm, (size_t)n * 4, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return fail_cuda("csr_band_lu_solve: reading perm", e);
    } else {
      std::copy(perm, perm + n, q.begin());
    }
    std::vector<char> seen((size_t)n, 0);
    for (int k = 0; k < n; ++k) {
      if (q[k] < 0 || q[k] >= n || seen[q[k]]) return fail_arg("csr_band_lu_solve: perm is not a permutation");
      seen[q[k]] = 1;
    }
  }
  Stager sg(st);
  const int hp = sg.in(indptr, (size_t)(n + 1) * 4), hi = sg.in(indices, (size_t)nnz * 4);
  const int hd = sg.in(data, (size_t)nnz * 8), hb = sg.in(b, (size_t)n * 8), hx = sg.out(x, (size_t)n * 8);
  const int hq = perm ? sg.in(perm, (size_t)n * 4) : -1;
  int rc = sg.commit();
  if (rc) return rc;
  BandLuInfo bi{};
  const int r = band_lu_solve(n, sg.dev<int>(hp), sg.dev<int>(hi), sg.dev<double>(hd), hq >= 0 ? sg.dev<int>(hq) : nullptr,
                              sg.dev<double>(hb), sg.dev<double>(hx), nb > 0 ? nb : 256, st, &bi);
  if (info) *info = bi.info;
  if (r == 1) return fail_arg("csr_band_lu_solve: singular matrix"), BCG_ERR_SINGULAR;
  if (r != 0) return fail_arg(band_lu_error()), BCG_ERR_CUDA;
  return sg.finish();
}

// ---- matrix-free implicit phase (srcfv/lhs/impli_matrix_free.F90:7) -------------
// dwi (intent inout in the reference, fully overwritten: interior = the
// increment after lmax sweeps, every ghost zero); dw is the right-hand side.
int bcg_impli_matrix_free_2d(double* dwi, const double* nx, const double* ny, const double* w, const double* dw,
                             const double* vol, const double* volf, double dtcoef, double cfl, double gam, double rgaz,
                             double prandtl, int lmax, int gh, double cv, double cs, double muref, double tref,
                             double s_suth, int im, int jm, int em) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (em != 5 || gh < 1 || im < 1 || jm < 1 || lmax < 0)
    return fail_arg("impli_matrix_free_2d: need em == 5, gh >= 1, im, jm >= 1, lmax >= 0");
  if (lmax > 0 && jm > impli_max_rows()) return fail_arg("impli_matrix_free_2d: jm above the sweep kernel's row limit");
  const size_t np = ncell(im, jm, gh), nn = nnode(im, jm, gh);
  cudaStream_t st = current_stream();
  Stager sg(st);
  const int hnx = sg.in(nx, nn * 2 * 8), hny = sg.in(ny, nn * 2 * 8), hw = sg.in(w, np * 5 * 8);
  const int hdw = sg.in(dw, np * 5 * 8), hvol = sg.in(vol, np * 8), hvolf = sg.in(volf, np * 2 * 8);
  const int hdwi = sg.out(dwi, np * 5 * 8);
  int rc = sg.commit();
  if (rc) return rc;
  ImpliArgs a{};
  a.im = im; a.jm = jm; a.gh = gh; a.lmax = lmax;
  a.dtcoef = dtcoef; a.cfl = cfl; a.gam = gam; a.rgaz = rgaz; a.prandtl = prandtl; a.cv = cv; a.cs = cs;
  a.muref = muref; a.tref = tref; a.s_suth = s_suth;
  a.nx = sg.dev<double>(hnx); a.ny = sg.dev<double>(hny); a.w = sg.dev<double>(hw); a.dw = sg.dev<double>(hdw);
  a.vol = sg.dev<double>(hvol); a.volf = sg.dev<double>(hvolf); a.dwi = sg.dev<double>(hdwi);
  a.scratch = (double*)pool_get(POOL_SCRATCH, impli_scratch_doubles(im, jm, gh) * 8);
  if (!a.scratch) return fail_arg("impli_matrix_free_2d: scratch allocation failed"), BCG_ERR_NOMEM;
  const cudaError_t e = run_impli(a, st);
  if (e != cudaSuccess) return fail_cuda("impli_matrix_free_2d", e);
  return sg.finish();
}

int bcg_flux_num_dnc5_2d_d(double* residu, double* residud, const double* w, const double* wd, const double* x0,
                           const double* y0, const double* nx, const double* ny, const double* xc, const double* yc,
                           const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                           double gam, double rgaz, double cs, double muref, double tref, double s_suth, double k2,
                           double k4, int im, int jm) {
  (void)x0; (void)y0; (void)xc; (void)yc;
  return residual_call(residu, residud, w, wd, 1, nx, ny, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref,
                       s_suth, k2, k4, im, jm);
}

int bcg_flux_num_dnc5_2d_dn(double* residu, double* residud, const double* w, const double* wd, int nd,
                            const double* x0, const double* y0, const double* nx, const double* ny, const double* xc,
                            const double* yc, const double* vol, const double* volf, int gh, double cp, double cv,
                            double prandtl, double gam, double rgaz, double cs, double muref, double tref,
                            double s_suth, double k2, double k4, int im, int jm) {
  (void)x0; (void)y0; (void)xc; (void)yc;
  return residual_call(residu, residud, w, wd, nd, nx, ny, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref,
                       tref, s_suth, k2, k4, im, jm);
}

// ---- spanwise operators (srcfv/dz/coeffs_5p_dz.F90:10, coeffs_5p_dz2.F90:10) --
// dz_out = Dz . wd (or Dzz . wd) on the interior; the ghosts of dz_out are
// left as they are (intent(inout) in the reference).
namespace {
int span_call(int op, double* dz_out, const double* w, const double* wd, int nd, const double* nx, const double* ny,
              const double* vol, int gh, double cp, double cv, double prandtl, double gam, double rgaz, double cs,
              double muref, double tref, double s_suth, int im, int jm) {
  const char* name = op == SPAN_DZ ? "coeffs_5p_dz" : "coeffs_5p_dz2";
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (!dims_ok(im, jm, gh)) return fail_arg("coeffs_5p_dz: need gh == 3 and im, jm >= 6");
  if (nd < 1) return fail_arg("coeffs_5p_dz: need at least one direction");
  if (!dz_out || !w || !wd) return fail_arg("coeffs_5p_dz: null array");
  if (op == SPAN_DZ && (!nx || !ny || !vol)) return fail_arg("coeffs_5p_dz: null metric array");
  const size_t np = ncell(im, jm, gh), nn = nnode(im, jm, gh);
  cudaStream_t st = current_stream();
  Stager sg(st);
  const int hw = sg.in(w, np * 5 * 8), hwd = sg.in(wd, np * 5 * 8 * (size_t)nd);
  int hnx = -1, hny = -1, hvol = -1;
  if (op == SPAN_DZ) { hnx = sg.in(nx, nn * 2 * 8); hny = sg.in(ny, nn * 2 * 8); hvol = sg.in(vol, np * 8); }
  const int ho = sg.out_interior(dz_out, im + 2 * gh, jm + 2 * gh, 5 * nd, gh, im, jm);
  int rc = sg.commit();
  if (rc) return rc;
  SpanArgs a{};
  a.im = im; a.jm = jm; a.gh = gh; a.op = op;
  a.phys = Phys{cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, 0.0, 0.0};
  a.w = sg.dev<double>(hw); a.dstride = np * 5;
  if (op == SPAN_DZ) { a.nx = sg.dev<double>(hnx); a.ny = sg.dev<double>(hny); a.vol = sg.dev<double>(hvol); }
  const double* wdd = sg.dev<double>(hwd);
  double* od = sg.dev<double>(ho);
  for (int k0 = 0; k0 < nd;) {
    const int kk = nd - k0 >= 4 ? 4 : (nd - k0 >= 2 ? 2 : 1);
    a.ndir = kk; a.wd = wdd + (size_t)k0 * np * 5; a.out = od + (size_t)k0 * np * 5;
    cudaError_t e = run_span(a, st);
    if (e != cudaSuccess) return fail_cuda(name, e);
    k0 += kk;
  }
  return sg.finish();
}
}  // namespace

int bcg_coeffs_5p_dz(double* dz_out, const double* w, const double* wd, const double* x0, const double* y0,
                     const double* nx, const double* ny, const double* xc, const double* yc, const double* vol,
                     const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz,
                     double cs, double muref, double tref, double s_suth, int im, int jm) {
  (void)x0; (void)y0; (void)xc; (void)yc; (void)volf;
  return span_call(SPAN_DZ, dz_out, w, wd, 1, nx, ny, vol, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth,
                   im, jm);
}

int bcg_coeffs_5p_dz2(double* dz2_out, const double* w, const double* wd, const double* x0, const double* y0,
                      const double* nx, const double* ny, const double* xc, const double* yc, const double* vol,
                      const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz,
                      double cs, double muref, double tref, double s_suth, int im, int jm) {
  (void)x0; (void)y0; (void)xc; (void)yc; (void)volf;
  return span_call(SPAN_DZZ, dz2_out, w, wd, 1, nx, ny, vol, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth,
                   im, jm);
}

int bcg_coeffs_5p_dz_dn(double* dz_out, const double* w, const double* wd, int nd, const double* x0,
                        const double* y0, const double* nx, const double* ny, const double* xc, const double* yc,
                        const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                        double gam, double rgaz, double cs, double muref, double tref, double s_suth, int im, int jm) {
  (void)x0; (void)y0; (void)xc; (void)yc; (void)volf;
  return span_call(SPAN_DZ, dz_out, w, wd, nd, nx, ny, vol, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth,
                   im, jm);
}

int bcg_coeffs_5p_dz2_dn(double* dz2_out, const double* w, const double* wd, int nd, const double* x0,
                         const double* y0, const double* nx, const double* ny, const double* xc, const double* yc,
                         const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                         double gam, double rgaz, double cs, double muref, double tref, double s_suth, int im,
                         int jm) {
  (void)x0; (void)y0; (void)xc; (void)yc; (void)volf;
  return span_call(SPAN_DZZ, dz2_out, w, wd, nd, nx, ny, vol, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref,
                   s_suth, im, jm);
}

// ---- adjoint (srcfv/adjoint/flux_num_dnc5_b.f90:15) ------------------------
// wb = (dR/dw)^T residub on every padded cell (wb overwritten); the interior
// of residub is zeroed, as the Tapenade routine does.  residu is unused.
namespace {
int adjoint_call(double* residub, const double* w, double* wb, const double* nx, const double* ny, const double* vol,
                 const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz, double cs,
                 double muref, double tref, double s_suth, double k2, double k4, int im, int jm, int nowall,
                 int nd = 1);
}

int bcg_flux_num_dnc5_2d_b(double* residu, double* residub, const double* w, double* wb, const double* x0,
                           const double* y0, const double* nx, const double* ny, const double* xc, const double* yc,
                           const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                           double gam, double rgaz, double cs, double muref, double tref, double s_suth, double k2,
                           double k4, int im, int jm) {
  (void)residu; (void)x0; (void)y0; (void)xc; (void)yc;
  return adjoint_call(residub, w, wb, nx, ny, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2,
                      k4, im, jm, 0);
}

// srcfv/adjoint/flux_num_dnc5_nowall_b.f90: the adjoint of the scheme without the wall rows
int bcg_flux_num_dnc5_nowall_2d_b(double* residu, double* residub, const double* w, double* wb, const double* x0,
                                  const double* y0, const double* nx, const double* ny, const double* xc,
                                  const double* yc, const double* vol, const double* volf, int gh, double cp,
                                  double cv, double prandtl, double gam, double rgaz, double cs, double muref,
                                  double tref, double s_suth, double k2, double k4, int im, int jm) {
  (void)residu; (void)x0; (void)y0; (void)xc; (void)yc;
  return adjoint_call(residub, w, wb, nx, ny, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2,
                      k4, im, jm, 1);
}

// nd cotangents in one call (no reference counterpart: the drivers call
// flux_num_dnc5_2d_b once per seed, cylinder.py:1116-1159): residub and wb
// hold nd consecutive (ni, nj, 5) blocks; the primal passes run once per
// launch and every cotangent's face records, gather and primitive reverse
// run as one grid row of the same kernels.
int bcg_flux_num_dnc5_2d_bn(double* residu, double* residub, const double* w, double* wb, int nd, const double* x0,
                            const double* y0, const double* nx, const double* ny, const double* xc, const double* yc,
                            const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                            double gam, double rgaz, double cs, double muref, double tref, double s_suth, double k2,
                            double k4, int im, int jm) {
  (void)residu; (void)x0; (void)y0; (void)xc; (void)yc;
  if (nd < 0) return fail_arg("flux_num_dnc5_2d_bn: negative cotangent count");
  if (nd == 0) return BCG_OK;
  return adjoint_call(residub, w, wb, nx, ny, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2,
                      k4, im, jm, 0, nd);
}

}  // extern "C"

namespace {
int adjoint_call(double* residub, const double* w, double* wb, const double* nx, const double* ny, const double* vol,
                 const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz, double cs,
                 double muref, double tref, double s_suth, double k2, double k4, int im, int jm, int nowall,
                 int nd) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (!dims_ok(im, jm, gh)) return fail_arg("flux_num_dnc5_2d_b: need gh == 3 and im, jm >= 6");
  if (!residub || !w || !wb) return fail_arg("flux_num_dnc5_2d_b: residub, w and wb are required");
  const size_t np = ncell(im, jm, gh), nn = nnode(im, jm, gh);
  cudaStream_t st = current_stream();
  Stager sg(st);
  const int hw = sg.in(w, np * 5 * 8), hnx = sg.in(nx, nn * 2 * 8), hny = sg.in(ny, nn * 2 * 8);
  const int hvol = sg.in(vol, np * 8), hvolf = sg.in(volf, np * 2 * 8);
  const int hrb = sg.inout(residub, np * 5 * 8 * (size_t)nd), hwb = sg.out(wb, np * 5 * 8 * (size_t)nd);
  int rc = sg.commit();
  if (rc) return rc;
  AdjointArgs a{};
  a.im = im; a.jm = jm; a.gh = gh;
  a.phys = Phys{cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4};
  a.w = sg.dev<double>(hw); a.nx = sg.dev<double>(hnx); a.ny = sg.dev<double>(hny);
  a.vol = sg.dev<double>(hvol); a.volf = sg.dev<double>(hvolf);
  a.nowall = nowall;
  a.cstride = np * 5;
  double* rb = sg.dev<double>(hrb);
  double* wbd = sg.dev<double>(hwb);
  // as many cotangents per launch as fit a 2 GiB scratch budget
  const size_t per = adjoint_cotangent_doubles(im, jm, gh);
  const int cmax = (int)std::max<size_t>(1, ((size_t)2 << 30) / (per * 8));
  for (int off = 0; off < nd;) {
    const int n = std::min(nd - off, cmax);
    a.ncot = n;
    a.rb = rb + (size_t)off * np * 5;
    a.wb = wbd + (size_t)off * np * 5;
    a.scratch = (double*)pool_get(POOL_SCRATCH, adjoint_scratch_doubles(im, jm, gh, n) * 8);
    if (!a.scratch) return fail_arg("scratch allocation failed"), BCG_ERR_NOMEM;
    cudaError_t e = run_adjoint(a, st);
    if (e != cudaSuccess) return fail_cuda("flux_num_dnc5_2d_b", e);
    off += n;
  }
  return sg.finish();
}
}  // namespace

extern "C" {

// ---- boundary conditions (srcfv/borders/*.F90, srcfv/tangent/bc_*_d.f90) ----
int bcg_bc_wall_viscous_adia_2d(double* w, const char* loc, double gam, const int* interf, int gh, int im, int jm) {
  return bc_call(BC_WALL, w, nullptr, nullptr, 0, loc, interf, nullptr, nullptr, gam, gh, im, jm, 5);
}
int bcg_bc_wall_viscous_adia_2d_d(double* w, double* wd, const char* loc, double gam, const int* interf, int gh,
                                  int im, int jm) {
  return bc_call(BC_WALL, w, wd, nullptr, 0, loc, interf, nullptr, nullptr, gam, gh, im, jm, 5);
}
int bcg_bc_no_reflexion_2d(double* w, const double* wbd, const char* loc, const int* interf, const double* nx,
                           const double* ny, double gam, int gh, int im, int jm, int lm) {
  return bc_call(BC_NOREF, w, nullptr, wbd, lm, loc, interf, nx, ny, gam, gh, im, jm, 5);
}
int bcg_bc_no_reflexion_2d_d(double* w, double* wd, const double* wbd, const char* loc, const int* interf,
                             const double* nx, const double* ny, double gam, int gh, int im, int jm, int lm) {
  return bc_call(BC_NOREF, w, wd, wbd, lm, loc, interf, nx, ny, gam, gh, im, jm, 5);
}
int bcg_bc_supandsubinlet_2d(double* w, const char* loc, const int* interf, const double* field, const double* nx,
                             const double* ny, double gam, int im, int jm, int lm, int gh) {
  return bc_call(BC_INLET, w, nullptr, field, lm, loc, interf, nx, ny, gam, gh, im, jm, 5);
}
int bcg_bc_supandsubinlet_2d_d(double* w, double* wd, const char* loc, const int* interf, const double* field,
                               const double* nx, const double* ny, double gam, int im, int jm, int lm, int gh) {
  return bc_call(BC_INLET, w, wd, field, lm, loc, interf, nx, ny, gam, gh, im, jm, 5);
}
int bcg_bc_extrapolate_o2_2d(double* w, const char* loc, const int* interf, int im, int jm, int gh, int em) {
  return bc_call(BC_EXTRAP, w, nullptr, nullptr, 0, loc, interf, nullptr, nullptr, 0.0, gh, im, jm, em);
}
int bcg_bc_extrapolate_o2_2d_d(double* w, double* wd, const char* loc, const int* interf, int im, int jm, int gh,
                               int em) {
  return bc_call(BC_EXTRAP, w, wd, nullptr, 0, loc, interf, nullptr, nullptr, 0.0, gh, im, jm, em);
}
int bcg_jn_match_2d(double* wr, const int* prr, int gh1r, int gh2r, int gh3r, int gh4r, int imr, int jmr,
                    const double* wd, const int* prd, int gh1d, int gh2d, int gh3d, int gh4d, int imd, int jmd,
                    const int* tr, int em) {
  return jn_call(wr, prr, gh1r, gh2r, gh3r, gh4r, imr, jmr, wd, prd, gh1d, gh2d, gh3d, gh4d, imd, jmd, tr, em);
}
// tangent of the join: the same copy applied to the state and to its tangent
// (srcfv/tangent/jn_match_2d_d.f90:11)
int bcg_jn_match_2d_d(double* wr, double* wrd, const int* prr, int gh1r, int gh2r, int gh3r, int gh4r, int imr,
                      int jmr, const double* wd, const double* wdd, const int* prd, int gh1d, int gh2d, int gh3d,
                      int gh4d, int imd, int jmd, const int* tr, int em) {
  int rc = jn_call(wr, prr, gh1r, gh2r, gh3r, gh4r, imr, jmr, wd, prd, gh1d, gh2d, gh3d, gh4d, imd, jmd, tr, em);
  if (rc) return rc;
  return jn_call(wrd, prr, gh1r, gh2r, gh3r, gh4r, imr, jmr, wdd, prd, gh1d, gh2d, gh3d, gh4d, imd, jmd, tr, em);
}
// ---- adjoints of the fills (srcfv/adjoint/*_b.f90); w is left unchanged ------
int bcg_bc_wall_viscous_adia_2d_b(double* w, double* wb, const char* loc, double gam, const int* interf, int gh,
                                  int im, int jm) {
  return bc_b_call(BC_WALL, w, wb, nullptr, 0, loc, interf, nullptr, nullptr, gam, gh, im, jm, 5);
}
int bcg_bc_no_reflexion_2d_b(double* w, double* wb, const double* wbd, const char* loc, const int* interf,
                             const double* nx, const double* ny, double gam, int gh, int im, int jm, int lm) {
  return bc_b_call(BC_NOREF, w, wb, wbd, lm, loc, interf, nx, ny, gam, gh, im, jm, 5);
}
int bcg_bc_supandsubinlet_2d_b(double* w, double* wb, const char* loc, const int* interf, const double* field,
                               const double* nx, const double* ny, double gam, int im, int jm, int lm, int gh) {
  return bc_b_call(BC_INLET, w, wb, field, lm, loc, interf, nx, ny, gam, gh, im, jm, 5);
}
int bcg_bc_extrapolate_o2_2d_b(double* w, double* wb, const char* loc, const int* interf, int im, int jm, int gh,
                               int em) {
  return bc_b_call(BC_EXTRAP, w, wb, nullptr, 0, loc, interf, nullptr, nullptr, 0.0, gh, im, jm, em);
}
int bcg_jn_match_2d_b(double* wr, double* wrb, const int* prr, int gh1r, int gh2r, int gh3r, int gh4r, int imr,
                      int jmr, const double* wd, double* wdb, const int* prd, int gh1d, int gh2d, int gh3d, int gh4d,
                      int imd, int jmd, const int* tr, int em) {
  (void)wr; (void)wd;
  return jn_b_call(wrb, prr, gh1r, gh2r, gh3r, gh4r, imr, jmr, wdb, prd, gh1d, gh2d, gh3d, gh4d, imd, jmd, tr, em);
}
// geometric join (srcfv/borders/jn_match_geom.F90:7-69): one-variable copy
int bcg_jn_match_geom_2d(double* wr, const int* prr, int gh1r, int gh2r, int gh3r, int gh4r, int imr, int jmr,
                         const double* wd, const int* prd, int gh1d, int gh2d, int gh3d, int gh4d, int imd, int jmd,
                         const int* tr) {
  if (tr && (tr[0] < 0 ? -tr[0] : tr[0]) != 1) return fail_arg("jn_match_geom_2d: only tr(1) = +-1 is supported");
  return jn_call(wr, prr, gh1r, gh2r, gh3r, gh4r, imr, jmr, wd, prd, gh1d, gh2d, gh3d, gh4d, imd, jmd, tr, 1);
}

}  // extern "C"

// ===========================================================================
// Colored Jacobian seeding / COO fill (misc/ComputeJacobian.f90)
// ===========================================================================
namespace {
int testvector_call(double* wd, int m, int l, int k, int gh, int im, int jm, int istart, int iend, int jstart,
                    int jend, bool partial) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (m < 0 || m > 4 || gh < 1 || im < 1 || jm < 1) return fail_arg("testvector: bad arguments");
  cudaStream_t st = current_stream();
  Stager sg(st);
  const int h = sg.out(wd, ncell(im, jm, gh) * 5 * 8);
  int rc = sg.commit();
  if (rc) return rc;
  cudaError_t e = launch_testvector(sg.dev<double>(h), m, l, k, gh, im, jm, istart, iend, jstart, jend, partial, st);
  if (e != cudaSuccess) return fail_cuda("testvector", e);
  return sg.finish();
}

// Only the 5*im*jm slots of seed (m,l,k[,n]) are touched, so host COO arrays
// are staged by that slice alone.
int jac_call(int mode, double* jac, int* ia, int* ja, const double* resd, int m, int l, int k, int gh, int im, int jm,
             long long nbentry, const double* coefdiag, double mini, int n) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (m < 0 || m > 4 || l < 0 || l > 2 * gh || k < 0 || k > 2 * gh || gh < 1 || im < 1 || jm < 1)
    return fail_arg("computejacobian: bad seed or extents");
  const long long base = jac_slot_base(mode, m, l, k, gh, im, jm, n);
  const long long nslot = 5LL * im * jm;
  if (base < 0 || base + nslot > nbentry) return fail_arg("computejacobian: COO arrays too short for this seed");
  cudaStream_t st = current_stream();
  Stager sg(st);
  const bool check = (mode == JAC_CHECK);
  const int hj = check ? sg.inout(jac + base, nslot * 8) : sg.out(jac + base, nslot * 8);
  const int hi = sg.out(ia + base, nslot * 4);
  const int hja = check ? sg.inout(ja + base, nslot * 4) : sg.out(ja + base, nslot * 4);
  const int hr = sg.in(resd, ncell(im, jm, gh) * 5 * 8);
  const int hc = coefdiag ? sg.in(coefdiag, (size_t)im * jm * 8) : -1;
  int rc = sg.commit();
  if (rc) return rc;
  JacArgs a{};
  a.mode = mode; a.m = m; a.l = l; a.k = k; a.gh = gh; a.im = im; a.jm = jm; a.n = n; a.mini = mini;
  a.resd = sg.dev<double>(hr); a.coefdiag = hc >= 0 ? sg.dev<double>(hc) : nullptr;
  a.jac = sg.dev<double>(hj); a.ia = sg.dev<int>(hi); a.ja = sg.dev<int>(hja);
  cudaError_t e = launch_computejacobian(a, st);
  if (e != cudaSuccess) return fail_cuda("computejacobian", e);
  return sg.finish();
}

int norm_call(int kind, double* o1, double* o2, int* imax, int* jmax, const double* rhs, int im, int jm, int gh) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (gh < 0 || im < 1 || jm < 1) return fail_arg("norm: bad extents");
  cudaStream_t st = current_stream();
  Stager sg(st);
  const int hr = sg.in(rhs, ncell(im, jm, gh) * 5 * 8);
  int rc = sg.commit();
  if (rc) return rc;
  const int nb = norm_partial_blocks(im, jm);
  double* dev = (double*)pool_get(POOL_AUX, (size_t)(nb * 20 + 16) * 8);
  if (!dev) return fail_arg("norm: allocation failed"), BCG_ERR_NOMEM;
  cudaError_t e = launch_norm(kind, sg.dev<double>(hr), im, jm, gh, dev, dev + 16, nb, st);
  if (e != cudaSuccess) return fail_cuda("norm", e);
  double out[15];
  e = cudaMemcpyAsync(out, dev, sizeof out, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail_cuda("norm readback", e);
  // outputs are small: written through the host (or copied to the device)
  double a5[5], b5[5];
  int i5[5], j5[5];
  for (int v = 0; v < 5; ++v) { a5[v] = out[v]; b5[v] = out[5 + v]; i5[v] = (int)out[5 + v]; j5[v] = (int)out[10 + v]; }
  auto put = [&](void* dst, const void* src, size_t bytes) {
    if (!dst) return cudaSuccess;
    if (is_device_ptr(dst)) return cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    std::memcpy(dst, src, bytes);
    return cudaSuccess;
  };
  if (kind == NORM_MAX) {
    if (put(o1, a5, sizeof a5) != cudaSuccess) return fail_cuda("norm output", cudaGetLastError());
    for (int v = 0; v < 5; ++v)
      if (i5[v] < 0) {  // never updated: leave the caller's indices untouched
        int cur_i[5], cur_j[5];
        if (imax && !is_device_ptr(imax)) std::memcpy(cur_i, imax, sizeof cur_i); else std::memset(cur_i, 0, sizeof cur_i);
        if (jmax && !is_device_ptr(jmax)) std::memcpy(cur_j, jmax, sizeof cur_j); else std::memset(cur_j, 0, sizeof cur_j);
        for (int u = 0; u < 5; ++u) if (i5[u] < 0) { i5[u] = cur_i[u]; j5[u] = cur_j[u]; }
        break;
      }
    if (put(imax, i5, sizeof i5) != cudaSuccess || put(jmax, j5, sizeof j5) != cudaSuccess)
      return fail_cuda("norm output", cudaGetLastError());
  } else {
    if (put(o1, a5, sizeof a5) != cudaSuccess || put(o2, b5, sizeof b5) != cudaSuccess)
      return fail_cuda("norm output", cudaGetLastError());
  }
  return sg.finish();
}
}  // namespace

extern "C" {
int bcg_testvector(double* wd, int m, int l, int k, int gh, int im, int jm) {
  return testvector_call(wd, m, l, k, gh, im, jm, 0, 0, 0, 0, false);
}
int bcg_testvector_partial(double* wd, int m, int l, int k, int gh, int im, int jm, int istart, int iend, int jstart,
                           int jend) {
  return testvector_call(wd, m, l, k, gh, im, jm, istart, iend, jstart, jend, true);
}
int bcg_computejacobianfromjv(double* jac, int* ia, int* ja, const double* resd, int m, int l, int k, int gh, int im,
                              int jm, long long nbentry) {
  return jac_call(JAC_PLAIN, jac, ia, ja, resd, m, l, k, gh, im, jm, nbentry, nullptr, 0.0, 0);
}
int bcg_computejacobianfromjv_relaxed(double* jac, int* ia, int* ja, const double* resd, int m, int l, int k, int gh,
                                      int im, int jm, long long nbentry, const double* coefdiag) {
  return jac_call(JAC_RELAXED, jac, ia, ja, resd, m, l, k, gh, im, jm, nbentry, coefdiag, 0.0, 0);
}
int bcg_computejacobianfromjv_relaxed_withjn(double* jac, int* ia, int* ja, const double* resd, int m, int l, int k,
                                             int gh, int im, int jm, long long nbentry, const double* coefdiag) {
  return jac_call(JAC_RELAXED_WITHJN, jac, ia, ja, resd, m, l, k, gh, im, jm, nbentry, coefdiag, 0.0, 0);
}
int bcg_computejacobianfromjv_withjn(double* jac, int* ia, int* ja, const double* resd, int m, int l, int k, int gh,
                                     int im, int jm, long long nbentry) {
  return jac_call(JAC_WITHJN, jac, ia, ja, resd, m, l, k, gh, im, jm, nbentry, nullptr, 0.0, 0);
}
int bcg_computejacobianfromjv_relaxed_withjnandcheck(double* jac, int* ia, int* ja, const double* resd, int m, int l,
                                                     int k, int gh, int im, int jm, long long nbentry,
                                                     const double* coefdiag, double mini, int n) {
  return jac_call(JAC_CHECK, jac, ia, ja, resd, m, l, k, gh, im, jm, nbentry, coefdiag, mini, n);
}
int bcg_computejacobianfromdz(double* jac, int* ia, int* ja, const double* dz, int m, int l, int k, int gh, int im,
                              int jm, long long nbentry) {
  return jac_call(JAC_DZ, jac, ia, ja, dz, m, l, k, gh, im, jm, nbentry, nullptr, 0.0, 0);
}

// ---- norms (srcfv/norm.F90:2-127) ------------------------------------------
int bcg_compute_norml2(double* norm, double* nmoy, const double* rhs, int im, int jm, int gh) {
  return norm_call(NORM_L2, norm, nmoy, nullptr, nullptr, rhs, im, jm, gh);
}
int bcg_compute_norml2inf(double* norm, double* ninf, const double* rhs, int im, int jm, int gh) {
  return norm_call(NORM_L2INF, norm, ninf, nullptr, nullptr, rhs, im, jm, gh);
}
int bcg_compute_maxnorm(double* norm, int* imax, int* jmax, const double* rhs, int im, int jm, int gh) {
  return norm_call(NORM_MAX, norm, nullptr, imax, jmax, rhs, im, jm, gh);
}
}  // extern "C"

// ===========================================================================
// Batched colored Jacobian of the boundary-layer configuration
// (BROADCAST_npz.py:1068-1137, 1206-1210; misc/PETSc_func.py:71-96)
// ===========================================================================
namespace {
int jacobian_outputs(JacobianArgs& a, Stager& sg, int* indptr, int* indices, double* data, long long capacity,
                     long long* nnz);

int jacobian_bl_csr(int op, const double* w, const double* nx, const double* ny, const double* vol,
                    const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz,
                    double cs, double muref, double tref, double s_suth, double k2, double k4, int im, int jm,
                    const int* interf_ilo, const int* interf_jhi, const int* interf_ihi, const int* interf_jlo,
                    const double* field, int lm_field, const double* wbd, int lm_wbd, const double* coefdiag,
                    double mini, int divide_by_vol, int* indptr, int* indices, double* data, long long capacity,
                    long long* nnz) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (!dims_ok(im, jm, gh)) return fail_arg("jacobian: need gh == 3 and im, jm >= 6");
  if (!nnz || !interf_ilo || !interf_jhi || !interf_ihi || !interf_jlo) return fail_arg("jacobian: null argument");
  const size_t np = ncell(im, jm, gh), nn = nnode(im, jm, gh);
  cudaStream_t st = current_stream();
  Stager sg(st);
  const int hw = sg.in(w, np * 5 * 8), hnx = sg.in(nx, nn * 2 * 8), hny = sg.in(ny, nn * 2 * 8);
  const int hvol = sg.in(vol, np * 8), hvolf = sg.in(volf, np * 2 * 8);
  const int hf = sg.in(field, (size_t)lm_field * gh * 5 * 8), hb = sg.in(wbd, (size_t)lm_wbd * 5 * 8);
  const int hc = coefdiag ? sg.in(coefdiag, (size_t)im * jm * 8) : -1;
  int rc = sg.commit();
  if (rc) return rc;
  JacobianArgs a{};
  a.im = im; a.jm = jm; a.gh = gh;
  a.phys = Phys{cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4};
  a.w = sg.dev<double>(hw); a.nx = sg.dev<double>(hnx); a.ny = sg.dev<double>(hny);
  a.vol = sg.dev<double>(hvol); a.volf = sg.dev<double>(hvolf);
  a.op = op;
  a.relaxed = coefdiag ? 1 : 0;
  a.coefdiag = hc >= 0 ? sg.dev<double>(hc) : nullptr;
  a.mini = mini; a.divide_by_vol = divide_by_vol; a.capacity = capacity; a.nnz = nnz;
  // boundary chain of the boundary-layer drivers (BROADCAST_npz.py:1079-1082)
  const struct { int kind; const char* loc; const int* it; const double* aux; int lm; } chain[4] = {
      {BC_INLET, "Ilo", interf_ilo, sg.dev<double>(hf), lm_field}, {BC_NOREF, "Jhi", interf_jhi, sg.dev<double>(hb), lm_wbd},
      {BC_EXTRAP, "Ihi", interf_ihi, nullptr, 0}, {BC_WALL, "Jlo", interf_jlo, nullptr, 0}};
  for (const auto& c : chain) {
    BcArgs b{};
    b.kind = c.kind; b.im = im; b.jm = jm; b.gh = gh; b.em = 5; b.lm = c.lm; b.gam = gam; b.aux = c.aux;
    b.nx = a.nx; b.ny = a.ny;
    if (!make_side(c.loc, c.it, &b.side) || !side_in_bounds(b.side, im, jm, gh))
      return fail_arg("jacobian: bad interface");
    a.bcs.push_back(b);
  }
  return jacobian_outputs(a, sg, indptr, indices, data, capacity, nnz);
}

// scratch, run and CSR outputs (host or device) of a prepared batched assembly
int jacobian_outputs(JacobianArgs& a, Stager& sg, int* indptr, int* indices, double* data, long long capacity,
                     long long* nnz) {
  const int im = a.im, jm = a.jm, gh = a.gh, nrow = 5 * im * jm;
  cudaStream_t st = current_stream();
  int rc = 0;
  a.scratch = (double*)pool_get(POOL_SCRATCH, jacobian_scratch_doubles(im, jm, gh, a.nzone == 2 ? 2 : 1) * 8);
  if (!a.scratch) return fail_arg("jacobian: scratch allocation failed"), BCG_ERR_NOMEM;
  a.iscratch = (int*)pool_get(POOL_AUX, jacobian_iscratch_ints(im, jm) * 4);
  if (!a.iscratch) return fail_arg("jacobian: scratch allocation failed"), BCG_ERR_NOMEM;
  // outputs: used in place when on the device, else produced in a device buffer
  const bool dev_out = is_device_ptr(indptr) && is_device_ptr(indices) && is_device_ptr(data);
  if (dev_out) {
    a.indptr = indptr; a.indices = indices; a.data = data;
    rc = run_jacobian(a, st);
    if (rc) return rc;
    return sg.finish();
  }
  // host outputs: the device copy is sized to the worst case, 245 entries per
  // row and zone
  const long long cap = (long long)nrow * 245 * (a.nzone == 2 ? 2 : 1);
  char* ob = (char*)pool_get(POOL_STAGE_OUT, (size_t)(nrow + 1) * 4 + (size_t)cap * 12 + 512);
  if (!ob) return fail_arg("jacobian: output allocation failed"), BCG_ERR_NOMEM;
  a.indptr = (int*)ob;
  a.indices = (int*)(ob + (((size_t)(nrow + 1) * 4 + 255) & ~(size_t)255));
  a.data = (double*)((char*)a.indices + (((size_t)cap * 4 + 255) & ~(size_t)255));
  a.capacity = cap;
  rc = run_jacobian(a, st);
  if (rc) return rc;
  if (*nnz > capacity) return fail_arg("jacobian: CSR capacity too small (see nnz)");
  cudaError_t e = cudaMemcpyAsync(indptr, a.indptr, (size_t)(nrow + 1) * 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(indices, a.indices, (size_t)*nnz * 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(data, a.data, (size_t)*nnz * 8, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail_cuda("jacobian: output copy", e);
  return sg.finish();
}
}  // namespace

extern "C" int bcg_jacobian_dnc5_bl_csr(const double* w, const double* nx, const double* ny, const double* vol,
                                        const double* volf, int gh, double cp, double cv, double prandtl, double gam,
                                        double rgaz, double cs, double muref, double tref, double s_suth, double k2,
                                        double k4, int im, int jm, const int* interf_ilo, const int* interf_jhi,
                                        const int* interf_ihi, const int* interf_jlo, const double* field,
                                        int lm_field, const double* wbd, int lm_wbd, const double* coefdiag,
                                        double mini, int divide_by_vol, int* indptr, int* indices, double* data,
                                        long long capacity, long long* nnz) {
  return jacobian_bl_csr(0, w, nx, ny, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4, im,
                         jm, interf_ilo, interf_jhi, interf_ihi, interf_jlo, field, lm_field, wbd, lm_wbd, coefdiag,
                         mini, divide_by_vol, indptr, indices, data, capacity, nnz);
}

// Batched assembly for the periodic O-mesh of cylinder.py:900-980: seeds,
// the tangent boundary chain of handleBC.applyBC (no-reflexion Jhi, wall Jlo,
// then the two periodic joins twice), flux_num_dnc5_2d_d and
// computejacobianfromjv[_relaxed]_withjn (columns wrap in i), CSR.
extern "C" int bcg_jacobian_dnc5_cyl_csr(const double* w, const double* nx, const double* ny, const double* vol,
                                         const double* volf, int gh, double cp, double cv, double prandtl,
                                         double gam, double rgaz, double cs, double muref, double tref,
                                         double s_suth, double k2, double k4, int im, int jm, const int* interf_jhi,
                                         const int* interf_jlo, const double* wbd, int lm_wbd, const int* prr1,
                                         const int* prd1, const int* prr2, const int* prd2, const int* tr,
                                         const double* coefdiag, double mini, int divide_by_vol, int* indptr,
                                         int* indices, double* data, long long capacity, long long* nnz) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (!dims_ok(im, jm, gh)) return fail_arg("jacobian: need gh == 3 and im, jm >= 6");
  if (!nnz || !interf_jhi || !interf_jlo || !prr1 || !prd1 || !prr2 || !prd2 || !tr)
    return fail_arg("jacobian: null argument");
  const size_t np = ncell(im, jm, gh), nn = nnode(im, jm, gh);
  cudaStream_t st = current_stream();
  Stager sg(st);
  const int hw = sg.in(w, np * 5 * 8), hnx = sg.in(nx, nn * 2 * 8), hny = sg.in(ny, nn * 2 * 8);
  const int hvol = sg.in(vol, np * 8), hvolf = sg.in(volf, np * 2 * 8);
  const int hb = sg.in(wbd, (size_t)lm_wbd * 5 * 8);
  const int hc = coefdiag ? sg.in(coefdiag, (size_t)im * jm * 8) : -1;
  int rc = sg.commit();
  if (rc) return rc;
  JacobianArgs a{};
  a.im = im; a.jm = jm; a.gh = gh;
  a.phys = Phys{cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4};
  a.w = sg.dev<double>(hw); a.nx = sg.dev<double>(hnx); a.ny = sg.dev<double>(hny);
  a.vol = sg.dev<double>(hvol); a.volf = sg.dev<double>(hvolf);
  a.op = 0; a.withjn = 1;
  // im not a multiple of the colour step: the driver's two azimuthal zones
  // (cylinder.py:899-938, Nzones), so that no colour has two seeds within a
  // stencil of each other across the periodic join
  if (im % (2 * gh + 1) != 0) { a.nzone = 2; a.imid = im / 2 / (2 * gh + 1) * (2 * gh + 1); }
  else a.nzone = 1;
  a.relaxed = coefdiag ? 1 : 0;
  a.coefdiag = hc >= 0 ? sg.dev<double>(hc) : nullptr;
  a.mini = mini; a.divide_by_vol = divide_by_vol; a.capacity = capacity; a.nnz = nnz;
  const struct { int kind; const char* loc; const int* it; const double* aux; int lm; } chain[2] = {
      {BC_NOREF, "Jhi", interf_jhi, sg.dev<double>(hb), lm_wbd}, {BC_WALL, "Jlo", interf_jlo, nullptr, 0}};
  for (const auto& c : chain) {
    BcArgs b{};
    b.kind = c.kind; b.im = im; b.jm = jm; b.gh = gh; b.em = 5; b.lm = c.lm; b.gam = gam; b.aux = c.aux;
    b.nx = a.nx; b.ny = a.ny;
    if (!make_side(c.loc, c.it, &b.side) || !side_in_bounds(b.side, im, jm, gh))
      return fail_arg("jacobian: bad interface");
    a.bcs.push_back(b);
  }
  JnArgs j1{}, j2{};
  rc = jn_args(prr1, gh, gh, gh, gh, im, jm, prd2, gh, gh, gh, gh, im, jm, tr, 5, &j1);
  if (rc) return rc;
  rc = jn_args(prr2, gh, gh, gh, gh, im, jm, prd1, gh, gh, gh, gh, im, jm, tr, 5, &j2);
  if (rc) return rc;
  for (int rep = 0; rep < 2; ++rep) { a.joins.push_back(j1); a.joins.push_back(j2); }
  return jacobian_outputs(a, sg, indptr, indices, data, capacity, nnz);
}

extern "C" int bcg_jacobian_dz_bl_csr(const double* w, const double* nx, const double* ny, const double* vol,
                                      const double* volf, int gh, double cp, double cv, double prandtl, double gam,
                                      double rgaz, double cs, double muref, double tref, double s_suth, int im, int jm,
                                      const int* interf_ilo, const int* interf_jhi, const int* interf_ihi,
                                      const int* interf_jlo, const double* field, int lm_field, const double* wbd,
                                      int lm_wbd, int which, double mini, int* indptr, int* indices, double* data,
                                      long long capacity, long long* nnz) {
  if (which != 1 && which != 2) return fail_arg("jacobian_dz: which must be 1 (Dz) or 2 (Dzz)");
  return jacobian_bl_csr(which == 1 ? SPAN_DZ : SPAN_DZZ, w, nx, ny, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs,
                         muref, tref, s_suth, 0.0, 0.0, im, jm, interf_ilo, interf_jhi, interf_ihi, interf_jlo, field,
                         lm_field, wbd, lm_wbd, nullptr, mini, 0, indptr, indices, data, capacity, nnz);
}

// ---- J, Dz and Dzz from one pass over the seeds, J(beta) as the epilogue ------
// (BROADCAST_npz.py:1068-1137 and 1221-1249, biglobal.py:82): the seeds and
// their linearised boundary chain once, then the residual tangent and both
// spanwise operators of every seeded state; device outputs only.
extern "C" int bcg_jacobian_span_bl_csr(const double* w, const double* nx, const double* ny, const double* vol,
                                        const double* volf, int gh, double cp, double cv, double prandtl, double gam,
                                        double rgaz, double cs, double muref, double tref, double s_suth, double k2,
                                        double k4, int im, int jm, const int* interf_ilo, const int* interf_jhi,
                                        const int* interf_ihi, const int* interf_jlo, const double* field,
                                        int lm_field, const double* wbd, int lm_wbd, double mini, int divide_by_vol,
                                        const unsigned long long* indptr3, const unsigned long long* indices3,
                                        const unsigned long long* data3, const long long* capacity3, long long* nnz3,
                                        int nbeta, const double* betas, int* b_indptr, int* b_indices,
                                        double* b_values, long long b_capacity, long long* b_nnz) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (!dims_ok(im, jm, gh)) return fail_arg("jacobian: need gh == 3 and im, jm >= 6");
  if (!indptr3 || !indices3 || !data3 || !capacity3 || !nnz3 || !interf_ilo || !interf_jhi || !interf_ihi ||
      !interf_jlo)
    return fail_arg("jacobian_span: null argument");
  for (int k = 0; k < 3; ++k)
    if (!is_device_ptr((const void*)indptr3[k]) || !is_device_ptr((const void*)indices3[k]) ||
        !is_device_ptr((const void*)data3[k]))
      return fail_arg("jacobian_span: the CSR outputs must be device arrays");
  if (nbeta > 0 && (!betas || !b_nnz || !is_device_ptr(b_indptr) || !is_device_ptr(b_indices) ||
                    !is_device_ptr(b_values)))
    return fail_arg("jacobian_span: J(beta) needs host betas and device outputs");
  const size_t np = ncell(im, jm, gh), nn = nnode(im, jm, gh);
  cudaStream_t st = current_stream();
  Stager sg(st);
  const int hw = sg.in(w, np * 5 * 8), hnx = sg.in(nx, nn * 2 * 8), hny = sg.in(ny, nn * 2 * 8);
  const int hvol = sg.in(vol, np * 8), hvolf = sg.in(volf, np * 2 * 8);
  const int hf = sg.in(field, (size_t)lm_field * gh * 5 * 8), hb = sg.in(wbd, (size_t)lm_wbd * 5 * 8);
  int rc = sg.commit();
  if (rc) return rc;
  JacobianArgs a{};
  a.im = im; a.jm = jm; a.gh = gh;
  a.phys = Phys{cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4};
  a.w = sg.dev<double>(hw); a.nx = sg.dev<double>(hnx); a.ny = sg.dev<double>(hny);
  a.vol = sg.dev<double>(hvol); a.volf = sg.dev<double>(hvolf);
  a.relaxed = 0; a.coefdiag = nullptr; a.mini = mini;
  a.nops = 3;
  const int ops[3] = {0, SPAN_DZ, SPAN_DZZ};
  for (int k = 0; k < 3; ++k) {
    a.ops[k] = ops[k];
    a.divide_v[k] = k == 0 ? divide_by_vol : 0;
    a.indptr_v[k] = (int*)indptr3[k]; a.indices_v[k] = (int*)indices3[k]; a.data_v[k] = (double*)data3[k];
    a.capacity_v[k] = capacity3[k]; a.nnz_v[k] = nnz3 + k;
  }
  const struct { int kind; const char* loc; const int* it; const double* aux; int lm; } chain[4] = {
      {BC_INLET, "Ilo", interf_ilo, sg.dev<double>(hf), lm_field}, {BC_NOREF, "Jhi", interf_jhi, sg.dev<double>(hb), lm_wbd},
      {BC_EXTRAP, "Ihi", interf_ihi, nullptr, 0}, {BC_WALL, "Jlo", interf_jlo, nullptr, 0}};
  for (const auto& c : chain) {
    BcArgs b{};
    b.kind = c.kind; b.im = im; b.jm = jm; b.gh = gh; b.em = 5; b.lm = c.lm; b.gam = gam; b.aux = c.aux;
    b.nx = a.nx; b.ny = a.ny;
    if (!make_side(c.loc, c.it, &b.side) || !side_in_bounds(b.side, im, jm, gh))
      return fail_arg("jacobian_span: bad interface");
    a.bcs.push_back(b);
  }
  a.scratch = (double*)pool_get(POOL_SCRATCH, jacobian_scratch_doubles(im, jm, gh, 1, 3) * 8);
  a.iscratch = (int*)pool_get(POOL_AUX, jacobian_iscratch_ints(im, jm) * 4);
  if (!a.scratch || !a.iscratch) return fail_arg("jacobian_span: scratch allocation failed"), BCG_ERR_NOMEM;
  rc = run_jacobian(a, st);
  if (rc) return rc;
  if (nbeta > 0) {
    const int nrow = 5 * im * jm;
    CsrBetaArgs ba{};
    ba.nrow = nrow;
    ba.j_p = a.indptr_v[0]; ba.j_i = a.indices_v[0]; ba.j_v = a.data_v[0];
    ba.dz_p = a.indptr_v[1]; ba.dz_i = a.indices_v[1]; ba.dz_v = a.data_v[1];
    ba.dzz_p = a.indptr_v[2]; ba.dzz_i = a.indices_v[2]; ba.dzz_v = a.data_v[2];
    ba.nbeta = nbeta;
    double* dbeta = (double*)pool_get(POOL_STAGE_OUT, (size_t)nbeta * 8);
    int* bscr = (int*)pool_get(POOL_AUX, csr_beta_iscratch_ints(nrow) * 4);
    if (!dbeta || !bscr) return fail_arg("jacobian_span: scratch allocation failed"), BCG_ERR_NOMEM;
    cudaError_t e = cudaMemcpyAsync(dbeta, betas, (size_t)nbeta * 8, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return fail_cuda("jacobian_span: betas", e);
    ba.betas = dbeta; ba.indptr = b_indptr; ba.indices = b_indices; ba.values = b_values; ba.capacity = b_capacity;
    ba.nnz = b_nnz; ba.iscratch = bscr;
    rc = run_csr_beta(ba, st);
    if (rc) return rc;
  }
  return sg.finish();
}

// ---- J(beta) = J - beta^2 Dzz + i beta Dz (biglobal.py:82) -------------------
// Three CSR matrices of nrow rows (sorted columns) combine on the union of
// their patterns for nbeta wavenumbers; values hold nbeta planes of nnz complex
// numbers (re, im interleaved), plane k at values + 2*k*nnz.  Inputs and
// outputs may be host or device arrays.
namespace {
long long csr_nnz(const int* indptr, int nrow, cudaStream_t st, int* rc) {
  int v = 0;
  if (is_device_ptr(indptr)) {
    cudaError_t e = cudaMemcpyAsync(&v, indptr + nrow, sizeof v, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { *rc = fail_cuda("csr_spanwise_beta: indptr", e); return -1; }
  } else {
    v = indptr[nrow];
  }
  *rc = BCG_OK;
  return v;
}
}  // namespace

extern "C" int bcg_csr_spanwise_beta(int nrow, const int* j_indptr, const int* j_indices, const double* j_data,
                                     const int* dz_indptr, const int* dz_indices, const double* dz_data,
                                     const int* dzz_indptr, const int* dzz_indices, const double* dzz_data,
                                     int nbeta, const double* betas, int* indptr, int* indices, double* values,
                                     long long capacity, long long* nnz) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (nrow < 1 || nbeta < 1 || !betas || !nnz || !j_indptr || !dz_indptr || !dzz_indptr)
    return fail_arg("csr_spanwise_beta: bad arguments");
  cudaStream_t st = current_stream();
  int rc = 0;
  const long long nj = csr_nnz(j_indptr, nrow, st, &rc);
  if (rc) return rc;
  const long long nz = csr_nnz(dz_indptr, nrow, st, &rc);
  if (rc) return rc;
  const long long nzz = csr_nnz(dzz_indptr, nrow, st, &rc);
  if (rc) return rc;
  Stager sg(st);
  const size_t pb = (size_t)(nrow + 1) * 4;
  const int h1 = sg.in(j_indptr, pb), h2 = sg.in(j_indices, (size_t)nj * 4), h3 = sg.in(j_data, (size_t)nj * 8);
  const int h4 = sg.in(dz_indptr, pb), h5 = sg.in(dz_indices, (size_t)nz * 4), h6 = sg.in(dz_data, (size_t)nz * 8);
  const int h7 = sg.in(dzz_indptr, pb), h8 = sg.in(dzz_indices, (size_t)nzz * 4);
  const int h9 = sg.in(dzz_data, (size_t)nzz * 8), hb = sg.in(betas, (size_t)nbeta * 8);
  rc = sg.commit();
  if (rc) return rc;
  CsrBetaArgs a{};
  a.nrow = nrow;
  a.j_p = sg.dev<int>(h1); a.j_i = sg.dev<int>(h2); a.j_v = sg.dev<double>(h3);
  a.dz_p = sg.dev<int>(h4); a.dz_i = sg.dev<int>(h5); a.dz_v = sg.dev<double>(h6);
  a.dzz_p = sg.dev<int>(h7); a.dzz_i = sg.dev<int>(h8); a.dzz_v = sg.dev<double>(h9);
  a.nbeta = nbeta; a.betas = sg.dev<double>(hb); a.nnz = nnz;
  a.iscratch = (int*)pool_get(POOL_AUX, csr_beta_iscratch_ints(nrow) * 4);
  if (!a.iscratch) return fail_arg("csr_spanwise_beta: scratch allocation failed"), BCG_ERR_NOMEM;
  const bool dev_out = is_device_ptr(indptr) && is_device_ptr(indices) && is_device_ptr(values);
  if (dev_out) {
    a.indptr = indptr; a.indices = indices; a.values = values; a.capacity = capacity;
    rc = run_csr_beta(a, st);
    if (rc) return rc;
    return sg.finish();
  }
  // host outputs: device buffers sized to the sum of the three patterns
  const long long cap = nj + nz + nzz;
  const size_t ib = (((size_t)(nrow + 1) * 4 + 255) & ~(size_t)255), xb = (((size_t)cap * 4 + 255) & ~(size_t)255);
  char* ob = (char*)pool_get(POOL_STAGE_OUT, ib + xb + (size_t)cap * 16 * nbeta + 256);
  if (!ob) return fail_arg("csr_spanwise_beta: output allocation failed"), BCG_ERR_NOMEM;
  a.indptr = (int*)ob; a.indices = (int*)(ob + ib); a.values = (double*)(ob + ib + xb); a.capacity = cap;
  rc = run_csr_beta(a, st);
  if (rc) return rc;
  if (*nnz > capacity) return fail_arg("csr_spanwise_beta: capacity too small (see nnz)");
  cudaError_t e = cudaMemcpyAsync(indptr, a.indptr, (size_t)(nrow + 1) * 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(indices, a.indices, (size_t)*nnz * 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(values, a.values, (size_t)*nnz * 16 * nbeta, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail_cuda("csr_spanwise_beta: output copy", e);
  return sg.finish();
}

// ---- uneven batch of grids (no reference counterpart: one grid per process
// there) ----------------------------------------------------------------------
namespace {
std::mutex g_batch_mu;
std::map<long long, BatchPlan*> g_batches;
long long g_batch_next = 1;
BatchPlan* batch_of(long long id) {
  std::lock_guard<std::mutex> lk(g_batch_mu);
  auto it = g_batches.find(id);
  return it == g_batches.end() ? nullptr : it->second;
}
}  // namespace

extern "C" int bcg_batch_create(int ngrid, const int* im, const int* jm, const double* phys, int ndir,
                                long long* plan) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (!plan) return fail_arg("batch_create: null plan");
  BatchPlan* p = nullptr;
  int rc = batch_create(ngrid, im, jm, phys, ndir, &p);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(g_batch_mu);
  *plan = g_batch_next++;
  g_batches[*plan] = p;
  return BCG_OK;
}

extern "C" int bcg_batch_set_arrays(long long plan, const unsigned long long* w, const unsigned long long* wd,
                                    const unsigned long long* nx, const unsigned long long* ny,
                                    const unsigned long long* vol, const unsigned long long* volf,
                                    const unsigned long long* res, const unsigned long long* resd) {
  BatchPlan* p = batch_of(plan);
  if (!p) return fail_arg("batch: unknown plan");
  return batch_set_arrays(p, w, wd, nx, ny, vol, volf, res, resd);
}

extern "C" int bcg_batch_configure(long long plan, int tile_faces, int tile_cells, int ctas_per_sm) {
  BatchPlan* p = batch_of(plan);
  if (!p) return fail_arg("batch: unknown plan");
  return batch_configure(p, tile_faces, tile_cells, ctas_per_sm);
}

extern "C" int bcg_batch_configure_host(long long plan, int tile_faces, int tile_cells, int ctas_per_sm) {
  BatchPlan* p = batch_of(plan);
  if (!p) return fail_arg("batch: unknown plan");
  return batch_configure_host(p, tile_faces, tile_cells, ctas_per_sm);
}

extern "C" int bcg_batch_run(long long plan, int use_graph) {
  BatchPlan* p = batch_of(plan);
  if (!p) return fail_arg("batch: unknown plan");
  return batch_run(p, use_graph, current_stream());
}

extern "C" int bcg_batch_run_pass(long long plan, int pass) {
  BatchPlan* p = batch_of(plan);
  if (!p) return fail_arg("batch: unknown plan");
  return batch_run_pass(p, pass, current_stream());
}

extern "C" int bcg_batch_run_host(long long plan, int nchunk, const unsigned long long* w,
                                  const unsigned long long* wd, const unsigned long long* nx,
                                  const unsigned long long* ny, const unsigned long long* vol,
                                  const unsigned long long* volf, const unsigned long long* res,
                                  const unsigned long long* resd) {
  BatchPlan* p = batch_of(plan);
  if (!p) return fail_arg("batch: unknown plan");
  return batch_run_host(p, nchunk, w, wd, nx, ny, vol, volf, res, resd, current_stream());
}

extern "C" int bcg_batch_device_bytes(long long plan, long long* bytes) {
  BatchPlan* p = batch_of(plan);
  if (!p || !bytes) return fail_arg("batch: unknown plan");
  *bytes = (long long)batch_device_bytes(p);
  return BCG_OK;
}

extern "C" int bcg_batch_destroy(long long plan) {
  BatchPlan* p = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_batch_mu);
    auto it = g_batches.find(plan);
    if (it == g_batches.end()) return fail_arg("batch: unknown plan");
    p = it->second;
    g_batches.erase(it);
  }
  cudaError_t e = cudaStreamSynchronize(current_stream());
  batch_destroy(p);
  return e == cudaSuccess ? BCG_OK : fail_cuda("batch_destroy", e);
}

// ===========================================================================
// Newton-Krylov solves (krylov.cu): FP32 band LU preconditioner, FP64 GMRES
// ===========================================================================
extern "C" int bcg_band32_factor(int n, const int* indptr, const int* indices, const double* data, const int* perm,
                                 int nb, long long* handle, int* info) {
  if (!has_device()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  const void* arrs[3] = {indptr, indices, data};
  for (const void* a : arrs)
    if (!a || !is_device_ptr(a)) return fail_arg("band32_factor: CSR arrays must be device pointers");
  if (perm && !is_device_ptr(perm)) return fail_arg("band32_factor: perm must be a device pointer");
  return band32_factor(n, indptr, indices, data, perm, nb, current_stream(), handle, info);
}

extern "C" int bcg_band32_solve(long long handle, const double* b, double* x) {
  if (!b || !x || !is_device_ptr(b) || !is_device_ptr(x)) return fail_arg("band32_solve: device vectors expected");
  return band32_solve(handle, b, x, current_stream());
}

extern "C" int bcg_band32_dims(long long handle, int* klku_nb) { return band32_dims(handle, klku_nb); }

extern "C" int bcg_band32_destroy(long long handle) { return band32_destroy(handle); }

extern "C" int bcg_gmres_solve(long long handle, int n, const int* indptr, const int* indices, const double* data,
                               const double* b, double* x, int restart, int maxit, double rtol, int* iters,
                               double* relres) {
  const void* arrs[5] = {indptr, indices, data, b, x};
  for (const void* a : arrs)
    if (!a || !is_device_ptr(a)) return fail_arg("gmres_solve: every array must be a device pointer");
  return gmres_solve(handle, n, indptr, indices, data, b, x, restart, maxit, rtol, current_stream(), iters, relres);
}

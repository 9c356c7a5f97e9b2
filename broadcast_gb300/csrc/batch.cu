// Residual (+ tangent) of many independent grids of uneven size, GB300 style.
//
// The reference runs one grid per process (BROADCAST_npz.py); a batch of
// boundary-layer instances of different sizes would leave most of a GB300
// idle per grid.  Here every pass of the DNC5 residual (primitives, Ducros
// gradients, interpolation rows, viscous point values, faces, balance; the same per-element bodies
// as the single-grid kernels, passes.cuh) is ONE persistent launch over a
// tile list that concatenates the tiles of all grids: each CTA walks tiles
// t = blockIdx.x, blockIdx.x + gridDim.x, ...; a tile belongs to one grid,
// found by binary search in the pass's tile-start table, whose descriptor
// (extents, coefficients, array addresses, scratch) the CTA stages in shared
// memory.  The launches can be captured once in a CUDA graph and replayed.
// Tile sizes and CTAs per SM are plan parameters, chosen by the autotuner in
// broadcast_gb300/batch.py.
#include <algorithm>
#include <vector>
#include "batch.h"
#include "passes.cuh"
#include "residual.h"
#include "runtime.h"

namespace bcg {

namespace {

enum { P_PRIM = 0, P_GRAD, P_QROWS, P_VPTS, P_FACES, P_BAL, NPASS };

struct GridDesc {
  Ext e;
  Coef c;
  const double* w;
  const double* wd;
  size_t dstride;
  const double* nx;
  const double* ny;
  const double* vol;
  const double* volf;
  double* res;
  double* resd;
  double* scratch;  // residual_scratch_doubles(im, jm, 3, K) doubles
  int grad;         // k2 != 0: the sensor pass is needed
};

template <class S>
struct Fields {
  Scratch<S> pr, gr, qr, hn;
};
template <class S>
BCG_HD Fields<S> fields_of(const GridDesc& G) {
  constexpr int NP = NDir<S>::value + 1;
  const Ext& e = G.e;
  const size_t nn = (size_t)(e.im + 1) * (e.jm + 1);
  Fields<S> f;
  f.pr = Scratch<S>{G.scratch, e.np};
  f.gr = Scratch<S>{G.scratch + (size_t)F_NPRIM * NP * e.np, e.np};
  f.qr = Scratch<S>{G.scratch + (size_t)(F_NPRIM + S_NSENS) * NP * e.np, e.np};
  f.hn = Scratch<S>{G.scratch + (size_t)(F_NPRIM + S_NSENS + Q_NQ) * NP * e.np, nn};
  return f;
}
template <class S> BCG_HD State<S> state_of(const GridDesc& G);
template <> BCG_HD State<double> state_of<double>(const GridDesc& G) { return State<double>{G.w}; }
template <> BCG_HD State<DK<1>> state_of<DK<1>>(const GridDesc& G) { return State<DK<1>>{G.w, G.wd, G.dstride}; }

// grid of tile t: the largest g with starts[g] <= t (starts has ngrid + 1 entries)
__device__ __forceinline__ int tile_grid(const long long* __restrict__ starts, int ngrid, long long t) {
  int lo = 0, hi = ngrid - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (starts[mid] <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// per grid (blockIdx.y): the count of warps that met a nonzero i-face ny or
// j-face nx component; zero means the grid is rectilinear
__global__ void __launch_bounds__(256) k_batch_rect(const GridDesc* __restrict__ descs, unsigned* __restrict__ rectnz) {
  const GridDesc& G = descs[blockIdx.y];
  const size_t nn = G.e.nn();
  unsigned bad = 0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += (size_t)gridDim.x * blockDim.x)
    bad |= (G.ny[k] != 0.0) | (G.nx[nn + k] != 0.0);
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicAdd(rectnz + blockIdx.y, 1u);
}

template <class S, int PASS, int BT>
__global__ void __launch_bounds__(BT) k_batch(const GridDesc* __restrict__ descs, const long long* __restrict__ starts,
                                              int ngrid, const unsigned* __restrict__ rectnz) {
  const long long* st = starts + (size_t)PASS * (ngrid + 1);
  const long long T = st[ngrid];
  __shared__ int s_g, s_rect;
  __shared__ FaceCtx<S> s_fc;           // curvilinear grids
  __shared__ FaceCtx<S, 3, true> s_fcr;  // rectilinear grids: the face kernel without the zero metric products
  __shared__ Scratch<S> s_hn;
  for (long long t = blockIdx.x; t < T; t += gridDim.x) {
    __syncthreads();  // the previous tile is done with the shared descriptor
    if (threadIdx.x == 0) {
      const int g = tile_grid(st, ngrid, t);
      s_g = g;
      if constexpr (PASS == P_FACES) {
        const GridDesc& G = descs[g];
        const Fields<S> f = fields_of<S>(G);
        auto fill = [&](auto& fc) {
          fc.e = G.e; fc.c = G.c; fc.w = state_of<S>(G);
          fc.pr = f.pr; fc.gr = f.gr; fc.qr = f.qr;
          fc.nx = G.nx; fc.ny = G.ny; fc.vol = G.vol; fc.volf = G.volf;
        };
        s_rect = rectnz[g] == 0;
        if (s_rect) fill(s_fcr); else fill(s_fc);
        s_hn = f.hn;
      }
    }
    __syncthreads();
    const int g = s_g;
    const long long el = (t - st[g]) * BT + threadIdx.x;
    if constexpr (PASS == P_FACES) {
      if (s_rect) {
        const Ext& e = s_fcr.e;
        if (el < (long long)(e.im + 1) * (e.jm + 1)) face_node<S, 3, true>(s_fcr, s_hn, (int)el);
      } else {
        const Ext& e = s_fc.e;
        if (el < (long long)(e.im + 1) * (e.jm + 1)) face_node<S>(s_fc, s_hn, (int)el);
      }
    } else {
      const GridDesc& G = descs[g];
      const Ext& e = G.e;
      const Fields<S> f = fields_of<S>(G);
      if constexpr (PASS == P_PRIM) {
        if (el < (long long)e.np) prim_cell<S>(e, G.c, state_of<S>(G), f.pr, (size_t)el);
      } else if constexpr (PASS == P_QROWS) {
        if (el < (long long)e.np) qrows_cell<S>(e, f.pr, f.qr, (size_t)el);
      } else if constexpr (PASS == P_VPTS) {
        if (el < (long long)e.np) vpts_cell<S>(e, f.qr, (size_t)el);
      } else if constexpr (PASS == P_GRAD) {
        if (el < (long long)(e.im + 2) * (e.jm + 2)) sensor_cell<S>(e, G.c, f.pr, f.gr, G.nx, G.ny, G.vol, (int)el);
      } else {
        if (el < (long long)e.im * e.jm) balance_cell<S>(e, f.hn, G.res, G.resd, G.dstride, (int)el);
      }
    }
  }
}

}  // namespace

struct BatchPlan {
  int ngrid = 0, K = 0;
  std::vector<GridDesc> h;
  GridDesc* d = nullptr;
  long long* dstarts = nullptr;
  double* scratch = nullptr;
  size_t scratch_doubles = 0;
  int tile_faces = 128, tile_cells = 256, ctas = 2, nsm = 0;
  int host_tile[3] = {0, 0, 0};  // tile shapes of the host-run chunk plans (0: the plan's own)
  long long ntiles[NPASS] = {0, 0, 0, 0, 0, 0};
  bool any_grad = false;
  cudaStream_t cap = nullptr;  // capture stream (the caller's may be the legacy default stream)
  cudaGraphExec_t exec = nullptr;
  bool owns_scratch = true;
  unsigned* rectnz = nullptr;  // per grid: nonzero i-face ny / j-face nx count of the last evaluation (0: rectilinear)
  bool owns_rectnz = true;
  // host-array runs (batch_run_host): device mirrors of every grid's arrays,
  // and the grids split into contiguous chunks, each a child plan over the
  // mirrors that shares this plan's scratch
  double* mirror = nullptr;
  std::vector<size_t> moff;          // per grid: offset of its mirrors (MIR_* order)
  std::vector<BatchPlan*> chunks;
  std::vector<int> chunk_lo;         // first grid of each chunk, then ngrid
  cudaStream_t hs[4] = {nullptr, nullptr, nullptr, nullptr};  // upload, download, two compute streams
  std::vector<cudaEvent_t> hev;      // start, per chunk uploaded, per chunk computed, downloads done
};

static long long pass_count(const Ext& e, int pass, bool grad) {
  switch (pass) {
    case P_PRIM: case P_QROWS: case P_VPTS: return (long long)e.np;
    case P_GRAD: return grad ? (long long)(e.im + 2) * (e.jm + 2) : 0;
    case P_FACES: return (long long)(e.im + 1) * (e.jm + 1);
    default: return (long long)e.im * e.jm;
  }
}

static int upload_starts(BatchPlan* p) {
  const int n = p->ngrid;
  std::vector<long long> st((size_t)NPASS * (n + 1));
  for (int pass = 0; pass < NPASS; ++pass) {
    const int bt = pass == P_FACES ? p->tile_faces : p->tile_cells;
    long long acc = 0;
    for (int g = 0; g < n; ++g) {
      st[(size_t)pass * (n + 1) + g] = acc;
      acc += (pass_count(p->h[g].e, pass, p->h[g].grad != 0) + bt - 1) / bt;
    }
    st[(size_t)pass * (n + 1) + n] = acc;
    p->ntiles[pass] = acc;
  }
  cudaError_t e = cudaMemcpy(p->dstarts, st.data(), st.size() * sizeof(long long), cudaMemcpyHostToDevice);
  return e == cudaSuccess ? BCG_OK : fail_cuda("batch: tile table", e);
}

int batch_create(int ngrid, const int* im, const int* jm, const double* phys, int ndir, BatchPlan** out) {
  if (ngrid < 1 || !im || !jm || !phys || !out) return fail_arg("batch: bad arguments");
  if (ndir != 0 && ndir != 1) return fail_arg("batch: ndir must be 0 or 1");
  BatchPlan* p = new BatchPlan();
  p->ngrid = ngrid; p->K = ndir;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&p->nsm, cudaDevAttrMultiProcessorCount, dev);
  p->h.resize(ngrid);
  std::vector<size_t> off(ngrid);
  for (int g = 0; g < ngrid; ++g) {
    if (im[g] < 6 || jm[g] < 6) { delete p; return fail_arg("batch: every grid needs im, jm >= 6"); }
    GridDesc& G = p->h[g];
    G = GridDesc{};
    G.e = make_ext(im[g], jm[g], 3);
    const double* ph = phys + (size_t)11 * g;
    const Phys P{ph[0], ph[1], ph[2], ph[3], ph[4], ph[5], ph[6], ph[7], ph[8], ph[9], ph[10]};
    G.c = make_coef(P);
    G.grad = (P.k2 != 0.0) ? 1 : 0;
    p->any_grad = p->any_grad || G.grad;
    G.dstride = G.e.np * 5;
    off[g] = p->scratch_doubles;
    p->scratch_doubles += (residual_scratch_doubles(im[g], jm[g], 3, ndir) + 31) & ~(size_t)31;
  }
  cudaError_t e = cudaMalloc(&p->scratch, p->scratch_doubles * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&p->d, sizeof(GridDesc) * ngrid);
  if (e == cudaSuccess) e = cudaMalloc(&p->dstarts, sizeof(long long) * NPASS * (ngrid + 1));
  if (e == cudaSuccess) e = cudaMalloc(&p->rectnz, sizeof(unsigned) * ngrid);
  if (e == cudaSuccess) e = cudaMemset(p->rectnz, 0xff, sizeof(unsigned) * ngrid);  // curvilinear until checked
  if (e != cudaSuccess) { batch_destroy(p); return fail_cuda("batch: device allocation", e), BCG_ERR_NOMEM; }
  for (int g = 0; g < ngrid; ++g) p->h[g].scratch = p->scratch + off[g];
  int rc = upload_starts(p);
  if (rc) { batch_destroy(p); return rc; }
  *out = p;
  return BCG_OK;
}

int batch_set_arrays(BatchPlan* p, const unsigned long long* w, const unsigned long long* wd,
                     const unsigned long long* nx, const unsigned long long* ny, const unsigned long long* vol,
                     const unsigned long long* volf, const unsigned long long* res, const unsigned long long* resd) {
  if (!w || !nx || !ny || !vol || !volf || !res || (p->K && (!wd || !resd))) return fail_arg("batch: null array table");
  for (int g = 0; g < p->ngrid; ++g) {
    GridDesc& G = p->h[g];
    G.w = (const double*)w[g]; G.wd = p->K ? (const double*)wd[g] : nullptr;
    G.nx = (const double*)nx[g]; G.ny = (const double*)ny[g];
    G.vol = (const double*)vol[g]; G.volf = (const double*)volf[g];
    G.res = (double*)res[g]; G.resd = p->K ? (double*)resd[g] : nullptr;
    const void* ptrs[8] = {G.w, G.nx, G.ny, G.vol, G.volf, G.res, p->K ? G.wd : G.w, p->K ? G.resd : G.res};
    for (const void* q : ptrs)
      if (!is_device_ptr(q)) return fail_arg("batch: every array must be a device pointer");
  }
  cudaError_t e = cudaMemcpy(p->d, p->h.data(), sizeof(GridDesc) * p->ngrid, cudaMemcpyHostToDevice);
  return e == cudaSuccess ? BCG_OK : fail_cuda("batch: descriptors", e);
}

static int check_tiles(int tile_faces, int tile_cells, int ctas_per_sm) {
  if (tile_faces != 64 && tile_faces != 128 && tile_faces != 256) return fail_arg("batch: tile_faces must be 64, 128 or 256");
  if (tile_cells != 128 && tile_cells != 256) return fail_arg("batch: tile_cells must be 128 or 256");
  if (ctas_per_sm < 1 || ctas_per_sm > 8) return fail_arg("batch: ctas_per_sm must be 1..8");
  return BCG_OK;
}

int batch_configure(BatchPlan* p, int tile_faces, int tile_cells, int ctas_per_sm) {
  int rc = check_tiles(tile_faces, tile_cells, ctas_per_sm);
  if (rc) return rc;
  p->tile_faces = tile_faces; p->tile_cells = tile_cells; p->ctas = ctas_per_sm;
  if (p->exec) { cudaGraphExecDestroy(p->exec); p->exec = nullptr; }
  if (!p->host_tile[0])  // the chunk plans follow unless they have shapes of their own
    for (BatchPlan* c : p->chunks) {
      rc = batch_configure(c, tile_faces, tile_cells, ctas_per_sm);
      if (rc) return rc;
    }
  return upload_starts(p);
}

int batch_configure_host(BatchPlan* p, int tile_faces, int tile_cells, int ctas_per_sm) {
  int rc = check_tiles(tile_faces, tile_cells, ctas_per_sm);
  if (rc) return rc;
  p->host_tile[0] = tile_faces; p->host_tile[1] = tile_cells; p->host_tile[2] = ctas_per_sm;
  for (BatchPlan* c : p->chunks) {
    rc = batch_configure(c, tile_faces, tile_cells, ctas_per_sm);
    if (rc) return rc;
  }
  return BCG_OK;
}

template <class S, int PASS, int BT>
static void launch_pass(const BatchPlan* p, int ctas, cudaStream_t st) {
  const long long T = p->ntiles[PASS];
  if (T == 0) return;
  const long long g = std::min<long long>(T, (long long)p->nsm * ctas);
  k_batch<S, PASS, BT><<<(unsigned)g, BT, 0, st>>>(p->d, p->dstarts, p->ngrid, p->rectnz);
}

// which grids are rectilinear, from their current metrics (before the
// primitives pass, so the face pass of the same evaluation reads the result)
static void launch_rect(const BatchPlan* p, cudaStream_t st) {
  cudaMemsetAsync(p->rectnz, 0, sizeof(unsigned) * p->ngrid, st);
  k_batch_rect<<<dim3(16, (unsigned)p->ngrid), 256, 0, st>>>(p->d, p->rectnz);
}

template <class S, int BT>
static void launch_cells(const BatchPlan* p, int pass, cudaStream_t st) {
  const int ctas = 2048 / BT;  // full residency of the light passes
  switch (pass) {
    case P_PRIM: launch_pass<S, P_PRIM, BT>(p, ctas, st); break;
    case P_GRAD: launch_pass<S, P_GRAD, BT>(p, ctas, st); break;
    case P_QROWS: launch_pass<S, P_QROWS, BT>(p, ctas, st); break;
    case P_VPTS: launch_pass<S, P_VPTS, BT>(p, ctas, st); break;
    default: launch_pass<S, P_BAL, BT>(p, ctas, st); break;
  }
}

template <class S>
static cudaError_t launch_all(const BatchPlan* p, cudaStream_t st) {
  const int passes[5] = {P_PRIM, P_GRAD, P_QROWS, P_VPTS, -1};
  launch_rect(p, st);
  for (int q : passes) {
    if (q < 0) break;
    if (q == P_GRAD && !p->any_grad) continue;
    if (p->tile_cells == 128) launch_cells<S, 128>(p, q, st); else launch_cells<S, 256>(p, q, st);
  }
  switch (p->tile_faces) {
    case 64: launch_pass<S, P_FACES, 64>(p, p->ctas, st); break;
    case 128: launch_pass<S, P_FACES, 128>(p, p->ctas, st); break;
    default: launch_pass<S, P_FACES, 256>(p, p->ctas, st); break;
  }
  if (p->tile_cells == 128) launch_cells<S, 128>(p, P_BAL, st); else launch_cells<S, 256>(p, P_BAL, st);
  return cudaGetLastError();
}

int batch_run_pass(BatchPlan* p, int pass, cudaStream_t st) {
  if (pass < 0 || pass >= NPASS) return fail_arg("batch: pass must be 0..5");
  if (!p->h.empty() && !p->h[0].w) return fail_arg("batch: arrays not set");
  auto one = [&](auto tag) {
    using S = decltype(tag);
    if (pass == P_GRAD && !p->any_grad) return;
    if (pass == P_FACES) {
      switch (p->tile_faces) {
        case 64: launch_pass<S, P_FACES, 64>(p, p->ctas, st); break;
        case 128: launch_pass<S, P_FACES, 128>(p, p->ctas, st); break;
        default: launch_pass<S, P_FACES, 256>(p, p->ctas, st); break;
      }
    } else if (p->tile_cells == 128) {
      launch_cells<S, 128>(p, pass, st);
    } else {
      launch_cells<S, 256>(p, pass, st);
    }
  };
  if (pass == P_PRIM) launch_rect(p, st);
  if (p->K) one(DK<1>{}); else one(0.0);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? BCG_OK : fail_cuda("batch: pass launch", e);
}

int batch_run(BatchPlan* p, int use_graph, cudaStream_t st) {
  if (!p->h.empty() && !p->h[0].w) return fail_arg("batch: arrays not set");
  auto launch = [&](cudaStream_t s) { return p->K ? launch_all<DK<1>>(p, s) : launch_all<double>(p, s); };
  if (!use_graph) {
    cudaError_t e = launch(st);
    return e == cudaSuccess ? BCG_OK : fail_cuda("batch: launch", e);
  }
  if (!p->exec) {
    // capture the pass launches once, on the plan's own stream (the caller's
    // may be the legacy default stream, which cannot be captured); the
    // descriptors the kernels read live in device memory, so new array
    // addresses need no new capture
    if (!p->cap) {
      cudaError_t e0 = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking);
      if (e0 != cudaSuccess) { p->cap = nullptr; return fail_cuda("batch: capture stream", e0); }
    }
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return fail_cuda("batch: begin capture", e);
    cudaError_t el = launch(p->cap);
    e = cudaStreamEndCapture(p->cap, &graph);
    if (el != cudaSuccess) { if (graph) cudaGraphDestroy(graph); return fail_cuda("batch: capture launch", el); }
    if (e != cudaSuccess) return fail_cuda("batch: end capture", e);
    e = cudaGraphInstantiate(&p->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) { p->exec = nullptr; return fail_cuda("batch: instantiate", e); }
  }
  cudaError_t e = cudaGraphLaunch(p->exec, st);
  return e == cudaSuccess ? BCG_OK : fail_cuda("batch: graph launch", e);
}

void batch_destroy(BatchPlan* p) {
  if (!p) return;
  for (BatchPlan* c : p->chunks) batch_destroy(c);
  for (cudaEvent_t ev : p->hev) cudaEventDestroy(ev);
  for (cudaStream_t s : p->hs)
    if (s) cudaStreamDestroy(s);
  if (p->mirror) cudaFree(p->mirror);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->cap) cudaStreamDestroy(p->cap);
  if (p->scratch && p->owns_scratch) cudaFree(p->scratch);
  if (p->d) cudaFree(p->d);
  if (p->dstarts) cudaFree(p->dstarts);
  if (p->rectnz && p->owns_rectnz) cudaFree(p->rectnz);
  delete p;
}

size_t batch_device_bytes(const BatchPlan* p) {
  size_t b = sizeof(GridDesc) * p->ngrid + sizeof(long long) * NPASS * (p->ngrid + 1) +
             (p->owns_rectnz ? sizeof(unsigned) * p->ngrid : 0);
  if (p->owns_scratch) b += p->scratch_doubles * sizeof(double);
  if (p->mirror) b += p->moff.back() * sizeof(double);
  for (const BatchPlan* c : p->chunks) b += batch_device_bytes(c);
  return b;
}

// ---------------------------------------------------------------------------
// Host-array runs.  Mirrors per grid, in this order: w, wd, nx, ny, vol, volf,
// res, resd (wd and resd only with a tangent); each starts on a 256-byte
// boundary.
namespace {
enum { MIR_W = 0, MIR_WD, MIR_NX, MIR_NY, MIR_VOL, MIR_VOLF, MIR_RES, MIR_RESD, MIR_N };

void mirror_sizes(const Ext& e, int K, size_t sz[MIR_N]) {
  const size_t np = e.np, nn = (size_t)(e.ni + 1) * (e.nj + 1);
  sz[MIR_W] = 5 * np; sz[MIR_WD] = K ? 5 * np : 0; sz[MIR_NX] = 2 * nn; sz[MIR_NY] = 2 * nn;
  sz[MIR_VOL] = np; sz[MIR_VOLF] = 2 * np; sz[MIR_RES] = 5 * np; sz[MIR_RESD] = K ? 5 * np : 0;
}
inline size_t al32(size_t n) { return (n + 31) & ~(size_t)31; }

// child plan over grids [g0, g1) of p: the parent's descriptors (with its
// scratch), arrays on the parent's mirrors, the parent's tile shapes
int make_chunk(BatchPlan* p, int g0, int g1, BatchPlan** out) {
  BatchPlan* c = new BatchPlan();
  c->ngrid = g1 - g0; c->K = p->K; c->nsm = p->nsm; c->any_grad = false;
  c->owns_scratch = false; c->scratch = p->scratch;
  c->owns_rectnz = false; c->rectnz = p->rectnz + g0;
  const bool own = p->host_tile[0] != 0;
  c->tile_faces = own ? p->host_tile[0] : p->tile_faces;
  c->tile_cells = own ? p->host_tile[1] : p->tile_cells;
  c->ctas = own ? p->host_tile[2] : p->ctas;
  c->h.assign(p->h.begin() + g0, p->h.begin() + g1);
  for (int g = 0; g < c->ngrid; ++g) {
    GridDesc& G = c->h[g];
    c->any_grad = c->any_grad || G.grad;
    double* m = p->mirror + p->moff[g0 + g];
    size_t sz[MIR_N];
    mirror_sizes(G.e, p->K, sz);
    double* at[MIR_N];
    for (int k = 0; k < MIR_N; ++k) { at[k] = m; m += al32(sz[k]); }
    G.w = at[MIR_W]; G.wd = p->K ? at[MIR_WD] : nullptr; G.nx = at[MIR_NX]; G.ny = at[MIR_NY];
    G.vol = at[MIR_VOL]; G.volf = at[MIR_VOLF]; G.res = at[MIR_RES]; G.resd = p->K ? at[MIR_RESD] : nullptr;
  }
  cudaError_t e = cudaMalloc(&c->d, sizeof(GridDesc) * c->ngrid);
  if (e == cudaSuccess) e = cudaMalloc(&c->dstarts, sizeof(long long) * NPASS * (c->ngrid + 1));
  if (e == cudaSuccess) e = cudaMemcpy(c->d, c->h.data(), sizeof(GridDesc) * c->ngrid, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) { batch_destroy(c); return fail_cuda("batch: chunk plan", e), BCG_ERR_NOMEM; }
  const int rc = upload_starts(c);
  if (rc) { batch_destroy(c); return rc; }
  *out = c;
  return BCG_OK;
}

// mirrors, chunk plans, streams and events for nchunk chunks (kept until the
// count changes or the plan is destroyed)
int prepare_host(BatchPlan* p, int nchunk) {
  if (!p->mirror) {
    p->moff.assign(p->ngrid + 1, 0);
    for (int g = 0; g < p->ngrid; ++g) {
      size_t sz[MIR_N], n = 0;
      mirror_sizes(p->h[g].e, p->K, sz);
      for (size_t x : sz) n += al32(x);
      p->moff[g + 1] = p->moff[g] + n;
    }
    cudaError_t e = cudaMalloc(&p->mirror, p->moff.back() * sizeof(double));
    if (e != cudaSuccess) { p->mirror = nullptr; return fail_cuda("batch: host-run mirrors", e), BCG_ERR_NOMEM; }
    for (cudaStream_t& s : p->hs) {
      e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
      if (e != cudaSuccess) { s = nullptr; return fail_cuda("batch: host-run streams", e); }
    }
  }
  if ((int)p->chunks.size() == nchunk) return BCG_OK;
  for (BatchPlan* c : p->chunks) batch_destroy(c);
  p->chunks.clear();
  for (cudaEvent_t ev : p->hev) cudaEventDestroy(ev);
  p->hev.clear();
  // contiguous ranges of about equal cell counts
  double tot = 0;
  for (const GridDesc& G : p->h) tot += (double)G.e.im * G.e.jm;
  p->chunk_lo.assign(1, 0);
  double acc = 0;
  for (int g = 0; g < p->ngrid; ++g) {
    acc += (double)p->h[g].e.im * p->h[g].e.jm;
    const int have = (int)p->chunk_lo.size();
    if (have < nchunk && g + 1 < p->ngrid && acc >= tot * have / nchunk) p->chunk_lo.push_back(g + 1);
  }
  p->chunk_lo.push_back(p->ngrid);
  const int nc = (int)p->chunk_lo.size() - 1;
  for (int c = 0; c < nc; ++c) {
    BatchPlan* ch = nullptr;
    const int rc = make_chunk(p, p->chunk_lo[c], p->chunk_lo[c + 1], &ch);
    if (rc) return rc;
    p->chunks.push_back(ch);
  }
  p->hev.assign(2 * nc + 2, nullptr);
  for (cudaEvent_t& ev : p->hev) {
    cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) { ev = nullptr; return fail_cuda("batch: host-run events", e); }
  }
  return BCG_OK;
}
}  // namespace

int batch_run_host(BatchPlan* p, int nchunk, const unsigned long long* w, const unsigned long long* wd,
                   const unsigned long long* nx, const unsigned long long* ny, const unsigned long long* vol,
                   const unsigned long long* volf, const unsigned long long* res, const unsigned long long* resd,
                   cudaStream_t st) {
  if (nchunk < 1 || nchunk > 16) return fail_arg("batch: nchunk must be 1..16");
  if (!w || !nx || !ny || !vol || !volf || !res || (p->K && (!wd || !resd))) return fail_arg("batch: null array table");
  for (int g = 0; g < p->ngrid; ++g) {
    const void* ptrs[8] = {(const void*)w[g], (const void*)nx[g], (const void*)ny[g], (const void*)vol[g],
                           (const void*)volf[g], (const void*)res[g], p->K ? (const void*)wd[g] : (const void*)w[g],
                           p->K ? (const void*)resd[g] : (const void*)res[g]};
    for (const void* q : ptrs)
      if (!q || is_device_ptr(q)) return fail_arg("batch: every array of a host run must be a host pointer");
  }
  int rc = prepare_host(p, std::min(nchunk, p->ngrid));
  if (rc) return rc;
  const int nc = (int)p->chunks.size();
  cudaStream_t up = p->hs[0], down = p->hs[1];
  cudaEvent_t* ev = p->hev.data();  // 0 start, 1 + c uploaded, 1 + nc + c computed, 1 + 2 nc downloads done
  // everything starts after the caller's earlier work on the library stream
  cudaError_t e = cudaEventRecord(ev[0], st);
  for (cudaStream_t s : p->hs)
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev[0], 0);
  if (e != cudaSuccess) return fail_cuda("batch: host run", e);
  const unsigned long long* src[6] = {w, p->K ? wd : nullptr, nx, ny, vol, volf};
  for (int c = 0; c < nc; ++c) {
    BatchPlan* ch = p->chunks[c];
    const int g0 = p->chunk_lo[c];
    for (int g = 0; g < ch->ngrid && e == cudaSuccess; ++g) {
      const GridDesc& G = ch->h[g];
      size_t sz[MIR_N];
      mirror_sizes(G.e, p->K, sz);
      double* dst[6] = {(double*)G.w, (double*)G.wd, (double*)G.nx, (double*)G.ny, (double*)G.vol, (double*)G.volf};
      for (int k = 0; k < 6 && e == cudaSuccess; ++k)
        if (sz[k]) e = cudaMemcpyAsync(dst[k], (const void*)src[k][g0 + g], sz[k] * sizeof(double),
                                       cudaMemcpyHostToDevice, up);
    }
    cudaStream_t comp = p->hs[2 + (c & 1)];
    if (e == cudaSuccess) e = cudaEventRecord(ev[1 + c], up);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(comp, ev[1 + c], 0);
    if (e != cudaSuccess) return fail_cuda("batch: host run upload", e);
    rc = batch_run(ch, 1, comp);
    if (rc) return rc;
    e = cudaEventRecord(ev[1 + nc + c], comp);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(down, ev[1 + nc + c], 0);
    for (int g = 0; g < ch->ngrid && e == cudaSuccess; ++g) {
      const GridDesc& G = ch->h[g];
      const Ext& x = G.e;
      e = copy_interior_planes((double*)res[g0 + g], G.res, x.ni, x.nj, 5, 3, x.im, x.jm, cudaMemcpyDeviceToHost, down);
      if (e == cudaSuccess && p->K)
        e = copy_interior_planes((double*)resd[g0 + g], G.resd, x.ni, x.nj, 5, 3, x.im, x.jm, cudaMemcpyDeviceToHost,
                                 down);
    }
    if (e != cudaSuccess) return fail_cuda("batch: host run download", e);
  }
  e = cudaEventRecord(ev[1 + 2 * nc], down);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev[1 + 2 * nc], 0);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? BCG_OK : fail_cuda("batch: host run", e);
}

}  // namespace bcg

// Colored Jacobian assembly of the DNC5 residual, all seeds in one call.
//
// Reference: the Newton loop of BROADCAST_npz.py:1068-1137 -- for every seed
// (m, l, k) in 5 x 7 x 7: testvector (misc/ComputeJacobian.f90:357), the
// linearised boundary chain (:1079-1082), the tangent residual (:1085),
// computejacobianfromjv_relaxed (:1127); then remove_zero_jac (|a| > 2e-16,
// :129-135 and :1136), the COO -> CSR conversion of createMatPetscCSR
// (misc/PETSc_func.py:71-96) and, for the stored matrix, Jac / vol of the row
// cell (:1206-1210).
//
// GB300 layout of the work: seeds run in groups of 4 as one 4-direction
// tangent pass (boundary chain and residual), their outputs are kept in HBM
// (245 padded states: 5.2 GB at 1024 x 512), and the CSR is then built row by
// row: the candidate columns of a row are known in closed form from the seed
// formulas, so each row is enumerated directly in ascending column order --
// no global sort, two passes (count, fill) around one exclusive scan.
#include <algorithm>
#include <cstdio>
#include <vector>
#include "assembly.h"
#include "bc.h"
#include "jacobian.h"
#include "residual.h"
#include "runtime.h"
#include "span.h"

namespace bcg {

namespace {

// seeded tangent states (testvector, or testvector_partial within the seed's
// zone: 0-based columns [0, imid) for zone 0, [imid, im) for zone 1); the
// seed table holds (m, l, k, zone) per seed
__global__ void k_seed4(double* __restrict__ wd, int nseed, const int* __restrict__ seeds, int gh, int im, int jm,
                        int imid) {
  const int ni = im + 2 * gh, nj = jm + 2 * gh;
  const size_t ns = (size_t)ni * nj * 5;
  const int step = 1 + 2 * gh;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < ns * nseed; q += (size_t)gridDim.x * blockDim.x) {
    const int s = (int)(q / ns);
    const size_t r = q % ns;
    const int i = (int)(r % ni) + 1 - gh, j = (int)((r / ni) % nj) + 1 - gh, v = (int)(r / ((size_t)ni * nj));
    const int m = seeds[4 * s], l = seeds[4 * s + 1], k = seeds[4 * s + 2], z = seeds[4 * s + 3];
    const int i0 = z ? imid : 0, i1 = z ? im : imid;  // zone columns [i0, i1), 0-based
    const bool on = (v == m) && j >= k + 1 && j <= jm && (j - k - 1) % step == 0 && i - 1 >= i0 && i - 1 < i1 &&
                    (i - 1 - i0 - l) % step == 0 && i - 1 - i0 - l >= 0;
    wd[q] = on ? 1.0 : 0.0;
  }
}

// One thread per row (cell i, j, variable e): enumerate the candidate entries
// in ascending column order.  pass 0 counts the kept entries, pass 1 writes.
// op 0 stores -resd (+coefdiag on the diagonal when relaxed), the fill of
// computejacobianfromjv(_relaxed) (ComputeJacobian.f90:292-355, 503-570);
// op != 0 stores +dz with the row window of computejacobianfromdz (:708-779).
__global__ void __launch_bounds__(128) k_csr_rows(int pass, int op, int withjn, int nzone, const double* __restrict__ resd_all,
                                                  int gh, int im, int jm, int relaxed,
                                                  const double* __restrict__ coefdiag, double mini,
                                                  const double* __restrict__ vol, int* __restrict__ count,
                                                  const long long* __restrict__ rowptr, int* __restrict__ indices,
                                                  double* __restrict__ data) {
  const int nrow = 5 * im * jm;
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= nrow) return;
  // reference row numbering: row = e + 5 (j-1) + 5 jm (i-1)
  const int e = row % 5, j = 1 + (row / 5) % jm, i = 1 + row / (5 * jm);
  const int ni = im + 2 * gh, nj = jm + 2 * gh;
  const size_t np = (size_t)ni * nj;
  const size_t cell = (size_t)(i + gh - 1) + (size_t)(j + gh - 1) * ni;
  const double cd = relaxed ? coefdiag[(i - 1) + (size_t)(j - 1) * im] : 0.0;
  const double vinv = vol ? 1.0 / vol[cell] : 1.0;
  // per (l, zone): the seed cell index (0-based) or -1; sorted by it
  constexpr int NC = 14;
  const int nc = 7 * nzone;
  int li[NC], lv[NC], ki[7], kv[7];
  const int step = 1 + 2 * gh;
  for (int c = 0; c < nc; ++c) {
    const int l = c % 7, z = c / 7;
    li[c] = c;
    int vali;
    if (nzone == 2) {
      // computejacobianfromjv_relaxed_withjnandcheck (ComputeJacobian.f90:1095-1204): zone 0 wraps the
      // columns past im - 2gh back to l, zone 1 those up to 2gh to the last seed of colour l
      if (l <= gh) vali = (i <= l + 1 + gh) ? l : (i - (l + 1) + gh) / step * step + l;
      else vali = (i <= l - gh) ? l : (i - (l + 1) + gh) / step * step + l;
      if (z == 0) {
        if (vali >= im - 2 * gh) vali = l;
      } else if (vali <= 2 * gh) {
        vali = im - (im % step) + l;
        if (vali > im - 1) vali -= step;
      }
      lv[c] = vali;
    } else if (!withjn) {
      if (l <= gh) vali = (i <= l + 1 + gh) ? l : (i - (l + 1) + gh) / step * step + l;
      else vali = (i <= l - gh) ? im + 1 : (i - (l + 1) + gh) / step * step + l;
      lv[c] = vali < im ? vali : -1;
    } else {
      // periodic in i (ComputeJacobian.f90:876-897): the seeded column left of
      // the first ones wraps to im-1-2gh+l, the one past im back to l
      if (l <= gh) vali = (i <= l + 1 + gh) ? l : (i - (l + 1) + gh) / step * step + l;
      else vali = (i <= l - gh) ? im - 1 - 2 * gh + l : (i - (l + 1) + gh) / step * step + l;
      if (vali >= im) vali = (vali - im <= gh - 1) ? l : -1;
      lv[c] = vali;
    }
  }
  for (int k = 0; k < 7; ++k) {
    ki[k] = k;
    int valj;
    if (op == 0 || k <= gh) valj = (j <= k + 1 + gh) ? k : (j - gh - (k + 1) + 2 * gh) / step * step + k;
    else valj = (j <= k - gh) ? jm + 1 : (j - (k + 1) + gh) / step * step + k;
    kv[k] = valj < jm ? valj : -1;
  }
  // insertion sorts
  for (int a = 1; a < nc; ++a)
    for (int b = a; b > 0 && lv[b - 1] > lv[b]; --b) { int t = lv[b]; lv[b] = lv[b - 1]; lv[b - 1] = t; t = li[b]; li[b] = li[b - 1]; li[b - 1] = t; }
  for (int a = 1; a < 7; ++a)
    for (int b = a; b > 0 && kv[b - 1] > kv[b]; --b) { int t = kv[b]; kv[b] = kv[b - 1]; kv[b - 1] = t; t = ki[b]; ki[b] = ki[b - 1]; ki[b - 1] = t; }
  long long out = pass ? rowptr[row] : 0;
  int n = 0;
  for (int a = 0; a < nc;) {
    // run of (l, zone) candidates with the same column (the periodic wrap when
    // im is not a multiple of 7, or the two zones): their slots are
    // duplicates, summed as the COO -> CSR conversion does, each slot
    // filtered on its own first
    int a2 = a + 1;
    while (a2 < nc && lv[a2] == lv[a]) ++a2;
    if (lv[a] < 0) { a = a2; continue; }
    for (int b = 0; b < 7; ++b) {
      if (kv[b] < 0) continue;
      const int k = ki[b];
      for (int m = 0; m < 5; ++m) {
        const int col = m + kv[b] * 5 + lv[a] * jm * 5;
        double sum = 0.0;
        bool kept = false;
        for (int q = a; q < a2; ++q) {
          const int l = li[q] % 7, z = li[q] / 7;
          const int seed = z * 245 + k + 7 * l + 49 * m;  // the reference's slot order, zone by zone
          const double r = resd_all[(size_t)seed * np * 5 + (size_t)e * np + cell];
          const double v = op ? r : ((relaxed && col == row) ? cd - r : -r);
          if (!(fabs(v) > mini)) continue;
          sum += v;
          kept = true;
        }
        if (!kept) continue;
        if (pass) { indices[out + n] = col; data[out + n] = sum * vinv; }
        ++n;
      }
    }
    a = a2;
  }
  if (!pass) count[row] = n;
}

// exclusive scan of per-row counts into int64 row pointers (3 kernels)
constexpr int kScanBlock = 1024;
__global__ void k_scan_block(const int* __restrict__ cnt, long long* __restrict__ ptr, long long* __restrict__ bsum,
                             int n) {
  __shared__ long long s[kScanBlock];
  const int t = threadIdx.x, g = blockIdx.x * kScanBlock + t;
  s[t] = (g < n) ? cnt[g] : 0;
  __syncthreads();
  for (int o = 1; o < kScanBlock; o <<= 1) {
    long long x = (t >= o) ? s[t - o] : 0;
    __syncthreads();
    s[t] += x;
    __syncthreads();
  }
  if (g < n) ptr[g] = s[t] - ((g < n) ? cnt[g] : 0);
  if (t == kScanBlock - 1) bsum[blockIdx.x] = s[t];
}
__global__ void k_scan_sums(long long* __restrict__ bsum, int nb, long long* __restrict__ total) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  long long acc = 0;
  for (int b = 0; b < nb; ++b) { const long long x = bsum[b]; bsum[b] = acc; acc += x; }
  *total = acc;
}
__global__ void k_scan_add(long long* __restrict__ ptr, const long long* __restrict__ bsum, int n,
                           const long long* __restrict__ total) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < n) ptr[g] += bsum[g / kScanBlock];
  if (g == n) ptr[n] = *total;
}
__global__ void k_ptr_to_int(const long long* __restrict__ p, int* __restrict__ out, int n) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g <= n) out[g] = (int)p[g];
}

}  // namespace

// seed groups of 4 per tangent launch: as many as fit an 8 GiB budget for
// their seeded states and residual scratch (all 61 at 256 x 256)
static int jacobian_groups(int im, int jm, int gh) {
  const size_t np = (size_t)(im + 2 * gh) * (jm + 2 * gh);
  const size_t per = (4 * np * 5 + residual_scratch_doubles(im, jm, gh, 4)) * 8;
  const size_t g = ((size_t)8 << 30) / per;
  return (int)std::max<size_t>(1, std::min<size_t>(61, g));
}

size_t jacobian_scratch_doubles(int im, int jm, int gh, int nzone, int nops) {
  const size_t np = (size_t)(im + 2 * gh) * (jm + 2 * gh);
  const size_t G = (size_t)jacobian_groups(im, jm, gh);
  return 245 * (size_t)nzone * (size_t)nops * np * 5  // outputs of every seed (per zone and operator)
         + 4 * G * np * 5  // seeded tangent states of G groups
         + np * 5          // state copy written by the linearised boundary fills
         + G * residual_scratch_doubles(im, jm, gh, 4);
}

int run_jacobian(const JacobianArgs& a, cudaStream_t st) {
  const int im = a.im, jm = a.jm, gh = a.gh;
  const size_t np = (size_t)(im + 2 * gh) * (jm + 2 * gh);
  const int nzone = a.nzone == 2 ? 2 : 1, nseed = 245 * nzone;
  const int nop = a.nops > 0 ? a.nops : 1;
  int opv[3] = {a.op, 0, 0};
  for (int k = 0; k < a.nops; ++k) opv[k] = a.ops[k];
  double* resd_all = a.scratch;  // nop blocks of nseed seed outputs
  const size_t oblk = (size_t)nseed * np * 5;
  double* wd4 = resd_all + (size_t)nop * oblk;
  double* wcopy = wd4 + 4 * (size_t)jacobian_groups(im, jm, gh) * np * 5;
  double* rscr = wcopy + np * 5;
  int* seeds_dev = a.iscratch;                        // 2 x 245 x 4
  long long* rowptr = (long long*)(a.iscratch + 2048);  // nrow + 1 (8-byte aligned offset)
  const int nrow = 5 * im * jm;
  long long* bsum = rowptr + nrow + 2;
  const int nb = (nrow + kScanBlock - 1) / kScanBlock;
  long long* total = bsum + nb + 1;
  int* count = (int*)(total + 2);
  // seed table in the reference's loop order: zone, then m, then l, then k
  std::vector<int> seeds((size_t)nseed * 4);
  for (int z = 0, s = 0; z < nzone; ++z)
    for (int m = 0; m < 5; ++m)
      for (int l = 0; l < 7; ++l)
        for (int k = 0; k < 7; ++k, ++s) { seeds[4 * s] = m; seeds[4 * s + 1] = l; seeds[4 * s + 2] = k; seeds[4 * s + 3] = z; }
  const int imid = nzone == 2 ? a.imid : im;
  cudaError_t e = cudaMemcpyAsync(seeds_dev, seeds.data(), seeds.size() * sizeof(int), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return fail_cuda("jacobian: seed table", e);
  e = cudaMemcpyAsync(wcopy, a.w, np * 5 * sizeof(double), cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return fail_cuda("jacobian: state copy", e);
  ResidualArgs ra{};
  ra.im = im; ra.jm = jm; ra.gh = gh; ra.phys = a.phys; ra.w = wcopy; ra.nx = a.nx; ra.ny = a.ny;
  ra.vol = a.vol; ra.volf = a.volf; ra.dstride = np * 5; ra.scratch = rscr; ra.res = nullptr;
  ra.rect = face_rectilinear(a.nx, a.ny, im, jm, gh, st) ? 1 : 0;
  // chunks of G groups of 4 seeds: seed, linearised boundary chain per group,
  // then one tangent launch per pass over the whole chunk (blockIdx.y = group);
  // the last seeds (245 = 61 * 4 + 1, 490 = 122 * 4 + 2) run as 1-direction chunks
  const int G = jacobian_groups(im, jm, gh);
  ra.ndir = 4;
  for (int s0 = 0; s0 < nseed;) {
    const int left = nseed - s0;
    const int kk = left >= 4 ? 4 : 1;
    const int ng = left >= 4 ? std::min(G, left / 4) : 1;
    const int ns = kk * ng;
    k_seed4<<<1024, 256, 0, st>>>(wd4, ns, seeds_dev + 4 * s0, gh, im, jm, imid);
    for (int g = 0; g < ng; ++g)
      for (const BcArgs& b0 : a.bcs) {
        BcArgs b = b0;
        b.ndir = kk; b.w = wcopy; b.wd = wd4 + (size_t)g * kk * np * 5; b.dstride = np * 5;
        e = launch_bc(b, st);
        if (e != cudaSuccess) return fail_cuda("jacobian: boundary fill", e);
      }
    // periodic joins of every seeded tangent (the primal copy is already joined)
    for (int d = 0; d < ns && !a.joins.empty(); ++d)
      for (const JnArgs& j0 : a.joins) {
        JnArgs jn = j0;
        jn.wr = wd4 + (size_t)d * np * 5;
        jn.wd = jn.wr;
        e = launch_jn_match(jn, st);
        if (e != cudaSuccess) return fail_cuda("jacobian: periodic join", e);
      }
    for (int k = 0; k < nop; ++k) {
      double* outk = resd_all + (size_t)k * oblk;
      if (opv[k] == 0) {
        ra.ndir = kk; ra.ngroup = ng;
        ra.wd = wd4;
        ra.resd = outk + (size_t)s0 * np * 5;
        e = run_residual(ra, st);
        if (e != cudaSuccess) return fail_cuda("jacobian: tangent residual", e);
      } else {
        for (int g = 0; g < ng; ++g) {
          SpanArgs sa{};
          sa.im = im; sa.jm = jm; sa.gh = gh; sa.op = opv[k]; sa.ndir = kk; sa.phys = a.phys; sa.w = wcopy;
          sa.wd = wd4 + (size_t)g * kk * np * 5; sa.dstride = np * 5; sa.nx = a.nx; sa.ny = a.ny; sa.vol = a.vol;
          sa.out = outk + (size_t)(s0 + g * kk) * np * 5;
          e = run_span(sa, st);
          if (e != cudaSuccess) return fail_cuda("jacobian: spanwise operator", e);
        }
      }
    }
    s0 += ns;
  }
  // CSR of each operator: count, scan, fill
  const int B = 128;
  for (int k = 0; k < nop; ++k) {
    const double* outk = resd_all + (size_t)k * oblk;
    const int opk = opv[k];
    const int relaxed = opk == 0 ? a.relaxed : 0;
    const int divide = a.nops > 0 ? a.divide_v[k] : a.divide_by_vol;
    int* indptr = a.nops > 0 ? a.indptr_v[k] : a.indptr;
    int* indices = a.nops > 0 ? a.indices_v[k] : a.indices;
    double* data = a.nops > 0 ? a.data_v[k] : a.data;
    const long long capacity = a.nops > 0 ? a.capacity_v[k] : a.capacity;
    long long* nnz_out = a.nops > 0 ? a.nnz_v[k] : a.nnz;
    k_csr_rows<<<(nrow + B - 1) / B, B, 0, st>>>(0, opk, a.withjn, nzone, outk, gh, im, jm, relaxed, a.coefdiag,
                                               a.mini, divide ? a.vol : nullptr, count, nullptr, nullptr, nullptr);
    k_scan_block<<<nb, kScanBlock, 0, st>>>(count, rowptr, bsum, nrow);
    k_scan_sums<<<1, 1, 0, st>>>(bsum, nb, total);
    k_scan_add<<<(nrow + 1 + 255) / 256, 256, 0, st>>>(rowptr, bsum, nrow, total);
    long long nnz = 0;
    e = cudaMemcpyAsync(&nnz, total, sizeof nnz, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail_cuda("jacobian: nnz", e);
    *nnz_out = nnz;
    if (nnz > capacity) return fail_arg("jacobian: CSR capacity too small (see nnz)");
    if (nnz >= (1LL << 31)) return fail_arg("jacobian: nnz exceeds 32-bit CSR indices");
    k_ptr_to_int<<<(nrow + 1 + 255) / 256, 256, 0, st>>>(rowptr, indptr, nrow);
    k_csr_rows<<<(nrow + B - 1) / B, B, 0, st>>>(1, opk, a.withjn, nzone, outk, gh, im, jm, relaxed, a.coefdiag,
                                               a.mini, divide ? a.vol : nullptr, count, rowptr, indices, data);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail_cuda("jacobian: csr", e);
  }
  return BCG_OK;
}

// ---------------------------------------------------------------------------
// Spanwise-wavenumber operator of the global stability problem
// (biglobal.py:82): J(beta) = J - beta^2 Dzz + i beta Dz, on the union of the
// three sparsity patterns, for several beta at once.  One thread per row
// merges the three sorted column lists; pass 0 counts, pass 1 writes.
namespace {
__global__ void __launch_bounds__(128) k_beta_rows(int pass, int nrow, const int* __restrict__ ja_p,
                                                   const int* __restrict__ ja_i, const double* __restrict__ ja_v,
                                                   const int* __restrict__ dz_p, const int* __restrict__ dz_i,
                                                   const double* __restrict__ dz_v, const int* __restrict__ dzz_p,
                                                   const int* __restrict__ dzz_i, const double* __restrict__ dzz_v,
                                                   int nbeta, const double* __restrict__ betas, long long nnz_u,
                                                   int* __restrict__ count, const long long* __restrict__ rowptr,
                                                   int* __restrict__ indices, double2* __restrict__ vals) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= nrow) return;
  int a = ja_p[row], ae = ja_p[row + 1], b = dz_p[row], be = dz_p[row + 1], c = dzz_p[row], ce = dzz_p[row + 1];
  const int BIG = 0x7fffffff;
  long long out = pass ? rowptr[row] : 0;
  int n = 0;
  while (a < ae || b < be || c < ce) {
    const int ca = a < ae ? ja_i[a] : BIG, cb = b < be ? dz_i[b] : BIG, cc = c < ce ? dzz_i[c] : BIG;
    const int col = min(ca, min(cb, cc));
    double vj = 0.0, vz = 0.0, vzz = 0.0;
    if (ca == col) vj = ja_v[a++];
    if (cb == col) vz = dz_v[b++];
    if (cc == col) vzz = dzz_v[c++];
    if (pass) {
      indices[out + n] = col;
      for (int k = 0; k < nbeta; ++k) {
        const double be_ = betas[k];
        vals[(size_t)k * nnz_u + out + n] = make_double2(vj - be_ * be_ * vzz, be_ * vz);
      }
    }
    ++n;
  }
  if (!pass) count[row] = n;
}
}  // namespace

int run_csr_beta(const CsrBetaArgs& a, cudaStream_t st) {
  const int nrow = a.nrow, B = 128;
  const int nb = (nrow + kScanBlock - 1) / kScanBlock;
  long long* rowptr = (long long*)a.iscratch;
  long long* bsum = rowptr + nrow + 2;
  long long* total = bsum + nb + 1;
  int* count = (int*)(total + 2);
  k_beta_rows<<<(nrow + B - 1) / B, B, 0, st>>>(0, nrow, a.j_p, a.j_i, a.j_v, a.dz_p, a.dz_i, a.dz_v, a.dzz_p,
                                               a.dzz_i, a.dzz_v, 0, nullptr, 0, count, nullptr, nullptr, nullptr);
  k_scan_block<<<nb, kScanBlock, 0, st>>>(count, rowptr, bsum, nrow);
  k_scan_sums<<<1, 1, 0, st>>>(bsum, nb, total);
  k_scan_add<<<(nrow + 1 + 255) / 256, 256, 0, st>>>(rowptr, bsum, nrow, total);
  long long nnz = 0;
  cudaError_t e = cudaMemcpyAsync(&nnz, total, sizeof nnz, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail_cuda("csr_spanwise_beta: nnz", e);
  *a.nnz = nnz;
  if (nnz > a.capacity) return fail_arg("csr_spanwise_beta: capacity too small (see nnz)");
  k_ptr_to_int<<<(nrow + 1 + 255) / 256, 256, 0, st>>>(rowptr, a.indptr, nrow);
  k_beta_rows<<<(nrow + B - 1) / B, B, 0, st>>>(1, nrow, a.j_p, a.j_i, a.j_v, a.dz_p, a.dz_i, a.dz_v, a.dzz_p,
                                               a.dzz_i, a.dzz_v, a.nbeta, a.betas, nnz, count, rowptr, a.indices,
                                               (double2*)a.values);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail_cuda("csr_spanwise_beta", e);
  return BCG_OK;
}

size_t csr_beta_iscratch_ints(int nrow) {
  const size_t nb = ((size_t)nrow + kScanBlock - 1) / kScanBlock;
  return 2 * ((size_t)nrow + 2 + nb + 1 + 2) + nrow + 64;
}

size_t jacobian_iscratch_ints(int im, int jm) {
  const size_t nrow = 5 * (size_t)im * jm;
  const size_t nb = (nrow + kScanBlock - 1) / kScanBlock;
  return 2048 + 2 * (nrow + 2 + nb + 1 + 2) + nrow + 64;
}

}  // namespace bcg

// One-time host-side pre-processing of the library: grid metrics
// (srcfv/geom/computegeom.F90:3-104), the boundary-layer inlet / far-field
// reference fields (set_bnd.f90:1-24) and the polynomial Blasius initial state
// (initialisation.f90:2-58).  These run once per grid, off the hot path, on
// host arrays (device arrays are copied through the host).
#include <cuda_runtime.h>
#include <cmath>
#include <cstring>
#include <vector>

namespace {

bool on_device(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// host view of an argument that may live on the device
struct HostView {
  double* user;
  std::vector<double> buf;
  bool dev;
  HostView(double* p, size_t n) : user(p), dev(on_device(p)) {
    if (dev) { buf.resize(n); cudaMemcpy(buf.data(), p, n * 8, cudaMemcpyDeviceToHost); }
  }
  double* h() { return dev ? buf.data() : user; }
  void back() { if (dev) cudaMemcpy(user, buf.data(), buf.size() * 8, cudaMemcpyHostToDevice); }
};

// linear extrapolation of ghost lines, a(g) = 2 a(g-1) - a(g-2)
struct A2 {
  double* p; int ni, lo;
  double& operator()(int i, int j) const { return p[(size_t)(i - lo) + (size_t)(j - lo) * ni]; }
};

}  // namespace

extern "C" {

int bcg_computegeom_2d(double* x0p, double* y0p, double* nxp, double* nyp, double* xcp, double* ycp, double* volp,
                       double* volfp, int im, int jm, int gh) {
  if (im < 2 || jm < 2 || gh < 1) return -1;
  const int lo = 1 - gh, nni = im + 2 * gh + 1, nnj = jm + 2 * gh + 1, ni = im + 2 * gh, nj = jm + 2 * gh;
  const size_t nn = (size_t)nni * nnj, nc = (size_t)ni * nj;
  HostView X0(x0p, nn), Y0(y0p, nn), NX(nxp, 2 * nn), NY(nyp, 2 * nn), XC(xcp, nc), YC(ycp, nc), VOL(volp, nc),
      VOLF(volfp, 2 * nc);
  A2 x0{X0.h(), nni, lo}, y0{Y0.h(), nni, lo}, xc{XC.h(), ni, lo}, yc{YC.h(), ni, lo}, vol{VOL.h(), ni, lo};
  A2 nx1{NX.h(), nni, lo}, nx2{NX.h() + nn, nni, lo}, ny1{NY.h(), nni, lo}, ny2{NY.h() + nn, nni, lo};
  A2 vf1{VOLF.h(), ni, lo}, vf2{VOLF.h() + nc, ni, lo};
  const int ihi_n = im + gh + 1, jhi_n = jm + gh + 1, ihi_c = im + gh, jhi_c = jm + gh;
  // node ghosts, twice per layer as in the reference
  for (int g = 1; g <= gh; ++g)
    for (int rep = 0; rep < 2; ++rep) {
      for (int j = lo; j <= jhi_n; ++j) x0(1 - g, j) = 2.0 * x0(2 - g, j) - x0(3 - g, j);
      for (int j = lo; j <= jhi_n; ++j) x0(im + 1 + g, j) = 2.0 * x0(im + g, j) - x0(im - 1 + g, j);
      for (int i = lo; i <= ihi_n; ++i) x0(i, 1 - g) = 2.0 * x0(i, 2 - g) - x0(i, 3 - g);
      for (int i = lo; i <= ihi_n; ++i) x0(i, jm + 1 + g) = 2.0 * x0(i, jm + g) - x0(i, jm - 1 + g);
      for (int i = lo; i <= ihi_n; ++i) y0(i, 1 - g) = 2.0 * y0(i, 2 - g) - y0(i, 3 - g);
      for (int i = lo; i <= ihi_n; ++i) y0(i, jm + 1 + g) = 2.0 * y0(i, jm + g) - y0(i, jm - 1 + g);
      for (int j = lo; j <= jhi_n; ++j) y0(1 - g, j) = 2.0 * y0(2 - g, j) - y0(3 - g, j);
      for (int j = lo; j <= jhi_n; ++j) y0(im + 1 + g, j) = 2.0 * y0(im + g, j) - y0(im - 1 + g, j);
    }
  // centres, areas (two triangles) and face normals x |face|
  for (int j = 1; j <= jm + 1; ++j)
    for (int i = 1; i <= im + 1; ++i) {
      const double xa = x0(i, j), ya = y0(i, j), xb = x0(i + 1, j), yb = y0(i + 1, j);
      const double xc1 = x0(i, j + 1), yc1 = y0(i, j + 1), xd = x0(i + 1, j + 1), yd = y0(i + 1, j + 1);
      xc(i, j) = 0.25 * (xa + xb + xc1 + xd);
      yc(i, j) = 0.25 * (ya + yb + yc1 + yd);
      const double q1 = 0.5 * std::fabs((xb - xa) * (yc1 - ya) - (xc1 - xa) * (yb - ya));
      const double q2 = 0.5 * std::fabs((xc1 - xd) * (yb - yd) - (xb - xd) * (yc1 - yd));
      vol(i, j) = q1 + q2;
      nx1(i, j) = y0(i, j + 1) - y0(i, j);
      ny1(i, j) = x0(i, j) - x0(i, j + 1);
      nx2(i, j) = y0(i, j) - y0(i + 1, j);
      ny2(i, j) = x0(i + 1, j) - x0(i, j);
    }
  for (int g = 1; g <= gh; ++g)
    for (int rep = 0; rep < 2; ++rep) {
      for (A2* a : {&xc, &yc}) {
        A2& c = *a;
        for (int j = lo; j <= jhi_c; ++j) c(1 - g, j) = 2.0 * c(2 - g, j) - c(3 - g, j);
        for (int j = lo; j <= jhi_c; ++j) c(im + g, j) = 2.0 * c(im - 1 + g, j) - c(im - 2 + g, j);
        for (int i = lo; i <= ihi_c; ++i) c(i, 1 - g) = 2.0 * c(i, 2 - g) - c(i, 3 - g);
        for (int i = lo; i <= ihi_c; ++i) c(i, jm + g) = 2.0 * c(i, jm - 1 + g) - c(i, jm - 2 + g);
      }
      for (int j = 1; j <= jm; ++j) vol(1 - g, j) = 2.0 * vol(2 - g, j) - vol(3 - g, j);
      for (int j = 1; j <= jm; ++j) vol(im + g, j) = 2.0 * vol(im - 1 + g, j) - vol(im - 2 + g, j);
      for (int i = lo; i <= ihi_c; ++i) vol(i, 1 - g) = 2.0 * vol(i, 2 - g) - vol(i, 3 - g);
      for (int i = lo; i <= ihi_c; ++i) vol(i, jm + g) = 2.0 * vol(i, jm - 1 + g) - vol(i, jm - 2 + g);
      for (A2* a : {&nx1, &nx2, &ny1, &ny2}) {
        A2& c = *a;
        for (int j = lo; j <= jhi_n; ++j) c(1 - g, j) = 2.0 * c(2 - g, j) - c(3 - g, j);
      }
      for (A2* a : {&nx1, &nx2, &ny1, &ny2}) {
        A2& c = *a;
        for (int j = lo; j <= jhi_n; ++j) c(im + 1 + g, j) = 2.0 * c(im + g, j) - c(im - 1 + g, j);
      }
      for (A2* a : {&nx1, &nx2, &ny1, &ny2}) {
        A2& c = *a;
        for (int i = lo; i <= ihi_n; ++i) c(i, 1 - g) = 2.0 * c(i, 2 - g) - c(i, 3 - g);
      }
      for (A2* a : {&nx1, &nx2, &ny1, &ny2}) {
        A2& c = *a;
        for (int i = lo; i <= ihi_n; ++i) c(i, jm + 1 + g) = 2.0 * c(i, jm + g) - c(i, jm - 1 + g);
      }
    }
  for (int j = 1; j <= jm + 1; ++j)
    for (int i = 1; i <= im + 1; ++i) {
      vf1(i, j) = 2.0 / (vol(i, j) + vol(i - 1, j));
      vf2(i, j) = 2.0 / (vol(i, j) + vol(i, j - 1));
    }
  X0.back(); Y0.back(); NX.back(); NY.back(); XC.back(); YC.back(); VOL.back(); VOLF.back();
  return 0;
}

// field(j,d,:) = w(1-d,j,:); wbd(i,:) = w(i-gh,jm,:)   (set_bnd.f90:1-24)
int bcg_set_bndbl_2d(const double* wp, double* fieldp, double* wbdp, int im, int jm, int gh) {
  if (im < 1 || jm < 1 || gh < 1) return -1;
  const int ni = im + 2 * gh, nj = jm + 2 * gh;
  const size_t nc = (size_t)ni * nj;
  HostView W(const_cast<double*>(wp), nc * 5), F(fieldp, (size_t)jm * gh * 5), B(wbdp, (size_t)(im + gh) * 5);
  const double* w = W.h();
  auto at = [&](int i, int j, int v) { return w[(size_t)(i + gh - 1) + (size_t)(j + gh - 1) * ni + (size_t)(v - 1) * nc]; };
  for (int j = 1; j <= jm; ++j)
    for (int d = 1; d <= gh; ++d)
      for (int v = 1; v <= 5; ++v) F.h()[(size_t)(j - 1) + (size_t)(d - 1) * jm + (size_t)(v - 1) * jm * gh] = at(1 - d, j, v);
  const int lm = im + gh;
  for (int i = 1; i <= lm; ++i)
    for (int v = 1; v <= 5; ++v) B.h()[(size_t)(i - 1) + (size_t)(v - 1) * lm] = at(i - gh, jm, v);
  F.back(); B.back();
  return 0;
}

// approximate Blasius profile 2e - 2e^3 + e^4 (initialisation.f90:2-58)
int bcg_initblfv(double muinf, const double* xcp, const double* ycp, double* wp, double* fieldp, int im, int gh,
                 int jm) {
  if (im < 3 || jm < 3 || gh < 1) return -1;
  const int ni = im + 2 * gh, nj = jm + 2 * gh;
  const size_t nc = (size_t)ni * nj;
  HostView XC(const_cast<double*>(xcp), nc), YC(const_cast<double*>(ycp), nc), W(wp, nc * 5), F(fieldp, (size_t)jm * gh * 5);
  auto c = [&](int i, int j) { return (size_t)(i + gh - 1) + (size_t)(j + gh - 1) * ni; };
  double* w = W.h();
  const double* xc = XC.h();
  const double* yc = YC.h();
  double* field = F.h();
  const double ro = w[c(3, 3)], rou = w[c(3, 3) + nc], roE = w[c(3, 3) + 4 * nc];
  const double ue = rou / ro, rou2 = 0.5 * rou * ue, xdm1 = std::sqrt(rou / muinf);
  auto prof = [&](double eta) { return eta < 1.0 ? 2.0 * eta - 2.0 * eta * eta * eta + eta * eta * eta * eta : 1.0; };
  for (int j = 1; j <= jm + gh; ++j)
    for (int i = 1 - gh; i <= im + gh; ++i) {
      const double ubl = prof(yc[c(i, j)] * xdm1 / std::sqrt(xc[c(i, j)])) * ue;
      w[c(i, j) + nc] = ro * ubl;
      w[c(i, j) + 4 * nc] = roE - rou2 + 0.5 * ro * ubl * ubl;
    }
  for (int i = 1 - gh; i <= im + gh; ++i) w[c(i, 0) + nc] = -w[c(i, 1) + nc];
  for (int j = 1; j <= jm; ++j)
    for (int i = 1 - gh; i <= 0; ++i) {
      // the reference multiplies by sqrt(xc) here (initialisation.f90:42)
      const double ubl = prof(yc[c(i, j)] * xdm1 * std::sqrt(xc[c(i, j)])) * ue;
      field[(size_t)(j - 1) + (size_t)(-i) * jm + (size_t)1 * jm * gh] = ro * ubl;
      field[(size_t)(j - 1) + (size_t)(-i) * jm + (size_t)4 * jm * gh] = roE - rou2 + 0.5 * ro * ubl * ubl;
    }
  W.back(); F.back();
  return 0;
}

}  // extern "C"

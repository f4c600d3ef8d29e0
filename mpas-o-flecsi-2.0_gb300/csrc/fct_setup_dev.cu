// FCT / del2 static coefficients computed on the GPU: the setup of
// apps/ocean/tasks/init_functions.cc:18-447 (the same steps as the host
// setup in fct_setup.cc), one thread per cell for the second-derivative
// least-squares fits and one per edge for the advection stencils, so that an
// ensemble of many meshes is set up in one call (one device allocation, one
// stream, every member's kernels queued back to back) instead of ~10 us per
// cell on a host core.
//
// Compiled with -fmad=false and the host setup's operation order: the
// integer outputs (stencil cells, counts, masks, levels, signs) equal the
// host's exactly; the floating-point ones differ from the host's (which
// equal the reference's bit for bit) only through the last-place
// differences between CUDA's acos / asin / sin / cos / atan2 / pow and the
// C library's.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <vector>

#include "device.cuh"
#include "mpaso_mesh.h"

namespace mpaso {
namespace {

constexpr int kME = 8, kME2 = 16, kNA = 6, kMM = kME + 1;
constexpr double kA = 6371000.0;           // mpasoflecsi/common/constants.hh:28
constexpr double kPi = 3.141592653589793;  // constants.hh:29

// error bits set by the kernels (the host setup's require() checks)
enum : unsigned {
  kErrEdgeIndex = 1u,
  kErrEdgeCells = 2u,
  kErrNeighbourhood = 4u,
  kErrBisect = 8u,
  kErrAdvCells = 16u,
};

__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }  // std::max
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }  // std::min

struct DevIn {
  int64_t nC, nE;
  const int64_t *c2e_off, *c2c_off, *e2v_off;
  const int32_t *c2e, *c2c, *e2v;
  const double *dcEdge, *dvEdge, *xCell, *yCell, *zCell, *xVertex, *yVertex, *zVertex;
  const int32_t *maxLevelCell, *boundaryCell;
  int on_sphere, nlev;
  double Lx, Ly, msd;
};

struct DevOut {
  int32_t *maxLevelEdgeTop, *nAdv, *advCells, *mask;
  double *msd, *sign, *d2, *advCoef, *advCoef3;
};

// Spherical triangle angle at a (mpasoflecsi/eqns/metrics.hh:25-73).
__device__ double sph_angle(const double *a, const double *b, const double *c) {
  const double sa = acos(smax(smin(b[0] * c[0] + b[1] * c[1] + b[2] * c[2], 1.0), -1.0));
  const double sb = acos(smax(smin(a[0] * c[0] + a[1] * c[1] + a[2] * c[2], 1.0), -1.0));
  const double sc = acos(smax(smin(a[0] * b[0] + a[1] * b[1] + a[2] * b[2], 1.0), -1.0));
  const double ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
  const double ac[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
  const double dx = (ab[1] * ac[2]) - (ab[2] * ac[1]);
  const double dy = (ab[2] * ac[0]) - (ab[0] * ac[2]);
  const double dz = (ab[0] * ac[1]) - (ab[1] * ac[0]);
  const double s = 0.5 * (sa + sb + sc);
  const double sin_angle = sqrt(smin(1.0, smax(0.0, (sin(s - sb) * sin(s - sc)) / (sin(sb) * sin(sc)))));
  const double ang = 2.0 * asin(smax(smin(sin_angle, 1.0), -1.0));
  return (dx * a[0] + dy * a[1] + dz * a[2] >= 0.0) ? ang : -ang;
}

// Great-circle arc length (metrics.hh:75-91).
__device__ double sph_arc(const double *a, const double *b) {
  const double c[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
  const double r = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  const double cl = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
  return r * 2. * asin(cl / (2. * r));
}

// Arc midpoint (metrics.hh:93-111); false where the reference asserts.
__device__ bool sph_bisect(const double *a, const double *b, double *c) {
  const double r = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  for (int k = 0; k < 3; ++k) c[k] = 0.5 * (a[k] + b[k]);
  if (c[0] == 0. || c[1] == 0. || c[2] == 0.) return false;
  const double d = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
  for (int k = 0; k < 3; ++k) c[k] = r * c[k] / d;
  return true;
}

__device__ __forceinline__ double wrap(double d, double L) { return L > 0 ? d - L * rint(d / L) : d; }

// Rows 3-5 of the inverse of the 6 x 6 normal matrix by scaled partial-
// pivoting elimination (mpasoflecsi/eqns/matrix.hh:52-167).  The host setup
// eliminates all six right-hand columns together and back-substitutes all six
// rows; every element here sees the same operations in the same order, one
// column at a time, and back-substitution stops after the three rows the
// second derivatives need (rows 5, 4, 3 come first and use no other row).
__device__ void invert6_rows345(double (&a)[kNA][kNA], double (&x)[3][kNA]) {
  constexpr int n = kNA;
  int idx[kNA];
  double scale[kNA];
  for (int i = 0; i < n; ++i) {
    idx[i] = i;
    double c1 = 0.;
    for (int j = 0; j < n; ++j) c1 = smax(c1, fabs(a[i][j]));
    scale[i] = c1;
  }
  for (int j = 0; j < n - 1; ++j) {
    int k = j;
    double best = 0.0;
    for (int i = j; i < n; ++i) {
      const double p = fabs(a[idx[i]][j]) / scale[idx[i]];
      if (p > best) best = p, k = i;
    }
    const int t = idx[j];
    idx[j] = idx[k], idx[k] = t;
    for (int i = j + 1; i < n; ++i) {
      const double pj = a[idx[i]][j] / a[idx[j]][j];
      a[idx[i]][j] = pj;
      for (int kk = j + 1; kk < n; ++kk) a[idx[i]][kk] = a[idx[i]][kk] - pj * a[idx[j]][kk];
    }
  }
  for (int col = 0; col < n; ++col) {
    double b[kNA], xc[kNA];
    for (int i = 0; i < n; ++i) b[i] = (i == col) ? 1. : 0.;
    for (int i = 0; i < n - 1; ++i)
      for (int j = i + 1; j < n; ++j) b[idx[j]] = b[idx[j]] - a[idx[j]][i] * b[idx[i]];
    xc[n - 1] = b[idx[n - 1]] / a[idx[n - 1]][n - 1];
    for (int j = n - 2; j >= 3; --j) {
      xc[j] = b[idx[j]];
      for (int k = j + 1; k < n; ++k) xc[j] = xc[j] - a[idx[j]][k] * xc[k];
      xc[j] = xc[j] / a[idx[j]][j];
    }
    x[0][col] = xc[3], x[1][col] = xc[4], x[2][col] = xc[5];
  }
}

// Column i of the fit's design matrix transposed: the monomials 1, x, y,
// x^2, x y, y^2 of point i (point 0, the cell itself, is the origin).
__device__ __forceinline__ double mono(int r, int i, const double *xp, const double *yp) {
  if (i == 0) return r == 0 ? 1.0 : 0.0;
  const double x = xp[i - 1], y = yp[i - 1];
  switch (r) {
    case 0: return 1.0;
    case 1: return x;
    case 2: return y;
    case 3: return x * x;
    case 4: return x * y;
    default: return y * y;
  }
}

__device__ __forceinline__ void unit_pos(const DevIn &in, int64_t c, double p[3]) {
  p[0] = in.xCell[c] / kA, p[1] = in.yCell[c] / kA, p[2] = in.zCell[c] / kA;
}

// cells(e) by transposition of c2e, ascending ids (mesh.cc:108-116): the
// smaller and the larger id of the cells that list the edge.
__global__ void k_edge_cells(DevIn in, int32_t *e2c0, int32_t *e2c1, int32_t *cnt, unsigned *err) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= in.nC) return;
  for (int64_t j = in.c2e_off[c]; j < in.c2e_off[c + 1]; ++j) {
    const int32_t e = in.c2e[j];
    if (e < 0 || e >= in.nE) {
      atomicOr(err, kErrEdgeIndex);
      continue;
    }
    atomicMin(e2c0 + e, (int32_t)c);
    atomicMax(e2c1 + e, (int32_t)c);
    atomicAdd(cnt + e, 1);
  }
}

// maxLevelEdgeTop (:18-27), meshScalingDel2 (:47-66, a constant: the
// reference takes cells 0 and 1 for every edge), highOrderAdvMask (:342-356).
__global__ void k_edge_levels(DevIn in, DevOut o, const int32_t *e2c0, const int32_t *e2c1, const int32_t *cnt,
                              unsigned *err) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= in.nE) return;
  if (cnt[e] < 2) {
    atomicOr(err, kErrEdgeCells);
    return;
  }
  const int32_t a = e2c0[e], b = e2c1[e];
  o.maxLevelEdgeTop[e] = max(in.maxLevelCell[a], in.maxLevelCell[b]);
  o.msd[e] = in.msd;
  for (int k = 0; k < in.nlev; ++k) {
    int m = 1;
    if (in.boundaryCell && (in.boundaryCell[(int64_t)a * in.nlev + k] == 1 ||
                            in.boundaryCell[(int64_t)b * in.nlev + k] == 1))
      m = 0;
    o.mask[e * in.nlev + k] = m;
  }
}

// edgeSignOnCell (:68-82) and derivTwo (:83-328), one thread per cell.  The
// per-thread arrays stay under the default 1 KB stack (neighbour positions
// are re-read from memory, the design matrix is generated from x, y), so a
// launch never makes the driver grow the local-memory reservation.
__global__ void __launch_bounds__(128) k_cell_fits(DevIn in, DevOut o, const int32_t *e2c0, unsigned *err) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= in.nC) return;
  const int64_t eb = in.c2e_off[c], cb = in.c2c_off[c];
  const int nEonC = (int)(in.c2e_off[c + 1] - eb);
  const int n = nEonC + 1;
  if (nEonC < 1 || n > kMM || in.c2c_off[c + 1] - cb != nEonC) {
    atomicOr(err, kErrNeighbourhood);
    return;
  }
  for (int j = 0; j < kME; ++j) o.sign[c * kME + j] = 0.0;
  for (int j = 0; j < nEonC; ++j) o.sign[c * kME + j] = (c == e2c0[in.c2e[eb + j]]) ? -1.0 : 1.0;
  double xp[kMM], yp[kMM], theta_t[kMM], pc0[3];
  for (int i = 0; i < kMM; ++i) theta_t[i] = 0.0;
  if (in.on_sphere) {
    unit_pos(in, c, pc0);
    const double pole[3] = {0.0, 0.0, 1.0};
    double p1[3], p2[3];
    unit_pos(in, in.c2c[cb], p1);
    double tt = (pc0[2] == 1.0) ? kPi / 2.0 : kPi / 2.0 - sph_angle(pc0, p1, pole);
    for (int i = 0; i < n - 1; ++i) {
      const int ip2 = (i + 2 > n - 1) ? 1 : i + 2;
      unit_pos(in, in.c2c[cb + i], p1);
      unit_pos(in, in.c2c[cb + ip2 - 1], p2);
      const double tv = sph_angle(pc0, p1, p2);
      const double dl = kA * sph_arc(pc0, p1) / 1.0;
      theta_t[i] = tt;
      xp[i] = cos(tt) * dl;
      yp[i] = sin(tt) * dl;
      tt = tt + tv;
    }
  } else {
    for (int i = 0; i < n - 1; ++i) {
      const int32_t nb = in.c2c[cb + i];
      xp[i] = wrap(in.xCell[nb] - in.xCell[c], in.Lx);
      yp[i] = wrap(in.yCell[nb] - in.yCell[c], in.Ly);
    }
  }
  // least-squares fit of a + b x + c y + d x^2 + e x y + f y^2 with unit
  // weights: (A^T A)^-1 A^T (the host's products with the identity weight
  // matrix are exact and left out)
  double N[kNA][kNA], inv[3][kNA];
  for (int r = 0; r < kNA; ++r)
    for (int q = 0; q < kNA; ++q) {
      double acc = 0.0;
      for (int i = 0; i < n; ++i) acc += mono(r, i, xp, yp) * mono(q, i, xp, yp);
      N[r][q] = acc;
    }
  invert6_rows345(N, inv);
  for (int i = 0; i < nEonC; ++i) {
    const int64_t e = in.c2e[eb + i];
    const int64_t vo = in.e2v_off[e];
    const int32_t va = in.e2v[vo], vb = in.e2v[vo + 1];
    double te;
    if (in.on_sphere) {
      double v1[3], v2[3], mid[3], p1[3];
      v1[0] = in.xVertex[va] / kA, v1[1] = in.yVertex[va] / kA, v1[2] = in.zVertex[va] / kA;
      v2[0] = in.xVertex[vb] / kA, v2[1] = in.yVertex[vb] / kA, v2[2] = in.zVertex[vb] / kA;
      if (!sph_bisect(v1, v2, mid)) {
        atomicOr(err, kErrBisect);
        return;
      }
      unit_pos(in, in.c2c[cb + i], p1);
      te = sph_angle(pc0, p1, mid) + theta_t[i];
    } else {
      const double xm = 0.5 * (wrap(in.xVertex[va] - in.xCell[c], in.Lx) + wrap(in.xVertex[vb] - in.xCell[c], in.Lx));
      const double ym = 0.5 * (wrap(in.yVertex[va] - in.yCell[c], in.Ly) + wrap(in.yVertex[vb] - in.yCell[c], in.Ly));
      te = atan2(ym, xm);
    }
    double c2t = cos(te), s2t = sin(te);
    const double cs = c2t * s2t;
    c2t = c2t * c2t;
    s2t = s2t * s2t;
    const int side = (c == e2c0[e]) ? 0 : 1;
    for (int j = 0; j < n; ++j) {
      double B[3];  // rows 3-5 of (A^T A)^-1 A^T, column j
      for (int r = 0; r < 3; ++r) {
        double acc = 0.0;
        for (int k = 0; k < kNA; ++k) acc += inv[r][k] * mono(k, j, xp, yp);
        B[r] = acc;
      }
      o.d2[(e * kME2 + j) * 2 + side] = 2. * c2t * B[0] + 2. * cs * B[1] + 2. * s2t * B[2];
    }
  }
}

__device__ __forceinline__ int find_in(const int32_t *l, int n, int32_t v) {
  int i = 0;
  while (i < n && l[i] != v) ++i;
  return i;
}

// advCellsForEdge, advCoef, advCoef_3rd (:357-445), one thread per edge.
__global__ void k_edge_stencils(DevIn in, DevOut o, const int32_t *e2c0, const int32_t *e2c1, unsigned *err) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= in.nE) return;
  double ac[kME2], a3[kME2];
  int32_t cl[2 * kME + 2];
  for (int i = 0; i < kME2; ++i) ac[i] = 0., a3[i] = 0.;
  const int32_t c1 = e2c0[e], c2 = e2c1[e];
  const int64_t b1 = in.c2c_off[c1], b2 = in.c2c_off[c2];
  const int n1 = (int)(in.c2c_off[c1 + 1] - b1), n2 = (int)(in.c2c_off[c2 + 1] - b2);
  if (n1 > kME || n2 > kME || in.c2e_off[c1 + 1] - in.c2e_off[c1] != n1 ||
      in.c2e_off[c2 + 1] - in.c2e_off[c2] != n2) {
    atomicOr(err, kErrNeighbourhood);
    return;
  }
  int n = 0;
  cl[n++] = c1, cl[n++] = c2;
  for (int j = 0; j < n1; ++j)
    if (find_in(cl, n, in.c2c[b1 + j]) == n) cl[n++] = in.c2c[b1 + j];
  for (int j = 0; j < n2; ++j)
    if (find_in(cl, n, in.c2c[b2 + j]) == n) cl[n++] = in.c2c[b2 + j];
  if (n > kME2) {
    atomicOr(err, kErrAdvCells);
    return;
  }
  o.nAdv[e] = n;
  for (int i = 0; i < kME2; ++i) o.advCells[e * kME2 + i] = i < n ? cl[i] : 0;
  const double *D = o.d2 + e * kME2 * 2;
  const int i1 = find_in(cl, n, c1);
  ac[i1] = ac[i1] + D[0], a3[i1] = a3[i1] + D[0];
  for (int j = 0; j < n1; ++j) {
    const int ix = find_in(cl, n, in.c2c[b1 + j]);
    ac[ix] = ac[ix] + D[(j + 1) * 2], a3[ix] = a3[ix] + D[(j + 1) * 2];
  }
  const int i2 = find_in(cl, n, c2);
  ac[i2] = ac[i2] + D[1], a3[i2] = a3[i2] - D[1];
  for (int j = 0; j < n2; ++j) {
    const int ix = find_in(cl, n, in.c2c[b2 + j]);
    ac[ix] = ac[ix] + D[(j + 1) * 2 + 1], a3[ix] = a3[ix] - D[(j + 1) * 2 + 1];
  }
  const double dc = in.dcEdge[e], dv = in.dvEdge[e];
  for (int i = 0; i < n; ++i) {
    ac[i] = -(dc * dc) * ac[i] / 12.0;
    a3[i] = -(dc * dc) * a3[i] / 12.0;
  }
  ac[i1] = ac[i1] + 0.5;
  ac[i2] = ac[i2] + 0.5;
  for (int i = 0; i < kME2; ++i) {
    o.advCoef[e * kME2 + i] = i < n ? dv * ac[i] : 0.0;
    o.advCoef3[e * kME2 + i] = i < n ? dv * a3[i] : 0.0;
  }
}

// Checks on the host everything the kernels index with, and the constant
// meshScalingDel2 (one value for every edge, from cells 0 and 1, as the
// reference takes it).
double validate(const mpaso_fct_setup_in &in, const mpaso_fct_setup_out &o) {
  const int64_t nC = in.nCells, nE = in.nEdges;
  require(nC > 0 && nE > 0 && in.nVertices > 0 && in.nlev >= 1, MPASO_ERR_ARG, "bad sizes");
  require(nC < INT_MAX && nE < INT_MAX, MPASO_ERR_ARG, "more than 2^31 cells or edges");
  require(in.c2e_off && in.c2c_off && in.e2v_off && in.c2e && in.c2c && in.e2v && in.dcEdge &&
              in.dvEdge && in.xCell && in.yCell && in.xVertex && in.yVertex && in.maxLevelCell,
          MPASO_ERR_ARG, "missing input array");
  require(!in.on_sphere || (in.zCell && in.zVertex), MPASO_ERR_ARG, "sphere needs z coordinates");
  require(o.maxLevelEdgeTop && o.meshScalingDel2 && o.edgeSignOnCell && o.derivTwo && o.nAdvCellsForEdge &&
              o.advCellsForEdge && o.highOrderAdvMask && o.advCoef && o.advCoef_3rd,
          MPASO_ERR_ARG, "missing output array");
  auto offsets_ok = [](const int64_t *off, int64_t n) {
    if (off[0] != 0) return false;
    for (int64_t i = 0; i < n; ++i)
      if (off[i + 1] < off[i]) return false;
    return true;
  };
  auto indices_ok = [](const int32_t *idx, int64_t n, int64_t hi) {
    for (int64_t i = 0; i < n; ++i)
      if (idx[i] < 0 || idx[i] >= hi) return false;
    return true;
  };
  require(offsets_ok(in.c2e_off, nC) && offsets_ok(in.c2c_off, nC) && offsets_ok(in.e2v_off, nE), MPASO_ERR_MESH,
          "connectivity offsets not ascending from 0");
  require(indices_ok(in.c2c, in.c2c_off[nC], nC), MPASO_ERR_MESH, "cell index out of range");
  require(indices_ok(in.e2v, in.e2v_off[nE], in.nVertices), MPASO_ERR_MESH, "vertex index out of range");
  for (int64_t e = 0; e < nE; ++e)
    require(in.e2v_off[e + 1] - in.e2v_off[e] >= 2, MPASO_ERR_MESH, "edge with fewer than two vertices");
  double msd = 1.0;
  if (in.meshDensity) {
    double maxDensity = 0.0;
    for (int64_t c = 0; c < nC; ++c)
      if (in.meshDensity[c] > maxDensity) maxDensity = in.meshDensity[c];
    const double rel = (in.meshDensity[0] + in.meshDensity[nC > 1 ? 1 : 0]) / (2.0 * maxDensity);
    msd = 1.0 / std::pow(rel, 0.25);
  }
  return msd;
}

// One device allocation carved into 256-byte aligned pieces.
struct Arena {
  size_t bytes = 0;
  char *base = nullptr;
  size_t take(size_t n) {
    const size_t at = bytes;
    bytes += (n + 255) / 256 * 256;
    return at;
  }
  template <class T> T *at(size_t off) const { return reinterpret_cast<T *>(base + off); }
};

// Per member: where each input and output sits in the arena.
struct Layout {
  size_t c2e_off, c2c_off, e2v_off, c2e, c2c, e2v, dc, dv, xc, yc, zc, xv, yv, zv, mlc, bc;
  size_t mlet, nadv, advc, mask, msd, sign, d2, ac, a3, e2c0, e2c1, cnt;
};

struct Call {
  cudaStream_t st = nullptr;
  Arena A;
  ~Call() {
    if (st) cudaStreamSynchronize(st);
    if (A.base) cudaFree(A.base);
    if (st) cudaStreamDestroy(st);
  }
};

void run_many(const mpaso_fct_setup_in *ins, mpaso_fct_setup_out *outs, int nm, int device) {
  std::vector<double> msd(nm);
  for (int i = 0; i < nm; ++i) {
    try {
      msd[i] = validate(ins[i], outs[i]);
    } catch (const error &e) {
      fail(e.code, "member " + std::to_string(i) + ": " + e.what());
    }
  }
  Call K;
  std::vector<Layout> lay(nm);
  for (int i = 0; i < nm; ++i) {
    const mpaso_fct_setup_in &in = ins[i];
    const size_t nC = in.nCells, nE = in.nEdges, nV = in.nVertices, L = in.nlev;
    Layout &l = lay[i];
    l.c2e_off = K.A.take((nC + 1) * 8), l.c2c_off = K.A.take((nC + 1) * 8), l.e2v_off = K.A.take((nE + 1) * 8);
    l.c2e = K.A.take(in.c2e_off[nC] * 4), l.c2c = K.A.take(in.c2c_off[nC] * 4), l.e2v = K.A.take(in.e2v_off[nE] * 4);
    l.dc = K.A.take(nE * 8), l.dv = K.A.take(nE * 8);
    l.xc = K.A.take(nC * 8), l.yc = K.A.take(nC * 8), l.zc = K.A.take(in.zCell ? nC * 8 : 0);
    l.xv = K.A.take(nV * 8), l.yv = K.A.take(nV * 8), l.zv = K.A.take(in.zVertex ? nV * 8 : 0);
    l.mlc = K.A.take(nC * 4), l.bc = K.A.take(in.boundaryCell ? nC * L * 4 : 0);
    l.mlet = K.A.take(nE * 4), l.nadv = K.A.take(nE * 4), l.advc = K.A.take(nE * kME2 * 4);
    l.mask = K.A.take(nE * L * 4), l.msd = K.A.take(nE * 8), l.sign = K.A.take(nC * kME * 8);
    l.d2 = K.A.take(nE * kME2 * 2 * 8), l.ac = K.A.take(nE * kME2 * 8), l.a3 = K.A.take(nE * kME2 * 8);
    l.e2c0 = K.A.take(nE * 4), l.e2c1 = K.A.take(nE * 4), l.cnt = K.A.take(nE * 4);
  }
  const size_t err_off = K.A.take(nm * sizeof(unsigned));
  MPASO_CUDA(cudaSetDevice(device));
  MPASO_CUDA(cudaStreamCreateWithFlags(&K.st, cudaStreamNonBlocking));
  MPASO_CUDA(cudaMalloc(&K.A.base, K.A.bytes));
  unsigned *err = K.A.at<unsigned>(err_off);
  MPASO_CUDA(cudaMemsetAsync(err, 0, nm * sizeof(unsigned), K.st));
  auto up = [&](size_t off, const void *h, size_t bytes) {
    if (h && bytes) MPASO_CUDA(cudaMemcpyAsync(K.A.base + off, h, bytes, cudaMemcpyHostToDevice, K.st));
  };
  std::vector<DevIn> din(nm);
  std::vector<DevOut> dout(nm);
  const int tpb = 128;
  for (int i = 0; i < nm; ++i) {  // uploads and the connectivity kernels of every member
    const mpaso_fct_setup_in &in = ins[i];
    const Layout &l = lay[i];
    const int64_t nC = in.nCells, nE = in.nEdges, nV = in.nVertices, L = in.nlev;
    up(l.c2e_off, in.c2e_off, (nC + 1) * 8), up(l.c2c_off, in.c2c_off, (nC + 1) * 8);
    up(l.e2v_off, in.e2v_off, (nE + 1) * 8);
    up(l.c2e, in.c2e, in.c2e_off[nC] * 4), up(l.c2c, in.c2c, in.c2c_off[nC] * 4), up(l.e2v, in.e2v, in.e2v_off[nE] * 4);
    up(l.dc, in.dcEdge, nE * 8), up(l.dv, in.dvEdge, nE * 8);
    up(l.xc, in.xCell, nC * 8), up(l.yc, in.yCell, nC * 8), up(l.zc, in.zCell, nC * 8);
    up(l.xv, in.xVertex, nV * 8), up(l.yv, in.yVertex, nV * 8), up(l.zv, in.zVertex, nV * 8);
    up(l.mlc, in.maxLevelCell, nC * 4), up(l.bc, in.boundaryCell, nC * L * 4);
    DevIn &d = din[i];
    d.nC = nC, d.nE = nE, d.on_sphere = in.on_sphere ? 1 : 0, d.nlev = (int)L, d.Lx = in.Lx, d.Ly = in.Ly;
    d.msd = msd[i];
    d.c2e_off = K.A.at<int64_t>(l.c2e_off), d.c2c_off = K.A.at<int64_t>(l.c2c_off);
    d.e2v_off = K.A.at<int64_t>(l.e2v_off), d.c2e = K.A.at<int32_t>(l.c2e), d.c2c = K.A.at<int32_t>(l.c2c);
    d.e2v = K.A.at<int32_t>(l.e2v), d.dcEdge = K.A.at<double>(l.dc), d.dvEdge = K.A.at<double>(l.dv);
    d.xCell = K.A.at<double>(l.xc), d.yCell = K.A.at<double>(l.yc);
    d.zCell = in.zCell ? K.A.at<double>(l.zc) : nullptr;
    d.xVertex = K.A.at<double>(l.xv), d.yVertex = K.A.at<double>(l.yv);
    d.zVertex = in.zVertex ? K.A.at<double>(l.zv) : nullptr;
    d.maxLevelCell = K.A.at<int32_t>(l.mlc), d.boundaryCell = in.boundaryCell ? K.A.at<int32_t>(l.bc) : nullptr;
    DevOut &g = dout[i];
    g.maxLevelEdgeTop = K.A.at<int32_t>(l.mlet), g.nAdv = K.A.at<int32_t>(l.nadv);
    g.advCells = K.A.at<int32_t>(l.advc), g.mask = K.A.at<int32_t>(l.mask), g.msd = K.A.at<double>(l.msd);
    g.sign = K.A.at<double>(l.sign), g.d2 = K.A.at<double>(l.d2), g.advCoef = K.A.at<double>(l.ac);
    g.advCoef3 = K.A.at<double>(l.a3);
    int32_t *e2c0 = K.A.at<int32_t>(l.e2c0), *e2c1 = K.A.at<int32_t>(l.e2c1), *cnt = K.A.at<int32_t>(l.cnt);
    MPASO_CUDA(cudaMemsetAsync(e2c0, 0x7f, nE * sizeof(int32_t), K.st));  // 0x7f7f7f7f: above any cell id
    MPASO_CUDA(cudaMemsetAsync(e2c1, 0xff, nE * sizeof(int32_t), K.st));  // -1
    MPASO_CUDA(cudaMemsetAsync(cnt, 0, nE * sizeof(int32_t), K.st));
    MPASO_CUDA(cudaMemsetAsync(g.d2, 0, nE * kME2 * 2 * sizeof(double), K.st));
    const unsigned gc = (unsigned)((nC + tpb - 1) / tpb), ge = (unsigned)((nE + tpb - 1) / tpb);
    k_edge_cells<<<gc, tpb, 0, K.st>>>(d, e2c0, e2c1, cnt, err + i);
    k_edge_levels<<<ge, tpb, 0, K.st>>>(d, g, e2c0, e2c1, cnt, err + i);
  }
  std::vector<unsigned> h_err(nm, 0);
  auto check_errors = [&](unsigned mask) {
    MPASO_CUDA(cudaMemcpyAsync(h_err.data(), err, nm * sizeof(unsigned), cudaMemcpyDeviceToHost, K.st));
    MPASO_CUDA(cudaStreamSynchronize(K.st));
    MPASO_CUDA(cudaGetLastError());
    static const struct {
      unsigned bit;
      const char *msg;
    } kMsg[] = {{kErrEdgeIndex, "edge index out of range"},
                {kErrEdgeCells, "edge without two cells"},
                {kErrNeighbourhood, "cell neighbourhood too large"},
                {kErrBisect, "arc_bisect: midpoint on a coordinate plane (the reference asserts here)"},
                {kErrAdvCells, "more than 16 advection cells on an edge"}};
    for (int i = 0; i < nm; ++i)
      for (const auto &m : kMsg)
        if (h_err[i] & m.bit & mask)
          fail(MPASO_ERR_MESH, (nm > 1 ? "member " + std::to_string(i) + ": " : std::string()) + m.msg);
  };
  // edges listed by two cells everywhere before any kernel follows e2c
  check_errors(kErrEdgeIndex | kErrEdgeCells);
  for (int i = 0; i < nm; ++i) {
    const int64_t nC = ins[i].nCells, nE = ins[i].nEdges;
    const Layout &l = lay[i];
    const unsigned gc = (unsigned)((nC + tpb - 1) / tpb), ge = (unsigned)((nE + tpb - 1) / tpb);
    const int32_t *e2c0 = K.A.at<int32_t>(l.e2c0), *e2c1 = K.A.at<int32_t>(l.e2c1);
    k_cell_fits<<<gc, tpb, 0, K.st>>>(din[i], dout[i], e2c0, err + i);
    k_edge_stencils<<<ge, tpb, 0, K.st>>>(din[i], dout[i], e2c0, e2c1, err + i);
  }
  check_errors(~0u);
  for (int i = 0; i < nm; ++i) {
    const int64_t nC = ins[i].nCells, nE = ins[i].nEdges, L = ins[i].nlev;
    const mpaso_fct_setup_out &o = outs[i];
    const DevOut &g = dout[i];
    auto down = [&](void *h, const void *dv, size_t bytes) {
      MPASO_CUDA(cudaMemcpyAsync(h, dv, bytes, cudaMemcpyDeviceToHost, K.st));
    };
    down(o.maxLevelEdgeTop, g.maxLevelEdgeTop, nE * sizeof(int32_t));
    down(o.meshScalingDel2, g.msd, nE * sizeof(double));
    down(o.edgeSignOnCell, g.sign, nC * kME * sizeof(double));
    down(o.derivTwo, g.d2, nE * kME2 * 2 * sizeof(double));
    down(o.nAdvCellsForEdge, g.nAdv, nE * sizeof(int32_t));
    down(o.advCellsForEdge, g.advCells, nE * kME2 * sizeof(int32_t));
    down(o.highOrderAdvMask, g.mask, nE * L * sizeof(int32_t));
    down(o.advCoef, g.advCoef, nE * kME2 * sizeof(double));
    down(o.advCoef_3rd, g.advCoef3, nE * kME2 * sizeof(double));
  }
  MPASO_CUDA(cudaStreamSynchronize(K.st));
}

}  // namespace
}  // namespace mpaso

extern "C" int mpaso_fct_setup_device(const mpaso_fct_setup_in *in, mpaso_fct_setup_out *out, int32_t device) {
  return mpaso::guarded("mpaso_fct_setup_device", [&] {
    mpaso::require(in && out, MPASO_ERR_ARG, "null argument");
    mpaso::run_many(in, out, 1, device);
  });
}

extern "C" int mpaso_fct_setup_device_many(const mpaso_fct_setup_in *ins, mpaso_fct_setup_out *outs, int32_t n,
                                           int32_t device) {
  return mpaso::guarded("mpaso_fct_setup_device_many", [&] {
    mpaso::require(ins && outs && n >= 1, MPASO_ERR_ARG, "bad argument");
    mpaso::run_many(ins, outs, n, device);
  });
}

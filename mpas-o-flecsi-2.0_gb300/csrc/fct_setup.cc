// FCT / del2 static coefficients on the host: the setup of
// apps/ocean/tasks/init_functions.cc:18-447, run once per mesh.
//
// The sphere branch evaluates the same floating-point operations in the same
// order as the reference (tangent-plane projection, 6-term least-squares fit
// solved through the partial-pivoting inverse of mpasoflecsi/eqns/matrix.hh,
// edge-angle second-derivative weights, advection coefficient assembly), so
// its output equals the reference's bit for bit (compiled with
// -ffp-contract=off).  The planar branch, which the reference leaves empty,
// fits the same polynomial in plane coordinates (minimum-image offsets on a
// periodic domain) and takes the edge angle from atan2 of the edge midpoint.
#include <algorithm>
#include <array>
#include <cmath>
#include <vector>

#include "common.hh"

namespace mpaso {
namespace {

constexpr int kME = 8, kME2 = 16, kNA = 6, kMM = kME + 1;
constexpr double kA = 6371000.0;           // mpasoflecsi/common/constants.hh:28
constexpr double kPi = 3.141592653589793;  // constants.hh:29

inline double smax(double a, double b) { return (a < b) ? b : a; }  // std::max
inline double smin(double a, double b) { return (b < a) ? b : a; }  // std::min

struct Csr {
  const int64_t *off;
  const int32_t *idx;
  int64_t b(int64_t i) const { return off[i]; }
  int64_t n(int64_t i) const { return off[i + 1] - off[i]; }
  int32_t at(int64_t i, int64_t j) const { return idx[off[i] + j]; }
};

// Spherical triangle angle at a (mpasoflecsi/eqns/metrics.hh:25-73).
double sph_angle(const double *a, const double *b, const double *c) {
  const double sa = std::acos(smax(smin(b[0] * c[0] + b[1] * c[1] + b[2] * c[2], 1.0), -1.0));
  const double sb = std::acos(smax(smin(a[0] * c[0] + a[1] * c[1] + a[2] * c[2], 1.0), -1.0));
  const double sc = std::acos(smax(smin(a[0] * b[0] + a[1] * b[1] + a[2] * b[2], 1.0), -1.0));
  const double ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
  const double ac[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
  const double dx = (ab[1] * ac[2]) - (ab[2] * ac[1]);
  const double dy = (ab[2] * ac[0]) - (ab[0] * ac[2]);
  const double dz = (ab[0] * ac[1]) - (ab[1] * ac[0]);
  const double s = 0.5 * (sa + sb + sc);
  const double sin_angle =
      std::sqrt(smin(1.0, smax(0.0, (std::sin(s - sb) * std::sin(s - sc)) / (std::sin(sb) * std::sin(sc)))));
  const double ang = 2.0 * std::asin(smax(smin(sin_angle, 1.0), -1.0));
  return (dx * a[0] + dy * a[1] + dz * a[2] >= 0.0) ? ang : -ang;
}

// Great-circle arc length (metrics.hh:75-91).
double sph_arc(const double *a, const double *b) {
  const double c[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
  const double r = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  const double cl = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
  return r * 2. * std::asin(cl / (2. * r));
}

// Arc midpoint (metrics.hh:93-111); fails where the reference's assertion does.
void sph_bisect(const double *a, const double *b, double *c) {
  const double r = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  for (int k = 0; k < 3; ++k) c[k] = 0.5 * (a[k] + b[k]);
  require(c[0] != 0. && c[1] != 0. && c[2] != 0., MPASO_ERR_MESH,
          "arc_bisect: midpoint on a coordinate plane (the reference asserts here)");
  const double d = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
  for (int k = 0; k < 3; ++k) c[k] = r * c[k] / d;
}

// C = A B with accumulation from zero in index order (mpasoflecsi/eqns/matrix.hh:28-43).
template <int RA, int CA, int CB>
void mm(int ra, int ca, int cb, const double (&A)[RA][CA], const double (&B)[CA][CB], double (&C)[RA][CB]) {
  for (int r = 0; r < ra; ++r)
    for (int c = 0; c < cb; ++c) {
      double acc = 0.0;
      for (int i = 0; i < ca; ++i) acc += A[r][i] * B[i][c];
      C[r][c] = acc;
    }
}

// Inverse of a (n x n) by scaled partial-pivoting elimination
// (matrix.hh:52-167: elgs + migs, T. Pang's method).
void invert(int n, double (&a)[kNA][kNA], double (&x)[kNA][kNA]) {
  int idx[kNA];
  double scale[kNA], b[kNA][kNA];
  for (int i = 0; i < n; ++i) {
    idx[i] = i;
    double c1 = 0.;
    for (int j = 0; j < n; ++j) c1 = smax(c1, std::fabs(a[i][j]));
    scale[i] = c1;
  }
  for (int j = 0; j < n - 1; ++j) {
    int k = j;
    double best = 0.0;
    for (int i = j; i < n; ++i) {
      const double p = std::fabs(a[idx[i]][j]) / scale[idx[i]];
      if (p > best) best = p, k = i;
    }
    std::swap(idx[j], idx[k]);
    for (int i = j + 1; i < n; ++i) {
      const double pj = a[idx[i]][j] / a[idx[j]][j];
      a[idx[i]][j] = pj;
      for (int kk = j + 1; kk < n; ++kk) a[idx[i]][kk] = a[idx[i]][kk] - pj * a[idx[j]][kk];
    }
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) b[i][j] = (i == j) ? 1. : 0.;
  for (int i = 0; i < n - 1; ++i)
    for (int j = i + 1; j < n; ++j)
      for (int k = 0; k < n; ++k) b[idx[j]][k] = b[idx[j]][k] - a[idx[j]][i] * b[idx[i]][k];
  for (int i = 0; i < n; ++i) {
    x[n - 1][i] = b[idx[n - 1]][i] / a[idx[n - 1]][n - 1];
    for (int j = n - 2; j >= 0; --j) {
      x[j][i] = b[idx[j]][i];
      for (int k = j + 1; k < n; ++k) x[j][i] = x[j][i] - a[idx[j]][k] * x[k][i];
      x[j][i] = x[j][i] / a[idx[j]][j];
    }
  }
}

double wrap(double d, double L) { return L > 0 ? d - L * std::nearbyint(d / L) : d; }

// derivTwo (init_functions.cc:83-328).
void second_derivative_weights(const mpaso_fct_setup_in &in, const Csr &c2e, const Csr &c2c,
                               const Csr &e2v, const std::vector<int32_t> &e2c0, double *d2) {
  std::fill(d2, d2 + in.nEdges * kME2 * 2, 0.0);
  for (int64_t c = 0; c < in.nCells; ++c) {
    const int nEonC = (int)c2e.n(c);
    const int n = nEonC + 1;
    require(n <= kMM && c2c.n(c) == nEonC, MPASO_ERR_MESH, "cell neighbourhood too large");
    int64_t cl[kMM];
    cl[0] = c;
    for (int i = 0; i < nEonC; ++i) cl[i + 1] = c2c.at(c, i);
    double xp[kMM], yp[kMM], theta_t[kMM] = {0};
    double pc[kMM][3];
    if (in.on_sphere) {
      for (int i = 0; i < n; ++i) {
        pc[i][0] = in.xCell[cl[i]] / kA, pc[i][1] = in.yCell[cl[i]] / kA, pc[i][2] = in.zCell[cl[i]] / kA;
      }
      const double pole[3] = {0.0, 0.0, 1.0};
      const double theta_abs = (pc[0][2] == 1.0) ? kPi / 2.0 : kPi / 2.0 - sph_angle(pc[0], pc[1], pole);
      double theta_v[kMM], dl[kMM];
      for (int i = 0; i < n - 1; ++i) {
        const int ip2 = (i + 2 > n - 1) ? 1 : i + 2;
        theta_v[i] = sph_angle(pc[0], pc[i + 1], pc[ip2]);
        dl[i] = kA * sph_arc(pc[0], pc[i + 1]) / 1.0;
      }
      theta_t[0] = theta_abs;
      for (int i = 1; i < n - 1; ++i) theta_t[i] = theta_t[i - 1] + theta_v[i - 1];
      for (int i = 0; i < n - 1; ++i) {
        xp[i] = std::cos(theta_t[i]) * dl[i];
        yp[i] = std::sin(theta_t[i]) * dl[i];
      }
    } else {
      for (int i = 0; i < n - 1; ++i) {
        xp[i] = wrap(in.xCell[cl[i + 1]] - in.xCell[c], in.Lx);
        yp[i] = wrap(in.yCell[cl[i + 1]] - in.yCell[c], in.Ly);
      }
    }
    // least-squares fit of a + b x + c y + d x^2 + e x y + f y^2 (mpas_poly_fit_2)
    const int ma = n;
    double A[kMM][kNA] = {{0}}, W[kMM][kMM] = {{0}};
    A[0][0] = 1.0, W[0][0] = 1.0;
    for (int i = 1; i < ma; ++i) {
      const double x = xp[i - 1], y = yp[i - 1];
      A[i][0] = 1.0, A[i][1] = x, A[i][2] = y, A[i][3] = x * x, A[i][4] = x * y, A[i][5] = y * y;
      W[i][i] = 1.0;
    }
    double At[kNA][kMM] = {{0}}, Wt[kMM][kMM] = {{0}}, Hm[kMM][kMM], AtH[kNA][kMM], AtHA[kNA][kNA],
           inv[kNA][kNA], B[kNA][kMM];
    for (int i = 0; i < ma; ++i)
      for (int j = 0; j < kNA; ++j) At[j][i] = A[i][j];
    for (int i = 0; i < ma; ++i)
      for (int j = 0; j < ma; ++j) Wt[j][i] = W[i][j];
    mm(ma, ma, ma, Wt, W, Hm);
    mm(kNA, ma, ma, At, Hm, AtH);
    mm(kNA, ma, kNA, AtH, A, AtHA);
    invert(kNA, AtHA, inv);
    mm(kNA, kNA, ma, inv, AtH, B);
    for (int i = 0; i < nEonC; ++i) {
      const int64_t e = c2e.at(c, i);
      double te;
      if (in.on_sphere) {
        double v1[3], v2[3], mid[3];
        const int32_t va = e2v.at(e, 0), vb = e2v.at(e, 1);
        v1[0] = in.xVertex[va] / kA, v1[1] = in.yVertex[va] / kA, v1[2] = in.zVertex[va] / kA;
        v2[0] = in.xVertex[vb] / kA, v2[1] = in.yVertex[vb] / kA, v2[2] = in.zVertex[vb] / kA;
        sph_bisect(v1, v2, mid);
        te = sph_angle(pc[0], pc[i + 1], mid) + theta_t[i];
      } else {
        const int32_t va = e2v.at(e, 0), vb = e2v.at(e, 1);
        const double xm = 0.5 * (wrap(in.xVertex[va] - in.xCell[c], in.Lx) + wrap(in.xVertex[vb] - in.xCell[c], in.Lx));
        const double ym = 0.5 * (wrap(in.yVertex[va] - in.yCell[c], in.Ly) + wrap(in.yVertex[vb] - in.yCell[c], in.Ly));
        te = std::atan2(ym, xm);
      }
      double c2t = std::cos(te), s2t = std::sin(te);
      const double cs = c2t * s2t;
      c2t = c2t * c2t;
      s2t = s2t * s2t;
      const int side = (c == e2c0[e]) ? 0 : 1;
      for (int j = 0; j < n; ++j)
        d2[(e * kME2 + j) * 2 + side] = 2. * c2t * B[3][j] + 2. * cs * B[4][j] + 2. * s2t * B[5][j];
    }
  }
}

int find(const int64_t *l, int n, int64_t v) {
  int i = 0;
  while (i < n && l[i] != v) ++i;
  return i;
}

void run(const mpaso_fct_setup_in &in, mpaso_fct_setup_out &o) {
  const int64_t nC = in.nCells, nE = in.nEdges;
  const int L = in.nlev;
  require(nC > 0 && nE > 0 && L >= 1, MPASO_ERR_ARG, "bad sizes");
  require(in.c2e_off && in.c2c_off && in.e2v_off && in.c2e && in.c2c && in.e2v && in.dcEdge &&
              in.dvEdge && in.xCell && in.yCell && in.xVertex && in.yVertex && in.maxLevelCell,
          MPASO_ERR_ARG, "missing input array");
  require(!in.on_sphere || (in.zCell && in.zVertex), MPASO_ERR_ARG, "sphere needs z coordinates");
  const Csr c2e{in.c2e_off, in.c2e}, c2c{in.c2c_off, in.c2c}, e2v{in.e2v_off, in.e2v};
  // cells(e) by transposition of c2e: ascending ids (mpasoflecsi/specialization/mesh.cc:108-116)
  std::vector<int32_t> e2c0(nE, -1), e2c1(nE, -1);
  for (int64_t c = 0; c < nC; ++c)
    for (int64_t j = 0; j < c2e.n(c); ++j) {
      const int32_t e = c2e.at(c, j);
      require(e >= 0 && e < nE, MPASO_ERR_MESH, "edge index out of range");
      if (e2c0[e] < 0)
        e2c0[e] = (int32_t)c;
      else
        e2c1[e] = (int32_t)c;
    }
  for (int64_t e = 0; e < nE; ++e)
    require(e2c0[e] >= 0 && e2c1[e] >= 0, MPASO_ERR_MESH, "edge without two cells");
  // maxLevelEdgeTop (:18-27): the larger of the two cells' levels, as the reference takes it
  for (int64_t e = 0; e < nE; ++e)
    o.maxLevelEdgeTop[e] = std::max(in.maxLevelCell[e2c0[e]], in.maxLevelCell[e2c1[e]]);
  // meshScalingDel2 (:47-66): cells 0 and 1 for every edge, as the reference does
  double maxDensity = 0.0;
  for (int64_t c = 0; c < nC; ++c)
    if (in.meshDensity && in.meshDensity[c] > maxDensity) maxDensity = in.meshDensity[c];
  for (int64_t e = 0; e < nE; ++e) {
    if (!in.meshDensity) {
      o.meshScalingDel2[e] = 1.0;
      continue;
    }
    const double rel = (in.meshDensity[0] + in.meshDensity[nC > 1 ? 1 : 0]) / (2.0 * maxDensity);
    o.meshScalingDel2[e] = 1.0 / std::pow(rel, 0.25);
  }
  // edgeSignOnCell (:68-82)
  for (int64_t c = 0; c < nC; ++c) {
    for (int j = 0; j < kME; ++j) o.edgeSignOnCell[c * kME + j] = 0.0;
    for (int64_t j = 0; j < c2e.n(c); ++j)
      o.edgeSignOnCell[c * kME + j] = (c == e2c0[c2e.at(c, j)]) ? -1.0 : 1.0;
  }
  second_derivative_weights(in, c2e, c2c, e2v, e2c0, o.derivTwo);
  // highOrderAdvMask, advCellsForEdge, advCoef, advCoef_3rd (:342-445)
  for (int64_t e = 0; e < nE; ++e) {
    double *ac = o.advCoef + e * kME2, *a3 = o.advCoef_3rd + e * kME2;
    for (int i = 0; i < kME2; ++i) ac[i] = 0., a3[i] = 0., o.advCellsForEdge[e * kME2 + i] = 0;
    for (int k = 0; k < L; ++k) {
      int mask = 1;
      if (in.boundaryCell && (in.boundaryCell[(int64_t)e2c0[e] * L + k] == 1 ||
                              in.boundaryCell[(int64_t)e2c1[e] * L + k] == 1))
        mask = 0;
      o.highOrderAdvMask[e * L + k] = mask;
    }
    const int64_t c1 = e2c0[e], c2 = e2c1[e];
    int64_t cl[2 * kME + 2];
    int n = 0;
    cl[n++] = c1, cl[n++] = c2;
    for (int64_t j = 0; j < c2c.n(c1); ++j)
      if (find(cl, n, c2c.at(c1, j)) == n) cl[n++] = c2c.at(c1, j);
    for (int64_t j = 0; j < c2c.n(c2); ++j)
      if (find(cl, n, c2c.at(c2, j)) == n) cl[n++] = c2c.at(c2, j);
    require(n <= kME2, MPASO_ERR_MESH, "more than 16 advection cells on an edge");
    o.nAdvCellsForEdge[e] = n;
    for (int i = 0; i < n; ++i) o.advCellsForEdge[e * kME2 + i] = (int32_t)cl[i];
    const double *D = o.derivTwo + e * kME2 * 2;
    int i1 = find(cl, n, c1);
    ac[i1] = ac[i1] + D[0], a3[i1] = a3[i1] + D[0];
    for (int64_t j = 0; j < c2e.n(c1); ++j) {
      const int ix = find(cl, n, c2c.at(c1, j));
      ac[ix] = ac[ix] + D[(j + 1) * 2], a3[ix] = a3[ix] + D[(j + 1) * 2];
    }
    const int i2 = find(cl, n, c2);
    ac[i2] = ac[i2] + D[1], a3[i2] = a3[i2] - D[1];
    for (int64_t j = 0; j < c2e.n(c2); ++j) {
      const int ix = find(cl, n, c2c.at(c2, j));
      ac[ix] = ac[ix] + D[(j + 1) * 2 + 1], a3[ix] = a3[ix] - D[(j + 1) * 2 + 1];
    }
    const double dc = in.dcEdge[e], dv = in.dvEdge[e];
    for (int i = 0; i < n; ++i) {
      ac[i] = -(dc * dc) * ac[i] / 12.0;
      a3[i] = -(dc * dc) * a3[i] / 12.0;
    }
    ac[i1] = ac[i1] + 0.5;
    ac[i2] = ac[i2] + 0.5;
    for (int i = 0; i < n; ++i) ac[i] = dv * ac[i], a3[i] = dv * a3[i];
  }
}

}  // namespace
}  // namespace mpaso

extern "C" int mpaso_fct_setup(const mpaso_fct_setup_in *in, mpaso_fct_setup_out *out) {
  return mpaso::guarded("mpaso_fct_setup", [&] {
    mpaso::require(in && out, MPASO_ERR_ARG, "null argument");
    mpaso::require(out->maxLevelEdgeTop && out->meshScalingDel2 && out->edgeSignOnCell && out->derivTwo &&
                       out->nAdvCellsForEdge && out->advCellsForEdge && out->highOrderAdvMask &&
                       out->advCoef && out->advCoef_3rd,
                   MPASO_ERR_ARG, "missing output array");
    mpaso::run(*in, *out);
  });
}

// Test-case initialisers and error norms on the device: the sw app's
// Williamson cases 1, 5 and 6 (apps/sw/tasks/testcase.cc:37-227) with the
// case-1 error norm (apps/sw/tasks/solve.cc:404-436), and the ocean app's
// cases 1-3 with their error norms (apps/ocean/tasks/testcase.cc:16-294).
//
// They write a state's fields in place, in the context's numbering, from the
// mesh geometry the caller gave once (mpaso_mesh_set_geometry), so a run --
// or each member of an ensemble -- starts without a host round trip.  The
// formulas are the reference's, in its order of operations; sin, cos, asin,
// pow and exp are CUDA's, which may differ from the host library's in the
// last place.  The norms are sums over cells reduced on the device in a fixed
// order (per-block partial sums, then one block over the partials).
#include <cstring>

#include "rk4.cuh"

namespace mpaso {

// Geometry the initialisers read, in the context's numbering.
struct DGeo {
  const double *latC, *lonC, *latV, *lonV, *latE, *lonE, *angE, *xC, *yC, *zC;
};

namespace {

constexpr int TPB = 256;
constexpr double kA = 6371000.0;             // mpasoflecsi/common/constants.hh:28
constexpr double kPi = 3.141592653589793;    // constants.hh:29
constexpr double kGravity = 9.80616;         // constants.hh:30-31
constexpr double kOmega = 7.29212e-5;        // constants.hh:32-33

DGeo geo_of(const MeshCtx &c) {
  require(c.geo != nullptr, MPASO_ERR_ARG, "no mesh geometry: call mpaso_mesh_set_geometry first");
  const double *g = c.geo;
  const int64_t nC = c.d.nC, nE = c.d.nE, nV = c.d.nV;
  DGeo o;
  o.latC = g, o.lonC = g + nC, o.latV = g + 2 * nC, o.lonV = g + 2 * nC + nV;
  o.latE = g + 2 * nC + 2 * nV, o.lonE = o.latE + nE, o.angE = o.lonE + nE;
  o.xC = o.angE + nE, o.yC = o.xC + nC, o.zC = o.yC + nC;
  return o;
}

__device__ __forceinline__ double sq(double x) { return x * x; }

// Great-circle distance (mpasoflecsi/eqns/metrics.hh:14-21).
__device__ double sphere_distance(double lat1, double lon1, double lat2, double lon2, double radius) {
  const double arg1 = sqrt(sq(sin(0.5 * (lat2 - lat1))) + cos(lat1) * cos(lat2) * sq(sin(0.5 * (lon2 - lon1))));
  return 2 * radius * asin(arg1);
}

// Arc length from (ax, ay, az) to (bx, by, bz) (metrics.hh:75-91).
__device__ double sphere_arc_length(double ax, double ay, double az, double bx, double by, double bz) {
  const double cx = bx - ax, cy = by - ay, cz = bz - az;
  const double r = sqrt(ax * ax + ay * ay + az * az);
  const double c = sqrt(cx * cx + cy * cy + cz * cz);
  return r * 2. * asin(c / (2. * r));
}

// ---------------------------------------------------------------- sw cases
// Cosine bell of case 1 (apps/sw/tasks/testcase.cc:68-76), centred at (0, lon_c).
__device__ double bell(double lat, double lon, double lon_c) {
  constexpr double h0 = 1000.0;
  const double r = sphere_distance(0.0, lon_c, lat, lon, kA);
  return r < kA / 3.0 ? (h0 / 2.0) * (1.0 + cos(kPi * r * 3.0 / kA)) : h0 / 2.0;
}

// Streamfunction at vertices of cases 1 and 5 (testcase.cc:54-59, 105-110).
__device__ double psi_solid(double latV, double lonV, double u0) {
  constexpr double alpha = 0.0;
  return -kA * u0 * (sin(latV) * cos(alpha) - cos(lonV) * cos(latV) * sin(alpha));
}

// Rossby-Haurwitz streamfunction of case 6 (testcase.cc:203-207).
__device__ double psi_rh(double latV, double lonV) {
  constexpr double w = 7.848e-6, K = 7.848e-6, R = 4.0;
  return -kA * kA * w * sin(latV) + kA * kA * K * pow(cos(latV), R) * sin(latV) * cos(R * lonV);
}

// Case 5 mountain distance and its tracer cones (testcase.cc:140-163).
__device__ double cone_r(double lat, double lon, double theta_c) {
  constexpr double lambda_c = 3.0 * kPi / 2.0, rr = kPi / 9.0;
  return sqrt(fmin(rr * rr, sq(lon - lambda_c) + sq(lat - theta_c)));
}

// Edges: u at every level from the vertex streamfunction,
// u = -(psi(v1) - psi(v0)) / dvEdge with (v0, v1) = vertices(e) (testcase.cc:61-66).
__global__ void k_sw_case_u(DMesh m, DGeo g, int which, int L, double *u) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= m.nE) return;
  const int2 v = m.voe[e];
  double p0, p1;
  if (which == 6) {
    p0 = psi_rh(g.latV[v.x], g.lonV[v.x]), p1 = psi_rh(g.latV[v.y], g.lonV[v.y]);
  } else {
    const double u0 = which == 1 ? 2.0 * kPi * kA / (12.0 * 86400.0) : 20.0;
    p0 = psi_solid(g.latV[v.x], g.lonV[v.x], u0), p1 = psi_solid(g.latV[v.y], g.lonV[v.y], u0);
  }
  const double ue = -1.0 * (p1 - p0) / m.dvEdge[e];
  for (int k = 0; k < L; ++k) u[e * L + k] = ue;
}

// Cells: h (and, case 5, the bottom topography and the two cone tracers).
__global__ void k_sw_case_h(DMesh m, DGeo g, int which, int L, int T, double *h, double *tr, double *hs_out) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= m.nC) return;
  const double lat = g.latC[c];
  double lon = g.lonC[c];
  double hc, t0 = 0.0, t1 = 0.0;
  if (which == 1) {
    hc = bell(lat, lon, 3.0 * kPi / 2.0);
  } else if (which == 5) {
    constexpr double u0 = 20, gh0 = 5960.0 * kGravity, hs0 = 2000, alpha = 0;
    constexpr double theta_c = kPi / 6.0, rr = kPi / 9.0;
    if (lon < 0) lon = lon + 2.0 * kPi;
    const double r = cone_r(lat, lon, theta_c);
    const double hs = hs0 * (1.0 - r / rr);
    hs_out[c] = hs;
    t0 = 1.0 - r / rr;
    t1 = 1.0 - cone_r(lat, lon, theta_c + kPi / 6.0) / rr;
    hc = (gh0 - (kA * kOmega * u0 + 0.5 * u0 * u0) *
                    sq(-cos(lon) * cos(lat) * sin(alpha) + sin(lat) * cos(alpha))) / kGravity;
    hc = hc - hs;
  } else {  // 6: Rossby-Haurwitz wave (testcase.cc:183-224)
    constexpr double h0 = 8000.0, w = 7.848e-6, K = 7.848e-6, R = 4.0;
    const double ct = cos(lat);
    const double aa = 0.5 * w * (2.0 * kOmega + w) * pow(ct, 2) +
                      0.25 * pow(K, 2) * pow(ct, (2 * R)) *
                          ((R + 1.0) * pow(ct, 2) + 2.0 * pow(R, 2) - R - 2.0 - 2.0 * pow(R, 2) * pow(ct, -2));
    const double bb = (2.0 * (kOmega + w) * K / ((R + 1.0) * (R + 2.0))) * pow(ct, R) *
                      ((pow(R, 2) + 2.0 * R + 2.0) - pow((R + 1.0) * ct, 2));
    const double cc = 0.25 * pow(K, 2) * pow(ct, (2.0 * R)) * ((R + 1.0) * pow(ct, 2) - R - 2.0);
    hc = (kGravity * h0 + kA * kA * aa + kA * kA * bb * cos(R * lon) + kA * kA * cc * cos(2.0 * R * lon)) /
         kGravity;
  }
  for (int k = 0; k < L; ++k) {
    h[c * L + k] = hc;
    for (int t = 0; t < T; ++t) tr[(c * L + k) * T + t] = t == 0 ? t0 : t == 1 ? t1 : 0.0;
  }
}

// Case 5: the state's per-edge bottom-depth difference hs(c2) - hs(c1).
__global__ void k_sw_case_dhs(DMesh m, const double *hs, double *dhs) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= m.nE) return;
  const int2 c = m.coe[e];
  dhs[e] = hs[c.y] - hs[c.x];
}

// ------------------------------------------------------------- ocean cases
constexpr double kDay = 86400.0;

// apps/ocean/tasks/testcase.cc:16-22
__device__ double rotation_velocity(double latE, double angleE) {
  constexpr double u0 = 2.0 * kPi * kA / 86400.0;
  return u0 * cos(latE) * cos(angleE);
}

// testcase.cc:24-34
__device__ double gaussian_dist(double xC) {
  constexpr double maxG = 21983.7698959881, Knorm = 20.0 / maxG, kappa = 10.0, T0 = 50.0;
  return T0 + Knorm * exp(kappa * xC / kA);
}

// testcase.cc:36-60
__device__ double slot_cyl_dist(double xC, double yC, double zC, double latC, double lonC) {
  const double aa = kA / 2., hw = kA / 12., bot = -kA / 3.;
  const double dist = sphere_arc_length(xC, yC, zC, kA, 0., 0.);
  double longC = lonC;
  if (longC > kPi) longC -= 2. * kPi;
  if (dist > aa) return 50.;
  if ((kA * latC > bot) && (kA * latC < aa) && (kA * fabs(longC) < hw)) return 50.;
  return 100.;
}

// testcase.cc:62-73
__device__ double harmonic_dist(double latC, double lonC, double coef, double elapsed) {
  const double cosLat = cos(latC);
  return 50. + 20. * cosLat * cosLat * cos(2. * lonC) * exp(-6.0 * coef * elapsed / (kA * kA));
}

// setup_case_1/2/3 (testcase.cc:96-173): u (edges), h = 1 and layerThicknessEdge
// = 0.5 (h1 + h2) = 1 (init_functions.cc:30-45), tracer 0 by case.
__global__ void k_oc_case(DMesh m, DGeo g, int which, int L, int T, double coef, double *u, double *hE,
                          double *h, double *tr) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < m.nE) {
    const double ue = which == 3 ? 0.0 : rotation_velocity(g.latE[i], g.angE[i]);
    for (int k = 0; k < L; ++k) u[i * L + k] = ue, hE[i * L + k] = 0.5 * (1. + 1.);
  }
  if (i < m.nC) {
    const double t0 = which == 1   ? gaussian_dist(g.xC[i])
                      : which == 2 ? slot_cyl_dist(g.xC[i], g.yC[i], g.zC[i], g.latC[i], g.lonC[i])
                                   : harmonic_dist(g.latC[i], g.lonC[i], coef, 0.0);
    for (int k = 0; k < L; ++k) {
      h[i * L + k] = 1.;
      for (int t = 0; t < T; ++t) tr[(i * L + k) * T + t] = t == 0 ? t0 : 0.0;
    }
  }
}

// ------------------------------------------------------------- error norms
// Per-cell terms summed over cells: sw case 1 {(h - h_true)^2 w, h_true^2 w, |h - h_true| / h_true}
// with w = cos(lat) / area (solve.cc:420-426); ocean cases {err^2, 0, |err|}, err = (tr - true) / true
// (testcase.cc:186-199, 230-247, 272-284).  Level 0, tracer 0.
__device__ void case_terms(const DMesh &m, const DGeo &g, int app, int which, double elapsed, double coef,
                           const double *h, const double *tr, int L, int T, int64_t c, double o[3]) {
  if (app == MPASO_APP_SW) {
    const double day_frac = elapsed / 86400 / 12;
    const double rot_ang = (3 * kPi / 2.) + 2 * kPi * day_frac;
    const double ht = bell(g.latC[c], g.lonC[c], rot_ang);
    const double w = cos(g.latC[c]) / m.areaCell[c];
    const double d = h[c * L] - ht;
    o[0] = sq(d) * w, o[1] = sq(ht) * w, o[2] = fabs(d) / ht;
    return;
  }
  const double rot = 2.0 * kPi * (elapsed / kDay);
  double t;
  if (which == 1) {
    const double xp = g.xC[c] * cos(-rot) - g.yC[c] * sin(-rot);
    t = gaussian_dist(xp);
  } else if (which == 2) {
    const double xp = g.xC[c] * cos(rot) + g.yC[c] * sin(rot);
    const double yp = -g.xC[c] * sin(rot) + g.yC[c] * cos(rot);
    t = slot_cyl_dist(xp, yp, g.zC[c], g.latC[c], g.lonC[c] - rot);
  } else {
    t = harmonic_dist(g.latC[c], g.lonC[c], coef, elapsed);
  }
  const double err = (tr[c * L * T] - t) / t;
  o[0] = err * err, o[1] = 0.0, o[2] = fabs(err);
}

constexpr int kErrBlocks = 304;  // 2 per SM on GB300; any count gives the same sums

__global__ void __launch_bounds__(TPB) k_case_error(DMesh m, DGeo g, int app, int which, double elapsed,
                                                    double coef, const double *h, const double *tr, int L,
                                                    int T, double *part) {
  __shared__ double s[3][TPB];
  double acc[3] = {0.0, 0.0, 0.0};
  for (int64_t c = blockIdx.x * (int64_t)TPB + threadIdx.x; c < m.nC; c += (int64_t)gridDim.x * TPB) {
    double o[3];
    case_terms(m, g, app, which, elapsed, coef, h, tr, L, T, c, o);
    acc[0] += o[0], acc[1] += o[1], acc[2] = fmax(acc[2], o[2]);
  }
  for (int q = 0; q < 3; ++q) s[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int w = TPB / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      s[0][threadIdx.x] += s[0][threadIdx.x + w];
      s[1][threadIdx.x] += s[1][threadIdx.x + w];
      s[2][threadIdx.x] = fmax(s[2][threadIdx.x], s[2][threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 3; ++q) part[blockIdx.x * 3 + q] = s[q][0];
}

// One thread adds the per-block partials in block order.
__global__ void k_case_error_sum(const double *part, int nb, double *out) {
  if (blockIdx.x || threadIdx.x) return;
  double a = 0.0, b = 0.0, mx = 0.0;
  for (int i = 0; i < nb; ++i) a += part[3 * i], b += part[3 * i + 1], mx = fmax(mx, part[3 * i + 2]);
  out[0] = a, out[1] = b, out[2] = mx;
}

double *aux_buffer(SwState &s, size_t bytes) {
  if (bytes > s.aux_bytes) {
    if (s.aux) {
      MPASO_CUDA(cudaStreamSynchronize(s.stream));
      MPASO_CUDA(cudaFree(s.aux));
      s.aux = nullptr, s.aux_bytes = 0;
    }
    if (cudaMalloc(&s.aux, bytes) != cudaSuccess) {
      cudaGetLastError();
      fail(MPASO_ERR_ALLOC, "device allocation of " + std::to_string(bytes) + " bytes failed");
    }
    s.aux_bytes = bytes;
  }
  return s.aux;
}

}  // namespace
}  // namespace mpaso

using namespace mpaso;

extern "C" {

int mpaso_mesh_set_geometry(mpaso_mesh m, const mpaso_geometry *g) {
  return guarded("mpaso_mesh_set_geometry", [&] {
    require(m && g, MPASO_ERR_ARG, "null argument");
    const double *src[10] = {g->latCell, g->lonCell, g->latVertex, g->lonVertex, g->latEdge,
                             g->lonEdge, g->angleEdge, g->xCell, g->yCell, g->zCell};
    for (const double *p : src) require(p != nullptr, MPASO_ERR_ARG, "null geometry array");
    MeshCtx &c = m->ctx;
    MPASO_CUDA(cudaSetDevice(c.device));
    const int64_t nC = c.d.nC, nE = c.d.nE, nV = c.d.nV;
    const int64_t n[10] = {nC, nC, nV, nV, nE, nE, nE, nC, nC, nC};
    const int ent[10] = {MPASO_CELLS, MPASO_CELLS, MPASO_VERTICES, MPASO_VERTICES, MPASO_EDGES,
                         MPASO_EDGES, MPASO_EDGES, MPASO_CELLS, MPASO_CELLS, MPASO_CELLS};
    const int64_t total = 5 * nC + 2 * nV + 3 * nE;
    if (!c.geo) {
      if (cudaMalloc(&c.geo, total * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        c.geo = nullptr;
        fail(MPASO_ERR_ALLOC, "device allocation of the mesh geometry failed");
      }
    }
    int64_t maxn = std::max(nC, std::max(nE, nV));
    double *stage = (double *)c.ensure_scratch(maxn * sizeof(double));
    int64_t off = 0;
    for (int q = 0; q < 10; ++q) {
      const double *s = src[q];
      if (!is_device_pointer(s)) {
        MPASO_CUDA(cudaMemcpyAsync(stage, s, n[q] * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        s = stage;
      }
      k_gather_rows_pub(s, c.geo + off, c.d_perm[ent[q]], n[q], 1, c.stream);
      MPASO_CUDA(cudaGetLastError());
      off += n[q];
    }
    MPASO_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int mpaso_state_setup_case(mpaso_state st, int32_t test_case, double coef) {
  return guarded("mpaso_state_setup_case", [&] {
    require(st != nullptr, MPASO_ERR_ARG, "null state");
    SwState &s = st->s;
    MeshCtx &c = s.mesh->ctx;
    MPASO_CUDA(cudaSetDevice(c.device));
    const DGeo g = geo_of(c);
    const DMesh &m = c.d;
    // the state's stream must see the geometry the mesh context's stream wrote
    MPASO_CUDA(cudaStreamSynchronize(c.stream));
    const int L = s.L, T = s.T;
    if (s.p.app == MPASO_APP_SW) {
      require(test_case == 1 || test_case == 5 || test_case == 6, MPASO_ERR_ARG,
              "sw test cases are 1, 5 and 6");
      k_sw_case_u<<<blocks_for(m.nE, TPB), TPB, 0, s.stream>>>(m, g, test_case, L, s.U[0]);
      double *hs = test_case == 5 ? aux_buffer(s, (size_t)m.nC * sizeof(double)) : nullptr;
      k_sw_case_h<<<blocks_for(m.nC, TPB), TPB, 0, s.stream>>>(m, g, test_case, L, T, s.H[0], s.TR0, hs);
      if (test_case == 5)
        k_sw_case_dhs<<<blocks_for(m.nE, TPB), TPB, 0, s.stream>>>(m, hs, (double *)s.st.dhs);
      s.diag_valid = false;
    } else {
      require(test_case >= 1 && test_case <= 3, MPASO_ERR_ARG, "ocean test cases are 1, 2 and 3");
      k_oc_case<<<blocks_for(std::max(m.nE, m.nC), TPB), TPB, 0, s.stream>>>(m, g, test_case, L, T, coef,
                                                                             s.U[0], s.HE, s.H[0], s.TR0);
      s.prep_dt = 0.0;  // thickness flux and 1/hProv of the new state are recomputed
    }
    MPASO_CUDA(cudaGetLastError());
    MPASO_CUDA(cudaStreamSynchronize(s.stream));
  });
}

int mpaso_state_case_error(mpaso_state st, int32_t test_case, double elapsed, double coef, double *err) {
  return guarded("mpaso_state_case_error", [&] {
    require(st && err, MPASO_ERR_ARG, "null argument");
    SwState &s = st->s;
    MeshCtx &c = s.mesh->ctx;
    MPASO_CUDA(cudaSetDevice(c.device));
    const DGeo g = geo_of(c);
    const DMesh &m = c.d;
    MPASO_CUDA(cudaStreamSynchronize(c.stream));
    if (s.p.app == MPASO_APP_SW)
      require(test_case == 1, MPASO_ERR_ARG, "the sw app's error norm is that of test case 1");
    else
      require(test_case >= 1 && test_case <= 3, MPASO_ERR_ARG, "ocean test cases are 1, 2 and 3");
    require(s.p.app == MPASO_APP_SW || s.T >= 1, MPASO_ERR_ARG, "state has no tracers");
    double *part = aux_buffer(s, (size_t)(3 * kErrBlocks + 3) * sizeof(double));
    k_case_error<<<kErrBlocks, TPB, 0, s.stream>>>(m, g, s.p.app, test_case, elapsed, coef, s.H[0], s.TR0, s.L,
                                                   std::max(s.T, 1), part);
    k_case_error_sum<<<1, 32, 0, s.stream>>>(part, kErrBlocks, part + 3 * kErrBlocks);
    MPASO_CUDA(cudaGetLastError());
    double sums[3];
    MPASO_CUDA(cudaMemcpyAsync(sums, part + 3 * kErrBlocks, sizeof(sums), cudaMemcpyDeviceToHost, s.stream));
    MPASO_CUDA(cudaStreamSynchronize(s.stream));
    if (s.p.app == MPASO_APP_SW) {
      // num /= 4 pi, den /= 4 pi, err = sqrt(num) / sqrt(den) (solve.cc:429-433)
      const double num = sums[0] / (4 * kPi), den = sums[1] / (4 * kPi);
      err[0] = std::sqrt(num) / std::sqrt(den);
    } else {
      err[0] = std::sqrt(sums[0]) / (double)m.nC;  // testcase.cc:199
    }
    err[1] = sums[2];
  });
}

}  // extern "C"

/* TEST INFRASTRUCTURE ONLY -- CPU oracle of the MPAS-O-FleCSI RK4 tendency path.
 *
 * A plain-C restatement of the reference's task loops with runtime level and
 * tracer counts.  Each function follows the reference lines it cites, in the
 * same floating-point evaluation order, so that it agrees bit for bit with the
 * reference sources compiled through oracle/shim/ (checked by
 * tests/test_oracle_pin.py).  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load this library; the product never does.
 *
 * Layouts are the reference's AoS: vlreal [n][L], vltracer [n][L][T],
 * metensor [n][8], me2tensor [n][16], vdtensor [n][3], derivtensor [n][16][2].
 * Build with -ffp-contract=off so no multiply-add is fused.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define MAXE 8
#define MAXE2 16

static __thread char g_err[256];
const char *orc_last_error(void) { return g_err; }
static int fail(const char *msg) {
  snprintf(g_err, sizeof g_err, "%s", msg);
  return 1;
}

int orc_compiled_levels(int32_t *nlev, int32_t *ntr, double *gravity) {
  *nlev = -1, *ntr = -1, *gravity = -1.0;
  return 0;
}

/* std::max / std::min semantics (first argument wins ties and NaN compares). */
static inline double smax(double a, double b) { return (a < b) ? b : a; }
static inline double smin(double a, double b) { return (b < a) ? b : a; }

#define OFF(m, c) ((m)->off[c])
#define IDX(m, c) ((m)->idx[c])
#define ROWB(m, c, i) ((m)->off[c][i])
#define ROWE(m, c, i) ((m)->off[c][(i) + 1])

/* ======================================================= sw tasks */

/* apps/sw/tasks/solve.cc:11-107 */
int orc_sw_compute_solve_diagnostics(const orc_mesh *m, const orc_static *s, const orc_config *c,
                                     const double *h, const double *u, double *h_edge,
                                     double *h_vertex, double *circulation, double *vorticity,
                                     double *ke, double *pv_edge, double *pv_vertex) {
  const int64_t L = c->nlev;
  for (int64_t e = 0; e < m->nE; ++e) { /* :31-39 */
    const int64_t c1 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e)];
    const int64_t c2 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e) + 1];
    for (int64_t k = 0; k < L; ++k) h_edge[e * L + k] = 0.5 * (h[c1 * L + k] + h[c2 * L + k]);
  }
  for (int64_t v = 0; v < m->nV; ++v) /* :42-46 */
    for (int64_t k = 0; k < L; ++k) circulation[v * L + k] = 0.0;
  for (int64_t e = 0; e < m->nE; ++e) { /* :47-55 */
    const int64_t v1 = IDX(m, ORC_E2V)[ROWB(m, ORC_E2V, e)];
    const int64_t v2 = IDX(m, ORC_E2V)[ROWB(m, ORC_E2V, e) + 1];
    for (int64_t k = 0; k < L; ++k) {
      circulation[v1 * L + k] = circulation[v1 * L + k] - s->dcEdge[e] * u[e * L + k];
      circulation[v2 * L + k] = circulation[v2 * L + k] + s->dcEdge[e] * u[e * L + k];
    }
  }
  for (int64_t v = 0; v < m->nV; ++v) /* :56-60 */
    for (int64_t k = 0; k < L; ++k) vorticity[v * L + k] = circulation[v * L + k] / s->areaTriangle[v];
  for (int64_t ic = 0; ic < m->nC; ++ic) { /* :63-77 */
    for (int64_t k = 0; k < L; ++k) ke[ic * L + k] = 0.0;
    for (int64_t j = ROWB(m, ORC_C2E, ic); j < ROWE(m, ORC_C2E, ic); ++j) {
      const int64_t e = IDX(m, ORC_C2E)[j];
      for (int64_t k = 0; k < L; ++k)
        ke[ic * L + k] += 0.25 * s->dcEdge[e] * s->dvEdge[e] * (u[e * L + k] * u[e * L + k]);
    }
    for (int64_t k = 0; k < L; ++k) ke[ic * L + k] /= s->areaCell[ic];
  }
  for (int64_t v = 0; v < m->nV; ++v) { /* :81-92 */
    const int32_t *vc = IDX(m, ORC_V2C) + ROWB(m, ORC_V2C, v);
    for (int64_t k = 0; k < L; ++k) {
      h_vertex[v * L + k] = 0.0;
      for (int i = 0; i < 3; ++i)
        h_vertex[v * L + k] += h[(int64_t)vc[i] * L + k] * s->kiteAreasOnVertex[v * 3 + i];
      h_vertex[v * L + k] /= s->areaTriangle[v];
      pv_vertex[v * L + k] = (s->fVertex[v] + vorticity[v * L + k]) / h_vertex[v * L + k];
    }
  }
  for (int64_t e = 0; e < m->nE; ++e) /* :95-99 */
    for (int64_t k = 0; k < L; ++k) pv_edge[e * L + k] = 0.0;
  for (int64_t v = 0; v < m->nV; ++v) /* :100-106 */
    for (int64_t j = ROWB(m, ORC_V2E, v); j < ROWE(m, ORC_V2E, v); ++j) {
      const int64_t e = IDX(m, ORC_V2E)[j];
      for (int64_t k = 0; k < L; ++k) pv_edge[e * L + k] += 0.5 * pv_vertex[v * L + k];
    }
  return 0;
}

/* apps/sw/tasks/solve.cc:169-234 */
int orc_sw_compute_tend(const orc_mesh *m, const orc_static *s, const orc_config *c,
                        const double *h_edge, const double *h, const double *u, const double *ke,
                        const double *pv_edge, double *tend_h, double *tend_u) {
  const int64_t L = c->nlev;
  const double g = c->gravity;
  for (int64_t ic = 0; ic < m->nC; ++ic)
    for (int64_t k = 0; k < L; ++k) tend_h[ic * L + k] = 0;
  for (int64_t e = 0; e < m->nE; ++e) { /* :191-201 */
    const int64_t c1 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e)];
    const int64_t c2 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e) + 1];
    for (int64_t k = 0; k < L; ++k) {
      const double flux = u[e * L + k] * s->dvEdge[e] * h_edge[e * L + k];
      tend_h[c1 * L + k] -= flux;
      tend_h[c2 * L + k] += flux;
    }
  }
  for (int64_t ic = 0; ic < m->nC; ++ic) /* :202-206 */
    for (int64_t k = 0; k < L; ++k) tend_h[ic * L + k] /= s->areaCell[ic];
  for (int64_t e = 0; e < m->nE; ++e)
    for (int64_t k = 0; k < L; ++k) tend_u[e * L + k] = 0.0;
  for (int64_t e = 0; e < m->nE; ++e) { /* :215-233 */
    const int64_t c1 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e)];
    const int64_t c2 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e) + 1];
    for (int64_t k = 0; k < L; ++k) {
      double q = 0;
      int64_t j = 0;
      for (int64_t p = ROWB(m, ORC_E2E, e); p < ROWE(m, ORC_E2E, e); ++p, ++j) {
        const int64_t eoe = IDX(m, ORC_E2E)[p];
        const double workpv = 0.5 * (pv_edge[e * L + k] + pv_edge[eoe * L + k]);
        q = q + s->weightsOnEdge[e * MAXE2 + j] * u[eoe * L + k] * workpv * h_edge[eoe * L + k];
      }
      tend_u[e * L + k] =
          q - (ke[c2 * L + k] - ke[c1 * L + k] +
               g * (h[c2 * L + k] + s->bottomDepth[c2] - h[c1 * L + k] - s->bottomDepth[c1])) /
                  s->dcEdge[e];
    }
  }
  return 0;
}

/* apps/sw/tasks/solve.cc:237-270 */
int orc_sw_compute_scalar_tend(const orc_mesh *m, const orc_static *s, const orc_config *c,
                               const double *h_edge, const double *u, const double *tracers,
                               double *tracer_tend) {
  const int64_t L = c->nlev, T = c->ntr;
  for (int64_t i = 0; i < m->nC * L * T; ++i) tracer_tend[i] = 0.0;
  for (int64_t e = 0; e < m->nE; ++e) {
    const int64_t c1 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e)];
    const int64_t c2 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e) + 1];
    for (int64_t k = 0; k < L; ++k)
      for (int64_t t = 0; t < T; ++t) {
        const double tracer_edge = 0.5 * (tracers[(c1 * L + k) * T + t] + tracers[(c2 * L + k) * T + t]);
        const double flux = u[e * L + k] * s->dvEdge[e] * h_edge[e * L + k] * tracer_edge;
        tracer_tend[(c1 * L + k) * T + t] -= flux / s->areaCell[c1];
        tracer_tend[(c2 * L + k) * T + t] += flux / s->areaCell[c2];
      }
  }
  return 0;
}

/* apps/sw/tasks/solve.cc:273-314 */
int orc_sw_compute_substep(const orc_mesh *m, const orc_config *c, double *u_provis,
                           const double *u_old, const double *u_tend, double *h_provis,
                           const double *h_old, const double *h_tend, double *tr_provis,
                           const double *tr_old, const double *tr_tend, double rkweight) {
  const int64_t L = c->nlev, T = c->ntr;
  for (int64_t i = 0; i < m->nE * L; ++i) u_provis[i] = u_old[i] + rkweight * u_tend[i];
  for (int64_t i = 0; i < m->nC * L; ++i) h_provis[i] = h_old[i] + rkweight * h_tend[i];
  for (int64_t i = 0; i < m->nC * L; ++i)
    for (int64_t t = 0; t < T; ++t)
      tr_provis[i * T + t] = (h_old[i] * tr_old[i * T + t] + rkweight * tr_tend[i * T + t]) / h_provis[i];
  if (c->pin_u)
    for (int64_t i = 0; i < m->nE * L; ++i) u_provis[i] = u_old[i];
  return 0;
}

/* apps/sw/tasks/solve.cc:317-341 */
int orc_sw_accumulate_update(const orc_mesh *m, const orc_config *c, double *u_new,
                             const double *u_tend, double *h_new, const double *h_tend,
                             double *tr_new, const double *tr_tend, double rkweight) {
  const int64_t L = c->nlev, T = c->ntr;
  for (int64_t i = 0; i < m->nE * L; ++i) u_new[i] += rkweight * u_tend[i];
  for (int64_t i = 0; i < m->nC * L; ++i) {
    h_new[i] += rkweight * h_tend[i];
    for (int64_t t = 0; t < T; ++t) tr_new[i * T + t] += rkweight * tr_tend[i * T + t];
  }
  return 0;
}

/* apps/sw/tasks/solve.cc:344-367 */
int orc_sw_finalize_timestep(const orc_mesh *m, const orc_config *c, const double *u_old,
                             double *u_new, const double *h_new, double *tr_new) {
  const int64_t L = c->nlev, T = c->ntr;
  for (int64_t i = 0; i < m->nC * L; ++i)
    for (int64_t t = 0; t < T; ++t) tr_new[i * T + t] /= h_new[i];
  if (c->pin_u)
    for (int64_t i = 0; i < m->nE * L; ++i) u_new[i] = u_old[i];
  return 0;
}

int orc_sw_del2_momentum_impl(const orc_mesh *m, const orc_static *s, const orc_config *c,
                              const double *u, const double *vorticity, double *tend_u);
int orc_sw_del2_momentum(const orc_mesh *m, const orc_static *s, const orc_config *c,
                         const double *u, const double *vorticity, double *tend_u) {
  return orc_sw_del2_momentum_impl(m, s, c, u, vorticity, tend_u);
}

/* ======================================================= ocean tasks */

/* apps/ocean/tasks/solve.cc:40-57 */
int orc_oc_normal_thickness_flux(const orc_mesh *m, const orc_config *c, const double *hEdge,
                                 const double *u, double *ntf) {
  for (int64_t i = 0; i < m->nE * c->nlev; ++i) ntf[i] = u[i] * hEdge[i];
  return 0;
}

/* apps/ocean/tasks/solve.cc:60-97 */
int orc_oc_provisional_layer_thicknesses(const orc_mesh *m, const orc_static *s,
                                         const orc_config *c, const double *h, const double *ntf,
                                         const double *w, double *hProv, double *hProvInv,
                                         double *hNewInv, double dt) {
  const int64_t L = c->nlev;
  (void)w;
  for (int64_t ic = 0; ic < m->nC; ++ic) {
    const double dtInvAreaCell = dt / s->areaCell[ic];
    const int64_t kmax = s->maxLevelCell[ic];
    for (int64_t k = 0; k < kmax; ++k) hProv[ic * L + k] = h[ic * L + k];
    int64_t je = 0;
    for (int64_t j = ROWB(m, ORC_C2E, ic); j < ROWE(m, ORC_C2E, ic); ++j, ++je) {
      const int64_t e = IDX(m, ORC_C2E)[j];
      const double signedFactor = dtInvAreaCell * s->dvEdge[e] * s->edgeSignOnCell[ic * MAXE + je];
      for (int64_t k = 0; k < kmax; ++k) hProv[ic * L + k] += signedFactor * ntf[e * L + k];
    }
    for (int64_t k = 0; k < kmax; ++k) {
      hProvInv[ic * L + k] = 1.0 / hProv[ic * L + k];
      hNewInv[ic * L + k] = 1.0 / (hProv[ic * L + k]);
    }
  }
  return 0;
}

/* apps/ocean/tasks/solve.cc:99-118 */
int orc_oc_low_order(const orc_mesh *m, const orc_static *s, const orc_config *c,
                     const double *ntf, const double *tracers, double *lo) {
  const int64_t L = c->nlev, T = c->ntr;
  for (int64_t e = 0; e < m->nE; ++e) {
    const int64_t c1 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e)];
    const int64_t c2 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e) + 1];
    for (int64_t k = 0; k < L; ++k) {
      const double ntf1 = smax(0.0, ntf[e * L + k]);
      const double ntf2 = smin(0.0, ntf[e * L + k]);
      for (int64_t t = 0; t < T; ++t)
        lo[(e * L + k) * T + t] = s->dvEdge[e] * (ntf1 * tracers[(c1 * L + k) * T + t] +
                                                  ntf2 * tracers[(c2 * L + k) * T + t]);
    }
  }
  return 0;
}

/* apps/ocean/tasks/solve.cc:120-167 (coef3rdOrder = 0.25, :11) */
int orc_oc_high_order(const orc_mesh *m, const orc_static *s, const orc_config *c,
                      const double *ntf, const double *tracers, double *ho) {
  const int64_t L = c->nlev, T = c->ntr;
  const double coef3rdOrder = 0.25;
  double *wgt = (double *)malloc(sizeof(double) * (size_t)(L * (2 + T)));
  if (!wgt) return fail("allocation");
  double *sgn = wgt + L, *flx = wgt + 2 * L;
  for (int64_t e = 0; e < m->nE; ++e) {
    for (int64_t k = 0; k < L; ++k) {
      const double f = ntf[e * L + k];
      wgt[k] = f * (double)s->highOrderAdvMask[e * L + k];
      sgn[k] = (f < 0.0) ? -1.0 : (double)(f > 0.);
      for (int64_t t = 0; t < T; ++t) flx[k * T + t] = 0.0;
    }
    for (int64_t i = 0; i < s->nAdvCellsForEdge[e]; ++i) {
      const int64_t iCell = s->advCellsForEdge[e * MAXE2 + i];
      const double coef1 = s->advCoef[e * MAXE2 + i];
      const double coef3 = s->advCoef_3rd[e * MAXE2 + i] * coef3rdOrder;
      for (int64_t k = 0; k < s->maxLevelCell[iCell]; ++k) {
        const double weightFactor = wgt[k] * (coef1 + coef3 * sgn[k]);
        for (int64_t t = 0; t < T; ++t)
          flx[k * T + t] += tracers[(iCell * L + k) * T + t] * weightFactor;
      }
    }
    for (int64_t k = 0; k < L; ++k)
      for (int64_t t = 0; t < T; ++t) ho[(e * L + k) * T + t] = flx[k * T + t];
  }
  free(wgt);
  return 0;
}

/* apps/ocean/tasks/solve.cc:169-285 */
int orc_oc_correct_and_rescale(const orc_mesh *m, const orc_static *s, const orc_config *c,
                               const double *hProvInv, const double *h, const double *ntf,
                               const double *lo, const double *tracers, double *ho,
                               double *flxIn, double *flxOut, double *tend, double *trMax,
                               double *trMin, double dt) {
  const int64_t L = c->nlev, T = c->ntr;
  const double eps = 1.e-10;
#define VT(a, i, k, t) (a)[((int64_t)(i) * L + (k)) * T + (t)]
  for (int64_t ic = 0; ic < m->nC; ++ic) { /* :195-214 */
    for (int64_t k = 0; k < s->maxLevelCell[ic]; ++k)
      for (int64_t t = 0; t < T; ++t) {
        VT(trMax, ic, k, t) = VT(tracers, ic, k, t);
        VT(trMin, ic, k, t) = VT(tracers, ic, k, t);
        VT(flxIn, ic, k, t) = 0.0;
        VT(flxOut, ic, k, t) = 0.0;
      }
    for (int64_t j = ROWB(m, ORC_C2C, ic); j < ROWE(m, ORC_C2C, ic); ++j) {
      const int64_t c2 = IDX(m, ORC_C2C)[j];
      const int64_t kmax = s->maxLevelCell[ic] < s->maxLevelCell[c2] ? s->maxLevelCell[ic]
                                                                      : s->maxLevelCell[c2];
      for (int64_t k = 0; k < kmax; ++k)
        for (int64_t t = 0; t < T; ++t) {
          VT(trMax, ic, k, t) = smax(VT(trMax, ic, k, t), VT(tracers, c2, k, t));
          VT(trMin, ic, k, t) = smin(VT(trMin, ic, k, t), VT(tracers, c2, k, t));
        }
    }
  }
  for (int64_t e = 0; e < m->nE; ++e) { /* :216-229 */
    const int64_t c1 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e)];
    const int64_t c2 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e) + 1];
    for (int64_t k = 0; k < s->maxLevelEdgeTop[e]; ++k) {
      const double tracerWeight = (double)((s->highOrderAdvMask[e * L + k] + 1) & 1) *
                                  (s->dvEdge[e] * 0.5) * ntf[e * L + k];
      for (int64_t t = 0; t < T; ++t) {
        VT(ho, e, k, t) += tracerWeight * (VT(tracers, c1, k, t) + VT(tracers, c2, k, t));
        VT(ho, e, k, t) -= VT(lo, e, k, t);
      }
    }
  }
  for (int64_t ic = 0; ic < m->nC; ++ic) { /* :232-267 */
    const double invAreaCell1 = 1.0 / s->areaCell[ic];
    int64_t je = 0;
    for (int64_t j = ROWB(m, ORC_C2E, ic); j < ROWE(m, ORC_C2E, ic); ++j, ++je) {
      const int64_t e = IDX(m, ORC_C2E)[j];
      const double signedFactor = s->edgeSignOnCell[ic * MAXE + je] * invAreaCell1;
      for (int64_t k = 0; k < s->maxLevelEdgeTop[e]; ++k)
        for (int64_t t = 0; t < T; ++t) {
          VT(tend, ic, k, t) += signedFactor * VT(lo, e, k, t);
          VT(flxIn, ic, k, t) += smax(0.0, signedFactor * VT(ho, e, k, t));
          VT(flxOut, ic, k, t) += smin(0.0, signedFactor * VT(ho, e, k, t));
        }
    }
    for (int64_t k = 0; k < s->maxLevelCell[ic]; ++k)
      for (int64_t t = 0; t < T; ++t) {
        const double hpi = hProvInv[ic * L + k];
        const double tracerUpwindNew = (VT(tracers, ic, k, t) * h[ic * L + k] + dt * VT(tend, ic, k, t)) * hpi;
        const double tracerMaxNew = tracerUpwindNew + dt * VT(flxIn, ic, k, t) * hpi;
        const double tracerMinNew = tracerUpwindNew + dt * VT(flxOut, ic, k, t) * hpi;
        double scaleFactor = (VT(trMax, ic, k, t) - tracerUpwindNew) / (tracerMaxNew - tracerUpwindNew + eps);
        VT(flxIn, ic, k, t) = smin(1.0, smax(0.0, scaleFactor));
        scaleFactor = (tracerUpwindNew - VT(trMin, ic, k, t)) / (tracerUpwindNew - tracerMinNew + eps);
        VT(flxOut, ic, k, t) = smin(1.0, smax(0.0, scaleFactor));
      }
  }
  for (int64_t e = 0; e < m->nE; ++e) { /* :270-282 */
    const int64_t c1 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e)];
    const int64_t c2 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e) + 1];
    for (int64_t k = 0; k < s->maxLevelEdgeTop[e]; ++k)
      for (int64_t t = 0; t < T; ++t)
        VT(ho, e, k, t) = smax(0.0, VT(ho, e, k, t)) * smin(VT(flxOut, c1, k, t), VT(flxIn, c2, k, t)) +
                          smin(0.0, VT(ho, e, k, t)) * smin(VT(flxIn, c1, k, t), VT(flxOut, c2, k, t));
  }
#undef VT
  return 0;
}

/* apps/ocean/tasks/solve.cc:287-326 */
int orc_oc_accumulate_fct(const orc_mesh *m, const orc_static *s, const orc_config *c,
                          const double *hProvInv, const double *h, const double *ho,
                          const double *tracers, double *tracersProv, double *tend, double dt) {
  const int64_t L = c->nlev, T = c->ntr;
  for (int64_t ic = 0; ic < m->nC; ++ic) {
    const double invAreaCell1 = 1.0 / s->areaCell[ic];
    int64_t je = 0;
    for (int64_t j = ROWB(m, ORC_C2E, ic); j < ROWE(m, ORC_C2E, ic); ++j, ++je) {
      const int64_t e = IDX(m, ORC_C2E)[j];
      const double signedFactor = s->edgeSignOnCell[ic * MAXE + je] * invAreaCell1;
      for (int64_t k = 0; k < s->maxLevelEdgeTop[e]; ++k)
        for (int64_t t = 0; t < T; ++t)
          tend[(ic * L + k) * T + t] += signedFactor * ho[(e * L + k) * T + t];
    }
    for (int64_t k = 0; k < s->maxLevelCell[ic]; ++k)
      for (int64_t t = 0; t < T; ++t)
        tracersProv[(ic * L + k) * T + t] =
            (tracers[(ic * L + k) * T + t] * h[ic * L + k] + dt * tend[(ic * L + k) * T + t]) *
            hProvInv[ic * L + k];
  }
  return 0;
}

/* apps/ocean/tasks/solve.cc:328-366 */
int orc_oc_hmix_del2(const orc_mesh *m, const orc_static *s, const orc_config *c,
                     const double *hEdge, const double *tracers, double *tend, double coef) {
  const int64_t L = c->nlev, T = c->ntr;
  for (int64_t ic = 0; ic < m->nC; ++ic) {
    const double invArea = 1.0 / s->areaCell[ic];
    int64_t je = 0;
    for (int64_t j = ROWB(m, ORC_C2E, ic); j < ROWE(m, ORC_C2E, ic); ++j, ++je) {
      const int64_t e = IDX(m, ORC_C2E)[j];
      const int64_t c1 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e)];
      const int64_t c2 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e) + 1];
      const double rho_scaling = s->meshScalingDel2[e] * coef * s->dvEdge[e] / s->dcEdge[e];
      for (int64_t k = 0; k < s->maxLevelEdgeTop[e]; ++k)
        for (int64_t t = 0; t < T; ++t) {
          const double tracer_turb_flux = tracers[(c2 * L + k) * T + t] - tracers[(c1 * L + k) * T + t];
          const double flux = hEdge[e * L + k] * tracer_turb_flux * rho_scaling;
          tend[(ic * L + k) * T + t] -= s->edgeSignOnCell[ic * MAXE + je] * flux * invArea;
        }
    }
  }
  return 0;
}

/* apps/ocean/tasks/solve.cc:368-399 */
int orc_oc_step_tracers_forward(const orc_mesh *m, const orc_config *c, const double *tend,
                                const double *tracers, double *tracersNew, double *tracersPrev,
                                double rk_weight, double rk_subweight) {
  const int64_t n = m->nC * c->nlev * c->ntr;
  for (int64_t i = 0; i < n; ++i) {
    tracersNew[i] += rk_weight * tend[i];
    tracersPrev[i] = tracers[i] + rk_subweight * tend[i];
  }
  return 0;
}

/* ======================================================= static setup */

/* mpasoflecsi/eqns/metrics.hh:25-73 */
static double sphere_angle(double ax, double ay, double az, double bx, double by, double bz,
                           double cx, double cy, double cz) {
  const double a = acos(smax(smin(bx * cx + by * cy + bz * cz, 1.0), -1.0));
  const double b = acos(smax(smin(ax * cx + ay * cy + az * cz, 1.0), -1.0));
  const double c = acos(smax(smin(ax * bx + ay * by + az * bz, 1.0), -1.0));
  const double ABx = bx - ax, ABy = by - ay, ABz = bz - az;
  const double ACx = cx - ax, ACy = cy - ay, ACz = cz - az;
  const double Dx = (ABy * ACz) - (ABz * ACy);
  const double Dy = (ABz * ACx) - (ABx * ACz);
  const double Dz = (ABx * ACy) - (ABy * ACx);
  const double s = 0.5 * (a + b + c);
  const double sin_angle = sqrt(smin(1.0, smax(0.0, (sin(s - b) * sin(s - c)) / (sin(b) * sin(c)))));
  if (Dx * ax + Dy * ay + Dz * az >= 0.0) return 2.0 * asin(smax(smin(sin_angle, 1.0), -1.0));
  return -2.0 * asin(smax(smin(sin_angle, 1.0), -1.0));
}

/* mpasoflecsi/eqns/metrics.hh:75-91 */
static double sphere_arc_length(double ax, double ay, double az, double bx, double by, double bz) {
  const double cx = bx - ax, cy = by - ay, cz = bz - az;
  const double r = sqrt(ax * ax + ay * ay + az * az);
  const double c = sqrt(cx * cx + cy * cy + cz * cz);
  return r * 2. * asin(c / (2. * r));
}

/* mpasoflecsi/eqns/metrics.hh:93-111 */
static int arc_bisect(double ax, double ay, double az, double bx, double by, double bz,
                      double *cx, double *cy, double *cz) {
  const double r = sqrt(ax * ax + ay * ay + az * az);
  *cx = 0.5 * (ax + bx);
  *cy = 0.5 * (ay + by);
  *cz = 0.5 * (az + bz);
  if (!(*cx != 0. && *cy != 0. && *cz != 0.)) return 1;
  const double d = sqrt(*cx * *cx + *cy * *cy + *cz * *cz);
  *cx = r * *cx / d;
  *cy = r * *cy / d;
  *cz = r * *cz / d;
  return 0;
}

#define NA 6   /* polynomial_order 2 -> 6 coefficients (init_functions.cc:215) */
#define MMAX 9 /* at most maxEdges + 1 points */

/* C[r][c] = sum_inner A[r][inner] * B[inner][c], accumulated from 0 in order
 * (mpasoflecsi/eqns/matrix.hh:28-43). */
static void matmul(int ra, int ca, const double *A, int cb, const double *B, double *C) {
  for (int r = 0; r < ra; ++r)
    for (int col = 0; col < cb; ++col) {
      double acc = 0.0;
      for (int in = 0; in < ca; ++in) acc += A[r * ca + in] * B[in * cb + col];
      C[r * cb + col] = acc;
    }
}

/* Partial-pivoting Gaussian elimination (mpasoflecsi/eqns/matrix.hh:52-105). */
static void elgs(int n, double *a, int *idx) {
  double cs[NA];
  for (int i = 0; i < n; ++i) idx[i] = i;
  for (int i = 0; i < n; ++i) {
    double c1 = 0.;
    for (int j = 0; j < n; ++j) c1 = smax(c1, fabs(a[i * n + j]));
    cs[i] = c1;
  }
  for (int j = 0; j < n - 1; ++j) {
    int k = j;
    double pi1 = 0.0;
    for (int i = j; i < n; ++i) {
      const double pi = fabs(a[idx[i] * n + j]) / cs[idx[i]];
      if (pi > pi1) {
        pi1 = pi;
        k = i;
      }
    }
    const int itmp = idx[j];
    idx[j] = idx[k];
    idx[k] = itmp;
    for (int i = j + 1; i < n; ++i) {
      const double pj = a[idx[i] * n + j] / a[idx[j] * n + j];
      a[idx[i] * n + j] = pj;
      for (int kk = j + 1; kk < n; ++kk) a[idx[i] * n + kk] = a[idx[i] * n + kk] - pj * a[idx[j] * n + kk];
    }
  }
}

/* Matrix inverse via elgs (mpasoflecsi/eqns/matrix.hh:125-167). */
static void migs(int n, double *a, double *x) {
  double b[NA * NA];
  int idx[NA];
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) b[i * n + j] = 0.;
  for (int i = 0; i < n; ++i) b[i * n + i] = 1.;
  elgs(n, a, idx);
  for (int i = 0; i < n - 1; ++i)
    for (int j = i + 1; j < n; ++j)
      for (int k = 0; k < n; ++k)
        b[idx[j] * n + k] = b[idx[j] * n + k] - a[idx[j] * n + i] * b[idx[i] * n + k];
  for (int i = 0; i < n; ++i) {
    x[(n - 1) * n + i] = b[idx[n - 1] * n + i] / a[idx[n - 1] * n + n - 1];
    for (int j = n - 2; j >= 0; j--) {
      x[j * n + i] = b[idx[j] * n + i];
      for (int k = j + 1; k < n; ++k) x[j * n + i] = x[j * n + i] - a[idx[j] * n + k] * x[k * n + i];
      x[j * n + i] = x[j * n + i] / a[idx[j] * n + j];
    }
  }
}

/* apps/ocean/tasks/init_functions.cc:83-328 (sphere branch; the reference
 * hard-codes on_a_sphere = true at :144). */
static int init_2nd_deriv(const orc_mesh *m, const orc_geom *g, double *derivTwo) {
  const double a = 6371000.0, pi = 3.141592653589793; /* constants.hh:28-29 */
  for (int64_t i = 0; i < m->nE * MAXE2 * 2; ++i) derivTwo[i] = 0.0;
  const int64_t nCells = m->nC;
  for (int64_t ic = 0; ic < m->nC; ++ic) {
    const int nEonC = (int)(ROWE(m, ORC_C2E, ic) - ROWB(m, ORC_C2E, ic));
    int64_t cell_list[MMAX];
    int nl = 0;
    cell_list[nl++] = ic;
    for (int64_t j = ROWB(m, ORC_C2C, ic); j < ROWE(m, ORC_C2C, ic); ++j) {
      if (nl >= MMAX) return fail("init_2nd_deriv: too many neighbours");
      cell_list[nl++] = IDX(m, ORC_C2C)[j];
    }
    const int n = nEonC + 1;
    int do_the_cell = 1;
    for (int i = 1; i < n; ++i)
      if (cell_list[i] < 0 || cell_list[i] >= nCells) {
        do_the_cell = 0;
        break;
      }
    if (!do_the_cell) continue;
    double xc[MMAX], yc[MMAX], zc[MMAX], theta_v[MMAX], theta_t[MMAX], dl_sphere[MMAX];
    double xp[MMAX], yp[MMAX];
    for (int i = 0; i < n; ++i) {
      xc[i] = g->xCell[cell_list[i]] / a;
      yc[i] = g->yCell[cell_list[i]] / a;
      zc[i] = g->zCell[cell_list[i]] / a;
    }
    double theta_abs;
    if (zc[0] == 1.0)
      theta_abs = pi / 2.0;
    else
      theta_abs = pi / 2.0 - sphere_angle(xc[0], yc[0], zc[0], xc[1], yc[1], zc[1], 0.0, 0.0, 1.0);
    const double length_scale = 1.0;
    for (int i = 0; i < n - 1; ++i) {
      int ip2 = i + 2;
      if (ip2 > n - 1) ip2 = 1;
      theta_v[i] = sphere_angle(xc[0], yc[0], zc[0], xc[i + 1], yc[i + 1], zc[i + 1], xc[ip2], yc[ip2], zc[ip2]);
      dl_sphere[i] = a * sphere_arc_length(xc[0], yc[0], zc[0], xc[i + 1], yc[i + 1], zc[i + 1]) / length_scale;
    }
    theta_t[0] = theta_abs;
    for (int i = 1; i < n - 1; ++i) theta_t[i] = theta_t[i - 1] + theta_v[i - 1];
    for (int i = 0; i < n - 1; ++i) {
      xp[i] = cos(theta_t[i]) * dl_sphere[i];
      yp[i] = sin(theta_t[i]) * dl_sphere[i];
    }
    /* mpas_poly_fit_2 (:206-270) */
    const int ma = n, na = NA;
    double aa[MMAX * NA] = {0}, ww[MMAX * MMAX] = {0};
    aa[0 * na + 0] = 1.0;
    ww[0] = 1.0;
    for (int i = 1; i < ma; ++i) {
      aa[i * na + 0] = 1.0;
      aa[i * na + 1] = xp[i - 1];
      aa[i * na + 2] = yp[i - 1];
      aa[i * na + 3] = xp[i - 1] * xp[i - 1];
      aa[i * na + 4] = xp[i - 1] * yp[i - 1];
      aa[i * na + 5] = yp[i - 1] * yp[i - 1];
      ww[i * ma + i] = 1.0;
    }
    double at[NA * MMAX], wt[MMAX * MMAX], hh[MMAX * MMAX], ath[NA * MMAX], atha[NA * NA],
        atha_inv[NA * NA], bb[NA * MMAX];
    for (int i = 0; i < ma; ++i)
      for (int j = 0; j < na; ++j) at[j * ma + i] = aa[i * na + j];
    for (int i = 0; i < ma; ++i)
      for (int j = 0; j < ma; ++j) wt[j * ma + i] = ww[i * ma + j];
    matmul(ma, ma, wt, ma, ww, hh);
    matmul(na, ma, at, ma, hh, ath);
    matmul(na, ma, ath, na, aa, atha);
    migs(na, atha, atha_inv);
    matmul(na, na, atha_inv, ma, ath, bb);
    for (int i = 0; i < nEonC; ++i) {
      const int64_t e1 = IDX(m, ORC_C2E)[ROWB(m, ORC_C2E, ic) + i];
      const int64_t va = IDX(m, ORC_E2V)[ROWB(m, ORC_E2V, e1)];
      const int64_t vb = IDX(m, ORC_E2V)[ROWB(m, ORC_E2V, e1) + 1];
      const double xv1 = g->xVertex[va] / a, yv1 = g->yVertex[va] / a, zv1 = g->zVertex[va] / a;
      const double xv2 = g->xVertex[vb] / a, yv2 = g->yVertex[vb] / a, zv2 = g->zVertex[vb] / a;
      double xec, yec, zec;
      if (arc_bisect(xv1, yv1, zv1, xv2, yv2, zv2, &xec, &yec, &zec))
        return fail("arc_bisect: A and B are diametrically opposite");
      double thetae_tmp = sphere_angle(xc[0], yc[0], zc[0], xc[i + 1], yc[i + 1], zc[i + 1], xec, yec, zec);
      thetae_tmp += theta_t[i];
      double cos2t = cos(thetae_tmp), sin2t = sin(thetae_tmp);
      const double costsint = cos2t * sin2t;
      cos2t = cos2t * cos2t;
      sin2t = sin2t * sin2t;
      const int side = (ic == IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e1)]) ? 0 : 1;
      for (int j = 0; j < n; ++j)
        derivTwo[(e1 * MAXE2 + j) * 2 + side] =
            2. * cos2t * bb[3 * ma + j] + 2. * costsint * bb[4 * ma + j] + 2. * sin2t * bb[5 * ma + j];
    }
  }
  return 0;
}

static int64_t find_idx(const int64_t *list, int64_t n, int64_t v) {
  int64_t i = 0;
  while (i < n && list[i] != v) ++i;
  return i;
}

/* apps/ocean/tasks/init_functions.cc:18-27, 47-82, 330-447 */
int orc_init_fct_statics(const orc_mesh *m, const orc_config *c, const orc_geom *g,
                         orc_setup_out *o) {
  const int64_t L = c->nlev;
  for (int64_t e = 0; e < m->nE; ++e) { /* :18-27 */
    const int64_t c1 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e)];
    const int64_t c2 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e) + 1];
    const int32_t a1 = g->maxLevelCell[c1], a2 = g->maxLevelCell[c2];
    o->maxLevelEdgeTop[e] = (a1 < a2) ? a2 : a1;
  }
  { /* :47-66 -- note: cells 0 and 1 for every edge, as the reference does */
    double maxDensity = 0.0;
    for (int64_t ic = 0; ic < m->nC; ++ic)
      if (g->meshDensity[ic] > maxDensity) maxDensity = g->meshDensity[ic];
    for (int64_t e = 0; e < m->nE; ++e) {
      const double relativeDensity = (g->meshDensity[0] + g->meshDensity[1]) / (2.0 * maxDensity);
      o->meshScalingDel2[e] = 1.0 / pow(relativeDensity, 0.25);
    }
  }
  for (int64_t ic = 0; ic < m->nC; ++ic) { /* :68-82 */
    int64_t j = 0;
    for (int64_t p = ROWB(m, ORC_C2E, ic); p < ROWE(m, ORC_C2E, ic); ++p, ++j) {
      const int64_t e = IDX(m, ORC_C2E)[p];
      o->edgeSignOnCell[ic * MAXE + j] = (ic == IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e)]) ? -1.0 : 1.0;
    }
  }
  if (init_2nd_deriv(m, g, o->derivTwo)) return 1;
  const double *derivTwo = o->derivTwo;
#define D2(e, j, s) derivTwo[((e) * MAXE2 + (j)) * 2 + (s)]
  for (int64_t e = 0; e < m->nE; ++e) { /* :342-356 */
    for (int i = 0; i < MAXE2; ++i) {
      o->advCoef[e * MAXE2 + i] = 0.;
      o->advCoef_3rd[e * MAXE2 + i] = 0.;
      o->advCellsForEdge[e * MAXE2 + i] = 0;
    }
    for (int64_t k = 0; k < L; ++k) {
      o->highOrderAdvMask[e * L + k] = 1;
      for (int64_t p = ROWB(m, ORC_E2C, e); p < ROWE(m, ORC_E2C, e); ++p)
        if (g->boundaryCell[(int64_t)IDX(m, ORC_E2C)[p] * L + k] == 1) o->highOrderAdvMask[e * L + k] = 0;
    }
  }
  for (int64_t e = 0; e < m->nE; ++e) { /* :358-445 */
    double *ac = o->advCoef + e * MAXE2, *a3 = o->advCoef_3rd + e * MAXE2;
    const int64_t cell1 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e)];
    const int64_t cell2 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e) + 1];
    int64_t cl[2 * MAXE + 2];
    int64_t n = 0;
    cl[n++] = cell1;
    cl[n++] = cell2;
    const int64_t nEonC1 = ROWE(m, ORC_C2E, cell1) - ROWB(m, ORC_C2E, cell1);
    for (int64_t p = ROWB(m, ORC_C2C, cell1); p < ROWE(m, ORC_C2C, cell1); ++p) {
      const int64_t cc = IDX(m, ORC_C2C)[p];
      if (find_idx(cl, n, cc) == n) cl[n++] = cc;
    }
    const int64_t nEonC2 = ROWE(m, ORC_C2E, cell2) - ROWB(m, ORC_C2E, cell2);
    for (int64_t p = ROWB(m, ORC_C2C, cell2); p < ROWE(m, ORC_C2C, cell2); ++p) {
      const int64_t cc = IDX(m, ORC_C2C)[p];
      if (find_idx(cl, n, cc) == n) cl[n++] = cc;
    }
    if (n > MAXE2) return fail("init_tracer_adv_coeff: more than 16 advection cells");
    o->nAdvCellsForEdge[e] = (int32_t)n;
    for (int64_t i = 0; i < n; ++i) o->advCellsForEdge[e * MAXE2 + i] = (int32_t)cl[i];
    int64_t idx = find_idx(cl, n, cell1);
    if (idx < n) {
      ac[idx] = ac[idx] + D2(e, 0, 0);
      a3[idx] = a3[idx] + D2(e, 0, 0);
    }
    for (int64_t i = 0; i < nEonC1; ++i) {
      const int64_t cc = IDX(m, ORC_C2C)[ROWB(m, ORC_C2C, cell1) + i];
      idx = find_idx(cl, n, cc);
      if (idx < n) {
        ac[idx] = ac[idx] + D2(e, i + 1, 0);
        a3[idx] = a3[idx] + D2(e, i + 1, 0);
      }
    }
    idx = find_idx(cl, n, cell2);
    if (idx < n) {
      ac[idx] = ac[idx] + D2(e, 0, 1);
      a3[idx] = a3[idx] - D2(e, 0, 1);
    }
    for (int64_t i = 0; i < nEonC2; ++i) {
      const int64_t cc = IDX(m, ORC_C2C)[ROWB(m, ORC_C2C, cell2) + i];
      idx = find_idx(cl, n, cc);
      if (idx < n) {
        ac[idx] = ac[idx] + D2(e, i + 1, 1);
        a3[idx] = a3[idx] - D2(e, i + 1, 1);
      }
    }
    const double dc = g->dcEdge[e], dv = g->dvEdge[e];
    for (int64_t i = 0; i < n; ++i) {
      ac[i] = -(dc * dc) * ac[i] / 12.0;
      a3[i] = -(dc * dc) * a3[i] / 12.0;
    }
    idx = find_idx(cl, n, cell1);
    if (idx < n) ac[idx] = ac[idx] + 0.5;
    idx = find_idx(cl, n, cell2);
    if (idx < n) ac[idx] = ac[idx] + 0.5;
    for (int64_t i = 0; i < n; ++i) {
      ac[i] = dv * ac[i];
      a3[i] = dv * a3[i];
    }
  }
#undef D2
  return 0;
}

/* apps/ocean/tasks/init_functions.cc:30-45 */
int orc_init_layer_thickness_edge(const orc_mesh *m, const orc_config *c, const double *h,
                                  const int32_t *maxLevelEdgeTop, double *hEdge) {
  const int64_t L = c->nlev;
  (void)maxLevelEdgeTop;
  for (int64_t e = 0; e < m->nE; ++e) {
    const int64_t c1 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e)];
    const int64_t c2 = IDX(m, ORC_E2C)[ROWB(m, ORC_E2C, e) + 1];
    for (int64_t k = 0; k < L; ++k) hEdge[e * L + k] = 0.5 * (h[c1 * L + k] + h[c2 * L + k]);
  }
  return 0;
}

/* ======================================================= drivers */

typedef struct {
  double *u[3], *h[3], *h_edge[3], *h_vertex[3], *ke[3], *pv_edge[3], *tr[3];
  double *circulation, *vorticity, *pv_vertex, *tend_h, *tend_u, *tend_tr;
  double *ntf, *hProv, *hProvInv, *hNewInv, *w, *lo, *ho, *flxIn, *flxOut, *trMax, *trMin, *trProv;
  double *block;
} sw_fields;

static int sw_alloc(sw_fields *S, int64_t nC, int64_t nE, int64_t nV, int64_t L, int64_t T) {
  const int64_t sz[] = {
      nE * L, nE * L, nE * L, nC * L, nC * L, nC * L, nE * L, nE * L, nE * L, nV * L, nV * L, nV * L,
      nC * L, nC * L, nC * L, nE * L, nE * L, nE * L, nC * L * T, nC * L * T, nC * L * T, /* 21 */
      nV * L, nV * L, nV * L, nC * L, nE * L, nC * L * T,                                   /* 27 */
      nE * L, nC * L, nC * L, nC * L, nC * L, nE * L * T, nE * L * T, nC * L * T, nC * L * T,
      nC * L * T, nC * L * T, nC * L * T}; /* 39 */
  int64_t tot = 0;
  for (int i = 0; i < 39; ++i) tot += sz[i];
  S->block = (double *)calloc((size_t)tot, sizeof(double));
  if (!S->block) return 1;
  double **slots[39] = {&S->u[0], &S->u[1], &S->u[2], &S->h[0], &S->h[1], &S->h[2],
                        &S->h_edge[0], &S->h_edge[1], &S->h_edge[2], &S->h_vertex[0],
                        &S->h_vertex[1], &S->h_vertex[2], &S->ke[0], &S->ke[1], &S->ke[2],
                        &S->pv_edge[0], &S->pv_edge[1], &S->pv_edge[2], &S->tr[0], &S->tr[1],
                        &S->tr[2], &S->circulation, &S->vorticity, &S->pv_vertex, &S->tend_h,
                        &S->tend_u, &S->tend_tr, &S->ntf, &S->hProv, &S->hProvInv, &S->hNewInv,
                        &S->w, &S->lo, &S->ho, &S->flxIn, &S->flxOut, &S->trMax, &S->trMin,
                        &S->trProv};
  double *p = S->block;
  for (int i = 0; i < 39; ++i) {
    *slots[i] = p;
    p += sz[i];
  }
  return 0;
}

enum { PREV = 0, NEXT = 1, PROVIS = 2 };

static int sw_diag(const orc_mesh *m, const orc_static *s, const orc_config *c, sw_fields *S, int t) {
  return orc_sw_compute_solve_diagnostics(m, s, c, S->h[t], S->u[t], S->h_edge[t], S->h_vertex[t],
                                          S->circulation, S->vorticity, S->ke[t], S->pv_edge[t],
                                          S->pv_vertex);
}

static int sw_tracer_tend(const orc_mesh *m, const orc_static *s, const orc_config *c,
                          sw_fields *S, double dt) {
  const int p = PROVIS;
  const int64_t L = c->nlev, T = c->ntr;
  if (c->fct) {
    memset(S->tend_tr, 0, sizeof(double) * (size_t)(m->nC * L * T)); /* solve.cc:28-38 */
    orc_oc_normal_thickness_flux(m, c, S->h_edge[p], S->u[p], S->ntf);
    orc_oc_provisional_layer_thicknesses(m, s, c, S->h[p], S->ntf, S->w, S->hProv, S->hProvInv,
                                         S->hNewInv, dt);
    orc_oc_low_order(m, s, c, S->ntf, S->tr[p], S->lo);
    if (orc_oc_high_order(m, s, c, S->ntf, S->tr[p], S->ho)) return 1;
    orc_oc_correct_and_rescale(m, s, c, S->hProvInv, S->h[p], S->ntf, S->lo, S->tr[p], S->ho,
                               S->flxIn, S->flxOut, S->tend_tr, S->trMax, S->trMin, dt);
    orc_oc_accumulate_fct(m, s, c, S->hProvInv, S->h[p], S->ho, S->tr[p], S->trProv, S->tend_tr, dt);
  } else {
    orc_sw_compute_scalar_tend(m, s, c, S->h_edge[p], S->u[p], S->tr[p], S->tend_tr);
  }
  if (c->hmix) orc_oc_hmix_del2(m, s, c, S->h_edge[p], S->tr[p], S->tend_tr, c->kappa);
  return 0;
}

/* apps/sw/run.cc:13-70 */
static int sw_advance(const orc_mesh *m, const orc_static *s, const orc_config *c, sw_fields *S,
                      double dt) {
  const int64_t nC = m->nC, nE = m->nE, L = c->nlev, T = c->ntr;
  /* init_provis (solve.cc:110-141) */
  memcpy(S->h[PROVIS], S->h[PREV], sizeof(double) * (size_t)(nC * L));
  memcpy(S->ke[PROVIS], S->ke[PREV], sizeof(double) * (size_t)(nC * L));
  memcpy(S->tr[PROVIS], S->tr[PREV], sizeof(double) * (size_t)(nC * L * T));
  memcpy(S->u[PROVIS], S->u[PREV], sizeof(double) * (size_t)(nE * L));
  memcpy(S->h_edge[PROVIS], S->h_edge[PREV], sizeof(double) * (size_t)(nE * L));
  memcpy(S->pv_edge[PROVIS], S->pv_edge[PREV], sizeof(double) * (size_t)(nE * L));
  /* setup_timestep (solve.cc:144-166) */
  memcpy(S->u[NEXT], S->u[PREV], sizeof(double) * (size_t)(nE * L));
  for (int64_t i = 0; i < nC * L; ++i) {
    S->h[NEXT][i] = S->h[PREV][i];
    for (int64_t t = 0; t < T; ++t) S->tr[NEXT][i * T + t] = S->tr[PREV][i * T + t] * S->h[PREV][i];
  }
  const double rk_w[4] = {dt / 6, dt / 3, dt / 3, dt / 6};
  const double rk_sub[4] = {dt / 2, dt / 2, dt, 0};
  for (int rk = 0; rk < 4; ++rk) {
    orc_sw_compute_tend(m, s, c, S->h_edge[PROVIS], S->h[PROVIS], S->u[PROVIS], S->ke[PROVIS],
                        S->pv_edge[PROVIS], S->tend_h, S->tend_u);
    if (c->nu != 0.0 && orc_sw_del2_momentum(m, s, c, S->u[PROVIS], S->vorticity, S->tend_u))
      return fail("del2 momentum");
    if (sw_tracer_tend(m, s, c, S, dt)) return 1;
    if (rk < 3) {
      orc_sw_compute_substep(m, c, S->u[PROVIS], S->u[PREV], S->tend_u, S->h[PROVIS], S->h[PREV],
                             S->tend_h, S->tr[PROVIS], S->tr[PREV], S->tend_tr, rk_sub[rk]);
      sw_diag(m, s, c, S, PROVIS);
    }
    orc_sw_accumulate_update(m, c, S->u[NEXT], S->tend_u, S->h[NEXT], S->tend_h, S->tr[NEXT],
                             S->tend_tr, rk_w[rk]);
  }
  orc_sw_finalize_timestep(m, c, S->u[PREV], S->u[NEXT], S->h[NEXT], S->tr[NEXT]);
  sw_diag(m, s, c, S, NEXT);
  /* timeshift (solve.cc:370-401) */
  memcpy(S->h[PREV], S->h[NEXT], sizeof(double) * (size_t)(nC * L));
  memcpy(S->ke[PREV], S->ke[NEXT], sizeof(double) * (size_t)(nC * L));
  memcpy(S->tr[PREV], S->tr[NEXT], sizeof(double) * (size_t)(nC * L * T));
  memcpy(S->u[PREV], S->u[NEXT], sizeof(double) * (size_t)(nE * L));
  memcpy(S->h_edge[PREV], S->h_edge[NEXT], sizeof(double) * (size_t)(nE * L));
  memcpy(S->pv_edge[PREV], S->pv_edge[NEXT], sizeof(double) * (size_t)(nE * L));
  return 0;
}

int orc_sw_run(const orc_mesh *m, const orc_static *s, const orc_config *c, double dt,
               int32_t nsteps, double *h, double *u, double *tracers) {
  const int64_t L = c->nlev, T = c->ntr;
  if (L < 1 || T < 0) return fail("bad level/tracer count");
  sw_fields S;
  if (sw_alloc(&S, m->nC, m->nE, m->nV, L, T)) return fail("allocation");
  memcpy(S.h[PREV], h, sizeof(double) * (size_t)(m->nC * L));
  memcpy(S.u[PREV], u, sizeof(double) * (size_t)(m->nE * L));
  memcpy(S.tr[PREV], tracers, sizeof(double) * (size_t)(m->nC * L * T));
  sw_diag(m, s, c, &S, PREV); /* apps/sw/run.cc:88-92 */
  int rc = 0;
  for (int32_t i = 0; i < nsteps && rc == 0; ++i) rc = sw_advance(m, s, c, &S, dt);
  memcpy(h, S.h[PREV], sizeof(double) * (size_t)(m->nC * L));
  memcpy(u, S.u[PREV], sizeof(double) * (size_t)(m->nE * L));
  memcpy(tracers, S.tr[PREV], sizeof(double) * (size_t)(m->nC * L * T));
  free(S.block);
  return rc;
}

/* apps/ocean/run.cc:10-50 */
int orc_ocean_run(const orc_mesh *m, const orc_static *s, const orc_config *c, double dt,
                  int32_t nsteps, const double *layerThickness, const double *layerThicknessEdge,
                  const double *normalVelocity, double *tracers) {
  const int64_t nC = m->nC, nE = m->nE, L = c->nlev, T = c->ntr;
  const int64_t nt = nC * L * T;
  double *blk = (double *)calloc((size_t)(9 * nt + 2 * nE * L * T + 5 * nC * L + nE * L), sizeof(double));
  if (!blk) return fail("allocation");
  double *tr_prev = blk, *tr_curr = tr_prev + nt, *tr_next = tr_curr + nt, *tr_prov = tr_next + nt;
  double *tend = tr_prov + nt, *flxIn = tend + nt, *flxOut = flxIn + nt, *trMax = flxOut + nt;
  double *trMin = trMax + nt, *lo = trMin + nt, *ho = lo + nE * L * T;
  double *hProv = ho + nE * L * T, *hProvInv = hProv + nC * L, *hNewInv = hProvInv + nC * L;
  double *w = hNewInv + nC * L, *ntf = w + nC * L;
  memcpy(tr_curr, tracers, sizeof(double) * (size_t)nt);
  const double rk_w[4] = {dt / 6, dt / 3, dt / 3, dt / 6};
  const double rk_sub[4] = {dt / 2, dt / 2, dt, 0};
  int rc = 0;
  for (int32_t step = 0; step < nsteps && rc == 0; ++step) {
    memcpy(tr_next, tr_curr, sizeof(double) * (size_t)nt); /* copy_tracers (solve.cc:13-26) */
    memcpy(tr_prev, tr_curr, sizeof(double) * (size_t)nt);
    for (int rk = 0; rk < 4; ++rk) {
      memset(tend, 0, sizeof(double) * (size_t)nt);
      if (c->fct) {
        orc_oc_normal_thickness_flux(m, c, layerThicknessEdge, normalVelocity, ntf);
        orc_oc_provisional_layer_thicknesses(m, s, c, layerThickness, ntf, w, hProv, hProvInv,
                                             hNewInv, dt);
        orc_oc_low_order(m, s, c, ntf, tr_prev, lo);
        rc = orc_oc_high_order(m, s, c, ntf, tr_prev, ho);
        orc_oc_correct_and_rescale(m, s, c, hProvInv, layerThickness, ntf, lo, tr_prev, ho,
                                   flxIn, flxOut, tend, trMax, trMin, dt);
        orc_oc_accumulate_fct(m, s, c, hProvInv, layerThickness, ho, tr_prev, tr_prov, tend, dt);
      }
      if (c->hmix) orc_oc_hmix_del2(m, s, c, layerThicknessEdge, tr_prev, tend, c->kappa);
      orc_oc_step_tracers_forward(m, c, tend, tr_curr, tr_next, tr_prev, rk_w[rk], rk_sub[rk]);
    }
    memcpy(tr_curr, tr_next, sizeof(double) * (size_t)nt); /* update_tracers (solve.cc:401-414) */
  }
  memcpy(tracers, tr_curr, sizeof(double) * (size_t)nt);
  free(blk);
  return rc;
}

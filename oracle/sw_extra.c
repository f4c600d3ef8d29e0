/* TEST INFRASTRUCTURE ONLY.  Terms the oracle drivers add that the reference
 * does not have; shared by the reference build and the restatement so both
 * drivers compose the same step.
 *
 * del2 momentum (parity unpinned: apps/sw/tasks/solve.cc:228-231 has no
 * viscosity).  Laplacian of the normal velocity as the gradient of divergence
 * minus the curl of vorticity:
 *   div(c)    = (1/areaCell) sum_{e in edges(c)} s(c,e) dvEdge u(e),
 *               s = +1 when c = cells(e)[0] (normal points out of c), else -1;
 *   tend_u(e) += nu ((div(c2) - div(c1))/dcEdge - (vort(v2) - vort(v1))/dvEdge),
 * with (c1, c2) = cells(e) and (v1, v2) = vertices(e); vort is the
 * diagnostic vorticity of apps/sw/tasks/solve.cc:56-60. */
#include <stdlib.h>

#include "oracle.h"

int orc_sw_del2_momentum_impl(const orc_mesh *m, const orc_static *s, const orc_config *c,
                              const double *u, const double *vorticity, double *tend_u) {
  const int64_t L = c->nlev;
  double *div = (double *)malloc(sizeof(double) * (size_t)(m->nC * L));
  if (!div) return 1;
  const int64_t *c2e_o = m->off[ORC_C2E], *e2c_o = m->off[ORC_E2C], *e2v_o = m->off[ORC_E2V];
  const int32_t *c2e = m->idx[ORC_C2E], *e2c = m->idx[ORC_E2C], *e2v = m->idx[ORC_E2V];
  for (int64_t ic = 0; ic < m->nC; ++ic) {
    for (int64_t k = 0; k < L; ++k) div[ic * L + k] = 0.0;
    for (int64_t j = c2e_o[ic]; j < c2e_o[ic + 1]; ++j) {
      const int64_t e = c2e[j];
      const double sgn = (e2c[e2c_o[e]] == ic) ? 1.0 : -1.0;
      for (int64_t k = 0; k < L; ++k) div[ic * L + k] += sgn * s->dvEdge[e] * u[e * L + k];
    }
    for (int64_t k = 0; k < L; ++k) div[ic * L + k] /= s->areaCell[ic];
  }
  for (int64_t e = 0; e < m->nE; ++e) {
    const int64_t c1 = e2c[e2c_o[e]], c2 = e2c[e2c_o[e] + 1];
    const int64_t v1 = e2v[e2v_o[e]], v2 = e2v[e2v_o[e] + 1];
    for (int64_t k = 0; k < L; ++k)
      tend_u[e * L + k] +=
          c->nu * ((div[c2 * L + k] - div[c1 * L + k]) / s->dcEdge[e] -
                   (vorticity[v2 * L + k] - vorticity[v1 * L + k]) / s->dvEdge[e]);
  }
  free(div);
  return 0;
}

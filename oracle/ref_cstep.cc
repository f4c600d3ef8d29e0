// TEST INFRASTRUCTURE ONLY.  Complex-step tangent of the reference's own sw
// RK4 step: apps/sw/tasks/solve.cc compiled unmodified against oracle/shim/
// with MPASO_REF_COMPLEX_STEP, so vlreal / vltracer hold complex numbers and
// every task evaluates on x + i eps dx.  Only +, -, * and / touch the state on
// this path (no min / max / abs), so Im(step(x + i eps dx)) / eps is the
// directional derivative to working precision (Squire & Trapp 1998) -- an
// FP64 tape over the reference step that the adjoint is checked against.
//
// The step is apps/sw/run.cc:13-70 with the centred tracer tendency
// (compute_scalar_tend) and no del2 momentum (the reference has none);
// tracers are passive and start at zero.  Built by oracle/build.py into
// oracle/_ref/libref_cstep_L<L>.so where the reference checkout exists.
#include <complex>
#include <cstring>
#include <string>
#include <vector>

#include "apps/sw/state.hh"
#include "apps/sw/tasks/solve.hh"
#include "oracle.h"

namespace {

using namespace mpas;
using cd = std::complex<double>;
thread_local std::string g_err;

template <class T> struct P {
  T *p;
  template <flecsi::partition_privilege_t A, flecsi::partition_privilege_t B>
  operator flecsi::accessor_t<T, A, B>() const {
    return {p};
  }
};
template <class T> P<T> F(const void *p) { return {(T *)p}; }
using D = double;

mesh::view view_of(const orc_mesh *m) {
  mesh::view v;
  v.nC = (std::size_t)m->nC, v.nE = (std::size_t)m->nE, v.nV = (std::size_t)m->nV;
  mesh::crs *dst[ORC_NCNX] = {&v.c2v, &v.c2e, &v.c2c, &v.e2v, &v.e2e, &v.v2c, &v.e2c, &v.v2e};
  for (int k = 0; k < ORC_NCNX; ++k) *dst[k] = {m->off[k], m->idx[k]};
  return v;
}

struct Sw {
  enum { prev = 0, next = 1, provis = 2 };
  std::vector<vlreal> u[3], h[3], h_edge[3], h_vertex[3], ke[3], pv_edge[3];
  std::vector<vltracer> tr[3];
  std::vector<vlreal> circulation, vorticity, pv_vertex, tend_h, tend_u;
  std::vector<vltracer> tend_tr;
  Sw(std::size_t nC, std::size_t nE, std::size_t nV) {
    for (int t = 0; t < 3; ++t) {
      u[t].assign(nE, vlreal{}), h[t].assign(nC, vlreal{}), h_edge[t].assign(nE, vlreal{});
      h_vertex[t].assign(nV, vlreal{}), ke[t].assign(nC, vlreal{}), pv_edge[t].assign(nE, vlreal{});
      tr[t].assign(nC, vltracer{});
    }
    circulation.assign(nV, vlreal{}), vorticity.assign(nV, vlreal{}), pv_vertex.assign(nV, vlreal{});
    tend_h.assign(nC, vlreal{}), tend_u.assign(nE, vlreal{}), tend_tr.assign(nC, vltracer{});
  }
};

void diag(mesh::view &mv, const orc_static *s, Sw &S, int t) {
  sw::task::compute_solve_diagnostics(
      mv, F<D>(s->dvEdge), F<D>(s->dcEdge), F<D>(s->areaCell), F<D>(s->areaTriangle),
      F<vdtensor<D>>(s->kiteAreasOnVertex), F<D>(s->fVertex), F<vlreal>(S.h[t].data()),
      F<vlreal>(S.u[t].data()), F<vlreal>(S.h_edge[t].data()), F<vlreal>(S.h_vertex[t].data()),
      F<vlreal>(S.circulation.data()), F<vlreal>(S.vorticity.data()), F<vlreal>(S.ke[t].data()),
      F<vlreal>(S.pv_edge[t].data()), F<vlreal>(S.pv_vertex.data()));
}

// apps/sw/run.cc:13-70
void advance(mesh::view &mv, const orc_static *s, Sw &S, double dt) {
  const int pr = Sw::prev, nx = Sw::next, pv = Sw::provis;
  sw::task::init_provis(mv, F<vlreal>(S.u[pr].data()), F<vlreal>(S.h[pr].data()),
                        F<vltracer>(S.tr[pr].data()), F<vlreal>(S.h_edge[pr].data()),
                        F<vlreal>(S.ke[pr].data()), F<vlreal>(S.pv_edge[pr].data()),
                        F<vlreal>(S.u[pv].data()), F<vlreal>(S.h[pv].data()),
                        F<vltracer>(S.tr[pv].data()), F<vlreal>(S.h_edge[pv].data()),
                        F<vlreal>(S.ke[pv].data()), F<vlreal>(S.pv_edge[pv].data()));
  sw::task::setup_timestep(mv, F<vlreal>(S.u[pr].data()), F<vlreal>(S.h[pr].data()),
                           F<vltracer>(S.tr[pr].data()), F<vlreal>(S.u[nx].data()),
                           F<vlreal>(S.h[nx].data()), F<vltracer>(S.tr[nx].data()));
  const double rk_w[4] = {dt / 6, dt / 3, dt / 3, dt / 6};
  const double rk_sub[4] = {dt / 2, dt / 2, dt, 0};
  for (int rk = 0; rk < 4; ++rk) {
    sw::task::compute_tend(mv, F<D>(s->areaCell), F<D>(s->dvEdge), F<D>(s->dcEdge),
                           F<me2tensor<D>>(s->weightsOnEdge), F<vlreal>(S.h_edge[pv].data()),
                           F<vlreal>(S.h[pv].data()), F<D>(s->bottomDepth),
                           F<vlreal>(S.u[pv].data()), F<vlreal>(S.ke[pv].data()),
                           F<vlreal>(S.pv_edge[pv].data()), F<vlreal>(S.tend_h.data()),
                           F<vlreal>(S.tend_u.data()));
    sw::task::compute_scalar_tend(mv, F<D>(s->areaCell), F<D>(s->dvEdge), F<vlreal>(S.h_edge[pv].data()),
                                  F<vlreal>(S.u[pv].data()), F<vltracer>(S.tr[pv].data()),
                                  F<vltracer>(S.tend_tr.data()));
    if (rk < 3) {
      sw::task::compute_substep(mv, F<vlreal>(S.u[pv].data()), F<vlreal>(S.u[pr].data()),
                                F<vlreal>(S.tend_u.data()), F<vlreal>(S.h[pv].data()),
                                F<vlreal>(S.h[pr].data()), F<vlreal>(S.tend_h.data()),
                                F<vltracer>(S.tr[pv].data()), F<vltracer>(S.tr[pr].data()),
                                F<vltracer>(S.tend_tr.data()), rk_sub[rk]);
      diag(mv, s, S, pv);
    }
    sw::task::accumulate_update(mv, F<vlreal>(S.u[nx].data()), F<vlreal>(S.tend_u.data()),
                                F<vlreal>(S.h[nx].data()), F<vlreal>(S.tend_h.data()),
                                F<vltracer>(S.tr[nx].data()), F<vltracer>(S.tend_tr.data()),
                                rk_w[rk]);
  }
  sw::task::finalize_timestep(mv, F<vlreal>(S.u[pr].data()), F<vlreal>(S.u[nx].data()),
                              F<vlreal>(S.h[nx].data()), F<vltracer>(S.tr[nx].data()));
  diag(mv, s, S, nx);
  sw::task::timeshift(mv, F<vlreal>(S.u[pr].data()), F<vlreal>(S.h[pr].data()),
                      F<vltracer>(S.tr[pr].data()), F<vlreal>(S.h_edge[pr].data()),
                      F<vlreal>(S.ke[pr].data()), F<vlreal>(S.pv_edge[pr].data()),
                      F<vlreal>(S.u[nx].data()), F<vlreal>(S.h[nx].data()),
                      F<vltracer>(S.tr[nx].data()), F<vlreal>(S.h_edge[nx].data()),
                      F<vlreal>(S.ke[nx].data()), F<vlreal>(S.pv_edge[nx].data()));
}

}  // namespace

extern "C" {

const char *orc_cstep_last_error(void) { return g_err.c_str(); }

int orc_cstep_levels(int32_t *nlev) {
  *nlev = (int32_t)nVertLevels;
  return 0;
}

// nsteps steps from (h, u) + i eps (dh, du); on return h, u hold the real
// part and dh, du the tangent Im / eps.  Arrays [n][nVertLevels].
int orc_cstep_sw_run(const orc_mesh *m, const orc_static *s, double dt, int32_t nsteps, double eps,
                     double *h, double *u, double *dh, double *du) {
  try {
    sw::inputs::test_case.set(sw::test::case6);  // wind not pinned
    auto mv = view_of(m);
    Sw S(mv.nC, mv.nE, mv.nV);
    const std::size_t L = nVertLevels;
    for (std::size_t c = 0; c < mv.nC; ++c)
      for (std::size_t k = 0; k < L; ++k) S.h[Sw::prev][c][k] = cd(h[c * L + k], eps * dh[c * L + k]);
    for (std::size_t e = 0; e < mv.nE; ++e)
      for (std::size_t k = 0; k < L; ++k) S.u[Sw::prev][e][k] = cd(u[e * L + k], eps * du[e * L + k]);
    diag(mv, s, S, Sw::prev);  // apps/sw/run.cc:88-92
    for (int i = 0; i < nsteps; ++i) advance(mv, s, S, dt);
    for (std::size_t c = 0; c < mv.nC; ++c)
      for (std::size_t k = 0; k < L; ++k) {
        const cd x = S.h[Sw::prev][c][k];
        h[c * L + k] = x.real(), dh[c * L + k] = x.imag() / eps;
      }
    for (std::size_t e = 0; e < mv.nE; ++e)
      for (std::size_t k = 0; k < L; ++k) {
        const cd x = S.u[Sw::prev][e][k];
        u[e * L + k] = x.real(), du[e * L + k] = x.imag() / eps;
      }
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return 1;
  }
}

}  // extern "C"

// TEST INFRASTRUCTURE ONLY.  Driver around the reference's own task sources
// (compiled unmodified against oracle/shim/): exposes the oracle.h C API,
// calling the reference task functions on caller memory, and composes them
// into the reference's RK4 drivers (apps/sw/run.cc:13-70,
// apps/ocean/run.cc:10-50).  Built by oracle/build.py (build_ref) into
// oracle/_ref/libref_L<L>_T<T>.so, one library per compile-time level/tracer
// count; never shipped, never linked into the product.
#include <cstring>
#include <string>
#include <vector>

#include "apps/ocean/tasks/init_functions.hh"
#include "apps/ocean/tasks/solve.hh"
#include "apps/sw/state.hh"
#include "apps/sw/tasks/solve.hh"
#include "oracle.h"

extern "C" int orc_sw_del2_momentum_impl(const orc_mesh *m, const orc_static *s,
                                         const orc_config *c, const double *u,
                                         const double *vorticity, double *tend_u);

namespace {

using namespace mpas;
thread_local std::string g_err;

// Caller memory -> any privilege of the shim accessor for element type T.
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

void check_cfg(const orc_config *c) {
  if (c->nlev != (int)nVertLevels || c->ntr != (int)maxTracers ||
      c->gravity != mpas_constants::gravity)
    throw std::runtime_error("config does not match this reference build (L=" +
                             std::to_string(nVertLevels) + ", T=" +
                             std::to_string(maxTracers) + ")");
}

void set_case(const orc_config *c) {
  sw::inputs::test_case.set(c->pin_u ? sw::test::case1 : sw::test::case6);
}

template <class Fn> int guard(Fn &&f) {
  try {
    f();
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return 1;
  }
}

// ---------------------------------------------------------------- sw driver
struct Sw {
  enum { prev = 0, next = 1, provis = 2 };
  std::size_t nC, nE, nV;
  std::vector<vlreal> u[3], h[3], h_edge[3], h_vertex[3], ke[3], pv_edge[3];
  std::vector<vltracer> tr[3];
  std::vector<vlreal> circulation, vorticity, pv_vertex, tend_h, tend_u;
  std::vector<vltracer> tend_tr;
  std::vector<vlreal> ntf, hProv, hProvInv, hNewInv, w;
  std::vector<vltracer> lo, ho, flxIn, flxOut, trMax, trMin, trProv;
  Sw(std::size_t c, std::size_t e, std::size_t v) : nC(c), nE(e), nV(v) {
    for (int t = 0; t < 3; ++t) {
      u[t].assign(nE, vlreal{}), h[t].assign(nC, vlreal{}), h_edge[t].assign(nE, vlreal{});
      h_vertex[t].assign(nV, vlreal{}), ke[t].assign(nC, vlreal{}), pv_edge[t].assign(nE, vlreal{});
      tr[t].assign(nC, vltracer{});
    }
    circulation.assign(nV, vlreal{}), vorticity.assign(nV, vlreal{}), pv_vertex.assign(nV, vlreal{});
    tend_h.assign(nC, vlreal{}), tend_u.assign(nE, vlreal{}), tend_tr.assign(nC, vltracer{});
    ntf.assign(nE, vlreal{}), hProv.assign(nC, vlreal{}), hProvInv.assign(nC, vlreal{});
    hNewInv.assign(nC, vlreal{}), w.assign(nC, vlreal{});
    lo.assign(nE, vltracer{}), ho.assign(nE, vltracer{}), flxIn.assign(nC, vltracer{});
    flxOut.assign(nC, vltracer{}), trMax.assign(nC, vltracer{}), trMin.assign(nC, vltracer{});
    trProv.assign(nC, vltracer{});
  }
};

void sw_diag(mesh::view &mv, const orc_static *s, Sw &S, int t) {
  sw::task::compute_solve_diagnostics(
      mv, F<D>(s->dvEdge), F<D>(s->dcEdge), F<D>(s->areaCell), F<D>(s->areaTriangle),
      F<vdtensor<D>>(s->kiteAreasOnVertex), F<D>(s->fVertex), F<vlreal>(S.h[t].data()),
      F<vlreal>(S.u[t].data()), F<vlreal>(S.h_edge[t].data()), F<vlreal>(S.h_vertex[t].data()),
      F<vlreal>(S.circulation.data()), F<vlreal>(S.vorticity.data()), F<vlreal>(S.ke[t].data()),
      F<vlreal>(S.pv_edge[t].data()), F<vlreal>(S.pv_vertex.data()));
}

void sw_tracer_tend(mesh::view &mv, const orc_mesh *m, const orc_static *s, const orc_config *c,
                    Sw &S, double dt) {
  const int pv = Sw::provis;
  if (c->fct) {
    ocean::task::reinitialize_tracer_tendencies(mv, F<vltracer>(S.tend_tr.data()));
    ocean::task::calc_normal_thickness_flux(mv, F<vlreal>(S.h_edge[pv].data()),
                                            F<vlreal>(S.u[pv].data()), F<vlreal>(S.ntf.data()));
    ocean::task::calc_provisional_layer_thicknesses(
        mv, F<int>(s->maxLevelCell), F<D>(s->areaCell), F<D>(s->dvEdge),
        F<metensor<D>>(s->edgeSignOnCell), F<vlreal>(S.h[pv].data()), F<vlreal>(S.ntf.data()),
        F<vlreal>(S.w.data()), F<vlreal>(S.hProv.data()), F<vlreal>(S.hProvInv.data()),
        F<vlreal>(S.hNewInv.data()), dt);
    ocean::task::calc_horiz_tracer_advection_flux_mono_low_order(
        mv, F<D>(s->dvEdge), F<vlreal>(S.ntf.data()), F<vltracer>(S.tr[pv].data()),
        F<vltracer>(S.lo.data()));
    ocean::task::calc_horiz_tracer_advection_flux_mono_high_order(
        mv, F<vltensor<int>>(s->highOrderAdvMask), F<D>(s->dvEdge), F<vlreal>(S.ntf.data()),
        F<me2tensor<D>>(s->advCoef), F<me2tensor<D>>(s->advCoef_3rd), F<int>(s->maxLevelCell),
        F<int>(s->nAdvCellsForEdge), F<me2tensor<int>>(s->advCellsForEdge),
        F<vltracer>(S.tr[pv].data()), F<vltracer>(S.ho.data()));
    ocean::task::correct_and_rescale_high_order_mono_horiz_flux(
        mv, F<metensor<D>>(s->edgeSignOnCell), F<vlreal>(S.hProvInv.data()),
        F<vlreal>(S.h[pv].data()), F<vlreal>(S.ntf.data()), F<D>(s->areaCell), F<D>(s->dvEdge),
        F<vltensor<int>>(s->highOrderAdvMask), F<int>(s->maxLevelCell),
        F<int>(s->maxLevelEdgeTop), F<vltracer>(S.lo.data()), F<vltracer>(S.tr[pv].data()),
        F<vltracer>(S.ho.data()), F<vltracer>(S.flxIn.data()), F<vltracer>(S.flxOut.data()),
        F<vltracer>(S.tend_tr.data()), F<vltracer>(S.trMax.data()),
        F<vltracer>(S.trMin.data()), dt);
    ocean::task::accumulate_horiz_tracer_advection_tend_mono_FCT(
        mv, F<metensor<D>>(s->edgeSignOnCell), F<vlreal>(S.hProvInv.data()),
        F<vlreal>(S.h[pv].data()), F<D>(s->areaCell), F<int>(s->maxLevelCell),
        F<int>(s->maxLevelEdgeTop), F<vltracer>(S.ho.data()), F<vltracer>(S.tr[pv].data()),
        F<vltracer>(S.trProv.data()), F<vltracer>(S.tend_tr.data()), dt);
  } else {
    sw::task::compute_scalar_tend(mv, F<D>(s->areaCell), F<D>(s->dvEdge),
                                  F<vlreal>(S.h_edge[pv].data()), F<vlreal>(S.u[pv].data()),
                                  F<vltracer>(S.tr[pv].data()), F<vltracer>(S.tend_tr.data()));
  }
  if (c->hmix)
    ocean::task::tracer_hmix_del2_tend(
        mv, F<D>(s->areaCell), F<D>(s->dcEdge), F<D>(s->dvEdge), F<D>(s->meshScalingDel2),
        F<int>(s->maxLevelEdgeTop), F<metensor<D>>(s->edgeSignOnCell),
        F<vlreal>(S.h_edge[pv].data()), F<vltracer>(S.tr[pv].data()),
        F<vltracer>(S.tend_tr.data()), c->kappa);
  (void)m;
}

// apps/sw/run.cc:13-70
void sw_advance(mesh::view &mv, const orc_mesh *m, const orc_static *s, const orc_config *c,
                Sw &S, double dt) {
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
    if (c->nu != 0.0) {
      if (orc_sw_del2_momentum_impl(m, s, c, (const double *)S.u[pv].data(),
                                    (const double *)S.vorticity.data(),
                                    (double *)S.tend_u.data()) != 0)
        throw std::runtime_error("del2 momentum failed");
    }
    sw_tracer_tend(mv, m, s, c, S, dt);
    if (rk < 3) {
      sw::task::compute_substep(mv, F<vlreal>(S.u[pv].data()), F<vlreal>(S.u[pr].data()),
                                F<vlreal>(S.tend_u.data()), F<vlreal>(S.h[pv].data()),
                                F<vlreal>(S.h[pr].data()), F<vlreal>(S.tend_h.data()),
                                F<vltracer>(S.tr[pv].data()), F<vltracer>(S.tr[pr].data()),
                                F<vltracer>(S.tend_tr.data()), rk_sub[rk]);
      sw_diag(mv, s, S, pv);
    }
    sw::task::accumulate_update(mv, F<vlreal>(S.u[nx].data()), F<vlreal>(S.tend_u.data()),
                                F<vlreal>(S.h[nx].data()), F<vlreal>(S.tend_h.data()),
                                F<vltracer>(S.tr[nx].data()), F<vltracer>(S.tend_tr.data()),
                                rk_w[rk]);
  }
  sw::task::finalize_timestep(mv, F<vlreal>(S.u[pr].data()), F<vlreal>(S.u[nx].data()),
                              F<vlreal>(S.h[nx].data()), F<vltracer>(S.tr[nx].data()));
  sw_diag(mv, s, S, nx);
  sw::task::timeshift(mv, F<vlreal>(S.u[pr].data()), F<vlreal>(S.h[pr].data()),
                      F<vltracer>(S.tr[pr].data()), F<vlreal>(S.h_edge[pr].data()),
                      F<vlreal>(S.ke[pr].data()), F<vlreal>(S.pv_edge[pr].data()),
                      F<vlreal>(S.u[nx].data()), F<vlreal>(S.h[nx].data()),
                      F<vltracer>(S.tr[nx].data()), F<vlreal>(S.h_edge[nx].data()),
                      F<vlreal>(S.ke[nx].data()), F<vlreal>(S.pv_edge[nx].data()));
}

}  // namespace

extern "C" {

const char *orc_last_error(void) { return g_err.c_str(); }

int orc_compiled_levels(int32_t *nlev, int32_t *ntr, double *gravity) {
  *nlev = (int32_t)nVertLevels, *ntr = (int32_t)maxTracers, *gravity = mpas_constants::gravity;
  return 0;
}

int orc_sw_compute_solve_diagnostics(const orc_mesh *m, const orc_static *s, const orc_config *c,
                                     const double *h, const double *u, double *h_edge,
                                     double *h_vertex, double *circulation, double *vorticity,
                                     double *ke, double *pv_edge, double *pv_vertex) {
  return guard([&] {
    check_cfg(c);
    auto mv = view_of(m);
    sw::task::compute_solve_diagnostics(
        mv, F<D>(s->dvEdge), F<D>(s->dcEdge), F<D>(s->areaCell), F<D>(s->areaTriangle),
        F<vdtensor<D>>(s->kiteAreasOnVertex), F<D>(s->fVertex), F<vlreal>(h), F<vlreal>(u),
        F<vlreal>(h_edge), F<vlreal>(h_vertex), F<vlreal>(circulation), F<vlreal>(vorticity),
        F<vlreal>(ke), F<vlreal>(pv_edge), F<vlreal>(pv_vertex));
  });
}

int orc_sw_compute_tend(const orc_mesh *m, const orc_static *s, const orc_config *c,
                        const double *h_edge, const double *h, const double *u, const double *ke,
                        const double *pv_edge, double *tend_h, double *tend_u) {
  return guard([&] {
    check_cfg(c);
    auto mv = view_of(m);
    sw::task::compute_tend(mv, F<D>(s->areaCell), F<D>(s->dvEdge), F<D>(s->dcEdge),
                           F<me2tensor<D>>(s->weightsOnEdge), F<vlreal>(h_edge), F<vlreal>(h),
                           F<D>(s->bottomDepth), F<vlreal>(u), F<vlreal>(ke), F<vlreal>(pv_edge),
                           F<vlreal>(tend_h), F<vlreal>(tend_u));
  });
}

int orc_sw_compute_scalar_tend(const orc_mesh *m, const orc_static *s, const orc_config *c,
                               const double *h_edge, const double *u, const double *tracers,
                               double *tracer_tend) {
  return guard([&] {
    check_cfg(c);
    auto mv = view_of(m);
    sw::task::compute_scalar_tend(mv, F<D>(s->areaCell), F<D>(s->dvEdge), F<vlreal>(h_edge),
                                  F<vlreal>(u), F<vltracer>(tracers), F<vltracer>(tracer_tend));
  });
}

int orc_sw_compute_substep(const orc_mesh *m, const orc_config *c, double *u_provis,
                           const double *u_old, const double *u_tend, double *h_provis,
                           const double *h_old, const double *h_tend, double *tr_provis,
                           const double *tr_old, const double *tr_tend, double rkweight) {
  return guard([&] {
    check_cfg(c);
    set_case(c);
    auto mv = view_of(m);
    sw::task::compute_substep(mv, F<vlreal>(u_provis), F<vlreal>(u_old), F<vlreal>(u_tend),
                              F<vlreal>(h_provis), F<vlreal>(h_old), F<vlreal>(h_tend),
                              F<vltracer>(tr_provis), F<vltracer>(tr_old), F<vltracer>(tr_tend),
                              rkweight);
  });
}

int orc_sw_accumulate_update(const orc_mesh *m, const orc_config *c, double *u_new,
                             const double *u_tend, double *h_new, const double *h_tend,
                             double *tr_new, const double *tr_tend, double rkweight) {
  return guard([&] {
    check_cfg(c);
    auto mv = view_of(m);
    sw::task::accumulate_update(mv, F<vlreal>(u_new), F<vlreal>(u_tend), F<vlreal>(h_new),
                                F<vlreal>(h_tend), F<vltracer>(tr_new), F<vltracer>(tr_tend),
                                rkweight);
  });
}

int orc_sw_finalize_timestep(const orc_mesh *m, const orc_config *c, const double *u_old,
                             double *u_new, const double *h_new, double *tr_new) {
  return guard([&] {
    check_cfg(c);
    set_case(c);
    auto mv = view_of(m);
    sw::task::finalize_timestep(mv, F<vlreal>(u_old), F<vlreal>(u_new), F<vlreal>(h_new),
                                F<vltracer>(tr_new));
  });
}

int orc_sw_del2_momentum(const orc_mesh *m, const orc_static *s, const orc_config *c,
                         const double *u, const double *vorticity, double *tend_u) {
  return orc_sw_del2_momentum_impl(m, s, c, u, vorticity, tend_u);
}

int orc_oc_normal_thickness_flux(const orc_mesh *m, const orc_config *c, const double *hEdge,
                                 const double *u, double *ntf) {
  return guard([&] {
    check_cfg(c);
    auto mv = view_of(m);
    ocean::task::calc_normal_thickness_flux(mv, F<vlreal>(hEdge), F<vlreal>(u), F<vlreal>(ntf));
  });
}

int orc_oc_provisional_layer_thicknesses(const orc_mesh *m, const orc_static *s,
                                         const orc_config *c, const double *h, const double *ntf,
                                         const double *w, double *hProv, double *hProvInv,
                                         double *hNewInv, double dt) {
  return guard([&] {
    check_cfg(c);
    auto mv = view_of(m);
    ocean::task::calc_provisional_layer_thicknesses(
        mv, F<int>(s->maxLevelCell), F<D>(s->areaCell), F<D>(s->dvEdge),
        F<metensor<D>>(s->edgeSignOnCell), F<vlreal>(h), F<vlreal>(ntf), F<vlreal>(w),
        F<vlreal>(hProv), F<vlreal>(hProvInv), F<vlreal>(hNewInv), dt);
  });
}

int orc_oc_low_order(const orc_mesh *m, const orc_static *s, const orc_config *c,
                     const double *ntf, const double *tracers, double *lo) {
  return guard([&] {
    check_cfg(c);
    auto mv = view_of(m);
    ocean::task::calc_horiz_tracer_advection_flux_mono_low_order(
        mv, F<D>(s->dvEdge), F<vlreal>(ntf), F<vltracer>(tracers), F<vltracer>(lo));
  });
}

int orc_oc_high_order(const orc_mesh *m, const orc_static *s, const orc_config *c,
                      const double *ntf, const double *tracers, double *ho) {
  return guard([&] {
    check_cfg(c);
    auto mv = view_of(m);
    ocean::task::calc_horiz_tracer_advection_flux_mono_high_order(
        mv, F<vltensor<int>>(s->highOrderAdvMask), F<D>(s->dvEdge), F<vlreal>(ntf),
        F<me2tensor<D>>(s->advCoef), F<me2tensor<D>>(s->advCoef_3rd), F<int>(s->maxLevelCell),
        F<int>(s->nAdvCellsForEdge), F<me2tensor<int>>(s->advCellsForEdge),
        F<vltracer>(tracers), F<vltracer>(ho));
  });
}

int orc_oc_correct_and_rescale(const orc_mesh *m, const orc_static *s, const orc_config *c,
                               const double *hProvInv, const double *h, const double *ntf,
                               const double *lo, const double *tracers, double *ho,
                               double *flxIn, double *flxOut, double *tend, double *trMax,
                               double *trMin, double dt) {
  return guard([&] {
    check_cfg(c);
    auto mv = view_of(m);
    ocean::task::correct_and_rescale_high_order_mono_horiz_flux(
        mv, F<metensor<D>>(s->edgeSignOnCell), F<vlreal>(hProvInv), F<vlreal>(h),
        F<vlreal>(ntf), F<D>(s->areaCell), F<D>(s->dvEdge), F<vltensor<int>>(s->highOrderAdvMask),
        F<int>(s->maxLevelCell), F<int>(s->maxLevelEdgeTop), F<vltracer>(lo),
        F<vltracer>(tracers), F<vltracer>(ho), F<vltracer>(flxIn), F<vltracer>(flxOut),
        F<vltracer>(tend), F<vltracer>(trMax), F<vltracer>(trMin), dt);
  });
}

int orc_oc_accumulate_fct(const orc_mesh *m, const orc_static *s, const orc_config *c,
                          const double *hProvInv, const double *h, const double *ho,
                          const double *tracers, double *tracersProv, double *tend, double dt) {
  return guard([&] {
    check_cfg(c);
    auto mv = view_of(m);
    ocean::task::accumulate_horiz_tracer_advection_tend_mono_FCT(
        mv, F<metensor<D>>(s->edgeSignOnCell), F<vlreal>(hProvInv), F<vlreal>(h),
        F<D>(s->areaCell), F<int>(s->maxLevelCell), F<int>(s->maxLevelEdgeTop), F<vltracer>(ho),
        F<vltracer>(tracers), F<vltracer>(tracersProv), F<vltracer>(tend), dt);
  });
}

int orc_oc_hmix_del2(const orc_mesh *m, const orc_static *s, const orc_config *c,
                     const double *hEdge, const double *tracers, double *tend, double coef) {
  return guard([&] {
    check_cfg(c);
    auto mv = view_of(m);
    ocean::task::tracer_hmix_del2_tend(mv, F<D>(s->areaCell), F<D>(s->dcEdge), F<D>(s->dvEdge),
                                       F<D>(s->meshScalingDel2), F<int>(s->maxLevelEdgeTop),
                                       F<metensor<D>>(s->edgeSignOnCell), F<vlreal>(hEdge),
                                       F<vltracer>(tracers), F<vltracer>(tend), coef);
  });
}

int orc_oc_step_tracers_forward(const orc_mesh *m, const orc_config *c, const double *tend,
                                const double *tracers, double *tracersNew, double *tracersPrev,
                                double rk_weight, double rk_subweight) {
  return guard([&] {
    check_cfg(c);
    auto mv = view_of(m);
    ocean::task::step_tracers_forward(mv, F<vltracer>(tend), F<vltracer>(tracers),
                                      F<vltracer>(tracersNew), F<vltracer>(tracersPrev),
                                      rk_weight, rk_subweight);
  });
}

int orc_init_fct_statics(const orc_mesh *m, const orc_config *c, const orc_geom *g,
                         orc_setup_out *o) {
  return guard([&] {
    check_cfg(c);
    auto mv = view_of(m);
    // apps/ocean/initialize.cc:88-102 (layerThicknessEdge is separate)
    ocean::task::init_maxLevelEdgeTop(mv, F<int>(g->maxLevelCell), F<int>(o->maxLevelEdgeTop));
    ocean::task::init_meshScalingDel2(mv, F<D>(g->meshDensity), F<D>(o->meshScalingDel2));
    ocean::task::init_edgeSignOnCell(mv, F<metensor<D>>(o->edgeSignOnCell));
    ocean::task::init_2nd_deriv(mv, F<D>(g->angleEdge), F<D>(g->dcEdge), F<D>(g->xCell),
                                F<D>(g->yCell), F<D>(g->zCell), F<D>(g->xVertex),
                                F<D>(g->yVertex), F<D>(g->zVertex), F<derivtensor>(o->derivTwo));
    ocean::task::init_tracer_adv_coeff(
        mv, F<int>(g->maxLevelCell), F<D>(g->dcEdge), F<D>(g->dvEdge),
        F<vltensor<int>>(g->boundaryCell), F<derivtensor>(o->derivTwo),
        F<int>(o->nAdvCellsForEdge), F<vltensor<int>>(o->highOrderAdvMask),
        F<me2tensor<int>>(o->advCellsForEdge), F<me2tensor<D>>(o->advCoef),
        F<me2tensor<D>>(o->advCoef_3rd));
  });
}

int orc_init_layer_thickness_edge(const orc_mesh *m, const orc_config *c, const double *h,
                                  const int32_t *maxLevelEdgeTop, double *hEdge) {
  return guard([&] {
    check_cfg(c);
    auto mv = view_of(m);
    ocean::task::init_layerThicknessEdge(mv, F<vlreal>(h), F<int>(maxLevelEdgeTop),
                                         F<vlreal>(hEdge));
  });
}

int orc_sw_run(const orc_mesh *m, const orc_static *s, const orc_config *c, double dt,
               int32_t nsteps, double *h, double *u, double *tracers) {
  return guard([&] {
    check_cfg(c);
    set_case(c);
    auto mv = view_of(m);
    Sw S(mv.nC, mv.nE, mv.nV);
    std::memcpy(S.h[Sw::prev].data(), h, mv.nC * sizeof(vlreal));
    std::memcpy(S.u[Sw::prev].data(), u, mv.nE * sizeof(vlreal));
    std::memcpy(S.tr[Sw::prev].data(), tracers, mv.nC * sizeof(vltracer));
    sw_diag(mv, s, S, Sw::prev);  // apps/sw/run.cc:88-92
    for (int i = 0; i < nsteps; ++i) sw_advance(mv, m, s, c, S, dt);
    std::memcpy(h, S.h[Sw::prev].data(), mv.nC * sizeof(vlreal));
    std::memcpy(u, S.u[Sw::prev].data(), mv.nE * sizeof(vlreal));
    std::memcpy(tracers, S.tr[Sw::prev].data(), mv.nC * sizeof(vltracer));
  });
}

// apps/ocean/run.cc:10-50
int orc_ocean_run(const orc_mesh *m, const orc_static *s, const orc_config *c, double dt,
                  int32_t nsteps, const double *layerThickness, const double *layerThicknessEdge,
                  const double *normalVelocity, double *tracers) {
  return guard([&] {
    check_cfg(c);
    auto mv = view_of(m);
    const std::size_t nC = mv.nC, nE = mv.nE;
    enum { prev = 0, curr = 1, next = 2, prov = 3 };
    std::vector<vltracer> tr[4];
    for (auto &t : tr) t.assign(nC, vltracer{});
    std::vector<vlreal> hProv(nC), hProvInv(nC), hNewInv(nC), w(nC), ntf(nE);
    std::vector<vltracer> tend(nC), lo(nE), ho(nE), flxIn(nC), flxOut(nC), trMax(nC), trMin(nC);
    std::memcpy(tr[curr].data(), tracers, nC * sizeof(vltracer));
    const double rk_w[4] = {dt / 6, dt / 3, dt / 3, dt / 6};
    const double rk_sub[4] = {dt / 2, dt / 2, dt, 0};
    for (int step = 0; step < nsteps; ++step) {
      ocean::task::copy_tracers(mv, F<vltracer>(tr[curr].data()), F<vltracer>(tr[next].data()),
                                F<vltracer>(tr[prev].data()));
      for (int rk = 0; rk < 4; ++rk) {
        ocean::task::reinitialize_tracer_tendencies(mv, F<vltracer>(tend.data()));
        if (c->fct) {
          ocean::task::calc_normal_thickness_flux(mv, F<vlreal>(layerThicknessEdge),
                                                  F<vlreal>(normalVelocity),
                                                  F<vlreal>(ntf.data()));
          ocean::task::calc_provisional_layer_thicknesses(
              mv, F<int>(s->maxLevelCell), F<D>(s->areaCell), F<D>(s->dvEdge),
              F<metensor<D>>(s->edgeSignOnCell), F<vlreal>(layerThickness),
              F<vlreal>(ntf.data()), F<vlreal>(w.data()), F<vlreal>(hProv.data()),
              F<vlreal>(hProvInv.data()), F<vlreal>(hNewInv.data()), dt);
          ocean::task::calc_horiz_tracer_advection_flux_mono_low_order(
              mv, F<D>(s->dvEdge), F<vlreal>(ntf.data()), F<vltracer>(tr[prev].data()),
              F<vltracer>(lo.data()));
          ocean::task::calc_horiz_tracer_advection_flux_mono_high_order(
              mv, F<vltensor<int>>(s->highOrderAdvMask), F<D>(s->dvEdge), F<vlreal>(ntf.data()),
              F<me2tensor<D>>(s->advCoef), F<me2tensor<D>>(s->advCoef_3rd),
              F<int>(s->maxLevelCell), F<int>(s->nAdvCellsForEdge),
              F<me2tensor<int>>(s->advCellsForEdge), F<vltracer>(tr[prev].data()),
              F<vltracer>(ho.data()));
          ocean::task::correct_and_rescale_high_order_mono_horiz_flux(
              mv, F<metensor<D>>(s->edgeSignOnCell), F<vlreal>(hProvInv.data()),
              F<vlreal>(layerThickness), F<vlreal>(ntf.data()), F<D>(s->areaCell),
              F<D>(s->dvEdge), F<vltensor<int>>(s->highOrderAdvMask), F<int>(s->maxLevelCell),
              F<int>(s->maxLevelEdgeTop), F<vltracer>(lo.data()), F<vltracer>(tr[prev].data()),
              F<vltracer>(ho.data()), F<vltracer>(flxIn.data()), F<vltracer>(flxOut.data()),
              F<vltracer>(tend.data()), F<vltracer>(trMax.data()), F<vltracer>(trMin.data()),
              dt);
          ocean::task::accumulate_horiz_tracer_advection_tend_mono_FCT(
              mv, F<metensor<D>>(s->edgeSignOnCell), F<vlreal>(hProvInv.data()),
              F<vlreal>(layerThickness), F<D>(s->areaCell), F<int>(s->maxLevelCell),
              F<int>(s->maxLevelEdgeTop), F<vltracer>(ho.data()), F<vltracer>(tr[prev].data()),
              F<vltracer>(tr[prov].data()), F<vltracer>(tend.data()), dt);
        }
        if (c->hmix)
          ocean::task::tracer_hmix_del2_tend(
              mv, F<D>(s->areaCell), F<D>(s->dcEdge), F<D>(s->dvEdge), F<D>(s->meshScalingDel2),
              F<int>(s->maxLevelEdgeTop), F<metensor<D>>(s->edgeSignOnCell),
              F<vlreal>(layerThicknessEdge), F<vltracer>(tr[prev].data()),
              F<vltracer>(tend.data()), c->kappa);
        ocean::task::step_tracers_forward(mv, F<vltracer>(tend.data()),
                                          F<vltracer>(tr[curr].data()),
                                          F<vltracer>(tr[next].data()),
                                          F<vltracer>(tr[prev].data()), rk_w[rk], rk_sub[rk]);
      }
      ocean::task::update_tracers(mv, F<vltracer>(tr[next].data()), F<vltracer>(tr[curr].data()));
    }
    std::memcpy(tracers, tr[curr].data(), nC * sizeof(vltracer));
  });
}

}  // extern "C"

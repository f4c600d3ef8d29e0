/*
 * oracle.h -- TEST INFRASTRUCTURE ONLY.  CPU oracle of the MPAS-O-FleCSI RK4
 * tendency path.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load the oracle libraries; the product never does.
 *
 * Two libraries export this same API:
 *   oracle/_ref/libref_L<L>_T<T>.so -- the reference's own task sources
 *       (apps/sw/tasks/solve.cc, apps/ocean/tasks/solve.cc,
 *       apps/ocean/tasks/init_functions.cc) compiled unmodified against the
 *       header shim in oracle/shim/, plus ref_driver.cc.  Levels and tracers
 *       are compile-time there (mpasoflecsi/common/constants.hh:16,18).
 *   oracle/_build/liboracle.so -- oracle.c, a plain-C restatement of the same
 *       task loops (runtime levels/tracers), the one that travels to the GPU
 *       host and serves as the CPU baseline there.
 *
 * All field arrays use the reference's per-entity AoS layouts:
 *   vlreal  [n][L], vltracer [n][L][T], metensor [n][8], me2tensor [n][16],
 *   vdtensor [n][3], derivtensor [n][16][2].
 * Every function returns 0 on success, nonzero on failure (orc_last_error()).
 */
#ifndef MPASO_ORACLE_H
#define MPASO_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Connectivity as the reference's mesh specialization holds it (0-based CRS):
 * file order for c2v, c2e, c2c, e2v, e2e; transposition (ascending ids) for
 * v2c, e2c, v2e (mpasoflecsi/specialization/mesh.cc:67-116). */
enum { ORC_C2V, ORC_C2E, ORC_C2C, ORC_E2V, ORC_E2E, ORC_V2C, ORC_E2C, ORC_V2E, ORC_NCNX };
typedef struct {
  int64_t nC, nE, nV;
  const int64_t *off[ORC_NCNX];
  const int32_t *idx[ORC_NCNX];
} orc_mesh;

/* Static (per-mesh) fields read by the tasks. */
typedef struct {
  const double *areaCell, *dvEdge, *dcEdge, *areaTriangle, *kiteAreasOnVertex, *fVertex;
  const double *weightsOnEdge; /* me2tensor */
  const double *bottomDepth;   /* h_s of the sw app */
  /* FCT / del2 statics (apps/ocean/state.hh:68-101) */
  const int32_t *maxLevelCell, *maxLevelEdgeTop, *nAdvCellsForEdge;
  const int32_t *advCellsForEdge;  /* me2tensor<int> */
  const int32_t *highOrderAdvMask; /* vltensor<int> */
  const double *edgeSignOnCell;    /* metensor */
  const double *advCoef, *advCoef_3rd; /* me2tensor */
  const double *meshScalingDel2;
} orc_static;

typedef struct {
  int32_t nlev, ntr;
  double gravity;
  int32_t fct;    /* sw: FCT tracer advection instead of compute_scalar_tend */
  int32_t hmix;   /* del2 tracer mixing */
  double kappa;   /* del2 tracer coefficient (m^2/s) */
  double nu;      /* del2 momentum viscosity (m^2/s); not in the reference */
  int32_t pin_u;  /* sw test case 1: wind held fixed (apps/sw/tasks/solve.cc:307-313,359-366) */
} orc_config;

const char *orc_last_error(void);
int orc_compiled_levels(int32_t *nlev, int32_t *ntr, double *gravity); /* -1 = runtime */

/* ---- sw tasks (apps/sw/tasks/solve.cc) ---- */
int orc_sw_compute_solve_diagnostics(const orc_mesh *m, const orc_static *s, const orc_config *c,
                                     const double *h, const double *u, double *h_edge,
                                     double *h_vertex, double *circulation, double *vorticity,
                                     double *ke, double *pv_edge, double *pv_vertex);
int orc_sw_compute_tend(const orc_mesh *m, const orc_static *s, const orc_config *c,
                        const double *h_edge, const double *h, const double *u, const double *ke,
                        const double *pv_edge, double *tend_h, double *tend_u);
int orc_sw_compute_scalar_tend(const orc_mesh *m, const orc_static *s, const orc_config *c,
                               const double *h_edge, const double *u, const double *tracers,
                               double *tracer_tend);
int orc_sw_compute_substep(const orc_mesh *m, const orc_config *c, double *u_provis,
                           const double *u_old, const double *u_tend, double *h_provis,
                           const double *h_old, const double *h_tend, double *tr_provis,
                           const double *tr_old, const double *tr_tend, double rkweight);
int orc_sw_accumulate_update(const orc_mesh *m, const orc_config *c, double *u_new,
                             const double *u_tend, double *h_new, const double *h_tend,
                             double *tr_new, const double *tr_tend, double rkweight);
int orc_sw_finalize_timestep(const orc_mesh *m, const orc_config *c, const double *u_old,
                             double *u_new, const double *h_new, double *tr_new);
/* del2 momentum: tend_u += nu*((div(c2)-div(c1))/dc - (vort(v2)-vort(v1))/dv).
 * Not in the reference (its compute_tend has no viscosity). */
int orc_sw_del2_momentum(const orc_mesh *m, const orc_static *s, const orc_config *c,
                         const double *u, const double *vorticity, double *tend_u);

/* ---- ocean tasks (apps/ocean/tasks/solve.cc) ---- */
int orc_oc_normal_thickness_flux(const orc_mesh *m, const orc_config *c, const double *hEdge,
                                 const double *u, double *ntf);
int orc_oc_provisional_layer_thicknesses(const orc_mesh *m, const orc_static *s,
                                         const orc_config *c, const double *h, const double *ntf,
                                         const double *w, double *hProv, double *hProvInv,
                                         double *hNewInv, double dt);
int orc_oc_low_order(const orc_mesh *m, const orc_static *s, const orc_config *c,
                     const double *ntf, const double *tracers, double *lo);
int orc_oc_high_order(const orc_mesh *m, const orc_static *s, const orc_config *c,
                      const double *ntf, const double *tracers, double *ho);
int orc_oc_correct_and_rescale(const orc_mesh *m, const orc_static *s, const orc_config *c,
                               const double *hProvInv, const double *h, const double *ntf,
                               const double *lo, const double *tracers, double *ho,
                               double *flxIn, double *flxOut, double *tend, double *trMax,
                               double *trMin, double dt);
int orc_oc_accumulate_fct(const orc_mesh *m, const orc_static *s, const orc_config *c,
                          const double *hProvInv, const double *h, const double *ho,
                          const double *tracers, double *tracersProv, double *tend, double dt);
int orc_oc_hmix_del2(const orc_mesh *m, const orc_static *s, const orc_config *c,
                     const double *hEdge, const double *tracers, double *tend, double coef);
int orc_oc_step_tracers_forward(const orc_mesh *m, const orc_config *c, const double *tend,
                                const double *tracers, double *tracersNew, double *tracersPrev,
                                double rk_weight, double rk_subweight);

/* ---- static setup (apps/ocean/tasks/init_functions.cc) ---- */
typedef struct {
  const double *angleEdge, *dcEdge, *dvEdge, *xCell, *yCell, *zCell, *xVertex, *yVertex, *zVertex;
  const double *meshDensity;
  const int32_t *maxLevelCell; /* [nC] */
  const int32_t *boundaryCell; /* vltensor<int> [nC][L] */
} orc_geom;
typedef struct {
  int32_t *maxLevelEdgeTop, *nAdvCellsForEdge, *advCellsForEdge, *highOrderAdvMask;
  double *meshScalingDel2, *edgeSignOnCell, *derivTwo, *advCoef, *advCoef_3rd;
} orc_setup_out;
int orc_init_fct_statics(const orc_mesh *m, const orc_config *c, const orc_geom *g,
                         orc_setup_out *o);
int orc_init_layer_thickness_edge(const orc_mesh *m, const orc_config *c, const double *h,
                                  const int32_t *maxLevelEdgeTop, double *hEdge);

/* ---- composed drivers ---- */
/* sw: apps/sw/run.cc:13-70 (+ the initial diagnostics of apps/sw/run.cc:88-92).
 * With fct=1 the tracer tendency is the ocean FCT sequence of
 * apps/ocean/run.cc:19-42 applied to the provisional sw state (layer thickness
 * = h[provis], layer thickness at edges = h_edge[provis], velocity = u[provis],
 * full dt), in place of compute_scalar_tend; hmix adds del2 tracer mixing and
 * nu > 0 adds del2 momentum after compute_tend.  h, u, tracers: in/out. */
int orc_sw_run(const orc_mesh *m, const orc_static *s, const orc_config *c, double dt,
               int32_t nsteps, double *h, double *u, double *tracers);
/* ocean: apps/ocean/run.cc:10-50 with monoAdvect = fct, hmix = hmix. */
int orc_ocean_run(const orc_mesh *m, const orc_static *s, const orc_config *c, double dt,
                  int32_t nsteps, const double *layerThickness, const double *layerThicknessEdge,
                  const double *normalVelocity, double *tracers);

#ifdef __cplusplus
}
#endif
#endif

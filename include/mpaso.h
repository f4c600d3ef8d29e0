/*
 * mpaso.h -- C ABI of libmpaso's GB300 (sm_103a) path for MPAS-O-FleCSI's
 * RK4 tendency tasks.
 *
 * Drop-in boundary: the reference launches its tasks through FleCSI,
 *   flecsi::execute<task::compute_tend>(m, areaCell(m), ...)  (apps/sw/run.cc:15-69,
 *   apps/ocean/run.cc:12-48),
 * with field accessors over per-entity AoS storage (mpasoflecsi/common/types.hh:31-46).
 * Each per-task entry below takes the same fields, in the same order and the
 * same AoS layouts, as raw pointers (host or device memory, detected per
 * pointer) in the reference's entity numbering.  Static mesh fields
 * (areaCell, dvEdge, dcEdge, weightsOnEdge, ...) are given once, at mesh
 * context creation; a task wrapper with the reference's signature passes the
 * per-step fields and ignores the static accessors.
 *
 * Internally the mesh is renumbered along a Hilbert curve (an exact integer
 * permutation, see mpaso_mesh_permutation), fields live in HBM in that order,
 * and every kernel gathers over precomputed connectivity without atomics.
 *
 * Conventions:
 *   - every call returns MPASO_OK (0) or an MPASO_ERR_* code (mpaso_mesh.h);
 *     mpaso_last_error() gives the calling thread's message; no exception
 *     crosses the ABI;
 *   - a context is used by one host thread at a time; distinct contexts may be
 *     used concurrently;
 *   - `stream` is a cudaStream_t (NULL = the context's own stream).  Calls
 *     with any host pointer are synchronous; calls with only device pointers
 *     are asynchronous on the stream.
 */
#ifndef MPASO_H
#define MPASO_H

#include <stdint.h>

#include "mpaso_mesh.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mpaso_mesh_s *mpaso_mesh;
typedef struct mpaso_state_s *mpaso_state;

/* Mesh description in the reference's terms.  Connectivity is FleCSI's CRS
 * (0-based) in file order: c2v = verticesOnCell, c2e = edgesOnCell,
 * c2c = cellsOnCell, e2v = verticesOnEdge, e2e = edgesOnEdge
 * (mpasoflecsi/specialization/mesh.cc:67-89).  The transposes v2c, e2c, v2e
 * are built inside, as mesh.cc:108-116 builds them (ascending ids). */
typedef struct {
  int64_t nCells, nEdges, nVertices;
  const int64_t *c2v_off, *c2e_off, *c2c_off, *e2v_off, *e2e_off;
  const int32_t *c2v, *c2e, *c2c, *e2v, *e2e;
  /* geometry (mpasoflecsi/specialization/mesh.hh:114-152) */
  const double *areaCell, *dvEdge, *dcEdge, *areaTriangle;
  const double *kiteAreasOnVertex; /* [nV][3] */
  const double *fVertex;
  const double *weightsOnEdge; /* [nE][16] */
  const double *bottomDepth;   /* h_s of the sw app; NULL = 0 */
  /* cell centres: used only to build the Hilbert ordering; NULL = keep order */
  const double *xCell, *yCell, *zCell;
  /* renumbering: 0 keep the numbering; 1 cells along a Hilbert curve, edges and
   * vertices after their cells; 2 cells, edges and vertices each along the
   * Hilbert curve of their own position; 3 cells in Morton order, edges and
   * vertices after their cells (results agree across orders to rounding) */
  int32_t reorder;
  /* FCT / del2 statics (apps/ocean/state.hh:68-101); NULL = not available */
  int32_t fct_nlev; /* level count of highOrderAdvMask */
  const int32_t *maxLevelCell, *maxLevelEdgeTop, *nAdvCellsForEdge;
  const int32_t *advCellsForEdge;  /* [nE][16] */
  const int32_t *highOrderAdvMask; /* [nE][fct_nlev] */
  const double *edgeSignOnCell;    /* [nC][8] */
  const double *advCoef, *advCoef_3rd; /* [nE][16] */
  const double *meshScalingDel2;
} mpaso_mesh_desc;

#define MPASO_CELLS 0
#define MPASO_EDGES 1
#define MPASO_VERTICES 2

/* Builds the device mesh context on `device` (-1 = current device). */
int mpaso_mesh_create(const mpaso_mesh_desc *desc, int device, mpaso_mesh *out);
/* Drops the caller's reference: the context is freed when it and every state
 * made on it (mpaso_state_create) have been destroyed, in any order. */
int mpaso_mesh_destroy(mpaso_mesh m);
/* new_to_old[new] = reference id, for MPASO_CELLS/EDGES/VERTICES. */
int mpaso_mesh_permutation(mpaso_mesh m, int32_t entity, int32_t *new_to_old);
/* Gravity used by compute_tend (the reference's mpas_constants::gravity,
 * mpasoflecsi/common/constants.hh:30-31; default 9.80616). */
int mpaso_mesh_set_gravity(mpaso_mesh m, double gravity);
/* Bytes of device memory held by the context. */
int mpaso_mesh_device_bytes(mpaso_mesh m, int64_t *bytes);

/* Ensemble of independent members on uneven meshes (no counterpart in the
 * reference, which runs one mesh): one context over the disjoint union of n
 * member descriptions, so one state and one graph-captured launch sequence
 * advance every member.  Reference numbering of the union = the members'
 * numberings concatenated in member order (fields are set and read as the
 * concatenation of the members' arrays); with reorder = 1 each member is
 * renumbered along its own Hilbert curve inside its own block.  Members must
 * agree on reorder and on having FCT statics (same fct_nlev); they share the
 * state parameters (dt, gravity, diffusion) and may mix planes and spheres. */
int mpaso_mesh_create_ensemble(const mpaso_mesh_desc *members, int32_t n, int device,
                               mpaso_mesh *out);
/* *n = member count (1 for a plain mesh); offsets (optional, 3 (n + 1)
 * int64) receive the first cell, edge and vertex of each member, then the
 * totals. */
int mpaso_mesh_members(mpaso_mesh m, int32_t *n, int64_t *offsets);

/* ------------------------------------------------------------------------
 * Per-task entries, one per reference task.  Arrays: vlreal [n][L],
 * vltracer [n][L][T], in the reference's numbering.  nlev / ntr are the
 * reference's nVertLevels / maxTracers (compile-time there).
 * ---------------------------------------------------------------------- */

/* apps/sw/tasks/solve.cc:11-107 */
int mpaso_sw_compute_solve_diagnostics(mpaso_mesh m, int32_t nlev, const double *h,
                                       const double *u, double *h_edge, double *h_vertex,
                                       double *circulation, double *vorticity, double *ke,
                                       double *pv_edge, double *pv_vertex, void *stream);
/* apps/sw/tasks/solve.cc:169-234 */
int mpaso_sw_compute_tend(mpaso_mesh m, int32_t nlev, const double *h_edge, const double *h,
                          const double *u, const double *ke, const double *pv_edge,
                          double *tend_h, double *tend_u, void *stream);
/* Allocation-free compute_tend (no counterpart in the reference).  Same
 * arguments and results as mpaso_sw_compute_tend, for callers that must not
 * allocate device memory during the call (a task inside a runtime that pools
 * all device memory, or code that cannot afford cudaMalloc's device-wide
 * synchronisation).  All seven arrays must be device memory.  Arguments are
 * staged through one static 32 MiB device array instead of allocated scratch,
 * which limits the mesh to (4 nEdges + 3 nCells) * nlev <= 4,194,304 doubles
 * (larger meshes get MPASO_ERR_ARG).  Each call looks up that array's
 * address (cudaGetSymbolAddress) unless its stream is being captured, when it
 * reuses the address of the last uncaptured call on that device: make the
 * first call on each device before any stream capture.  The array is not
 * counted by mpaso_mesh_device_bytes.  Every call shares the array, so calls
 * whose GPU work overlaps race. */
int mpaso_sw_compute_tend_noalloc(mpaso_mesh m, int32_t nlev, const double *h_edge,
                                  const double *h, const double *u, const double *ke,
                                  const double *pv_edge, double *tend_h, double *tend_u,
                                  void *stream);
/* apps/sw/tasks/solve.cc:237-270 */
int mpaso_sw_compute_scalar_tend(mpaso_mesh m, int32_t nlev, int32_t ntr, const double *h_edge,
                                 const double *u, const double *tracers, double *tracer_tend,
                                 void *stream);
/* apps/sw/tasks/solve.cc:273-314; pin_u = 1 reproduces test case 1 */
int mpaso_sw_compute_substep(mpaso_mesh m, int32_t nlev, int32_t ntr, double *u_provis,
                             const double *u_old, const double *u_tend, double *h_provis,
                             const double *h_old, const double *h_tend, double *tracers_provis,
                             const double *tracers_old, const double *tracers_tend,
                             double rkweight, int32_t pin_u, void *stream);
/* apps/sw/tasks/solve.cc:317-341 */
int mpaso_sw_accumulate_update(mpaso_mesh m, int32_t nlev, int32_t ntr, double *u_new,
                               const double *u_tend, double *h_new, const double *h_tend,
                               double *tracers_new, const double *tracers_tend, double rkweight,
                               void *stream);
/* apps/sw/tasks/solve.cc:344-367 */
int mpaso_sw_finalize_timestep(mpaso_mesh m, int32_t nlev, int32_t ntr, const double *u_old,
                               double *u_new, const double *h_new, double *tracers_new,
                               int32_t pin_u, void *stream);

/* apps/ocean/tasks/solve.cc:40-57 */
int mpaso_oc_calc_normal_thickness_flux(mpaso_mesh m, int32_t nlev,
                                        const double *layerThicknessEdge,
                                        const double *normalVelocity,
                                        double *normalThicknessFlux, void *stream);
/* apps/ocean/tasks/solve.cc:60-97 (w is unused, as in the reference) */
int mpaso_oc_calc_provisional_layer_thicknesses(mpaso_mesh m, int32_t nlev,
                                                const double *layerThickness,
                                                const double *normalThicknessFlux,
                                                double *hProv, double *hProvInv, double *hNewInv,
                                                double dt, void *stream);
/* apps/ocean/tasks/solve.cc:99-118 */
int mpaso_oc_calc_horiz_tracer_advection_flux_mono_low_order(
    mpaso_mesh m, int32_t nlev, int32_t ntr, const double *normalThicknessFlux,
    const double *tracers, double *lowOrderFlux, void *stream);
/* apps/ocean/tasks/solve.cc:120-167 */
int mpaso_oc_calc_horiz_tracer_advection_flux_mono_high_order(
    mpaso_mesh m, int32_t nlev, int32_t ntr, const double *normalThicknessFlux,
    const double *tracers, double *highOrderFlux, void *stream);
/* apps/ocean/tasks/solve.cc:169-285 */
int mpaso_oc_correct_and_rescale_high_order_mono_horiz_flux(
    mpaso_mesh m, int32_t nlev, int32_t ntr, const double *hProvInv, const double *layerThickness,
    const double *normalThicknessFlux, const double *lowOrderFlux, const double *tracers,
    double *highOrderFlux, double *flxIn, double *flxOut, double *tend, double *tracerMax,
    double *tracerMin, double dt, void *stream);
/* apps/ocean/tasks/solve.cc:287-326 */
int mpaso_oc_accumulate_horiz_tracer_advection_tend_mono_FCT(
    mpaso_mesh m, int32_t nlev, int32_t ntr, const double *hProvInv, const double *layerThickness,
    const double *highOrderFlux, const double *tracers, double *tracersProv, double *tend,
    double dt, void *stream);
/* apps/ocean/tasks/solve.cc:328-366 */
int mpaso_oc_tracer_hmix_del2_tend(mpaso_mesh m, int32_t nlev, int32_t ntr,
                                   const double *layerThicknessEdge, const double *tracers,
                                   double *tend, double coef, void *stream);
/* apps/ocean/tasks/solve.cc:368-399 */
int mpaso_oc_step_tracers_forward(mpaso_mesh m, int32_t nlev, int32_t ntr, const double *tend,
                                  const double *tracers, double *tracersNew, double *tracersPrev,
                                  double rk_weight, double rk_subweight, void *stream);

/* ------------------------------------------------------------------------
 * Fused RK4 path: state resident in HBM, one call advances nsteps.
 * ---------------------------------------------------------------------- */
#define MPASO_APP_SW 0    /* apps/sw/run.cc:13-70 (+ FCT tracer coupling) */
#define MPASO_APP_OCEAN 1 /* apps/ocean/run.cc:10-50 */

typedef struct {
  int32_t app;
  int32_t nlev, ntr;
  double gravity; /* sw */
  int32_t fct;    /* FCT tracer advection (sw: replaces compute_scalar_tend) */
  int32_t hmix;   /* del2 tracer mixing */
  double kappa;   /* del2 tracer coefficient, m^2/s */
  double nu;      /* del2 momentum viscosity, m^2/s (sw; not in the reference) */
  int32_t pin_u;  /* sw test case 1 */
} mpaso_params;

#define MPASO_FIELD_H 0                    /* sw h / ocean layerThickness [nC][L] */
#define MPASO_FIELD_U 1                    /* sw u / ocean normalVelocity [nE][L] */
#define MPASO_FIELD_TRACERS 2              /* [nC][L][T] */
#define MPASO_FIELD_LAYER_THICKNESS_EDGE 3 /* ocean layerThicknessEdge [nE][L] */
/* sw diagnostics of the current state, read-only (get / snapshot): the
 * vorticity and pv_vertex fields compute_solve_diagnostics produces
 * (apps/sw/tasks/solve.cc:56-60, 90) and the sw history output writes as
 * "vorticity" / "potential_vorticity" (mpasoflecsi/io/desc.hh:46-56) */
#define MPASO_FIELD_VORTICITY 4            /* [nV][L] */
#define MPASO_FIELD_PV_VERTEX 5            /* [nV][L] */

int mpaso_state_create(mpaso_mesh m, const mpaso_params *p, mpaso_state *out);
int mpaso_state_destroy(mpaso_state s);
/* Copy a field in (reference numbering, host or device memory). */
int mpaso_state_set(mpaso_state s, int32_t field, const double *data);
/* Copy a field out (reference numbering, host or device memory). */
int mpaso_state_get(mpaso_state s, int32_t field, double *data);
/* Scan the prognostic fields (h, u, tracers; the ocean's edge thickness) on
 * the device for NaN or infinity: MPASO_OK, or MPASO_ERR_NUMERIC with the
 * first offending field, entity (reference numbering), level and tracer in
 * mpaso_last_error().  No counterpart in the reference, which has no such
 * check; a blow-up there shows as NaN in the error norms of
 * apps/sw/finalize.cc:21-23. */
int mpaso_state_check_finite(mpaso_state s);
/* Advance nsteps RK4 steps of size dt; asynchronous on the state's stream. */
int mpaso_rk4_step(mpaso_state s, double dt, int32_t nsteps);
/* Same, replayed from a CUDA graph of one step (captured on first use for dt). */
int mpaso_rk4_step_graph(mpaso_state s, double dt, int32_t nsteps);
/* One call through the boundary with host buffers: copy in, nsteps, copy out.
 * Mapped page-locked buffers are read and written in place by the exchange's
 * kernels (one pass per field each way); other buffers are staged. */
int mpaso_rk4_step_host(mpaso_state s, double dt, int32_t nsteps, double *h, double *u,
                        double *tracers);
/* The same exchange queued on the state's stream without waiting for it
 * (page-locked buffers only): calls run in order, each copying in what the
 * previous one copied out, so a time loop of these keeps the GPU busy while
 * the host returns at once.  The buffers must not be touched until
 * mpaso_state_sync returns. */
int mpaso_rk4_step_host_async(mpaso_state s, double dt, int32_t nsteps, double *h, double *u,
                              double *tracers);
int mpaso_state_sync(mpaso_state s);
/* History output without stalling the time loop (the reference writes each
 * output step synchronously: the field_output_wrapper task of apps/sw/run.cc:10
 * via write_timestep, mpasoflecsi/io/helpers.hh:127-151): enqueues a copy of `field`
 * as it stands after the work already queued on the state's stream into
 * host memory `data` (reference numbering) and returns at once.  A side
 * stream permutes the field into one of two device buffers used in turn and
 * copies it out; later steps wait only for the permutation, not for the copy.
 * `data` should be page-locked for the copy to be asynchronous, and must not
 * be read before mpaso_state_snapshot_wait returns.  No counterpart in the
 * reference's task interface. */
int mpaso_state_snapshot(mpaso_state s, int32_t field, double *data);
int mpaso_state_snapshot_wait(mpaso_state s);
int mpaso_state_stream(mpaso_state s, void **stream);
/* Per-kernel timing: runs nsteps steps (not from a graph) with CUDA events
 * around every launch on the state's stream and returns, for each of the
 * *nkinds kernel kinds of a stage (at most 8), the mean duration of one
 * launch in ms.  names (optional) receives a ','-separated list of kinds. */
int mpaso_state_profile(mpaso_state s, double dt, int32_t nsteps, double *ms_per_launch,
                        int32_t *nkinds, char *names, int32_t names_len);
/* Kernel launches issued per RK4 step by mpaso_rk4_step. */
int mpaso_state_launches_per_step(mpaso_state s, int32_t *n);
int mpaso_state_device_bytes(mpaso_state s, int64_t *bytes);

/* Launch configuration of the kernels of an RK stage, as 12 ints:
 * config[0..2] = 1 where the kernel's stencil loop is unrolled at compile
 * time (only meaningful where the mesh's widest stencil is 10: the sphere),
 * config[3..5] = threads per block (64, 128 or 256), config[6..8] = 1 where
 * the kernel runs with registers capped at 40 per thread (1536 threads per
 * SM; sw app with at most 1 tracer; otherwise ignored), config[9] = static
 * array kept resident in the L2 cache's persisting portion (sw app): 0 none,
 * 1 the FCT advection coefficients, 2 the TRiSK weights; config[10] = 1
 * when consecutive stage kernels use programmatic dependent launch (a kernel
 * is scheduled while its predecessor drains and waits for it in hardware; sw
 * app); config[11] = 1 for the four-launch schedule of the sw app with
 * tracers (the tracer fluxes move from the first kernel into the edge threads
 * of the second, the limiter into a kernel of its own).  Results do not
 * depend on the threads per block, the L2 choice, the launch overlap or the
 * schedule; the other variants may
 * differ in the last bits.  No counterpart in the reference (its tasks have
 * no device launch shape).  Setting it drops any captured step graph; a
 * persisting L2 reservation is per device context, so at most one state per
 * device should use config[9] != 0, and destroying it releases the
 * reservation. */
int mpaso_state_launch_config(mpaso_state s, int32_t *config);
int mpaso_state_set_launch_config(mpaso_state s, const int32_t *config);
/* The same with n >= 12 ints, the 13th being the threads per edge-level of
 * the TRiSK loop in the second stage kernel (sw app, at most one tracer): 1,
 * 2 or 4 lanes share an edge's stencil and add their partial sums by warp
 * shuffles (results differ in the last bits).  Entries past 13 read as
 * nothing and are written as 0.  The autotuner times the lane counts with
 * the second kernel's other variants; the 12-int calls leave it as it is. */
int mpaso_state_launch_config_ex(mpaso_state s, int32_t *config, int32_t n);
int mpaso_state_set_launch_config_ex(mpaso_state s, const int32_t *config, int32_t n);
/* Per-mesh autotuner: for each stage kernel in turn, times every variant
 * (unrolled or not x capped or not x 64/128/256 threads, and for the second
 * kernel of the sw app 1, 2 or 4 threads per edge-level) over nsteps steps
 * of size dt and keeps the fastest, then picks the L2 residency choice on
 * the whole stage, the schedule on the whole stage and the launch overlap on
 * uninterrupted steps.  The prognostic state is saved first and restored on
 * return, so the call leaves (h, u, tracers) unchanged; it allocates one
 * temporary copy of them.  config (may be NULL) receives the chosen
 * configuration (12 ints).  Call it outside stream capture. */
int mpaso_state_autotune(mpaso_state s, double dt, int32_t nsteps, int32_t *config);

/* Adjoint of the RK4 step.  No counterpart in the reference, which has no
 * adjoint: these differentiate what mpaso_rk4_step computes for app =
 * MPASO_APP_SW (apps/sw/run.cc:10-60) with pin_u = 0, and, through
 * mpaso_rk4_vjp_tracers, the tracers of app = MPASO_APP_OCEAN
 * (apps/ocean/run.cc:10-50), whose thickness and velocity are prescribed
 * inputs: there gh / gu may be NULL and gh0 / gu0 (when given) receive zeros.
 *
 * mpaso_rk4_forward: advances the state nsteps steps of size dt like
 * mpaso_rk4_step, keeping a checkpoint of (h, u, tracers) every ckpt_every
 * steps.  ckpt_every = 0 stores the whole window instead (every stage state
 * and the intermediates the reverse sweep reads, 4 nsteps + 1 tape slots),
 * so the vjp recomputes nothing: HBM for time, where the window fits.
 * mpaso_rk4_vjp: given the cotangents gh (nCells x nlev) and gu (nEdges x
 * nlev) of the state after the forward run, writes dJ/dh0 and dJ/du0 of the
 * state before it into gh0 / gu0 (reference ordering; host or device
 * pointers).  (h, u) do not depend on the tracers, so this reverse leaves
 * them out.  Stage states are recomputed segment by segment from the
 * checkpoints.
 * mpaso_rk4_vjp_tracers: the same with the tracers: gtr / gtr0 are the
 * cotangents of the final / initial tracer concentrations (nCells x nlev x
 * ntr), and gh0 includes what h contributes through the tracer transport.
 * With fct = 1 the FCT limiter (apps/ocean/tasks/solve.cc:169-326) is
 * differentiated on the branch its forward evaluation takes (each max, min,
 * clamp and sign as evaluated, ties to the reference's first argument);
 * hmix del2 mixing and the centred flux of fct = 0 are linear in the
 * tracers.
 * Device memory: ceil(N / ckpt_every) + 4 ckpt_every + 2 copies of (h, u),
 * 4 ckpt_every + 1 copies of two vertex fields (the taped pv and
 * kite-summed thickness), and about 20 work arrays of one level-field each;
 * with tracers also ceil(N / ckpt_every) + 4 ckpt_every + 1 copies of the
 * tracers, 4 ckpt_every copies of two edge-tracer fields (fluxes A, LO) and
 * of the two limiter factors, and about 15 work arrays of one level-tracer
 * field.  On meshes under 2^20 cell-levels with two segments or more, the
 * 4 ckpt_every (+ 1) taped copies are held twice: the reverse sweep
 * recomputes the next segment into the second set while it reverses the
 * current one (same gradient, bit for bit). */
int mpaso_rk4_forward(mpaso_state s, double dt, int32_t nsteps, int32_t ckpt_every);
int mpaso_rk4_vjp(mpaso_state s, const double *gh, const double *gu, double *gh0, double *gu0);
int mpaso_rk4_vjp_tracers(mpaso_state s, const double *gh, const double *gu, const double *gtr,
                          double *gh0, double *gu0, double *gtr0);
int mpaso_adjoint_device_bytes(mpaso_state s, int64_t *bytes);

/* nsteps RK4 steps of an sw state (any context, ensembles included; up to
 * 3 tracers) in ONE persistent cooperative launch: a grid the SMs hold at
 * once loops over the steps, stages and the three phases of each stage, with
 * a grid barrier between phases.  No counterpart in the reference.  Every
 * barrier wait is bounded: after `spin_limit` polls (0: 2^26, seconds) it
 * gives up and the call returns MPASO_ERR_TIMEOUT, the state then partly
 * advanced.  `extra_arrivals` must be 0 in use; a positive value makes every
 * wait expect arrivals that never come, which exercises that bound.  Same
 * results as mpaso_rk4_step_graph. */
int mpaso_rk4_step_persistent(mpaso_state s, double dt, int32_t nsteps, int64_t spin_limit,
                              int32_t extra_arrivals);

/* ------------------------------------------------------------------------
 * Test cases on the device.  The reference sets up its test cases and
 * computes their error norms as host tasks: apps/sw/tasks/testcase.cc:37-227
 * (Williamson cases 1, 5, 6) with compute_error (apps/sw/tasks/solve.cc:404-436),
 * and apps/ocean/tasks/testcase.cc:96-294 (cases 1-3, calc_error_case_1/2/3).
 * These entries do the same on a state's device fields.  The geometry they
 * read is given once per mesh context, in reference numbering (host or
 * device arrays; for an ensemble context, the members' arrays concatenated). */
typedef struct {
  const double *latCell, *lonCell;     /* [nCells] */
  const double *latVertex, *lonVertex; /* [nVertices] */
  const double *latEdge, *lonEdge, *angleEdge; /* [nEdges] */
  const double *xCell, *yCell, *zCell; /* [nCells] */
} mpaso_geometry;
int mpaso_mesh_set_geometry(mpaso_mesh m, const mpaso_geometry *g);

/* Writes the test case's initial h, u and tracers into the state (every
 * level gets the reference's level-0 fields; tracers the case does not set
 * are zero).  sw state: cases 1, 5, 6 (case 5 also sets the state's bottom
 * topography, the mountain); ocean state: cases 1, 2, 3 (h = 1,
 * layerThicknessEdge = 1; `coef` is case 3's del2 coefficient). */
int mpaso_state_setup_case(mpaso_state s, int32_t test_case, double coef);
/* Error norms of the state against the case's analytic solution after
 * `elapsed` seconds, level 0 and tracer 0: err[0] = the reference's norm
 * (sw case 1: the normalised l2 error of h; ocean: sqrt(sum err^2) / nCells of
 * the pointwise relative error), err[1] = the largest pointwise relative
 * error. */
int mpaso_state_case_error(mpaso_state s, int32_t test_case, double elapsed, double coef, double *err);

/* Device / runtime queries (no GPU needed: report 0 devices). */
int mpaso_device_count(int32_t *n);
const char *mpaso_build_info(void);

#ifdef __cplusplus
}
#endif
#endif

// Fused RK4 path: state context, stage parameters and the FCT / del2 device
// code shared by the sw driver (rk4.cu) and the ocean tracer driver (ocean.cu).
#pragma once

#include <vector>

#include "device.cuh"
#include "task_io.cuh"

namespace mpaso {

constexpr long long kSignBit = (long long)0x8000000000000000ULL;

// Fast FP64 reciprocal: hardware approximation (rcp.approx.ftz.f64) refined
// by two Newton-Raphson steps r <- r + r (1 - b r); within a few ulp of 1/b
// for normal b.
__device__ __forceinline__ double rcp_nr(double b) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(b));
  double e = fma(-b, r, 1.0);
  r = fma(r, e, r);
  e = fma(-b, r, 1.0);
  return fma(r, e, r);
}

__device__ __forceinline__ long long sign_mask(double s) { return dbits(s) & kSignBit; }

// Load of a value an earlier kernel wrote: through the read-only
// (non-coherent) path when RO, else a plain load -- inside the persistent
// kernel, where an earlier phase of the same launch wrote it.
template <bool RO, class V> __device__ __forceinline__ V ld_in(const V *p) {
  if constexpr (RO)
    return __ldg(p);
  else
    return *p;
}

// Programmatic dependent launch: a kernel launched with the
// programmatic-serialization attribute may be scheduled while its
// predecessor's last blocks still run; it waits here (a hardware dependency,
// no polling) until the predecessor has completed and its writes are
// visible, then lets its own successor start launching.  Without the
// attribute both instructions return at once.  Every kernel launched with
// the attribute starts with this, before touching memory.
__device__ __forceinline__ void stage_prologue() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launch with programmatic dependent launch when `pdl` (the attribute travels
// into captured graphs).
template <class... K, class... A>
void launch_pdl(void (*kern)(K...), int64_t n, int threads, bool pdl, cudaStream_t st, A... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks_for(n, threads));
  cfg.blockDim = dim3(threads);
  cfg.stream = st;
  cudaLaunchAttribute at;
  at.id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at.val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = pdl ? &at : nullptr;
  cfg.numAttrs = pdl ? 1 : 0;
  MPASO_CUDA(cudaLaunchKernelEx(&cfg, kern, args...));
}

// Timing mark after a stage kernel (SwState::prof_events): an event node of
// the step graph being captured for the per-kernel profile.
inline void prof_mark(cudaEvent_t ev, cudaStream_t st) {
  MPASO_CUDA(cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal));
}

// Per-state derived statics (device arrays), built once at state creation.
// The sw kernels carry the doubled thickness flux F2 = u (h1 + h2) = 2 F and
// the doubled edge PV Pv = pv_a + pv_b = 2 pv_e; the power-of-two factors are
// folded into the scaled copies below, which changes no rounding.
struct DStat {
  const double *sdv;   // [maxEoC][nC] edgeSignOnCell * dvEdge (0 in pad slots)
  const double *sdvi;  // [maxEoC][nC] 0.5 * edgeSignOnCell * dvEdge / areaCell (tend_h from F2)
  const double *kw;    // [nE] 0.25 * dcEdge * dvEdge
  const double *sdc;   // [3][nV] circulation sign * dcEdge
  const double *dhs;   // [nE] bottomDepth(c2) - bottomDepth(c1)
  const double *kd;    // [nE] meshScalingDel2 * kappa * dvEdge / dcEdge
  const double *kdh;   // [nE] kd / 2 (del2 flux from h1 + h2)
  const double *dvh;   // [nE] dvEdge / 2 (fluxes from F2)
  const double *woe8;  // [maxEoE][nE] weightsOnEdge / 8 (PV flux from F2, Pv)
  // [maxAdv][nE] pairs {advCoef + 0.25 advCoef_3rd, advCoef - 0.25 advCoef_3rd}, halved
  // (cpm2, sw kernels) or not (cpm1, ocean kernels); one 16-byte load per slot, the
  // flux sign picks the member.
  const double2 *cpm2, *cpm1;
  const double *nuInva;  // [nC] nu / areaCell
  const double *nuDv;    // [nE] nu / dvEdge
};

// One RK stage's pointers and weights.
struct Stage {
  int stage;            // 0..3
  double w_sub, w_acc;  // substep and accumulation weights (apps/sw/run.cc:23-24)
  double dt, g, nu;
  int fct, hmix, visc, pin_u;
  int centred;          // without FCT: the sw app's centred tracer flux (1) or no advection (0, ocean)
  const double *u_in, *h_in, *tr_in;        // stage input
  const double *u_prev, *h_prev, *tr_prev;  // step start
  double *u_out, *h_out, *tr_out;           // next stage input (stages 0..2)
  double *u_acc, *h_acc, *trh_acc;          // RK accumulators
  double *u_new, *h_new, *tr_new;           // step result (stage 3)
  double *pv, *vort, *bern;                 // diagnostics of the stage input (bern: ke - nu div)
  double *F;                                // ocean: thickness flux u h_e
  double2 *FG;                              // sw: {F2, F2 Pv} per edge, gathered together
  double *pve, *A, *LO, *DF;                // edge intermediates
  double2 *R2;                              // {R+, R-} limiter factors per cell and tracer
  double *tLO;                              // cell intermediates
  const double *hE, *hpi;                   // ocean: layerThicknessEdge, 1/hProv
  double *tape_pv, *tape_hs;                // adjoint taping: pv and kite-summed h of the next state
  double *tape_hpi;                         // adjoint taping: 1/hProv of the stage (FCT)
  double *tape_s1;                          // adjoint taping: sum_j W_j F2_j / 8 of each edge
  double *hpw;                              // sw four-launch schedule: 1/hProv from K2 to the limiter
};

// Buffers and step parameters a captured host-exchange graph was built for.
struct XKey {
  const void *h = nullptr, *u = nullptr, *tr = nullptr;
  double dt = 0.0;
  int nsteps = -1;
  bool operator==(const XKey &o) const {
    return h == o.h && u == o.u && tr == o.tr && dt == o.dt && nsteps == o.nsteps;
  }
};

// State context (sw or ocean app).
struct SwState {
  mpaso_mesh mesh = nullptr;
  mpaso_params p{};
  int L = 1, T = 0;
  cudaStream_t stream = nullptr;
  void *arena = nullptr;
  size_t arena_bytes = 0;
  double *U[4]{}, *H[4]{}, *TR0 = nullptr, *TRA = nullptr, *TRB = nullptr, *TRH = nullptr;
  double *HE = nullptr, *HPI = nullptr;
  double *pv = nullptr, *vort = nullptr, *bern = nullptr;
  double *F = nullptr, *pve = nullptr, *A = nullptr, *LO = nullptr, *DF = nullptr;
  double2 *FG = nullptr, *R2 = nullptr;
  double *tLO = nullptr;
  DStat st{};
  bool diag_valid = false;  // sw: diagnostics of U[0]/H[0] current
  double prep_dt = 0.0;     // ocean: dt of the cached F / 1/hProv (0 = stale)
  cudaGraphExec_t graph = nullptr;
  double graph_dt = 0.0;
  // device staging of mpaso_rk4_step_host (reference-ordered h, u, tracers)
  double *io_stage = nullptr;
  size_t io_bytes = 0;
  // mpaso_rk4_step_host with page-locked buffers: the captured exchange graph,
  // a DAG over the state stream and two side streams (one per field) so each
  // field's copy and permutation overlap the others'
  cudaGraphExec_t xg = nullptr;
  XKey xkey{};
  cudaStream_t x_side[2] = {nullptr, nullptr};
  cudaEvent_t x_ev[7] = {};
  // when set, recorded on the stage stream right after the tendency kernel of
  // each stage launched (h and u of that stage's output are final there)
  cudaEvent_t k2_mark = nullptr;
  // history output (mpaso_state_snapshot): side stream, two staging buffers
  // used in turn, events ordering them against the stepping stream
  cudaStream_t out_stream = nullptr;
  double *out_buf[2] = {nullptr, nullptr};
  size_t out_bytes = 0;
  int out_next = 0;
  cudaEvent_t out_ready = nullptr, out_read[2] = {nullptr, nullptr}, out_done[2] = {nullptr, nullptr};
  // per-launch timing: event nodes recorded after every kernel of a stage
  // while the profiled step graph is captured (time_stage_kernels)
  cudaEvent_t *prof_events = nullptr;
  // adjoint buffers (checkpoints, stage tape, cotangents); see adjoint.cu
  struct AdjBuffers *adj = nullptr;
  // launch configuration of the three stage kernels (autotuned): stencil
  // unrolled at compile time (1) or runtime width (0), threads per block, and
  // registers capped for full occupancy (1) or not (0)
  int tune_unroll[3] = {1, 1, 1};
  int tune_tpb[3] = {256, 256, 256};
  int tune_occ[3] = {0, 0, 0};
  // L2 residency of one static array across the step: 0 none, 1 the advection
  // coefficient pairs (read by K1), 2 the TRiSK weights (read by K2); the
  // window is attached to that kernel's launches (see set_l2_window)
  int tune_l2 = 0;
  cudaAccessPolicyWindow l2win{};
  // stage kernels launched with programmatic dependent launch (sw app; off
  // unless the autotuner measures it faster)
  int tune_pdl = 0;
  // sw with tracers: four launches per stage (tracer fluxes in K2's edge
  // threads, limiter in its own kernel) instead of three
  int tune_split = 0;
  double *HPW = nullptr;
  // threads per edge-level of the TRiSK loop in the second stage kernel (sw
  // app, at most one tracer): 1, 2 or 4
  int tune_lanes = 1;
  // grid barrier of the persistent step: arrival count, error flag
  unsigned int *pbar = nullptr;
  // small device buffer of the test-case set-up and error norms (testcases.cu)
  double *aux = nullptr;
  size_t aux_bytes = 0;
  ~SwState();
};

// Allocates the state buffers listed as (pointer, doubles) in one arena.
void alloc_arena(SwState &s, std::vector<std::pair<double **, int64_t>> &bufs);
void build_stat(SwState &s);
void stat_buffers(SwState &s, std::vector<std::pair<double **, int64_t>> &bufs);
void free_adjoint(SwState &s);
void sw_stage_ptrs(SwState &s, int rk, double dt, const double *u_in, const double *h_in,
                   const double *u_prev, const double *h_prev, double *u_out, double *h_out,
                   double *u_acc, double *h_acc, double *u_new, double *h_new, double *tape_pv,
                   double *tape_hs, double *tape_s1, cudaStream_t st);
void sw_diag_ptrs(SwState &s, const double *u, const double *h, double *tape_pv, double *tape_hs,
                  cudaStream_t st);
void sw_steps_pub(SwState &s, double dt, int nsteps, cudaStream_t st);
// nsteps graph-replayed steps on the state's stream (the step graph is cached)
void sw_steps_graph(SwState &s, double dt, int nsteps);
Stage sw_make_stage(SwState &s, int rk, double dt);
void sw_launch_stage(SwState &s, const Stage &S, cudaStream_t st);
Stage ocean_make_stage(SwState &s, int rk, double dt);
void ocean_launch_stage(SwState &s, const Stage &S, cudaStream_t st);
void ocean_recompute(SwState &s, double dt, cudaStream_t st);
void ocean_prepare(SwState &s, double dt, cudaStream_t st);
void drop_adjoint_graph(SwState &s);

// ---------------------------------------------------------------------------
// FCT / del2 tracer device code (apps/ocean/tasks/solve.cc:99-366).

// Edge fluxes for tracers of the stage input: low-order flux LO, anti-
// diffusive flux A = HO - LO, del2 flux DF = h_e (tr2 - tr1) kappa ...
// The thickness flux arrives as F = s * u h_e (s = 1 or 2) and the edge
// thickness as hx = s * h_e; dv, cp, cm, kd are the matching 1/s copies.
// NA > 0: compile-time advection-stencil width (the mesh's maxAdv); 0 = runtime.
template <int T, int NA, bool RO = true>
__device__ __forceinline__ void edge_tracer_fluxes(const DMesh &m, const Stage &S, int L, int e, int k,
                                                   int64_t i, int64_t i1, int64_t i2, double F,
                                                   double hx, const double *dv, const double2 *cpm,
                                                   const double *kd) {
  double t1[T], t2[T];
#pragma unroll
  for (int t = 0; t < T; ++t) t1[t] = ld_in<RO>(&S.tr_in[i1 * T + t]), t2[t] = ld_in<RO>(&S.tr_in[i2 * T + t]);
  const double dvF = __ldcs(&dv[e]) * F;
  if (S.fct) {
    // low order: dv (max(0,F) tr1 + min(0,F) tr2) == dv F tr_upwind (ocean solve.cc:110-113)
    const bool up1 = dgt0(F);
    // high order: F mask sum_a tr_a (advCoef_a + 0.25 advCoef_3rd_a sign(F)) (solve.cc:137-165)
    const bool neg = dlt0(F);
    double s[T];
#pragma unroll
    for (int t = 0; t < T; ++t) s[t] = 0.0;
    const int na = NA > 0 ? NA : m.maxAdv;
#pragma unroll
    for (int a = 0; a < na; ++a) {
      const int cell = __ldcs(&m.advCells[(int64_t)a * m.nE + e]);
      const double2 c2 = __ldcs(&cpm[(int64_t)a * m.nE + e]);
      const double cf = neg ? c2.y : c2.x;
      const double *tr = S.tr_in + ((int64_t)cell * L + k) * T;
#pragma unroll
      for (int t = 0; t < T; ++t) s[t] = fma(cf, ld_in<RO>(&tr[t]), s[t]);
    }
    const int mask = __ldcs(&m.hoMask[(int64_t)e * m.fctLev + k]);
    // A = HO - LO, HO = F s; edges without the high-order mask take the centred
    // flux (solve.cc:222-225).  A branch, not a select: the mask is set almost
    // everywhere, and the centred flux would cost three more FP64 instructions
    if (mask) {
#pragma unroll
      for (int t = 0; t < T; ++t) {
        const double lo = dvF * (up1 ? t1[t] : t2[t]);
        S.LO[i * T + t] = lo;
        S.A[i * T + t] = fma(F, s[t], -lo);
      }
    } else {
#pragma unroll
      for (int t = 0; t < T; ++t) {
        const double lo = dvF * (up1 ? t1[t] : t2[t]);
        S.LO[i * T + t] = lo;
        S.A[i * T + t] = fma(0.5 * dvF, t1[t] + t2[t], -lo);
      }
    }
  } else if (S.centred) {
    // centred flux of compute_scalar_tend (apps/sw/tasks/solve.cc:255-269)
#pragma unroll
    for (int t = 0; t < T; ++t) S.LO[i * T + t] = (0.5 * dvF) * (t1[t] + t2[t]);
  } else {
    // the ocean app advects tracers only through FCT (apps/ocean/run.cc:20-38)
#pragma unroll
    for (int t = 0; t < T; ++t) S.LO[i * T + t] = 0.0;
  }
  if (S.hmix) {
    const double hk = hx * __ldcs(&kd[e]);
#pragma unroll
    for (int t = 0; t < T; ++t) S.DF[i * T + t] = hk * (t2[t] - t1[t]);
  }
}

// Loop over the edge slots of a cell.  NC > 0 unrolls NC slots at compile
// time so every slot's loads issue together: pad slots repeat valid indices
// (own cell, slot-0 edge, zero weights) and `valid` masks what they would
// add.  NC = 0 loops to the cell's own edge count.  With every real slot
// valid, both forms add the same terms in the same order.
template <int NC, class Body>
__device__ __forceinline__ void for_slots(int n, Body &&body) {
  if constexpr (NC > 0) {
#pragma unroll
    for (int j = 0; j < NC; ++j) body(j, j < n);
  } else {
    for (int j = 0; j < n; ++j) body(j, true);
  }
}

// v in a real slot, +0 in a pad slot (a select on the integer pipe)
__device__ __forceinline__ double dmask(double v, bool valid) { return valid ? v : 0.0; }

// Cell bounds, upwind tendency and limiter factors R+ / R- (ocean solve.cc:194-267).
template <int T, int NC>
__device__ __forceinline__ void cell_limiter(const DMesh &m, const Stage &S, int L, int c, int k,
                                             int64_t i, double hin, double hpi) {
  const int n = m.nEoC[c];
  double tl[T];
#pragma unroll
  for (int t = 0; t < T; ++t) tl[t] = 0.0;
  if (!S.fct) {
    for_slots<NC>(n, [&](int j, bool ok) {
      const int64_t s = (int64_t)j * m.nC + c;
      const int64_t ie0 = ((int64_t)m.eoc[s] * L + k) * T;
      const long long sm = sign_mask(m.eocSign[s]);
#pragma unroll
      for (int t = 0; t < T; ++t) tl[t] += dmask(dflip(S.LO[ie0 + t], sm), ok);
    });
#pragma unroll
    for (int t = 0; t < T; ++t) S.tLO[i * T + t] = tl[t];  // area-weighted; divided by the area later
    return;
  }
  double trc[T], mx[T], mn[T], fi[T], fo[T];
#pragma unroll
  for (int t = 0; t < T; ++t) {
    trc[t] = S.tr_in[i * T + t];
    mx[t] = trc[t], mn[t] = trc[t], fi[t] = 0.0, fo[t] = 0.0;
  }
  for_slots<NC>(n, [&](int j, bool ok) {
    const int64_t s = (int64_t)j * m.nC + c;
    const int64_t in0 = ((int64_t)m.coc[s] * L + k) * T;  // pads: the cell itself
    const int64_t ie0 = ((int64_t)m.eoc[s] * L + k) * T;
    const long long sm = sign_mask(m.eocSign[s]);
#pragma unroll
    for (int t = 0; t < T; ++t) {
      const double x = S.tr_in[in0 + t];
      mx[t] = dmax(mx[t], x);
      mn[t] = dmin(mn[t], x);
      tl[t] += dmask(dflip(S.LO[ie0 + t], sm), ok);
      // flxIn gets the positive signed fluxes, flxOut the others: one add into
      // the accumulator the sign selects (integer-pipe select, same sums)
      const double ax = dmask(dflip(S.A[ie0 + t], sm), ok);
      const bool in = dgt0(ax);
      const double acc = (in ? fi[t] : fo[t]) + ax;
      fi[t] = in ? acc : fi[t];
      fo[t] = in ? fo[t] : acc;
    }
  });
  const double dtia = S.dt * m.invAreaCell[c];  // dt / area
  const double dthi = dtia * hpi;               // dt / (area hProv)
  const double eps = 1.e-10;
#pragma unroll
  for (int t = 0; t < T; ++t) {
    // trUp = (tr h + dt tend) / hProv; trMaxNew - trUp = dt flxIn / hProv, with
    // tend, flxIn, flxOut the area-weighted sums tl, fi, fo divided by the area
    const double up = fma(dtia, tl[t], trc[t] * hin) * hpi;
    const double np = mx[t] - up, dp = fma(dthi, fi[t], eps);
    const double nm = up - mn[t], dm = fma(-dthi, fo[t], eps);
    // clamp01(n / d): 0 when n <= 0, 1 when n >= d, the quotient otherwise
    double rp = dgt0(np) ? 1.0 : 0.0, rm = dgt0(nm) ? 1.0 : 0.0;
    if (dgt0(np) && dkey(np) < dkey(dp)) rp = dclamp01(np * rcp_nr(dp));
    if (dgt0(nm) && dkey(nm) < dkey(dm)) rm = dclamp01(nm * rcp_nr(dm));
    S.R2[i * T + t] = make_double2(rp, rm);
    S.tLO[i * T + t] = tl[t];
  }
}

// Tracer tendency of a cell: upwind part + limited anti-diffusive fluxes
// (ocean solve.cc:269-326) - del2 mixing (solve.cc:340-364).  One pass over
// the cell's edges for all tracers; the limiter factors of the cell across
// each edge come from one 16-byte gather.  With (c1, c2) = cells(e), the
// reference limits A by min(R-(c1), R+(c2)) for A > 0 and min(R+(c1), R-(c2))
// otherwise, i.e. by min(R- upstream, R+ downstream).
struct NoEdgeHook {
  __device__ void operator()(int64_t, int, bool) const {}
};

// `hook(slot, edge, valid)` runs once per edge slot of the cell inside the
// same loop (the sw driver folds the next state's cell diagnostics into it).
template <int T, int NC, class Hook = NoEdgeHook>
__device__ __forceinline__ void cell_tracer_tend(const DMesh &m, const Stage &S, int L, int c, int k,
                                                 int64_t i, double *tend, Hook &&hook = Hook()) {
  const int n = m.nEoC[c];
  double2 own[T];
#pragma unroll
  for (int t = 0; t < T; ++t) {
    tend[t] = S.tLO[i * T + t];  // area-weighted upwind part
    if (S.fct) own[t] = S.R2[i * T + t];
  }
  for_slots<NC>(n, [&](int j, bool ok) {
    const int64_t s = (int64_t)j * m.nC + c;
    const int e = m.eoc[s];
    hook(s, e, ok);
    const long long sm = sign_mask(m.eocSign[s]);
    const int nb = m.nbr[s];
    const bool own_first = nb & 1;
    const int64_t ie0 = ((int64_t)e * L + k) * T, jn = ((int64_t)(nb >> 1) * L + k) * T;
#pragma unroll
    for (int t = 0; t < T; ++t) {
      double x = 0.0;
      if (S.fct) {
        const double a = S.A[ie0 + t];
        const double2 o = S.R2[jn + t];
        const double r = dgt0(a) == own_first ? dmin(own[t].y, o.x) : dmin(o.y, own[t].x);
        x = S.hmix ? fma(a, r, -S.DF[ie0 + t]) : a * r;  // limited flux - del2 flux in one FMA
      } else if (S.hmix) {
        x = -S.DF[ie0 + t];
      }
      tend[t] += dmask(dflip(x, sm), ok);
    }
  });
  const double inva = m.invAreaCell[c];
#pragma unroll
  for (int t = 0; t < T; ++t) tend[t] *= inva;
}

}  // namespace mpaso

struct mpaso_state_s {
  mpaso::SwState s;
};

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

// Per-state derived statics (device arrays), built once at state creation.
// The sw kernels carry the doubled thickness flux F2 = u (h1 + h2) = 2 F and
// the doubled edge PV Pv = pv_a + pv_b = 2 pv_e; the power-of-two factors are
// folded into the scaled copies below, which changes no rounding.
struct DStat {
  const double *sdv;   // [maxEoC][nC] edgeSignOnCell * dvEdge (0 in pad slots)
  const double *sdvi;  // [maxEoC][nC] 0.5 * edgeSignOnCell * dvEdge / areaCell (tend_h from F2)
  const double *kw;    // [nE] 0.25 * dcEdge * dvEdge
  const double *sdc;   // [3][nV] circulation sign * dcEdge
  const double *gbd;   // [nC] gravity * bottomDepth
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
  const double *u_in, *h_in, *tr_in;        // stage input
  const double *u_prev, *h_prev, *tr_prev;  // step start
  double *u_out, *h_out, *tr_out;           // next stage input (stages 0..2)
  double *u_acc, *h_acc, *trh_acc;          // RK accumulators
  double *u_new, *h_new, *tr_new;           // step result (stage 3)
  double *pv, *vort, *bern;                 // diagnostics of the stage input
  double *F, *G, *pve, *A, *LO, *DF;        // edge intermediates
  double *Rp, *Rm, *tLO;                    // cell intermediates
  const double *hE, *hpi;                   // ocean: layerThicknessEdge, 1/hProv
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
  double *F = nullptr, *G = nullptr, *pve = nullptr, *A = nullptr, *LO = nullptr, *DF = nullptr;
  double *Rp = nullptr, *Rm = nullptr, *tLO = nullptr;
  DStat st{};
  bool diag_valid = false;  // sw: diagnostics of U[0]/H[0] current
  double prep_dt = 0.0;     // ocean: dt of the cached F / 1/hProv (0 = stale)
  cudaGraphExec_t graph = nullptr;
  double graph_dt = 0.0;
  // optional per-launch timing: events recorded after every kernel of a stage
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
  ~SwState();
};

// Allocates the state buffers listed as (pointer, doubles) in one arena.
void alloc_arena(SwState &s, std::vector<std::pair<double **, int64_t>> &bufs);
void build_stat(SwState &s);
void stat_buffers(SwState &s, std::vector<std::pair<double **, int64_t>> &bufs);
void free_adjoint(SwState &s);
void sw_stage_ptrs(SwState &s, int rk, double dt, const double *u_in, const double *h_in,
                   const double *u_prev, const double *h_prev, double *u_out, double *h_out,
                   double *u_acc, double *h_acc, double *u_new, double *h_new, cudaStream_t st);
void sw_diag_ptrs(SwState &s, const double *u, const double *h, cudaStream_t st);
void sw_steps_pub(SwState &s, double dt, int nsteps, cudaStream_t st);

// ---------------------------------------------------------------------------
// FCT / del2 tracer device code (apps/ocean/tasks/solve.cc:99-366).

// Edge fluxes for tracers of the stage input: low-order flux LO, anti-
// diffusive flux A = HO - LO, del2 flux DF = h_e (tr2 - tr1) kappa ...
// The thickness flux arrives as F = s * u h_e (s = 1 or 2) and the edge
// thickness as hx = s * h_e; dv, cp, cm, kd are the matching 1/s copies.
// NA > 0: compile-time advection-stencil width (the mesh's maxAdv); 0 = runtime.
template <int T, int NA>
__device__ __forceinline__ void edge_tracer_fluxes(const DMesh &m, const Stage &S, int L, int e, int k,
                                                   int64_t i, int64_t i1, int64_t i2, double F,
                                                   double hx, const double *dv, const double2 *cpm,
                                                   const double *kd) {
  double t1[T], t2[T];
#pragma unroll
  for (int t = 0; t < T; ++t) t1[t] = S.tr_in[i1 * T + t], t2[t] = S.tr_in[i2 * T + t];
  const double dvF = dv[e] * F;
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
      const int cell = m.advCells[(int64_t)a * m.nE + e];
      const double2 c2 = cpm[(int64_t)a * m.nE + e];
      const double cf = neg ? c2.y : c2.x;
      const double *tr = S.tr_in + ((int64_t)cell * L + k) * T;
#pragma unroll
      for (int t = 0; t < T; ++t) s[t] = fma(cf, tr[t], s[t]);
    }
    const int mask = m.hoMask[(int64_t)e * m.fctLev + k];
    const double wgt = mask ? F : 0.0;
#pragma unroll
    for (int t = 0; t < T; ++t) {
      const double lo = dvF * (up1 ? t1[t] : t2[t]);
      double ho = wgt * s[t];
      if (!mask) ho = fma(0.5 * dvF, t1[t] + t2[t], ho);  // solve.cc:222-225
      S.LO[i * T + t] = lo;
      S.A[i * T + t] = ho - lo;
    }
  } else {
    // centred flux of compute_scalar_tend (apps/sw/tasks/solve.cc:255-269)
#pragma unroll
    for (int t = 0; t < T; ++t) S.LO[i * T + t] = (0.5 * dvF) * (t1[t] + t2[t]);
  }
  if (S.hmix) {
    const double hk = hx * kd[e];
#pragma unroll
    for (int t = 0; t < T; ++t) S.DF[i * T + t] = hk * (t2[t] - t1[t]);
  }
}

// Cell bounds, upwind tendency and limiter factors R+ / R- (ocean solve.cc:194-267).
template <int T>
__device__ __forceinline__ void cell_limiter(const DMesh &m, const Stage &S, int L, int c, int k,
                                             int64_t i, double hin, double hpi) {
  const int n = m.nEoC[c];
  const double inva = m.invAreaCell[c];
  if (!S.fct) {
#pragma unroll
    for (int t = 0; t < T; ++t) {
      double tl = 0.0;
      for (int j = 0; j < n; ++j) {
        const int e = m.eoc[(int64_t)j * m.nC + c];
        tl += dflip(S.LO[((int64_t)e * L + k) * T + t], sign_mask(m.eocSign[(int64_t)j * m.nC + c]));
      }
      S.tLO[i * T + t] = tl;  // area-weighted; cell_tracer_tend divides by the area
    }
    return;
  }
  const double dtia = S.dt * inva;  // dt / area
  const double dthi = dtia * hpi;   // dt / (area hProv)
  const double eps = 1.e-10;
#pragma unroll
  for (int t = 0; t < T; ++t) {
    const double trc = S.tr_in[i * T + t];
    double mx = trc, mn = trc, tl = 0.0, fi = 0.0, fo = 0.0;
    for (int j = 0; j < n; ++j) {
      const int nb = m.coc[(int64_t)j * m.nC + c];
      const double x = S.tr_in[((int64_t)nb * L + k) * T + t];
      mx = dmax(mx, x);
      mn = dmin(mn, x);
      const int e = m.eoc[(int64_t)j * m.nC + c];
      const long long sm = sign_mask(m.eocSign[(int64_t)j * m.nC + c]);
      const int64_t ie = ((int64_t)e * L + k) * T + t;
      tl += dflip(S.LO[ie], sm);
      const double ax = dflip(S.A[ie], sm);
      fi += dpos(ax);
      fo += dneg(ax);
    }
    // trUp = (tr h + dt tend) / hProv; trMaxNew - trUp = dt flxIn / hProv, with
    // tend, flxIn, flxOut the area-weighted sums tl, fi, fo divided by the area
    const double up = fma(dtia, tl, trc * hin) * hpi;
    const double np = mx - up, dp = fma(dthi, fi, eps);
    const double nm = up - mn, dm = fma(-dthi, fo, eps);
    // clamp01(n / d): 0 when n <= 0, 1 when n >= d, the quotient otherwise
    double rp = dgt0(np) ? 1.0 : 0.0, rm = dgt0(nm) ? 1.0 : 0.0;
    if (dgt0(np) && dkey(np) < dkey(dp)) rp = dclamp01(np * rcp_nr(dp));
    if (dgt0(nm) && dkey(nm) < dkey(dm)) rm = dclamp01(nm * rcp_nr(dm));
    S.Rp[i * T + t] = rp;
    S.Rm[i * T + t] = rm;
    S.tLO[i * T + t] = tl;
  }
}

// Tracer tendency of a cell: upwind part + limited anti-diffusive fluxes
// (ocean solve.cc:269-326) - del2 mixing (solve.cc:340-364).
template <int T>
__device__ __forceinline__ void cell_tracer_tend(const DMesh &m, const Stage &S, int L, int c,
                                                 int k, int64_t i, double *tend) {
  const int n = m.nEoC[c];
  const double inva = m.invAreaCell[c];
#pragma unroll
  for (int t = 0; t < T; ++t) {
    double acc = S.tLO[i * T + t];  // area-weighted upwind part
    for (int j = 0; j < n; ++j) {
      const int e = m.eoc[(int64_t)j * m.nC + c];
      const long long sm = sign_mask(m.eocSign[(int64_t)j * m.nC + c]);
      const int64_t ie = ((int64_t)e * L + k) * T + t;
      double x = 0.0;
      if (S.fct) {
        const int2 cc = m.coe[e];
        const int64_t j1 = ((int64_t)cc.x * L + k) * T + t, j2 = ((int64_t)cc.y * L + k) * T + t;
        const double a = S.A[ie];
        // max(0,A) min(R-(c1), R+(c2)) + min(0,A) min(R+(c1), R-(c2))  (solve.cc:276-279)
        const double r = dgt0(a) ? dmin(S.Rm[j1], S.Rp[j2]) : dmin(S.Rp[j1], S.Rm[j2]);
        x = a * r;
      }
      if (S.hmix) x -= S.DF[ie];
      acc += dflip(x, sm);
    }
    tend[t] = acc * inva;
  }
}

}  // namespace mpaso

struct mpaso_state_s {
  mpaso::SwState s;
};

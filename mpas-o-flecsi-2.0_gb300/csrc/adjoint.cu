// Hand-written adjoint (vector-Jacobian product) of the fused sw RK4 step for
// (h, u) and, optionally, the tracers (FCT advection + del2 mixing), with
// uniform checkpointing.
//
// Forward per stage (rk4.cu), in the quantities the adjoint needs:
//   circ_v = sum sdc u,  hs_v = sum kite h,  pv_v = (f A + circ) / hs
//   he_e = (h1 + h2)/2,  F_e = u he,  pve_e = (pv_a + pv_b)/2
//   tend_u_e = (pve_e S1_e + S2_e)/2 - invDc ((ke2 - ke1) + g (h2 - h1 + dhs))
//              + nu (invDc (div2 - div1) - invDv (vort_b - vort_a)),
//     S1_e = sum_j W_ej F_j,  S2_e = sum_j W_ej F_j pve_j   (apps/sw/tasks/solve.cc:215-233)
//   tend_h_c = inva sum sdv F                                (solve.cc:185-206)
//   ke_c = inva sum kw u^2,  div_c = -inva sum sdv u,  vort_v = circ / A
//
// Every scatter of the transposed operator becomes a gather over reverse
// connectivity: edgesOnEdge is symmetric (e' in eoe(e) <=> e in eoe(e')), so
// the transposed TRiSK stencil of e is its own stencil with the partner's
// weight (DMesh::woeT); thickness-to-vertex sums are gathered per cell through
// (vertex, kite) slots (DMesh::vocR/kiteR).  No atomics.
//
// RK4 reverse sweep for one step y -> y' = y + dt/6 (k1 + 2 k2 + 2 k3 + k4),
// given lam = dJ/dy':
//   mu4 = J4^T (dt/6 lam)
//   mu3 = J3^T (dt/3 lam + dt mu4)
//   mu2 = J2^T (dt/3 lam + dt/2 mu3)
//   mu1 = J1^T (dt/6 lam + dt/2 mu2)
//   dJ/dy = lam + mu1 + mu2 + mu3 + mu4,
// with J_s the Jacobian of the tendency at stage state s.  Stage states are
// recomputed segment by segment from checkpoints kept every `ckpt_every`
// steps and taped for the segment being reversed.
//
// Tracers.  The sw step is linear-RK in (u, h, q = h tr) (apps/sw/tasks/
// solve.cc:162, 300-302, 337, 354): stage inputs tr_s = q_s / h_s, the
// tracer tendency Tq(u_s, h_s, tr_s) feeds q like tend_h feeds h.  So the
// same RK recursion runs on (lam_q, acc_q, lk_q), and a stage adds
//   mu_q = (dTq/dtr)^T lk_q / h_s,
//   mu_h += (dTq/dh)^T lk_q - sum_t (dTq/dtr)^T lk_q tr_s / h_s,
//   mu_u += (dTq/du)^T lk_q,
// with (q, h) <-> (tr, h) converted only at the ends of the window.  The FCT
// limiter (apps/ocean/tasks/solve.cc:169-326) is differentiated on the branch
// its forward evaluation takes: every max / min / clamp / sign picks the
// argument the forward picked (ties as the reference's max / min: the first
// argument), and the derivative flows through that argument only.  The
// stage's fluxes A, LO and limiter factors R+/R- are taped by the recompute;
// bounds, provisional thickness and upwind values are recomputed.
#include <cstring>

#include "rk4.cuh"

namespace mpaso {

// One set of tape arrays (a segment's stage states and intermediates).
struct TapeSet {
  double *u, *h, *pv, *hs, *s1, *tr, *A, *LO, *tLO, *hpi;
  double2 *R2;
};

struct AdjBuffers {
  void *arena = nullptr;
  size_t bytes = 0;
  // two tape sets on meshes too small to fill the GPU: the reverse sweep
  // recomputes segment s - 1 into one on a side stream while it reverses
  // segment s from the other (`tape[1]` unused otherwise); the tp_* pointers
  // below are the set in use
  bool dbl = false;
  TapeSet tape[2] = {};
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_tape = nullptr, ev_rev = nullptr;
  int N = 0, k = 0, nck = 0, cap_ck = 0, cap_k = 0;
  double dt = 0.0;
  bool have_forward = false;
  double *ck_u = nullptr, *ck_h = nullptr;  // checkpoints [nck][nE L], [nck][nC L]
  double *tp_u = nullptr, *tp_h = nullptr;  // stage-state tape [4k + 1][...]
  double *uacc = nullptr, *hacc = nullptr;
  double *tp_pv = nullptr, *tp_hs = nullptr;  // pv, kite-summed h of every tape slot [4k + 1][nV L]
  double *tp_s1 = nullptr;  // the forward's TRiSK sum sum_j W_j F_j / 4 of every stage [4k][nE L]
  double *pve = nullptr;
  double2 *FP = nullptr;  // {F, P} per edge, gathered together by B1
  double *lam_u = nullptr, *lam_h = nullptr, *acc_u = nullptr, *acc_h = nullptr;
  double *lk_u = nullptr, *lk_h = nullptr, *mu_u = nullptr, *mu_h = nullptr;
  double *lhe = nullptr, *lpve = nullptr, *lke = nullptr, *ldiv = nullptr, *lcirc = nullptr, *lhs = nullptr;
  // tracers (allocated when the state has any): checkpoints and stage tape of
  // the concentrations, the stage fluxes and limiter factors, cotangents of
  // q = h tr, and the limiter adjoint's per-cell / per-edge intermediates
  double *ck_tr = nullptr, *tp_tr = nullptr;  // [nck][nC L T], [4k + 1][nC L T]
  double *tp_A = nullptr, *tp_LO = nullptr;   // [4k][nE L T]
  double2 *tp_R2 = nullptr;                   // [4k][nC L T] {R+, R-}
  double *tp_tLO = nullptr;                   // [4k][nC L T] area-weighted upwind sums
  double *tp_hpi = nullptr;                   // [4k][nC L] 1/hProv
  double *trhacc = nullptr;
  double *lam_q = nullptr, *acc_q = nullptr, *lk_q = nullptr, *gq = nullptr;
  double *ltl = nullptr, *ltrs = nullptr;
  double2 *lfio = nullptr, *lmm = nullptr;
  int2 *amm = nullptr;
  double *muh_t = nullptr, *lFt = nullptr, *lhet = nullptr;
  double2 *p12 = nullptr, *lho = nullptr;
  // the whole reverse sweep, captured once per (N, k, dt, tracers) and replayed
  cudaGraphExec_t rev = nullptr;
  int rev_N = 0, rev_k = 0, rev_tr = 0;
  bool rev_stored = false, rev_skip = false;
  // the checkpointing forward taped its last segment (tracers taped: last_tr);
  // the reverse sweep then starts without recomputing that segment
  bool last_taped = false;
  int last_tr = 0;
  double rev_dt = 0.0;
  int tr = 0;  // the sweep being run reverses the tracers too
  // ckpt_every = 0: the forward tapes the whole window (one segment), the
  // reverse sweep recomputes nothing; the taping forward is a captured graph
  bool stored = false, stored_tr = false;
  cudaGraphExec_t fwd = nullptr;
  int fwd_N = 0;
  double fwd_dt = 0.0;
};

void drop_adjoint_graph(SwState &s) {
  if (s.adj && s.adj->rev) {
    cudaGraphExecDestroy(s.adj->rev);
    s.adj->rev = nullptr;
  }
  if (s.adj && s.adj->fwd) {
    cudaGraphExecDestroy(s.adj->fwd);
    s.adj->fwd = nullptr;
  }
}

void free_adjoint(SwState &s) {
  if (s.adj) {
    drop_adjoint_graph(s);
    if (s.adj->arena) cudaFree(s.adj->arena);
    for (cudaEvent_t e : {s.adj->ev_fork, s.adj->ev_tape, s.adj->ev_rev})
      if (e) cudaEventDestroy(e);
    if (s.adj->side) cudaStreamDestroy(s.adj->side);
    delete s.adj;
    s.adj = nullptr;
  }
}

namespace {

constexpr int TPB = 256;

struct AdjArgs {
  const double *u, *h;                        // stage state
  const double *pv, *hs;                      // taped pv, kite-summed h of the stage state
  const double *s1;                           // taped TRiSK sum of the stage (sum W F / 4)
  double *pve;                                // edge pv of the stage state
  double2 *FP;                                // {F = u he, P = lk_u pve} per edge
  const double *un, *hn, *pvn;                // state of the next stage to reverse (prep)
  int prep;                                   // B3 prepares FP, pve of that stage
  double *lk_u, *lk_h;                        // cotangent of the stage tendency (in), next one (out)
  double *mu_u, *mu_h;                        // J^T lk
  double *lhe, *lpve, *lke, *ldiv, *lcirc, *lhs;
  double *lam_u, *lam_h, *acc_u, *acc_h;
  const double *lFt, *lhet, *muh_t;           // tracer terms (null without tracers)
  int rk, visc;
  double dt, g, nu;
};

// Tracer part of one stage's reverse (see the header).
struct TrArgs {
  const double *u, *h, *tr;        // stage input (tape)
  const double *A, *LO;            // stage fluxes (tape)
  const double2 *R2;               // stage limiter factors (tape)
  const double *hpi, *tLO;         // stage 1/hProv and upwind sum (tape; area-weighted unless ocean)
  const double *kd;                // del2 coefficient per edge
  double *lk_h;                    // thickness-tendency cotangent, + dt lambda_hProv in place
  double *lk_q, *gq, *lam_q, *acc_q;
  double *ltl, *ltrs;              // per cell and tracer: upwind-sum and own-tracer cotangents
  double2 *lfio, *lmm;             // {flxIn, flxOut} and {max, min} bound cotangents
  int2 *amm;                       // cells holding the {max, min} bound
  double *muh_t, *lFt, *lhet;
  double2 *p12, *lho;              // per edge and tracer: parts for cells(e); lambda_HO F by sign of F
  const double *Fx, *hEx;          // ocean: the prescribed thickness flux and edge thickness
  int T, rk, fct, hmix, ocean;     // ocean: tracers only, h / u prescribed, no q = h tr
  int centred;                     // without FCT: the sw app's centred flux (1) or no advection (0, ocean)
  double dt;
};

// Edge quantities of a stage state that B1 gathers: F = u he, pve from the taped
// vertex pv, and P = lk_u pve (lk_u: the stage tendency's cotangent).
__device__ __forceinline__ void prep_edge(const DMesh &m, const AdjArgs &a, int L, int e, int k, int64_t i,
                                          const double *u, const double *h, const double *pv, double lk) {
  const int2 c = m.coe[e];
  const int2 v = m.voe[e];
  const double he = 0.5 * (h[(int64_t)c.x * L + k] + h[(int64_t)c.y * L + k]);
  const double pve = 0.5 * (pv[(int64_t)v.x * L + k] + pv[(int64_t)v.y * L + k]);
  a.pve[i] = pve;
  a.FP[i] = make_double2(u[i] * he, lk * pve);
}

// PREP (edges): the above for the first stage reversed in a segment (later
// stages get it from the B3 before them).
__global__ void __launch_bounds__(TPB) k_adj_prep(DMesh m, AdjArgs a, int L) {
  stage_prologue();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nE * L) return;
  const int e = (int)(i / L), k = (int)(i - (int64_t)e * L);
  prep_edge(m, a, L, e, k, i, a.u, a.h, a.pv, a.lk_u[i]);
}

// B1 (edges): transposed PV flux, d tend_h / dF, chain through F = u he.
// NW = 10: the edgesOnEdge stencil unrolled at compile time (10-slot meshes).
// `tr`: the tracer part's thickness-flux and edge-thickness cotangents lFt,
// lhet of this edge (from TB) are added.
template <int NW>
__device__ __forceinline__ void b1_item(const DMesh &m, const AdjArgs &a, int L, int64_t i, bool tr, double lFt,
                                        double lhet) {
  const int e = (int)(i / L), k = (int)(i - (int64_t)e * L);
  // S1 = sum_j W_j F_j comes from the forward's tape (4 x its W/8 . 2F sum, exact)
  const double s1 = 4.0 * a.s1[i];
  double t1 = 0.0, t2 = 0.0;
  const int ne = NW > 0 ? NW : m.maxEoE;
#pragma unroll
  for (int j = 0; j < ne; ++j) {
    const int64_t s = (int64_t)j * m.nE + e;
    const int64_t io = (int64_t)m.eoe[s] * L + k;
    const double wt = m.woeT[s];
    t1 = fma(wt, a.lk_u[io], t1);
    t2 = fma(wt, a.FP[io].y, t2);
  }
  const int2 c = m.coe[e];
  const int64_t i1 = (int64_t)c.x * L + k, i2 = (int64_t)c.y * L + k;
  const double he = 0.5 * (a.h[i1] + a.h[i2]);
  const double Fe = a.FP[i].x, pve = a.pve[i], ue = a.u[i];
  const double dth = a.lk_h[i2] * m.invAreaCell[c.y] - a.lk_h[i1] * m.invAreaCell[c.x];
  double lF = fma(0.5, fma(pve, t1, t2), m.dvEdge[e] * dth);
  a.lpve[i] = 0.5 * fma(a.lk_u[i], s1, Fe * t1);
  if (tr) {
    lF += lFt;
    a.mu_u[i] = lF * he;
    a.lhe[i] = fma(lF, ue, lhet);
  } else {
    a.mu_u[i] = lF * he;
    a.lhe[i] = lF * ue;
  }
}

template <int NW>
__global__ void __launch_bounds__(TPB) k_adj_b1(DMesh m, AdjArgs a, int L) {
  stage_prologue();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nE * L) return;
  const bool tr = a.lFt != nullptr;
  b1_item<NW>(m, a, L, i, tr, tr ? a.lFt[i] : 0.0, tr ? a.lhet[i] : 0.0);
}

// B2 (cells + vertices): gradient terms, h_e -> h, pv -> (circ, hs).
// `muh`: the tracer part's thickness cotangent of this cell (0 without tracers).
__device__ __forceinline__ void b2_cell_item(const DMesh &m, const AdjArgs &a, int L, int64_t i, double muh) {
  {
    const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
    double G = 0.0, sl = 0.0;
    auto slot = [&](int j, bool ok) {
      const int64_t s = (int64_t)j * m.nC + c;
      const int e = m.eoc[s];
      const int64_t ie = (int64_t)e * L + k;
      G += dmask(dflip(m.invDcEdge[e] * a.lk_u[ie], sign_mask(m.eocSign[s])), ok);
      sl += dmask(a.lhe[ie], ok);
    };
    if (m.maxEoC <= 6)
      for_slots<6>(m.nEoC[c], slot);
    else
      for_slots<0>(m.nEoC[c], slot);
    a.mu_h[i] = fma(0.5, sl, -a.g * G) + muh;
    a.lke[i] = -G;
    if (a.visc) a.ldiv[i] = a.nu * G;
  }
}

__device__ __forceinline__ void b2_vertex_item(const DMesh &m, const AdjArgs &a, int L, int64_t i) {
  const int v = (int)(i / L), k = (int)(i - (int64_t)v * L);
  double lpv = 0.0, lvort = 0.0;
#pragma unroll
  for (int j = 0; j < kVertexDegree; ++j) {
    const int64_t s = (int64_t)j * m.nV + v;
    const int e = m.eov[s];
    const int64_t ie = (int64_t)e * L + k;
    lpv += a.lpve[ie];
    if (a.visc) lvort += dflip(m.invDvEdge[e] * a.lk_u[ie], sign_mask(m.eovSign[s]));
  }
  lpv *= 0.5;
  const double rh = rcp_nr(a.hs[i]);
  double lc = lpv * rh;
  if (a.visc) lc = fma(-a.nu * lvort, m.invAreaTriangle[v], lc);
  a.lcirc[i] = lc;
  a.lhs[i] = -lpv * a.pv[i] * rh;
}

__global__ void __launch_bounds__(TPB) k_adj_b2(DMesh m, AdjArgs a, int L) {
  stage_prologue();
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nCL = (int64_t)m.nC * L;
  if (i < nCL) {
    b2_cell_item(m, a, L, i, a.muh_t ? a.muh_t[i] : 0.0);
    return;
  }
  i -= nCL;
  if (i < (int64_t)m.nV * L) b2_vertex_item(m, a, L, i);
}

// RK4 cotangent bookkeeping for one element once mu is complete.
__device__ __forceinline__ double combine(int rk, double dt, int64_t i, double mu, double *lam, double *acc,
                                          double *lk) {
  double l;
  switch (rk) {
    case 3:
      acc[i] = lam[i] + mu;
      l = fma(dt, mu, (dt / 3) * lam[i]);
      break;
    case 2:
      acc[i] += mu;
      l = fma(dt / 2, mu, (dt / 3) * lam[i]);
      break;
    case 1:
      acc[i] += mu;
      l = fma(dt / 2, mu, (dt / 6) * lam[i]);
      break;
    default: {
      const double ln = acc[i] + mu;
      lam[i] = ln;
      l = (dt / 6) * ln;
    }
  }
  lk[i] = l;
  return l;
}

// B3 (cells + edges): thickness through kites; u through circulation, KE and
// divergence; then the RK combination.
__device__ __forceinline__ void b3_cell_item(const DMesh &m, const AdjArgs &a, int L, int64_t i) {
  const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
  double mh = a.mu_h[i];
  for (int j = 0; j < m.maxEoC; ++j) {
    const int64_t s = (int64_t)j * m.nC + c;
    mh = fma(m.kiteR[s], a.lhs[(int64_t)m.vocR[s] * L + k], mh);
  }
  combine(a.rk, a.dt, i, mh, a.lam_h, a.acc_h, a.lk_h);
}

__device__ __forceinline__ void b3_edge_item(const DMesh &m, const DStat &st, const AdjArgs &a, int L, int64_t i) {
  const int e = (int)(i / L), k = (int)(i - (int64_t)e * L);
  const int2 c = m.coe[e];
  const int2 v = m.voe[e];
  const int64_t i1 = (int64_t)c.x * L + k, i2 = (int64_t)c.y * L + k;
  const double ia1 = m.invAreaCell[c.x], ia2 = m.invAreaCell[c.y];
  double mu = a.mu_u[i];
  mu = fma(m.dcEdge[e], a.lcirc[(int64_t)v.y * L + k] - a.lcirc[(int64_t)v.x * L + k], mu);
  mu = fma(2.0 * a.u[i] * st.kw[e], fma(a.lke[i1], ia1, a.lke[i2] * ia2), mu);
  if (a.visc) mu = fma(-m.dvEdge[e], fma(a.ldiv[i2], ia2, -a.ldiv[i1] * ia1), mu);
  const double lk = combine(a.rk, a.dt, i, mu, a.lam_u, a.acc_u, a.lk_u);
  // the next stage's B1 inputs (B1 of this stage has completed)
  if (a.prep) prep_edge(m, a, L, e, k, i, a.un, a.hn, a.pvn, lk);
}

__global__ void __launch_bounds__(TPB) k_adj_b3(DMesh m, DStat st, AdjArgs a, int L) {
  stage_prologue();
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nCL = (int64_t)m.nC * L;
  if (i < nCL) {
    b3_cell_item(m, a, L, i);
    return;
  }
  i -= nCL;
  if (i < (int64_t)m.nE * L) b3_edge_item(m, st, a, L, i);
}


// ---------------------------------------------------------------------------
// Tracer reverse, three launches per stage ahead of B1: TA (cells) the FCT
// limiter, TB (edges) the fluxes, TC (cells) the gathers and the q update.
// g = lk_q / areaCell is kept beside lk_q (the tendency's per-area cotangent).

// The NL lanes of a cell are adjacent and NL-aligned in a warp; kernels
// retire whole groups, so a group's mask names live threads only.
template <int NL> __device__ __forceinline__ unsigned group_mask() {
  return ((1u << NL) - 1u) << ((threadIdx.x & 31u) & ~(unsigned)(NL - 1));
}

// Sum over the NL lanes of a cell.
template <int NL> __device__ __forceinline__ double lane_sum(double v) {
  const unsigned gm = group_mask<NL>();
#pragma unroll
  for (int o = NL / 2; o > 0; o >>= 1) v += __shfl_xor_sync(gm, v, o);
  return v;
}

// TA (cells, FCT only): the bounds with the cells that hold them, the upwind
// value and the limiter quotients of the stage (apps/ocean/tasks/solve.cc:
// 194-267; 1/hProv and the upwind sum are taped by the recompute), and the
// cotangents of R+ / R- that the limited fluxes of the cell's edges send back
// through the factor each used (solve.cc:270-282), taken down to the bounds,
// the upwind sum, flxIn / flxOut and hProv.  NL lanes per cell share its edge
// slots; the bounds merge as (value, slot) with the lower slot (the cell
// itself first) winning ties, which is the reference's sequential max / min.
template <int NL, int NC>
__device__ __forceinline__ void tr_a_item(const DMesh &m, const TrArgs &a, int L, int64_t g) {
  const int lane = (int)(g & (NL - 1));
  const int64_t i = g / NL;
  const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
  const int n = m.nEoC[c], T = a.T;
  const double hin = a.h[i], hpi = a.hpi[i];
  const double dtia = a.dt * m.invAreaCell[c];
  const double dthi = dtia * hpi;
  const double eps = 1.e-10;
  double lhpi = 0.0, lh = 0.0;
  for (int t = 0; t < T; ++t) {
    const int64_t it = i * T + t;
    const double trc = a.tr[it], gc = a.gq[it];
    const double2 own = a.R2[it];
    double mx = trc, mn = trc, fi = 0.0, fo = 0.0, lrp = 0.0, lrm = 0.0;
    int smx = -1, smn = -1;
    auto slot = [&](int j, bool ok) {
      // compares, selects and sign flips on the integer pipe (rk4.cuh helpers),
      // one add per slot for flxIn / flxOut; pad slots (own cell, slot-0 edge)
      // are masked and cannot win a bound
      const int64_t s = (int64_t)j * m.nC + c;
      const double aa = a.A[((int64_t)m.eoc[s] * L + k) * T + t];
      const double sa = dmask(dflip(aa, sign_mask(m.eocSign[s])), ok);
      const bool in = dgt0(sa);
      const double f = (in ? fi : fo) + sa;
      fi = in ? f : fi, fo = in ? fo : f;
      const double x = a.tr[((int64_t)m.coc[s] * L + k) * T + t];
      if (dkey(mx) < dkey(x)) mx = x, smx = j;
      if (dkey(x) < dkey(mn)) mn = x, smn = j;
      // which of this cell's factors the limited flux of e used: A > 0 takes
      // min(R-(c1), R+(c2)), A < 0 min(R+(c1), R-(c2)), the first on ties
      const int nb = m.nbr[s];
      const bool first = nb & 1;
      const int64_t jo = ((int64_t)(nb >> 1) * L + k) * T + t;
      const double2 ot = a.R2[jo];
      int sel = 0;  // 1: R+ of this cell, 2: R- of this cell
      if (!ok)
        ;
      else if (dgt0(aa))
        sel = first ? (dkey(ot.x) < dkey(own.y) ? 0 : 2) : (dkey(own.x) < dkey(ot.y) ? 1 : 0);
      else if (dlt0(aa))
        sel = first ? (dkey(ot.y) < dkey(own.x) ? 0 : 1) : (dkey(own.y) < dkey(ot.x) ? 2 : 0);
      if (sel) {  // one subtraction and one fma into the factor's sum (selected operands)
        const double go = a.gq[jo];
        const double G = (first ? go : gc) - (first ? gc : go);  // g(c2) - g(c1)
        const double acc = fma(G, aa, sel == 1 ? lrp : lrm);
        lrp = sel == 1 ? acc : lrp;
        lrm = sel == 1 ? lrm : acc;
      }
    };
    if constexpr (NL == 1)
      for_slots<NC>(n, slot);
    else
      for (int j = lane; j < n; j += NL) slot(j, true);
    const unsigned gm = group_mask<NL>();
#pragma unroll
    for (int o = NL / 2; o > 0; o >>= 1) {
      const double xm = __shfl_xor_sync(gm, mx, o), xn = __shfl_xor_sync(gm, mn, o);
      const int sm = __shfl_xor_sync(gm, smx, o), sn = __shfl_xor_sync(gm, smn, o);
      if (dkey(mx) < dkey(xm) || (dkey(xm) == dkey(mx) && sm < smx)) mx = xm, smx = sm;
      if (dkey(xn) < dkey(mn) || (dkey(xn) == dkey(mn) && sn < smn)) mn = xn, smn = sn;
    }
    fi = lane_sum<NL>(fi), fo = lane_sum<NL>(fo), lrp = lane_sum<NL>(lrp), lrm = lane_sum<NL>(lrm);
    if (lane) continue;
    // upwind sum: area-weighted from the sw kernels, divided by the area (as
    // the reference's tend holds it) from the ocean kernels
    const double num = fma(a.ocean ? a.dt : dtia, a.tLO[it], trc * hin);
    const double up = num * hpi;
    double lup = 0.0, ldp = 0.0, ldm = 0.0;
    double2 lb = make_double2(0.0, 0.0);  // cotangents of the max / min bounds
    // R = min(1, max(0, n / d)) passes a derivative only strictly inside (0, 1),
    // read off the factor the forward computed
    constexpr long long kOne = 0x3ff0000000000000LL;
    if (dgt0(own.x) && dkey(own.x) < kOne) {  // R+ = (max - up) / (dthi flxIn + eps)
      const double dp = fma(dthi, fi, eps), r = rcp_nr(dp), q = lrp * r;
      lb.x = q, lup = -q, ldp = -q * (mx - up) * r;
    }
    if (dgt0(own.y) && dkey(own.y) < kOne) {  // R- = (up - min) / (-dthi flxOut + eps)
      const double dm = fma(-dthi, fo, eps), r = rcp_nr(dm), q = lrm * r;
      lb.y = -q, lup += q, ldm = -q * (up - mn) * r;
    }
    a.lfio[it] = make_double2(ldp * dthi, -ldm * dthi);
    a.ltrs[it] = lup * hin * hpi;
    a.ltl[it] = lup * dthi;
    a.lmm[it] = lb;
    a.amm[it] = make_int2(smx < 0 ? c : m.coc[(int64_t)smx * m.nC + c], smn < 0 ? c : m.coc[(int64_t)smn * m.nC + c]);
    lh = fma(lup * trc, hpi, lh);
    lhpi = fma(lup, num, lhpi);
    lhpi = fma(fma(ldp, fi, -ldm * fo), dtia, lhpi);
  }
  if (lane || a.ocean) return;  // ocean: h and the thickness flux are prescribed
  // hProv = h + dt tend_h: its cotangent goes to h and to the thickness tendency
  const double lhp = -lhpi * hpi * hpi;
  a.muh_t[i] = lh + lhp;
  a.lk_h[i] = fma(a.dt, lhp, a.lk_h[i]);
}

template <int NL, int NC>
__global__ void __launch_bounds__(TPB) k_adj_tr_a(DMesh m, TrArgs a, int L) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g / NL >= (int64_t)m.nC * L) return;  // whole groups: all lanes of a live cell stay
  tr_a_item<NL, NC>(m, a, L, g);
}

// B3 of this reversed stage with TA of the next one (the stage before it in the
// forward, same segment): TA of a cell-level reads, of what B3 writes, only
// the thickness-tendency cotangent of its own cell, so one thread does both.
template <int NC>
__global__ void __launch_bounds__(TPB) k_adj_b3_tra(DMesh m, DStat st, AdjArgs a, TrArgs tn, int L) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nCL = (int64_t)m.nC * L;
  if (i < nCL) {
    b3_cell_item(m, a, L, i);
    tr_a_item<1, NC>(m, tn, L, i);
    return;
  }
  i -= nCL;
  if (i < (int64_t)m.nE * L) b3_edge_item(m, st, a, L, i);
}

// TB (edges): the cotangents of the stage's edge fluxes.  FCT: the limited
// antidiffusive flux A' and the cell sums (tLO, flxIn, flxOut) give A and LO;
// LO = dv F tr_upwind and HO = F S (S the advection-stencil sum of the
// tracer, or dv (tr1 + tr2) / 2 where the high-order mask is 0) give F and
// the tracers (solve.cc:99-167, 216-229).  S is read back as HO / F = (A +
// LO) / F from the taped fluxes (the stencil is summed only where F = 0).
// Without FCT: the centred flux of apps/sw/tasks/solve.cc:237-270 (sw) or no
// advection (ocean, whose advection is the FCT task alone).  del2 mixing
// (ocean solve.cc:328-366) adds to h_e and the tracers.  Per edge and
// tracer the parts for cells(e) go to p12 and lambda_HO F, split by the sign
// of F, to lho (TC gathers them); per edge the thickness-flux and
// edge-thickness cotangents summed over tracers go to lFt / lhet (B1 adds them).
__device__ __forceinline__ void tr_b_item(const DMesh &m, const TrArgs &a, int L, int64_t i, double &lF_out,
                                          double &lhe_out) {
  const int e = (int)(i / L), k = (int)(i - (int64_t)e * L), T = a.T;
  const int2 c = m.coe[e];
  const int64_t i1 = (int64_t)c.x * L + k, i2 = (int64_t)c.y * L + k;
  const double he = a.ocean ? a.hEx[i] : 0.5 * (a.h[i1] + a.h[i2]);
  const double F = a.ocean ? a.Fx[i] : a.u[i] * he, dv = m.dvEdge[e];
  const bool pos = dgt0(F), neg = dlt0(F);
  const int mask = a.fct ? m.hoMask[(int64_t)e * m.fctLev + k] : 0;
  const double kd = a.hmix ? a.kd[e] : 0.0;
  const double rF = (pos || neg) ? rcp_nr(F) : 0.0;
  double lF = 0.0, lhe = 0.0;
  for (int t = 0; t < T; ++t) {
    const int64_t i1t = i1 * T + t, i2t = i2 * T + t, it = i * T + t;
    const double tr1 = a.tr[i1t], tr2 = a.tr[i2t];
    const double G = a.gq[i2t] - a.gq[i1t];
    double p1 = 0.0, p2 = 0.0;
    if (a.fct) {
      const double aa = a.A[it], lo = a.LO[it];
      // the branch the flux sign took, as one subtraction and one fma whose
      // operands the sign selects (integer-pipe selects, the same arithmetic
      // per lane), so a warp with both signs issues them once
      const bool ap = dgt0(aa), an = dlt0(aa);
      double lA = 0.0;
      if (ap || an) {
        const double2 r1 = a.R2[i1t], r2 = a.R2[i2t], f1 = a.lfio[i1t], f2 = a.lfio[i2t];
        const double rmin = ap ? dmin(r1.y, r2.x) : dmin(r1.x, r2.y);
        lA = fma(G, rmin, (ap ? f2.x : f2.y) - (ap ? f1.y : f1.x));
      }
      const double lLO = G + (a.ltl[i2t] - a.ltl[i1t]) - lA;
      if (pos || neg) {  // the upwind value's cotangent, on the side the flux sign picks
        const double q = lLO * dv;
        lF = fma(q, pos ? tr1 : tr2, lF);
        const double pq = q * F;
        p1 = pos ? pq : 0.0;
        p2 = pos ? 0.0 : pq;
      }
      double S;
      if (pos || neg) {
        S = (aa + lo) * rF;
      } else if (mask) {  // F = 0: the stencil with the centred coefficients
        S = 0.0;
        for (int sl = 0; sl < m.nAdv[e]; ++sl) {
          const int64_t sa = (int64_t)sl * m.nE + e;
          S = fma(m.advCoef[sa], a.tr[((int64_t)m.advCells[sa] * L + k) * T + t], S);
        }
      } else {
        S = 0.5 * dv * (tr1 + tr2);
      }
      lF = fma(lA, S, lF);
      const double lAF = lA * F;
      if (mask) {
        a.lho[it] = make_double2(pos ? lAF : 0.0, neg ? lAF : 0.0);
      } else {
        const double q = 0.5 * dv * lAF;
        p1 += q, p2 += q;
        a.lho[it] = make_double2(0.0, 0.0);
      }
    } else if (a.centred) {
      const double hd = 0.5 * dv;
      lF = fma(G * hd, tr1 + tr2, lF);
      p1 = p2 = G * hd * F;
    }
    if (a.hmix) {  // tend -= inva sum sign DF, DF = h_e (tr2 - tr1) kd
      lhe = fma(-G * kd, tr2 - tr1, lhe);
      const double q = G * he * kd;
      p1 += q, p2 -= q;
    }
    a.p12[it] = make_double2(p1, p2);
  }
  lF_out = lF, lhe_out = lhe;
}

__global__ void __launch_bounds__(TPB) k_adj_tr_b(DMesh m, TrArgs a, int L) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nE * L) return;
  double lF, lhe;
  tr_b_item(m, a, L, i, lF, lhe);
  if (a.ocean) return;
  a.lFt[i] = lF;
  a.lhet[i] = lhe;
}

// TC (cells): the tracer cotangent of the stage input, gathered from the
// upwind value, the edges of the cell, the advection stencils that read it
// (DMesh::advRe / advRc) and the bounds it holds for itself and its distinct
// neighbours (DMesh::cocU); then q = h tr is converted and the RK bookkeeping
// of q runs (g = lk_q / areaCell for the next stage beside it).  NL lanes per
// cell split the gathers and sum by shuffles.
// Returns true on the lane that holds the cell's thickness cotangent mh_out.
template <int NL>
__device__ __forceinline__ bool tr_c_item(const DMesh &m, const TrArgs &a, int L, int64_t g, double &mh_out) {
  const int lane = (int)(g & (NL - 1));
  const int64_t i = g / NL;
  const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
  const int n = m.nEoC[c], T = a.T;
  const double hinv = a.ocean ? 1.0 : rcp_nr(a.h[i]), inva = m.invAreaCell[c];
  double mh = a.fct && !a.ocean ? a.muh_t[i] : 0.0;
  for (int t = 0; t < T; ++t) {
    const int64_t it = i * T + t;
    double lt = 0.0;
    for (int j = lane; j < n; j += NL) {
      const int64_t s = (int64_t)j * m.nC + c;
      const double2 p = a.p12[((int64_t)m.eoc[s] * L + k) * T + t];
      lt += (m.nbr[s] & 1) ? p.x : p.y;
      if (a.fct) {
        const int oc = m.cocU[s];
        if (oc >= 0) {
          const int64_t ot = ((int64_t)oc * L + k) * T + t;
          const int2 ao = a.amm[ot];
          if (ao.x == c) lt += a.lmm[ot].x;
          if (ao.y == c) lt += a.lmm[ot].y;
        }
      }
    }
    if (a.fct)
      for (int j0 = lane; j0 < m.maxAdvR; j0 += 4 * NL) {
        // four entries per lane in flight: indices first, then the gathers
        int e[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int j = j0 + u * NL;
          e[u] = j < m.maxAdvR ? m.advRe[(int64_t)j * m.nC + c] : -1;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if (e[u] < 0) continue;
          // one of {F > 0 part, F < 0 part} is +0: pick the other with its coefficient
          const double2 w = m.advRc[(int64_t)(j0 + u * NL) * m.nC + c];
          const double2 l = a.lho[((int64_t)e[u] * L + k) * T + t];
          const bool p = dbits(l.x) != 0;
          lt = fma(p ? w.x : w.y, p ? l.x : l.y, lt);
        }
        if (e[3] < 0) break;
      }
    lt = lane_sum<NL>(lt);
    if (lane) continue;
    if (a.fct) {
      lt += a.ltrs[it];
      const int2 am = a.amm[it];
      const double2 lb = a.lmm[it];
      if (am.x == c) lt += lb.x;
      if (am.y == c) lt += lb.y;
    }
    const double mq = lt * hinv;  // sw: tr = q / h; ocean: the state is tr itself
    if (!a.ocean) mh = fma(-mq, a.tr[it], mh);
    a.gq[it] = combine(a.rk, a.dt, it, mq, a.lam_q, a.acc_q, a.lk_q) * inva;
  }
  mh_out = mh;
  return lane == 0;
}

template <int NL>
__global__ void __launch_bounds__(TPB) k_adj_tr_c(DMesh m, TrArgs a, int L) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g / NL >= (int64_t)m.nC * L) return;  // whole groups: all lanes of a live cell stay
  double mh;
  if (tr_c_item<NL>(m, a, L, g, mh) && !a.ocean) a.muh_t[g / NL] = mh;
}

// The sw app with tracers, fused by item: TB and B1 of one edge-level in one
// thread (the tracer part's flux cotangents pass in registers) ...
template <int NW>
__global__ void __launch_bounds__(TPB) k_adj_trb_b1(DMesh m, TrArgs t, AdjArgs a, int L) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nE * L) return;
  double lF, lhe;
  tr_b_item(m, t, L, i, lF, lhe);
  b1_item<NW>(m, a, L, i, true, lF, lhe);
}

// ... and TC and B2: the NL lanes of a cell-level do TC, its first lane then
// the cell part of B2 with the thickness cotangent in hand; the threads past
// the cells do B2's vertices.
template <int NL>
__global__ void __launch_bounds__(TPB) k_adj_trc_b2(DMesh m, TrArgs t, AdjArgs a, int L) {
  int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nCL = (int64_t)m.nC * L;
  if (g < nCL * NL) {
    double mh;
    if (tr_c_item<NL>(m, t, L, g, mh)) b2_cell_item(m, a, L, g / NL, mh);
    return;
  }
  g -= nCL * NL;
  if (g < (int64_t)m.nV * L) b2_vertex_item(m, a, L, g);
}

// Window ends: lambda_q = lambda_tr / h, lambda_h -= sum_t lambda_tr tr / h
// (out = 0), and lambda_tr = lambda_q h, lambda_h += sum_t lambda_q tr (out = 1).
__global__ void k_adj_q_convert(int64_t nCL, int T, const double *h, const double *tr, double *lam_q,
                                double *lam_h, int out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nCL) return;
  const double hi = h[i];
  double lh = lam_h[i];
  for (int t = 0; t < T; ++t) {
    const int64_t it = i * T + t;
    if (out) {
      lh = fma(lam_q[it], tr[it], lh);
      lam_q[it] *= hi;
    } else {
      const double q = lam_q[it] / hi;
      lh = fma(-q, tr[it], lh);
      lam_q[it] = q;
    }
  }
  lam_h[i] = lh;
}

// lk_q = c lam_q and g = lk_q / areaCell
__global__ void k_adj_init_q(DMesh m, int L, int T, const double *lam, double *lk, double *g, double c) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nC * L * T) return;
  const double l = c * lam[i];
  lk[i] = l;
  g[i] = l * m.invAreaCell[i / ((int64_t)L * T)];
}

__global__ void k_adj_init(int64_t n, const double *lam, double *lk, double c) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) lk[i] = c * lam[i];
}

void ensure_buffers(SwState &s, int N, int k) {
  const DMesh &m = s.mesh->ctx.d;
  const int64_t L = s.L, eu = (int64_t)m.nE * L, ch = (int64_t)m.nC * L, vv = (int64_t)m.nV * L;
  const int nck = (N + k - 1) / k + 1;
  // a second tape set where the window has two segments or more and the
  // stages leave most of the GPU idle (under 2^20 cell-levels)
  const bool dbl = k < N && (int64_t)m.nC * L < (1LL << 20);
  AdjBuffers *A = s.adj;
  if (A && A->cap_ck >= nck && A->cap_k >= k && (A->dbl || !dbl)) return;
  free_adjoint(s);
  A = s.adj = new AdjBuffers();
  A->dbl = dbl;
  // the ocean app differentiates its tracers only: no (h, u) tape or cotangents
  const int64_t hu = s.p.app == MPASO_APP_OCEAN ? 0 : 1;
  std::vector<std::pair<double **, int64_t>> bufs = {
      {&A->ck_u, hu * nck * eu}, {&A->ck_h, hu * nck * ch}, {&A->tp_u, hu * (4LL * k + 1) * eu},
      {&A->tp_h, hu * (4LL * k + 1) * ch}, {&A->uacc, hu * eu}, {&A->hacc, hu * ch},
      {&A->tp_pv, hu * (4LL * k + 1) * vv}, {&A->tp_hs, hu * (4LL * k + 1) * vv}, {&A->tp_s1, hu * 4LL * k * eu},
      {(double **)&A->FP, hu * 2 * eu}, {&A->pve, hu * eu}, {&A->lam_u, hu * eu}, {&A->lam_h, hu * ch},
      {&A->acc_u, hu * eu}, {&A->acc_h, hu * ch}, {&A->lk_u, hu * eu}, {&A->lk_h, hu * ch}, {&A->mu_u, hu * eu},
      {&A->mu_h, hu * ch}, {&A->lhe, hu * eu}, {&A->lpve, hu * eu}, {&A->lke, hu * ch}, {&A->ldiv, hu * ch},
      {&A->lcirc, hu * vv}, {&A->lhs, hu * vv}};
  if (s.T > 0) {
    const int64_t cT = ch * s.T, eT = eu * s.T;
    const std::vector<std::pair<double **, int64_t>> tb = {
        {&A->ck_tr, nck * cT}, {&A->tp_tr, (4LL * k + 1) * cT}, {&A->tp_A, 4LL * k * eT},
        {&A->tp_LO, 4LL * k * eT}, {(double **)&A->tp_R2, 8LL * k * cT}, {&A->tp_tLO, 4LL * k * cT},
        {&A->tp_hpi, hu * 4LL * k * ch}, {&A->trhacc, cT}, {&A->lam_q, cT}, {&A->acc_q, cT}, {&A->lk_q, cT},
        {&A->gq, cT}, {&A->ltl, cT}, {&A->ltrs, cT}, {(double **)&A->lfio, 2 * cT},
        {(double **)&A->lmm, 2 * cT}, {(double **)&A->amm, cT}, {&A->muh_t, hu * ch}, {&A->lFt, hu * eu},
        {&A->lhet, hu * eu}, {(double **)&A->lho, 2 * eT}, {(double **)&A->p12, 2 * eT}};
    bufs.insert(bufs.end(), tb.begin(), tb.end());
  }
  TapeSet &t1 = A->tape[1];
  if (dbl) {
    const std::vector<std::pair<double **, int64_t>> tb = {
        {&t1.u, hu * (4LL * k + 1) * eu}, {&t1.h, hu * (4LL * k + 1) * ch}, {&t1.pv, hu * (4LL * k + 1) * vv},
        {&t1.hs, hu * (4LL * k + 1) * vv}, {&t1.s1, hu * 4LL * k * eu}};
    bufs.insert(bufs.end(), tb.begin(), tb.end());
    if (s.T > 0) {
      const int64_t cT = ch * s.T, eT = eu * s.T;
      const std::vector<std::pair<double **, int64_t>> tt = {
          {&t1.tr, (4LL * k + 1) * cT}, {&t1.A, 4LL * k * eT}, {&t1.LO, 4LL * k * eT},
          {(double **)&t1.R2, 8LL * k * cT}, {&t1.tLO, 4LL * k * cT}, {&t1.hpi, hu * 4LL * k * ch}};
      bufs.insert(bufs.end(), tt.begin(), tt.end());
    }
  }
  size_t total = 0;
  for (auto &b : bufs) total += ((size_t)std::max<int64_t>(b.second, 1) * 8 + 255) & ~size_t(255);
  if (cudaMalloc(&A->arena, total) != cudaSuccess) {
    cudaGetLastError();
    fail(MPASO_ERR_ALLOC, "device allocation of the adjoint buffers failed (" + std::to_string(total) +
                              " bytes)");
  }
  A->bytes = total;
  MPASO_CUDA(cudaMemsetAsync(A->arena, 0, total, s.stream));
  char *p = (char *)A->arena;
  for (auto &b : bufs) {
    *b.first = (double *)p;
    p += ((size_t)std::max<int64_t>(b.second, 1) * 8 + 255) & ~size_t(255);
  }
  A->tape[0] = TapeSet{A->tp_u, A->tp_h, A->tp_pv, A->tp_hs, A->tp_s1, A->tp_tr,
                       A->tp_A, A->tp_LO, A->tp_tLO, A->tp_hpi, A->tp_R2};
  if (dbl) {
    MPASO_CUDA(cudaStreamCreateWithFlags(&A->side, cudaStreamNonBlocking));
    for (cudaEvent_t *e : {&A->ev_fork, &A->ev_tape, &A->ev_rev})
      MPASO_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  }
  A->cap_ck = nck;
  A->cap_k = k;
}

// Makes tape set b the one the tp_* pointers name.
void use_tape(AdjBuffers &A, int b) {
  const TapeSet &t = A.tape[b];
  A.tp_u = t.u, A.tp_h = t.h, A.tp_pv = t.pv, A.tp_hs = t.hs, A.tp_s1 = t.s1, A.tp_tr = t.tr;
  A.tp_A = t.A, A.tp_LO = t.LO, A.tp_tLO = t.tLO, A.tp_hpi = t.hpi, A.tp_R2 = t.R2;
}

// Reverse of the stage whose input state is tape slot j; `first`: no B3 before
// it prepared its edge quantities; `prep_next`: prepare those of slot j - 1.
// Tracer arguments of the reversed stage whose input state is tape slot j.
TrArgs tr_args(SwState &s, AdjBuffers &A, int rk, int j) {
  const DMesh &m = s.mesh->ctx.d;
  const int64_t nE = (int64_t)m.nE * s.L, nC = (int64_t)m.nC * s.L;
  const int64_t cT = nC * s.T, eT = nE * s.T;
  TrArgs t{};
  t.u = A.tp_u + (size_t)j * nE, t.h = A.tp_h + (size_t)j * nC, t.tr = A.tp_tr + (size_t)j * cT;
  t.A = A.tp_A + (size_t)j * eT, t.LO = A.tp_LO + (size_t)j * eT, t.R2 = A.tp_R2 + (size_t)j * cT;
  t.hpi = A.tp_hpi + (size_t)j * nC, t.tLO = A.tp_tLO + (size_t)j * cT;
  if (s.p.app == MPASO_APP_OCEAN) {  // prescribed thickness, edge thickness, flux and 1/hProv
    t.ocean = 1, t.h = s.H[0], t.hpi = s.HPI, t.Fx = s.F, t.hEx = s.HE;
  }
  t.kd = s.st.kd, t.lk_h = A.lk_h, t.lk_q = A.lk_q, t.gq = A.gq, t.lam_q = A.lam_q, t.acc_q = A.acc_q;
  t.ltl = A.ltl, t.ltrs = A.ltrs, t.lfio = A.lfio, t.lmm = A.lmm, t.amm = A.amm;
  t.muh_t = A.muh_t, t.lFt = A.lFt, t.lhet = A.lhet, t.p12 = A.p12, t.lho = A.lho;
  t.T = s.T, t.rk = rk, t.fct = s.p.fct ? 1 : 0, t.hmix = s.p.hmix ? 1 : 0, t.dt = A.dt;
  t.centred = !t.fct && !t.ocean;
  return t;
}

// `tra_done`: TA of this stage already ran with the previous reversed stage's
// B3; returns whether this stage's B3 ran TA of the next one.
bool stage_vjp(SwState &s, AdjBuffers &A, int rk, int j, bool first, bool prep_next, cudaStream_t st,
               bool tra_done) {
  const DMesh &m = s.mesh->ctx.d;
  const int L = s.L;
  const int64_t nE = (int64_t)m.nE * L, nC = (int64_t)m.nC * L, nV = (int64_t)m.nV * L;
  AdjArgs a{};
  a.u = A.tp_u + (size_t)j * nE, a.h = A.tp_h + (size_t)j * nC;
  a.pv = A.tp_pv + (size_t)j * nV, a.hs = A.tp_hs + (size_t)j * nV;
  a.s1 = A.tp_s1 + (size_t)j * nE;
  a.FP = A.FP, a.pve = A.pve;
  a.lk_u = A.lk_u, a.lk_h = A.lk_h, a.mu_u = A.mu_u, a.mu_h = A.mu_h;
  a.lhe = A.lhe, a.lpve = A.lpve, a.lke = A.lke, a.ldiv = A.ldiv, a.lcirc = A.lcirc, a.lhs = A.lhs;
  a.lam_u = A.lam_u, a.lam_h = A.lam_h, a.acc_u = A.acc_u, a.acc_h = A.acc_h;
  a.rk = rk, a.visc = s.p.nu != 0.0, a.dt = A.dt, a.g = s.p.gravity, a.nu = s.p.nu;
  a.prep = prep_next ? 1 : 0;
  if (prep_next) {
    a.un = A.tp_u + (size_t)(j - 1) * nE, a.hn = A.tp_h + (size_t)(j - 1) * nC;
    a.pvn = A.tp_pv + (size_t)(j - 1) * nV;
  }
  // plain stream order: programmatic dependent launch made this 25% slower (measured)
  const bool pdl = false;
  const bool ocean = s.p.app == MPASO_APP_OCEAN;
  if (first && !ocean) launch_pdl(k_adj_prep, nE, TPB, pdl, st, m, a, L);
  if (A.tr) {
    const TrArgs t = tr_args(s, A, rk, j);
    constexpr int NLA = 1, NLC = 2;  // lanes per cell (measured best at level 6)
    if (t.fct && !tra_done) {
      if (m.maxEoC <= 6)
        launch_pdl(k_adj_tr_a<NLA, 6>, nC * NLA, TPB, pdl, st, m, t, L);
      else
        launch_pdl(k_adj_tr_a<NLA, 0>, nC * NLA, TPB, pdl, st, m, t, L);
    }
    // two lanes per cell-level hide gather latency on small meshes; with a
    // million cell-levels or more there is parallelism enough, and the
    // second lane only idles through the per-cell tail on the FP64 pipe
    const bool one_lane = nC >= (1 << 20);
    if (!ocean) {
      // sw: TB with B1 and TC with B2 as two fused launches, then B3
      if (m.maxEoE == 10)
        launch_pdl(k_adj_trb_b1<10>, nE, TPB, pdl, st, m, t, a, L);
      else
        launch_pdl(k_adj_trb_b1<0>, nE, TPB, pdl, st, m, t, a, L);
      if (one_lane)
        launch_pdl(k_adj_trc_b2<1>, nC + nV, TPB, pdl, st, m, t, a, L);
      else
        launch_pdl(k_adj_trc_b2<NLC>, nC * NLC + nV, TPB, pdl, st, m, t, a, L);
      if (t.fct && prep_next) {  // with TA of the next reversed stage (slot j - 1)
        const TrArgs tn = tr_args(s, A, rk > 0 ? rk - 1 : 3, j - 1);
        if (m.maxEoC <= 6)
          launch_pdl(k_adj_b3_tra<6>, nC + nE, TPB, pdl, st, m, s.st, a, tn, L);
        else
          launch_pdl(k_adj_b3_tra<0>, nC + nE, TPB, pdl, st, m, s.st, a, tn, L);
        return true;
      }
      launch_pdl(k_adj_b3, nC + nE, TPB, pdl, st, m, s.st, a, L);
      return false;
    }
    launch_pdl(k_adj_tr_b, nE, TPB, pdl, st, m, t, L);
    if (one_lane)
      launch_pdl(k_adj_tr_c<1>, nC, TPB, pdl, st, m, t, L);
    else
      launch_pdl(k_adj_tr_c<NLC>, nC * NLC, TPB, pdl, st, m, t, L);
  }
  if (ocean) return false;  // the ocean's h and u are prescribed: nothing more to reverse
  if (m.maxEoE == 10)
    launch_pdl(k_adj_b1<10>, nE, TPB, pdl, st, m, a, L);
  else
    launch_pdl(k_adj_b1<0>, nE, TPB, pdl, st, m, a, L);
  launch_pdl(k_adj_b2, nC + nV, TPB, pdl, st, m, a, L);
  launch_pdl(k_adj_b3, nC + nE, TPB, pdl, st, m, s.st, a, L);
  return false;
}

void tape_segment(SwState &s, AdjBuffers &A, int n, bool with_tr, cudaStream_t st);

// Captures (once per window length and dt) and replays the taping forward of
// the store-the-window mode, then leaves the final state in the state's buffers.
void forward_stored(SwState &s, double dt, int N) {
  AdjBuffers &A = *s.adj;
  const DMesh &m = s.mesh->ctx.d;
  const size_t eu = (size_t)m.nE * s.L, ch = (size_t)m.nC * s.L, ct = ch * s.T;
  const bool with_tr = s.T > 0;
  if (A.fwd && (A.fwd_N != N || A.fwd_dt != dt)) {
    cudaGraphExecDestroy(A.fwd);
    A.fwd = nullptr;
  }
  if (!A.fwd) {
    cudaGraph_t g;
    MPASO_CUDA(cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeThreadLocal));
    try {
      const bool hu = s.p.app == MPASO_APP_SW;  // the ocean's h and u are prescribed
      if (!hu) ocean_recompute(s, dt, s.stream);
      if (hu) {
        MPASO_CUDA(cudaMemcpyAsync(A.tp_u, s.U[0], eu * 8, cudaMemcpyDeviceToDevice, s.stream));
        MPASO_CUDA(cudaMemcpyAsync(A.tp_h, s.H[0], ch * 8, cudaMemcpyDeviceToDevice, s.stream));
      }
      if (with_tr) MPASO_CUDA(cudaMemcpyAsync(A.tp_tr, s.TR0, ct * 8, cudaMemcpyDeviceToDevice, s.stream));
      tape_segment(s, A, N, with_tr, s.stream);
      if (hu) {
        MPASO_CUDA(cudaMemcpyAsync(s.U[0], A.tp_u + 4 * (size_t)N * eu, eu * 8, cudaMemcpyDeviceToDevice, s.stream));
        MPASO_CUDA(cudaMemcpyAsync(s.H[0], A.tp_h + 4 * (size_t)N * ch, ch * 8, cudaMemcpyDeviceToDevice, s.stream));
      }
      if (with_tr)
        MPASO_CUDA(cudaMemcpyAsync(s.TR0, A.tp_tr + 4 * (size_t)N * ct, ct * 8, cudaMemcpyDeviceToDevice, s.stream));
    } catch (...) {
      cudaStreamEndCapture(s.stream, &g);
      cudaGetLastError();
      throw;
    }
    MPASO_CUDA(cudaStreamEndCapture(s.stream, &g));
    const cudaError_t e = cudaGraphInstantiate(&A.fwd, g, 0);
    cudaGraphDestroy(g);
    MPASO_CUDA(e);
    A.fwd_N = N, A.fwd_dt = dt;
  }
  MPASO_CUDA(cudaGraphLaunch(A.fwd, s.stream));
  s.diag_valid = false;  // the taping stages wrote the state's diagnostic scratch
  A.stored_tr = with_tr;
}

void forward(SwState &s, double dt, int N, int k) {
  void tape_segment(SwState &, AdjBuffers &, int, bool, cudaStream_t);
  const bool ocean = s.p.app == MPASO_APP_OCEAN;
  require(!ocean || s.T > 0, MPASO_ERR_ARG, "the ocean app's adjoint differentiates its tracers: ntr >= 1");
  require(!s.p.pin_u, MPASO_ERR_ARG, "the adjoint does not support a pinned wind (test case 1)");
  require(N >= 1 && k >= 0, MPASO_ERR_ARG, "nsteps must be >= 1 and ckpt_every >= 0");
  const bool stored = k == 0;
  if (stored) k = N;
  ensure_buffers(s, N, k);
  AdjBuffers &A = *s.adj;
  use_tape(A, 0);
  A.stored = stored;
  if (stored) {
    A.N = N, A.k = N, A.dt = dt, A.nck = 1;
    forward_stored(s, dt, N);
    A.have_forward = true;
    return;
  }
  const DMesh &m = s.mesh->ctx.d;
  const size_t eu = (size_t)m.nE * s.L * 8, ch = (size_t)m.nC * s.L * 8;
  A.N = N, A.k = k, A.dt = dt, A.nck = (N + k - 1) / k;
  if (!ocean) {
    MPASO_CUDA(cudaMemcpyAsync(A.ck_u, s.U[0], eu, cudaMemcpyDeviceToDevice, s.stream));
    MPASO_CUDA(cudaMemcpyAsync(A.ck_h, s.H[0], ch, cudaMemcpyDeviceToDevice, s.stream));
  }
  const size_t ct = ch * s.T;
  if (s.T) MPASO_CUDA(cudaMemcpyAsync(A.ck_tr, s.TR0, ct, cudaMemcpyDeviceToDevice, s.stream));
  A.last_taped = false;
  for (int done = 0, c = 1; done < N; ++c) {
    const int n = std::min(k, N - done);
    if (done + n < N) {
      sw_steps_graph(s, dt, n);
    } else {
      // the last segment with its tape, which the reverse sweep needs first:
      // from the state through tape slots 0..4n, and the final state back
      const bool tr = s.T > 0;
      const size_t cb = ct;
      if (ocean) ocean_prepare(s, dt, s.stream);
      if (!ocean) {
        MPASO_CUDA(cudaMemcpyAsync(A.tp_u, s.U[0], eu, cudaMemcpyDeviceToDevice, s.stream));
        MPASO_CUDA(cudaMemcpyAsync(A.tp_h, s.H[0], ch, cudaMemcpyDeviceToDevice, s.stream));
      }
      if (tr) MPASO_CUDA(cudaMemcpyAsync(A.tp_tr, s.TR0, cb, cudaMemcpyDeviceToDevice, s.stream));
      tape_segment(s, A, n, tr, s.stream);
      if (!ocean) {
        MPASO_CUDA(cudaMemcpyAsync(s.U[0], A.tp_u + (size_t)4 * n * m.nE * s.L, eu, cudaMemcpyDeviceToDevice,
                                   s.stream));
        MPASO_CUDA(cudaMemcpyAsync(s.H[0], A.tp_h + (size_t)4 * n * m.nC * s.L, ch, cudaMemcpyDeviceToDevice,
                                   s.stream));
      }
      if (tr)
        MPASO_CUDA(cudaMemcpyAsync(s.TR0, A.tp_tr + (size_t)4 * n * m.nC * s.L * s.T, cb,
                                   cudaMemcpyDeviceToDevice, s.stream));
      MPASO_CUDA(cudaGetLastError());
      s.diag_valid = false;  // the state's diagnostics buffers held the tape's stages
      A.last_taped = true, A.last_tr = tr ? 1 : 0;
    }
    done += n;
    if (done < N && !ocean) {
      MPASO_CUDA(cudaMemcpyAsync(A.ck_u + (size_t)c * m.nE * s.L, s.U[0], eu, cudaMemcpyDeviceToDevice, s.stream));
      MPASO_CUDA(cudaMemcpyAsync(A.ck_h + (size_t)c * m.nC * s.L, s.H[0], ch, cudaMemcpyDeviceToDevice, s.stream));
    }
    if (done < N) {
      if (s.T)
        MPASO_CUDA(cudaMemcpyAsync(A.ck_tr + (size_t)c * m.nC * s.L * s.T, s.TR0, ct, cudaMemcpyDeviceToDevice,
                                   s.stream));
    }
  }
  A.have_forward = true;
}

// Taping run of n steps from tape slot 0 (state there already): slot 4t + rk
// receives the input of stage rk of step t, plus the stage's pv and kite-summed
// thickness, and with tracers the stage's fluxes, limiter factors, upwind sums
// and 1/hProv.  with_tr: the tracer-carrying stage kernels (else (h, u) only).
void tape_segment(SwState &s, AdjBuffers &A, int n, bool with_tr, cudaStream_t st) {
  const DMesh &m = s.mesh->ctx.d;
  const int64_t eu = (int64_t)m.nE * s.L, ch = (int64_t)m.nC * s.L;
  const int64_t cT = ch * s.T, eT = eu * s.T;
  const int64_t vv = (int64_t)m.nV * s.L;
  if (s.p.app == MPASO_APP_OCEAN) {  // tracers only, over the prescribed flux and 1/hProv
    for (int t = 0; t < n; ++t) {
      double *ytr = A.tp_tr + (size_t)4 * t * cT;
      for (int rk = 0; rk < 4; ++rk) {
        const int j = 4 * t + rk;
        Stage S = ocean_make_stage(s, rk, A.dt);
        S.tr_in = ytr + (size_t)rk * cT, S.tr_prev = ytr;
        S.tr_out = rk < 3 ? ytr + (size_t)(rk + 1) * cT : nullptr;
        S.trh_acc = A.trhacc, S.tr_new = rk == 3 ? ytr + (size_t)4 * cT : nullptr;
        S.A = A.tp_A + (size_t)j * eT, S.LO = A.tp_LO + (size_t)j * eT, S.R2 = A.tp_R2 + (size_t)j * cT;
        S.tLO = A.tp_tLO + (size_t)j * cT;
        ocean_launch_stage(s, S, st);
      }
    }
    return;
  }
  sw_diag_ptrs(s, A.tp_u, A.tp_h, A.tp_pv, A.tp_hs, st);
  for (int t = 0; t < n; ++t) {
    double *yu = A.tp_u + (size_t)4 * t * eu, *yh = A.tp_h + (size_t)4 * t * ch;
    for (int rk = 0; rk < 4; ++rk) {
      double *iu = yu + (size_t)rk * eu, *ih = yh + (size_t)rk * ch;
      double *ou = yu + (size_t)(rk + 1) * eu, *oh = yh + (size_t)(rk + 1) * ch;
      const size_t next = (size_t)(4 * t + rk + 1) * vv;  // tape slot of the stage's output
      if (!with_tr) {
        sw_stage_ptrs(s, rk, A.dt, iu, ih, yu, yh, rk < 3 ? ou : nullptr, rk < 3 ? oh : nullptr, A.uacc, A.hacc,
                      rk == 3 ? ou : nullptr, rk == 3 ? oh : nullptr, A.tp_pv + next, A.tp_hs + next,
                      A.tp_s1 + (size_t)(4 * t + rk) * eu, st);
        continue;
      }
      // with tracers: the state's own stage kernels, every pointer on the tape
      const int j = 4 * t + rk;
      double *ytr = A.tp_tr + (size_t)4 * t * cT;
      Stage S = sw_make_stage(s, rk, A.dt);
      S.u_in = iu, S.h_in = ih, S.tr_in = ytr + (size_t)rk * cT;
      S.u_prev = yu, S.h_prev = yh, S.tr_prev = ytr;
      S.u_out = rk < 3 ? ou : nullptr, S.h_out = rk < 3 ? oh : nullptr;
      S.tr_out = rk < 3 ? ytr + (size_t)(rk + 1) * cT : nullptr;
      S.u_acc = A.uacc, S.h_acc = A.hacc, S.trh_acc = A.trhacc;
      S.u_new = rk == 3 ? ou : nullptr, S.h_new = rk == 3 ? oh : nullptr;
      S.tr_new = rk == 3 ? ytr + (size_t)4 * cT : nullptr;
      S.A = A.tp_A + (size_t)j * eT, S.LO = A.tp_LO + (size_t)j * eT, S.R2 = A.tp_R2 + (size_t)j * cT;
      S.tLO = A.tp_tLO + (size_t)j * cT, S.tape_hpi = A.tp_hpi + (size_t)j * ch;
      S.tape_pv = A.tp_pv + next, S.tape_hs = A.tp_hs + next, S.tape_s1 = A.tp_s1 + (size_t)j * eu;
      sw_launch_stage(s, S, st);
    }
  }
}

void reverse_body(SwState &s) {
  AdjBuffers &A = *s.adj;
  const DMesh &m = s.mesh->ctx.d;
  const int64_t eu = (int64_t)m.nE * s.L, ch = (int64_t)m.nC * s.L;
  const int64_t cT = ch * s.T;
  const cudaStream_t st = s.stream;
  const bool ocean = s.p.app == MPASO_APP_OCEAN;
  // With two tape sets, segment seg's tape is set (nck - 1 - seg) mod 2 (the
  // last segment in set 0, where the checkpointing forward tapes it), and the
  // side stream recomputes segment seg - 1 while this stream reverses segment
  // seg: the reverse reads only its tape set and its own buffers, the
  // recompute only writes the other set and the forward's scratch, and no two
  // recomputes run at once.
  const bool dbl = A.dbl && !A.stored && A.nck > 1;
  auto set_of = [&](int seg) { return dbl ? (A.nck - 1 - seg) & 1 : 0; };
  auto recompute = [&](int seg, cudaStream_t q) {  // taping recompute of a segment from its checkpoint
    const int n = std::min(A.k, A.N - seg * A.k);
    if (!ocean) {
      MPASO_CUDA(cudaMemcpyAsync(A.tp_u, A.ck_u + (size_t)seg * eu, eu * 8, cudaMemcpyDeviceToDevice, q));
      MPASO_CUDA(cudaMemcpyAsync(A.tp_h, A.ck_h + (size_t)seg * ch, ch * 8, cudaMemcpyDeviceToDevice, q));
    }
    if (A.tr)
      MPASO_CUDA(cudaMemcpyAsync(A.tp_tr, A.ck_tr + (size_t)seg * cT, cT * 8, cudaMemcpyDeviceToDevice, q));
    tape_segment(s, A, n, A.tr != 0, q);
  };
  if (ocean) ocean_recompute(s, A.dt, st);  // the prescribed flux and 1/hProv the stages used
  for (int seg = A.nck - 1; seg >= 0; --seg) {
    const int s0 = seg * A.k, n = std::min(A.k, A.N - s0);
    const bool last = seg == A.nck - 1;
    if (!A.stored) {
      if (last) {
        use_tape(A, set_of(seg));
        if (!A.rev_skip) recompute(seg, st);
        if (dbl) {  // the side stream joins after this stream's recompute
          MPASO_CUDA(cudaEventRecord(A.ev_fork, st));
          MPASO_CUDA(cudaStreamWaitEvent(A.side, A.ev_fork, 0));
        }
      } else if (dbl) {
        MPASO_CUDA(cudaStreamWaitEvent(st, A.ev_tape, 0));  // this segment's tape, from the side stream
      } else {
        recompute(seg, st);
      }
    }
    if (dbl && seg >= 1) {
      // the next segment's tape into the set the reverse of segment seg + 1 used
      if (!last) MPASO_CUDA(cudaStreamWaitEvent(A.side, A.ev_rev, 0));
      use_tape(A, set_of(seg - 1));
      recompute(seg - 1, A.side);
      MPASO_CUDA(cudaEventRecord(A.ev_tape, A.side));
    }
    use_tape(A, set_of(seg));
    if (last) {
      // cotangents of the final state (tape slot 4n): tracers to q = h tr, then
      // the first reversed stage's lk = dt/6 lam
      if (A.tr && !ocean)
        k_adj_q_convert<<<blocks_for(ch, TPB), TPB, 0, st>>>(ch, s.T, A.tp_h + (size_t)4 * n * ch,
                                                              A.tp_tr + (size_t)4 * n * cT, A.lam_q, A.lam_h, 0);
      if (!ocean) {
        k_adj_init<<<blocks_for(eu, TPB), TPB, 0, st>>>(eu, A.lam_u, A.lk_u, A.dt / 6);
        k_adj_init<<<blocks_for(ch, TPB), TPB, 0, st>>>(ch, A.lam_h, A.lk_h, A.dt / 6);
      }
      if (A.tr)
        k_adj_init_q<<<blocks_for(cT, TPB), TPB, 0, st>>>(m, s.L, s.T, A.lam_q, A.lk_q, A.gq, A.dt / 6);
    }
    bool tra_done = false;  // TA of the next reversed stage already ran with B3
    for (int t = n - 1; t >= 0; --t)
      for (int rk = 3; rk >= 0; --rk) {
        const int j = 4 * t + rk;
        tra_done = stage_vjp(s, A, rk, j, t == n - 1 && rk == 3, j > 0, st, tra_done);
      }
    if (dbl) MPASO_CUDA(cudaEventRecord(A.ev_rev, st));
  }
  // q = h tr at the window's start (tape slot 0 of segment 0 holds checkpoint 0)
  use_tape(A, set_of(0));
  if (A.tr && !ocean)
    k_adj_q_convert<<<blocks_for(ch, TPB), TPB, 0, st>>>(ch, s.T, A.tp_h, A.tp_tr, A.lam_q, A.lam_h, 1);
  use_tape(A, 0);  // the forward tapes into set 0
  MPASO_CUDA(cudaGetLastError());
}

// The reverse sweep is ~800 launches per segment of small kernels: captured
// once as a graph for the current (N, k, dt) and buffers, then replayed.
void reverse(SwState &s) {
  AdjBuffers &A = *s.adj;
  // the forward's tape of the last segment serves one reverse sweep of the same
  // tracer mode (the sweep's recomputes overwrite it)
  const bool skip = !A.stored && A.last_taped && A.last_tr == (A.tr ? 1 : 0);
  A.last_taped = false;
  if (A.rev && (A.rev_N != A.N || A.rev_k != A.k || A.rev_dt != A.dt || A.rev_tr != A.tr ||
                A.rev_stored != A.stored || A.rev_skip != skip)) {
    cudaGraphExecDestroy(A.rev);
    A.rev = nullptr;
  }
  if (!A.rev) {
    A.rev_skip = skip;  // read by reverse_body
    cudaGraph_t g;
    MPASO_CUDA(cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeThreadLocal));
    try {
      reverse_body(s);
    } catch (...) {
      cudaStreamEndCapture(s.stream, &g);
      cudaGetLastError();
      throw;
    }
    MPASO_CUDA(cudaStreamEndCapture(s.stream, &g));
    const cudaError_t e = cudaGraphInstantiate(&A.rev, g, 0);
    cudaGraphDestroy(g);
    MPASO_CUDA(e);
    A.rev_N = A.N, A.rev_k = A.k, A.rev_dt = A.dt, A.rev_tr = A.tr, A.rev_stored = A.stored;
  }
  MPASO_CUDA(cudaGraphLaunch(A.rev, s.stream));
  s.diag_valid = false;
}

// Reference-ordered rows of `row` doubles (host or device) <-> internal order.
void to_internal(SwState &s, const double *src, double *dst, int entity, int64_t row) {
  MeshCtx &ctx = s.mesh->ctx;
  const int64_t n = entity == MPASO_CELLS ? ctx.d.nC : ctx.d.nE;
  const double *p = src;
  double *stage = nullptr;
  if (!is_device_pointer(src)) {
    MPASO_CUDA(cudaMallocAsync((void **)&stage, (size_t)n * row * 8, s.stream));
    MPASO_CUDA(cudaMemcpyAsync(stage, src, (size_t)n * row * 8, cudaMemcpyHostToDevice, s.stream));
    p = stage;
  }
  k_gather_rows_pub(p, dst, ctx.d_perm[entity], n, row, s.stream);
  if (stage) MPASO_CUDA(cudaFreeAsync(stage, s.stream));
}

void from_internal(SwState &s, const double *src, double *dst, int entity, int64_t row) {
  MeshCtx &ctx = s.mesh->ctx;
  const int64_t n = entity == MPASO_CELLS ? ctx.d.nC : ctx.d.nE;
  const bool dev = is_device_pointer(dst);
  double *out = dst;
  if (!dev) MPASO_CUDA(cudaMallocAsync((void **)&out, (size_t)n * row * 8, s.stream));
  k_scatter_rows_pub(src, out, ctx.d_perm[entity], n, row, s.stream);
  if (!dev) {
    MPASO_CUDA(cudaMemcpyAsync(dst, out, (size_t)n * row * 8, cudaMemcpyDeviceToHost, s.stream));
    MPASO_CUDA(cudaFreeAsync(out, s.stream));
  }
}

}  // namespace
}  // namespace mpaso

using namespace mpaso;

extern "C" {

int mpaso_rk4_forward(mpaso_state s, double dt, int32_t nsteps, int32_t ckpt_every) {
  return guarded("mpaso_rk4_forward", [&] {
    require(s != nullptr, MPASO_ERR_ARG, "null state");
    MPASO_CUDA(cudaSetDevice(s->s.mesh->ctx.device));
    forward(s->s, dt, nsteps, ckpt_every);
  });
}

int mpaso_rk4_vjp(mpaso_state s, const double *gh, const double *gu, double *gh0, double *gu0) {
  return guarded("mpaso_rk4_vjp", [&] {
    require(s && gh && gu && gh0 && gu0, MPASO_ERR_ARG, "null argument");
    SwState &S = s->s;
    require(S.p.app == MPASO_APP_SW, MPASO_ERR_ARG,
            "the ocean app's thickness and velocity are prescribed: use mpaso_rk4_vjp_tracers");
    require(S.adj && S.adj->have_forward, MPASO_ERR_ARG, "mpaso_rk4_vjp needs a preceding mpaso_rk4_forward");
    MPASO_CUDA(cudaSetDevice(S.mesh->ctx.device));
    to_internal(S, gu, S.adj->lam_u, MPASO_EDGES, S.L);
    to_internal(S, gh, S.adj->lam_h, MPASO_CELLS, S.L);
    S.adj->tr = 0;
    reverse(S);
    from_internal(S, S.adj->lam_u, gu0, MPASO_EDGES, S.L);
    from_internal(S, S.adj->lam_h, gh0, MPASO_CELLS, S.L);
    MPASO_CUDA(cudaStreamSynchronize(S.stream));
  });
}

int mpaso_rk4_vjp_tracers(mpaso_state s, const double *gh, const double *gu, const double *gtr, double *gh0,
                          double *gu0, double *gtr0) {
  return guarded("mpaso_rk4_vjp_tracers", [&] {
    require(s && gtr && gtr0, MPASO_ERR_ARG, "null argument");
    SwState &S = s->s;
    const bool ocean = S.p.app == MPASO_APP_OCEAN;
    require(ocean || (gh && gu && gh0 && gu0), MPASO_ERR_ARG, "null argument");
    require(S.T > 0, MPASO_ERR_ARG, "mpaso_rk4_vjp_tracers needs a state with tracers");
    require(S.adj && S.adj->have_forward, MPASO_ERR_ARG,
            "mpaso_rk4_vjp_tracers needs a preceding mpaso_rk4_forward");
    require(!S.p.fct || S.mesh->ctx.has_fct, MPASO_ERR_ARG, "FCT statics missing from the mesh");
    require(!S.adj->stored || S.adj->stored_tr, MPASO_ERR_ARG, "the stored window holds no tracers");
    MPASO_CUDA(cudaSetDevice(S.mesh->ctx.device));
    const int64_t LT = (int64_t)S.L * S.T;
    if (!ocean) {
      to_internal(S, gu, S.adj->lam_u, MPASO_EDGES, S.L);
      to_internal(S, gh, S.adj->lam_h, MPASO_CELLS, S.L);
    }
    to_internal(S, gtr, S.adj->lam_q, MPASO_CELLS, LT);
    S.adj->tr = 1;
    reverse(S);
    if (!ocean) {
      from_internal(S, S.adj->lam_u, gu0, MPASO_EDGES, S.L);
      from_internal(S, S.adj->lam_h, gh0, MPASO_CELLS, S.L);
    } else {  // prescribed fields: no cotangent is computed for them
      const MeshCtx &ctx = S.mesh->ctx;
      for (auto [p, n] : {std::make_pair(gh0, (int64_t)ctx.d.nC * S.L), std::make_pair(gu0, (int64_t)ctx.d.nE * S.L)}) {
        if (!p) continue;
        if (is_device_pointer(p))
          MPASO_CUDA(cudaMemsetAsync(p, 0, (size_t)n * 8, S.stream));
        else
          std::memset(p, 0, (size_t)n * 8);
      }
    }
    from_internal(S, S.adj->lam_q, gtr0, MPASO_CELLS, LT);
    MPASO_CUDA(cudaStreamSynchronize(S.stream));
  });
}

int mpaso_adjoint_device_bytes(mpaso_state s, int64_t *bytes) {
  return guarded("mpaso_adjoint_device_bytes", [&] {
    require(s && bytes, MPASO_ERR_ARG, "null argument");
    *bytes = s->s.adj ? (int64_t)s->s.adj->bytes : 0;
  });
}

}  // extern "C"

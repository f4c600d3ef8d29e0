// Fused RK4 tracer step of the ocean app (apps/ocean/run.cc:10-50): FCT
// horizontal advection with a prescribed velocity and layer thickness, plus
// del2 tracer mixing, on the renumbered HBM layout.
//
// The velocity and thickness never change, so the normal thickness flux
// (apps/ocean/tasks/solve.cc:40-57) and 1/hProv (solve.cc:60-97) are computed
// once per dt.  Each RK stage is then three launches:
//   K1 edges : low-order flux, anti-diffusive flux, del2 flux (solve.cc:99-167, 216-229, 328-366)
//   K2 cells : bounds, upwind tendency, limiter factors (solve.cc:194-267)
//   K3 cells : limited tendency, del2 tendency and step_tracers_forward
//              (solve.cc:269-326, 328-366, 368-399)
//
// Reference rounding.  These kernels evaluate every product, sum and quotient
// of the reference tasks in the reference's order, each rounded on its own
// (this file is compiled with -fmad=false and writes no fma), and divide where
// the reference divides.  Fusion only moves where a value is computed: an
// edge's fluxes are formed once and gathered by both cells, and a cell's
// sums run over its edges in the reference's edge order.  The only liberties
// are ones that cannot change a value: a product with a factor that is exactly
// zero is left out of a sum (x + 0 = x), a flux is added only to the one of
// flxIn / flxOut its sign selects (the other gains +0), and a clamped
// quotient whose numerator is <= 0 or >= its (positive) denominator is not
// divided out.  The result equals the reference task sequence value for value
// (signs of zero aside).  That is what the limiter needs: on tracer plateaus
// its quotient (max - upwind) / (dt flxIn / hProv + 1e-10) divides
// rounding-level differences by the regulariser, so any other rounding of the
// chain moves the step by far more than its own rounding.
#include "rk4.cuh"

namespace mpaso {
namespace {

constexpr int TPB = 256;

// Statics of the ocean kernels in the reference's rounding (written over the
// state's cpm1 / kd after build_stat):
//   cpm1[a][e] = {advCoef + 0.25 advCoef_3rd, advCoef - 0.25 advCoef_3rd}, the
//     factor coef1 + coef3 sgn of solve.cc:150-153 for sgn = +1 / -1;
//   kd[e] = meshScalingDel2 kappa dvEdge / dcEdge (solve.cc:352), divided.
__global__ void k_oc_stat(DMesh m, double kappa, double2 *cpm, double *rho) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < (int64_t)m.maxAdv * m.nE) {
    const double coef1 = m.advCoef[i], coef3 = m.advCoef3[i] * 0.25;
    cpm[i] = make_double2(coef1 + coef3, coef1 - coef3);
  }
  if (i < m.nE) rho[i] = m.meshScalingDel2[i] * kappa * m.dvEdge[i] / m.dcEdge[i];
}

// F = u hE (solve.cc:49-54); hProv = h + sum_e (dt / area) dv edgeSign F in the
// cell's edge order, 1/hProv (solve.cc:73-95).
__global__ void k_oc_prep(DMesh m, int L, const double *u, const double *h, const double *hE, double *F,
                          double *hpi, double dt) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nEL = (int64_t)m.nE * L;
  if (i < nEL) {
    F[i] = u[i] * hE[i];
    return;
  }
  i -= nEL;
  if (i >= (int64_t)m.nC * L) return;
  const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
  const int n = m.nEoC[c];
  const double dtInvAreaCell = dt / m.areaCell[c];
  double hp = h[i];
  for (int j = 0; j < n; ++j) {
    const int64_t s = (int64_t)j * m.nC + c;
    const int e = m.eoc[s];
    const double sf = dtInvAreaCell * m.dvEdge[e] * m.eocSign[s];
    const int64_t ie = (int64_t)e * L + k;
    hp += sf * (u[ie] * hE[ie]);
  }
  hpi[i] = 1.0 / hp;
}

// K1: per edge-level, for every tracer, the low-order flux LO
// (solve.cc:106-116), the high-order flux corrected for FCT, A = HO - LO
// (solve.cc:143-165, 216-229), and the del2 flux DF = hE (tr2 - tr1) rho
// (solve.cc:350-356).  NA > 0: advection stencils of exactly NA slots (pads
// carry zero coefficients), unrolled; 0: the mesh's padded width at run time.
template <int T, int NA>
__global__ void __launch_bounds__(TPB) k_oc_edges(DMesh m, DStat st, Stage S, int L) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nE * L) return;
  const int e = (int)(i / L), k = (int)(i - (int64_t)e * L);
  const int2 c = m.coe[e];
  const int64_t i1 = ((int64_t)c.x * L + k) * T, i2 = ((int64_t)c.y * L + k) * T;
  double t1[T], t2[T];
#pragma unroll
  for (int t = 0; t < T; ++t) t1[t] = S.tr_in[i1 + t], t2[t] = S.tr_in[i2 + t];
  if (S.fct) {
    const double f = S.F[i];
    const int mask = m.hoMask[(int64_t)e * m.fctLev + k];
    // wgtTmp = f mask (solve.cc:145): for a mask of 1 f itself, for 0 the zero
    // with f's sign, on the integer pipe (other masks: the product)
    const double wgt = mask == 1 ? f : mask == 0 ? bitsd(dbits(f) & kSignBit) : f * (double)mask;
    // sgnTmp = sign(f) picks the factor coef1 + coef3 sgn; where f = 0 the
    // weight wgt is a zero and so is every weightFactor, whichever is picked
    const bool neg = dlt0(f);
    double flx[T];
#pragma unroll
    for (int t = 0; t < T; ++t) flx[t] = 0.0;
    const int na = NA > 0 ? NA : m.maxAdv;
#pragma unroll
    for (int a = 0; a < na; ++a) {
      const int64_t sa = (int64_t)a * m.nE + e;
      const int cell = m.advCells[sa];
      const double2 cf = st.cpm1[sa];
      const double wf = wgt * (neg ? cf.y : cf.x);  // weightFactor (solve.cc:155)
      const double *tr = S.tr_in + ((int64_t)cell * L + k) * T;
#pragma unroll
      for (int t = 0; t < T; ++t) flx[t] += tr[t] * wf;
    }
    const double dv = m.dvEdge[e];
    // LO = dv (max(0, f) tr1 + min(0, f) tr2): one of the two products is a zero
    const bool up1 = dgt0(f);
    // tracerWeight of solve.cc:222-223 is a zero on edges whose high-order mask
    // is set (their high-order flux gains nothing); on the others the centred
    // flux, with ((mask + 1) & 1) = 1.  A branch, not a select: the mask is set
    // almost everywhere, so warps skip this work instead of issuing it
    if (!mask) {
      const double tw = (dv * 0.5) * f;
#pragma unroll
      for (int t = 0; t < T; ++t) flx[t] = flx[t] + tw * (t1[t] + t2[t]);
    }
#pragma unroll
    for (int t = 0; t < T; ++t) {
      const double lo = dv * (f * (up1 ? t1[t] : t2[t]));
      S.LO[i * T + t] = lo;
      S.A[i * T + t] = flx[t] - lo;
    }
  }
  if (S.hmix) {
    const double hr = S.hE[i];
    const double rho = st.kd[e];
#pragma unroll
    for (int t = 0; t < T; ++t) S.DF[i * T + t] = hr * (t2[t] - t1[t]) * rho;
  }
}

// min(1, max(0, num / den)) for den > 0, divided only strictly inside (0, 1):
// num <= 0 gives 0 and num >= den gives 1 exactly as the clamped quotient does.
__device__ __forceinline__ double clamp_quotient(double num, double den) {
  if (!dgt0(den)) return dclamp01(num / den);
  if (!dgt0(num)) return 0.0;
  if (!(dkey(num) < dkey(den))) return 1.0;
  return dclamp01(num / den);
}

// K2: per cell-level, for every tracer, the bounds over the cell and its
// neighbours (solve.cc:194-214), the upwind tendency and flxIn / flxOut over
// the cell's edges (solve.cc:232-249) and the limiter factors R+ / R-
// (solve.cc:251-265).  Writes R2 = {R+, R-} and tLO = the upwind tendency
// (divided by the area, as the reference's tend holds it).
template <int T, int NC>
__global__ void __launch_bounds__(TPB) k_oc_cells(DMesh m, Stage S, int L) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nC * L || !S.fct) return;
  const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
  const int n = m.nEoC[c];
  const double invAreaCell1 = m.invAreaCell[c];  // 1 / areaCell
  double trc[T], mx[T], mn[T], td[T], fi[T], fo[T];
#pragma unroll
  for (int t = 0; t < T; ++t) {
    trc[t] = S.tr_in[i * T + t];
    mx[t] = trc[t], mn[t] = trc[t], td[t] = 0.0, fi[t] = 0.0, fo[t] = 0.0;
  }
  for_slots<NC>(n, [&](int j, bool ok) {
    const int64_t s = (int64_t)j * m.nC + c;
    const int64_t in0 = ((int64_t)m.coc[s] * L + k) * T;  // pads: the cell itself
    const int64_t ie0 = ((int64_t)m.eoc[s] * L + k) * T;
    const long long sm = sign_mask(m.eocSign[s]);  // signedFactor = +-invAreaCell1
#pragma unroll
    for (int t = 0; t < T; ++t) {
      const double x = S.tr_in[in0 + t];
      mx[t] = dmax(mx[t], x);
      mn[t] = dmin(mn[t], x);
      if (ok) {
        td[t] += dflip(invAreaCell1 * S.LO[ie0 + t], sm);
        const double ax = dflip(invAreaCell1 * S.A[ie0 + t], sm);
        // flxIn += max(0, ax), flxOut += min(0, ax): one add into the sum the
        // sign selects (integer-pipe selects; a zero ax changes neither sum,
        // so none is kept), instead of an add in each of two divergent branches
        const bool in = dgt0(ax), out = dlt0(ax);
        const double acc = (in ? fi[t] : fo[t]) + ax;
        fi[t] = in ? acc : fi[t];
        fo[t] = out ? acc : fo[t];
      }
    }
  });
  const double h = S.h_in[i], hpi = S.hpi[i], dt = S.dt;
  const double eps = 1.e-10;
#pragma unroll
  for (int t = 0; t < T; ++t) {
    const double up = (trc[t] * h + dt * td[t]) * hpi;  // tracerUpwindNew
    const double mxn = up + dt * fi[t] * hpi;            // tracerMaxNew
    const double mnn = up + dt * fo[t] * hpi;            // tracerMinNew
    const double rp = clamp_quotient(mx[t] - up, (mxn - up) + eps);
    const double rm = clamp_quotient(up - mn[t], (up - mnn) + eps);
    S.R2[i * T + t] = make_double2(rp, rm);
    S.tLO[i * T + t] = td[t];
  }
}

// K3: per cell-level, for every tracer, the tendency: the upwind part, the
// limited anti-diffusive fluxes (solve.cc:270-282, 296-309) and the del2
// mixing (solve.cc:340-364), each summed over the cell's edges in order, then
// step_tracers_forward (solve.cc:368-399).  The limited flux of an edge,
// max(0, A) min(R-(c1), R+(c2)) + min(0, A) min(R+(c1), R-(c2)) with
// (c1, c2) = cells(e), is A times the one minimum its sign selects.
template <int T, int NC>
__global__ void __launch_bounds__(TPB) k_oc_final(DMesh m, Stage S, int L) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nC * L) return;
  const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
  const int n = m.nEoC[c];
  const double invAreaCell1 = m.invAreaCell[c];
  double td[T];
  double2 own[T];
#pragma unroll
  for (int t = 0; t < T; ++t) {
    td[t] = S.fct ? S.tLO[i * T + t] : 0.0;
    if (S.fct) own[t] = S.R2[i * T + t];
  }
  if (S.fct) {
    for_slots<NC>(n, [&](int j, bool ok) {
      if (!ok) return;
      const int64_t s = (int64_t)j * m.nC + c;
      const long long sm = sign_mask(m.eocSign[s]);
      const int nb = m.nbr[s];
      const bool first = nb & 1;  // c is cells(e)[0]
      const int64_t ie0 = ((int64_t)m.eoc[s] * L + k) * T, jn = ((int64_t)(nb >> 1) * L + k) * T;
#pragma unroll
      for (int t = 0; t < T; ++t) {
        const double a = S.A[ie0 + t];
        const double2 o = S.R2[jn + t];
        const double2 r1 = first ? own[t] : o, r2 = first ? o : own[t];  // {R+, R-} of c1, c2
        // one product with the minimum the sign selects (integer-pipe selects);
        // a zero flux enters as +0, whose products are the +0 the reference's
        // max(0, A) / min(0, A) terms give
        const bool pos = dgt0(a);
        const double rmin = pos ? dmin(r1.y, r2.x) : dmin(r1.x, r2.y);
        const double hl = (dgt0(a) || dlt0(a) ? a : 0.0) * rmin;
        td[t] += dflip(invAreaCell1 * hl, sm);
      }
    });
  }
  if (S.hmix) {
    for_slots<NC>(n, [&](int j, bool ok) {
      if (!ok) return;
      const int64_t s = (int64_t)j * m.nC + c;
      const long long sm = sign_mask(m.eocSign[s]);
      const int64_t ie0 = ((int64_t)m.eoc[s] * L + k) * T;
#pragma unroll
      for (int t = 0; t < T; ++t) td[t] -= dflip(S.DF[ie0 + t] * invAreaCell1, sm);
    });
  }
#pragma unroll
  for (int t = 0; t < T; ++t) {
    const int64_t j = i * T + t;
    const double cur = S.tr_prev[j];
    switch (S.stage) {  // tracersNew += w tend; tracersPrev = tracers + w_sub tend
      case 0:
        S.trh_acc[j] = cur + S.w_acc * td[t];
        S.tr_out[j] = cur + S.w_sub * td[t];
        break;
      case 3:
        S.tr_new[j] = S.trh_acc[j] + S.w_acc * td[t];
        break;
      default:
        S.trh_acc[j] = S.trh_acc[j] + S.w_acc * td[t];
        S.tr_out[j] = cur + S.w_sub * td[t];
    }
  }
}

Stage ocean_stage(SwState &s, int rk, double dt) {
  const double rk_w[4] = {dt / 6, dt / 3, dt / 3, dt / 6};  // apps/ocean/run.cc:15-16
  const double rk_sub[4] = {dt / 2, dt / 2, dt, 0};
  Stage S{};
  S.stage = rk, S.w_sub = rk_sub[rk], S.w_acc = rk_w[rk], S.dt = dt;
  S.fct = s.p.fct, S.hmix = s.p.hmix;
  double *trs[4] = {s.TR0, s.TRA, s.TRB, s.TRA};
  S.tr_in = trs[rk];
  S.tr_out = rk < 3 ? trs[rk + 1] : nullptr;
  S.tr_prev = s.TR0, S.trh_acc = s.TRH, S.tr_new = s.TR0;
  S.h_in = s.H[0], S.u_in = s.U[0];
  S.F = s.F, S.A = s.A, S.LO = s.LO, S.DF = s.DF, S.R2 = s.R2, S.tLO = s.tLO;
  S.hE = s.HE, S.hpi = s.HPI;
  return S;
}

template <int T> void ocean_stage_T(SwState &s, const Stage &S, cudaStream_t st) {
  const DMesh &m = s.mesh->ctx.d;
  const int L = s.L;
  cudaEvent_t *ev = s.prof_events;
  const int b0 = s.tune_tpb[0], b1 = s.tune_tpb[1], b2 = s.tune_tpb[2];
  if (m.maxAdv == 10 && s.tune_unroll[0])
    k_oc_edges<T, 10><<<blocks_for((int64_t)m.nE * L, b0), b0, 0, st>>>(m, s.st, S, L);
  else
    k_oc_edges<T, 0><<<blocks_for((int64_t)m.nE * L, b0), b0, 0, st>>>(m, s.st, S, L);
  if (ev) prof_mark(ev[0], st);
  const bool c6 = m.maxEoC <= 6;
  if (c6 && s.tune_unroll[1])
    k_oc_cells<T, 6><<<blocks_for((int64_t)m.nC * L, b1), b1, 0, st>>>(m, S, L);
  else
    k_oc_cells<T, 0><<<blocks_for((int64_t)m.nC * L, b1), b1, 0, st>>>(m, S, L);
  if (ev) prof_mark(ev[1], st);
  if (c6 && s.tune_unroll[2])
    k_oc_final<T, 6><<<blocks_for((int64_t)m.nC * L, b2), b2, 0, st>>>(m, S, L);
  else
    k_oc_final<T, 0><<<blocks_for((int64_t)m.nC * L, b2), b2, 0, st>>>(m, S, L);
  if (ev) prof_mark(ev[2], st);
}

}  // namespace

void ocean_create(SwState &s) {
  const DMesh &m = s.mesh->ctx.d;
  const int64_t L = s.L, T = s.T, nC = m.nC, nE = m.nE;
  std::vector<std::pair<double **, int64_t>> bufs = {
      {&s.U[0], nE * L}, {&s.H[0], nC * L}, {&s.HE, nE * L}, {&s.HPI, nC * L},
      {&s.TR0, nC * L * T}, {&s.TRA, nC * L * T}, {&s.TRB, nC * L * T}, {&s.TRH, nC * L * T},
      {&s.F, nE * L}, {&s.A, nE * L * T}, {&s.LO, nE * L * T}, {&s.DF, nE * L * T},
      {(double **)&s.R2, 2 * nC * L * T}, {&s.tLO, nC * L * T}};
  stat_buffers(s, bufs);
  alloc_arena(s, bufs);
  build_stat(s);
  const int64_t n = std::max<int64_t>((int64_t)m.maxAdv * nE, nE);
  k_oc_stat<<<blocks_for(n, TPB), TPB, 0, s.stream>>>(m, s.p.kappa, (double2 *)s.st.cpm1, (double *)s.st.kd);
  MPASO_CUDA(cudaGetLastError());
}

void ocean_recompute(SwState &s, double dt, cudaStream_t st);

void ocean_prepare(SwState &s, double dt, cudaStream_t st) {
  if (s.prep_dt != dt) ocean_recompute(s, dt, st);
}

// Thickness flux and 1/hProv of the stored (h, u), unconditionally (also from
// inside a stream capture, after new h / u were gathered in).
void ocean_recompute(SwState &s, double dt, cudaStream_t st) {
  const DMesh &m = s.mesh->ctx.d;
  k_oc_prep<<<blocks_for(((int64_t)m.nE + m.nC) * s.L, TPB), TPB, 0, st>>>(m, s.L, s.U[0], s.H[0], s.HE, s.F,
                                                                        s.HPI, dt);
  MPASO_CUDA(cudaGetLastError());
  s.prep_dt = dt;
}

void ocean_one_stage(SwState &s, int rk, double dt, cudaStream_t st) {
  const Stage S = ocean_stage(s, rk, dt);
  switch (s.T) {
    case 1: ocean_stage_T<1>(s, S, st); break;
    case 2: ocean_stage_T<2>(s, S, st); break;
    case 3: ocean_stage_T<3>(s, S, st); break;
    case 4: ocean_stage_T<4>(s, S, st); break;
    case 5: ocean_stage_T<5>(s, S, st); break;
    case 6: ocean_stage_T<6>(s, S, st); break;
    case 7: ocean_stage_T<7>(s, S, st); break;
    case 8: ocean_stage_T<8>(s, S, st); break;
    default: fail(MPASO_ERR_ARG, "ocean app needs 1..8 tracers");
  }
}

void ocean_steps(SwState &s, double dt, int nsteps, cudaStream_t st) {
  ocean_prepare(s, dt, st);
  for (int n = 0; n < nsteps; ++n)
    for (int rk = 0; rk < 4; ++rk) ocean_one_stage(s, rk, dt, st);
  MPASO_CUDA(cudaGetLastError());
}

int ocean_launches_per_step(const SwState &) { return 12; }

// A stage with the state's weights and buffers, and its launch, for callers
// that redirect some of its pointers (the adjoint's taping recompute).
Stage ocean_make_stage(SwState &s, int rk, double dt) { return ocean_stage(s, rk, dt); }
void ocean_launch_stage(SwState &s, const Stage &S, cudaStream_t st) {
  switch (s.T) {
    case 1: ocean_stage_T<1>(s, S, st); break;
    case 2: ocean_stage_T<2>(s, S, st); break;
    case 3: ocean_stage_T<3>(s, S, st); break;
    case 4: ocean_stage_T<4>(s, S, st); break;
    case 5: ocean_stage_T<5>(s, S, st); break;
    case 6: ocean_stage_T<6>(s, S, st); break;
    case 7: ocean_stage_T<7>(s, S, st); break;
    case 8: ocean_stage_T<8>(s, S, st); break;
    default: fail(MPASO_ERR_ARG, "ocean app needs 1..8 tracers");
  }
}

}  // namespace mpaso

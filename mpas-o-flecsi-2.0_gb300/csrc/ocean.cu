// Fused RK4 tracer step of the ocean app (apps/ocean/run.cc:10-50): FCT
// horizontal advection with a prescribed velocity and layer thickness, plus
// del2 tracer mixing, on the renumbered HBM layout.
//
// The velocity and thickness never change, so the normal thickness flux
// (apps/ocean/tasks/solve.cc:40-57) and 1/hProv (solve.cc:60-97) are computed
// once per dt.  Each RK stage is then three launches:
//   K1 edges : low-order flux, anti-diffusive flux, del2 flux (solve.cc:99-167, 216-229, 328-366)
//   K2 cells : bounds, upwind tendency, limiter factors (solve.cc:194-267)
//   K3 cells : limited tendency and step_tracers_forward (solve.cc:269-326, 368-399)
#include "rk4.cuh"

namespace mpaso {
namespace {

constexpr int TPB = 256;

// F = u hE; 1/hProv = 1 / (h + dt/area sum_e edgeSign dv F).
__global__ void k_oc_prep(DMesh m, DStat st, int L, const double *u, const double *h,
                          const double *hE, double *F, double *hpi, double dt) {
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
  double acc = 0.0;
  for (int j = 0; j < n; ++j) {
    const int e = m.eoc[(int64_t)j * m.nC + c];
    acc = fma(st.sdv[(int64_t)j * m.nC + c], u[(int64_t)e * L + k] * hE[(int64_t)e * L + k], acc);
  }
  hpi[i] = 1.0 / fma(dt * m.invAreaCell[c], acc, h[i]);
}

template <int T, int NA>
__global__ void __launch_bounds__(TPB) k_oc_edges(DMesh m, DStat st, Stage S, int L) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nE * L) return;
  const int e = (int)(i / L), k = (int)(i - (int64_t)e * L);
  const int2 c = m.coe[e];
  edge_tracer_fluxes<T, NA>(m, S, L, e, k, i, (int64_t)c.x * L + k, (int64_t)c.y * L + k, S.F[i], S.hE[i],
                            m.dvEdge, st.cpm1, st.kd);
}

// NC = 6: cell loops unrolled over 6 slots (meshes with at most 6 edges per cell)
template <int T, int NC>
__global__ void __launch_bounds__(TPB) k_oc_cells(DMesh m, Stage S, int L) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nC * L) return;
  const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
  cell_limiter<T, NC>(m, S, L, c, k, i, S.h_in[i], S.hpi[i]);
}

template <int T, int NC>
__global__ void __launch_bounds__(TPB) k_oc_final(DMesh m, Stage S, int L) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nC * L) return;
  const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
  double tend[T];
  cell_tracer_tend<T, NC>(m, S, L, c, k, i, tend);
#pragma unroll
  for (int t = 0; t < T; ++t) {
    const int64_t j = i * T + t;
    const double cur = S.tr_prev[j];
    switch (S.stage) {  // tracersNew += w tend; tracersPrev = tracers + w_sub tend
      case 0:
        S.trh_acc[j] = fma(S.w_acc, tend[t], cur);
        S.tr_out[j] = fma(S.w_sub, tend[t], cur);
        break;
      case 3:
        S.tr_new[j] = fma(S.w_acc, tend[t], S.trh_acc[j]);
        break;
      default:
        S.trh_acc[j] = fma(S.w_acc, tend[t], S.trh_acc[j]);
        S.tr_out[j] = fma(S.w_sub, tend[t], cur);
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
  if (ev) MPASO_CUDA(cudaEventRecord(ev[0], st));
  const bool c6 = m.maxEoC <= 6;
  if (c6 && s.tune_unroll[1])
    k_oc_cells<T, 6><<<blocks_for((int64_t)m.nC * L, b1), b1, 0, st>>>(m, S, L);
  else
    k_oc_cells<T, 0><<<blocks_for((int64_t)m.nC * L, b1), b1, 0, st>>>(m, S, L);
  if (ev) MPASO_CUDA(cudaEventRecord(ev[1], st));
  if (c6 && s.tune_unroll[2])
    k_oc_final<T, 6><<<blocks_for((int64_t)m.nC * L, b2), b2, 0, st>>>(m, S, L);
  else
    k_oc_final<T, 0><<<blocks_for((int64_t)m.nC * L, b2), b2, 0, st>>>(m, S, L);
  if (ev) MPASO_CUDA(cudaEventRecord(ev[2], st));
}

}  // namespace

void ocean_create(SwState &s) {
  const DMesh &m = s.mesh->ctx.d;
  const int64_t L = s.L, T = s.T, nC = m.nC, nE = m.nE, nV = m.nV;
  std::vector<std::pair<double **, int64_t>> bufs = {
      {&s.U[0], nE * L}, {&s.H[0], nC * L}, {&s.HE, nE * L}, {&s.HPI, nC * L},
      {&s.TR0, nC * L * T}, {&s.TRA, nC * L * T}, {&s.TRB, nC * L * T}, {&s.TRH, nC * L * T},
      {&s.F, nE * L}, {&s.A, nE * L * T}, {&s.LO, nE * L * T}, {&s.DF, nE * L * T},
      {(double **)&s.R2, 2 * nC * L * T}, {&s.tLO, nC * L * T}};
  stat_buffers(s, bufs);
  alloc_arena(s, bufs);
  build_stat(s);
}

void ocean_recompute(SwState &s, double dt, cudaStream_t st);

void ocean_prepare(SwState &s, double dt, cudaStream_t st) {
  if (s.prep_dt != dt) ocean_recompute(s, dt, st);
}

// Thickness flux and 1/hProv of the stored (h, u), unconditionally (also from
// inside a stream capture, after new h / u were gathered in).
void ocean_recompute(SwState &s, double dt, cudaStream_t st) {
  const DMesh &m = s.mesh->ctx.d;
  k_oc_prep<<<blocks_for(((int64_t)m.nE + m.nC) * s.L, TPB), TPB, 0, st>>>(m, s.st, s.L, s.U[0], s.H[0],
                                                                        s.HE, s.F, s.HPI, dt);
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

// Fused RK4 path of the sw app (apps/sw/run.cc:13-70) with the FCT tracer
// coupling, del2 tracer mixing and del2 momentum, on the renumbered HBM layout.
//
// Per RK stage three launches, no copies:
//   K1 edge pre-pass   : thickness flux F = u h_e, F pv_e, FCT low/high-order
//                        fluxes -> anti-diffusive flux A, del2 tracer flux
//                        (apps/ocean/tasks/solve.cc:40-167, 216-229, 328-366);
//   K2 edges + cells   : tend_u from edgesOnEdge x weightsOnEdge, KE and
//                        geopotential gradient (apps/sw/tasks/solve.cc:215-233),
//                        u update; tend_h (solve.cc:185-206), h update, FCT
//                        bounds and limiter factors (ocean solve.cc:194-267);
//   K3 cells + vertices: limited fluxes -> tracer tendency (ocean solve.cc:
//                        269-326), thickness-weighted tracer update
//                        (sw solve.cc:273-367), then the diagnostics of the next
//                        stage's state (sw solve.cc:11-107).
// The state rotates through four buffers per field, so the step needs no
// init_provis / setup_timestep / timeshift copies.
//
// GB300 executes FP64 at ~1/64 of its FP32 rate, so these kernels are bound by
// FP64 issue: multiplications by +-1 are sign-bit flips, min/max/clamp/
// upwind selection are integer operations on the bit patterns, divisions by
// static quantities use precomputed reciprocals, and the dynamic ones use
// rcp_nr.  Results match the reference task sequence to rounding (about 1e-15
// relative per step), not bit for bit.
#include <cstring>
#include <map>
#include <mutex>
#include <utility>

#include "rk4.cuh"

namespace mpaso {
namespace {

constexpr int TPB = 256;
// Launch-shape variants of the stage kernels (picked per mesh by the autotuner):
// NW = 10: edgesOnEdge and advection stencils of exactly 10 slots (hexagon /
// pentagon meshes), unrolled at compile time; NW = 0: runtime widths.
// OC = 1: registers capped at 40 so 1536 threads fit an SM (more warps to hide
// gather latency, less ILP per warp); OC = 0: the compiler's choice.
constexpr int kOccMaxT = 1;  // OC = 1 variants exist up to this many tracers (beyond, they spill)
constexpr int kLanesMaxT = 1;  // variants with 2 or 4 lanes per edge exist up to this many tracers
#define MPASO_BOUNDS(OC) __launch_bounds__(TPB, (OC) ? 1536 / TPB : 0)


// ------------------------------------------------------------- K1: edges
// One edge-level of the pre-pass.  RO: inputs through the read-only path
// (false inside the persistent kernel).
template <int T, int NW, bool RO>
__device__ __forceinline__ void edge_pre_item(const DMesh &m, const DStat &st, const Stage &S, int L, int64_t i) {
  const int e = (int)(i / L), k = (int)(i - (int64_t)e * L);
  const int2 c = __ldcs(&m.coe[e]);
  const int2 v = __ldcs(&m.voe[e]);
  const int64_t i1 = (int64_t)c.x * L + k, i2 = (int64_t)c.y * L + k;
  const double hs = ld_in<RO>(&S.h_in[i1]) + ld_in<RO>(&S.h_in[i2]);  // 2 h_edge
  const double F = ld_in<RO>(&S.u_in[i]) * hs;                         // 2 u h_edge
  const double pv2 = ld_in<RO>(&S.pv[(int64_t)v.x * L + k]) + ld_in<RO>(&S.pv[(int64_t)v.y * L + k]);  // 2 pv_edge
  S.FG[i] = make_double2(F, F * pv2);
  S.pve[i] = pv2;
  if constexpr (T > 0) edge_tracer_fluxes<T, NW, RO>(m, S, L, e, k, i, i1, i2, F, hs, st.dvh, st.cpm2, st.kdh);
}

template <int T, int NW, int OC>
__global__ void MPASO_BOUNDS(OC) k_sw_edge_pre(DMesh m, DStat st, Stage S, int L) {
  stage_prologue();
  // grid-stride over edge-levels: launched on at most the blocks the SMs hold
  // at once, so the work ends without a partial last wave (measured 37.4 ->
  // 36.0 us at level 7; the mixed edge / cell kernels below lost this way)
  const int64_t nEL = (int64_t)m.nE * L;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nEL; i += (int64_t)gridDim.x * blockDim.x)
    edge_pre_item<T, NW, true>(m, st, S, L, i);
}

// ------------------------------------------------------ K2: edges + cells
// SPLIT = 1 (the four-launch schedule): K1 computed only F, F Pv and Pv_e; the
// edge threads here add the tracer fluxes (their stencil gathers overlap the
// TRiSK arithmetic) and the cell threads leave the limiter, which needs every
// edge's fluxes, to k_sw_limit.  Same arithmetic either way.
// LANES (1, 2 or 4) threads per edge-level share its TRiSK stencil: lane j
// sums slots j, j + LANES, ..., and the partial sums meet by warp shuffles
// (the sum is reassociated, so results differ in the last bits).  More lanes
// mean more FP64 issue per edge (the edge's own arithmetic runs on every lane)
// but more gathers in flight; they pay only where the mesh is too small to
// fill the GPU, which the autotuner measures.
template <int LANES> __device__ __forceinline__ double lane_total(double x) {
  if constexpr (LANES > 1) {
    const unsigned grp = (LANES == 2 ? 0x3u : 0xfu) << (threadIdx.x & 31 & ~(LANES - 1));
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1) x += __shfl_xor_sync(grp, x, o);
  }
  return x;
}

template <int T, int NW, int SPLIT, int LANES = 1>
__device__ __forceinline__ void tend_item(const DMesh &m, const DStat &st, const Stage &S, int L, int64_t i) {
  const int64_t nEL = (int64_t)m.nE * L;
  if (i < nEL * LANES) {
    const int lane = (int)(i & (LANES - 1));
    i /= LANES;
    const int e = (int)(i / L), k = (int)(i - (int64_t)e * L);
    // q = sum_j W_j F_j (pv_e + pv_j) / 2 = (Pv_e sum W/8 F2_j + sum W/8 F2_j Pv_j)
    double s1 = 0.0, s2 = 0.0;
    const int ne = NW > 0 ? NW : m.maxEoE;
#pragma unroll
    for (int j = lane; j < ne; j += LANES) {
      const int eo = __ldcs(&m.eoe[(int64_t)j * m.nE + e]);
      const double w = __ldcs(&st.woe8[(int64_t)j * m.nE + e]);
      const int64_t io = (int64_t)eo * L + k;
      const double2 fg = S.FG[io];
      s1 = fma(w, fg.x, s1);
      s2 = fma(w, fg.y, s2);
    }
    s1 = lane_total<LANES>(s1);
    s2 = lane_total<LANES>(s2);
    if (lane) return;
    const double q = fma(S.pve[i], s1, s2);
    if (S.tape_s1) S.tape_s1[i] = s1;
    const int2 c = m.coe[e];
    const int64_t i1 = (int64_t)c.x * L + k, i2 = (int64_t)c.y * L + k;
    // - (ke2 - ke1 + g (h2 + b2 - h1 - b1)) / dc + nu (div2 - div1) / dc, with the
    // kinetic and divergence parts as one difference of kdiv = ke - nu div; the
    // geopotential stays a thickness difference, exact where h is uniform
    const double h1 = S.h_in[i1], h2 = S.h_in[i2];
    const double dh = (h2 - h1) + st.dhs[e];
    double tend = fma(-m.invDcEdge[e], fma(S.g, dh, S.bern[i2] - S.bern[i1]), q);
    if (S.visc) {  // - nu (vort_b - vort_a) / dv
      const int2 v = m.voe[e];
      tend = fma(-st.nuDv[e], S.vort[(int64_t)v.y * L + k] - S.vort[(int64_t)v.x * L + k], tend);
    }
    const double up = S.u_prev[i];
    switch (S.stage) {
      case 0:
        S.u_out[i] = S.pin_u ? up : fma(S.w_sub, tend, up);
        S.u_acc[i] = fma(S.w_acc, tend, up);
        break;
      case 3:
        S.u_new[i] = S.pin_u ? up : fma(S.w_acc, tend, S.u_acc[i]);
        break;
      default:
        S.u_out[i] = S.pin_u ? up : fma(S.w_sub, tend, up);
        S.u_acc[i] = fma(S.w_acc, tend, S.u_acc[i]);
    }
    if constexpr (SPLIT && T > 0)
      edge_tracer_fluxes<T, NW>(m, S, L, e, k, i, i1, i2, S.FG[i].x, h1 + h2, st.dvh, st.cpm2, st.kdh);
    return;
  }
  i -= nEL * LANES;
  if (i >= (int64_t)m.nC * L) return;
  constexpr int NC = NW > 0 ? 6 : 0;  // the unrolled variant also unrolls the cell loops
  const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
  const int n = m.nEoC[c];
  double tend_h = 0.0;  // sum edgeSign dv F / area, from F2 with the halved weights (0 in pads)
  for_slots<NC>(n, [&](int j, bool) {
    const int64_t s = (int64_t)j * m.nC + c;
    tend_h = fma(st.sdvi[s], S.FG[(int64_t)m.eoc[s] * L + k].x, tend_h);
  });
  const double hp = S.h_prev[i];
  switch (S.stage) {
    case 0:
      S.h_out[i] = fma(S.w_sub, tend_h, hp);
      S.h_acc[i] = fma(S.w_acc, tend_h, hp);
      break;
    case 3:
      S.h_new[i] = fma(S.w_acc, tend_h, S.h_acc[i]);
      break;
    default:
      S.h_out[i] = fma(S.w_sub, tend_h, hp);
      S.h_acc[i] = fma(S.w_acc, tend_h, S.h_acc[i]);
  }
  if constexpr (T > 0) {
    // provisional thickness (apps/ocean/tasks/solve.cc:60-97): h + dt tend_h
    const double hin = S.h_in[i];
    const double hpi = S.fct ? rcp_nr(fma(S.dt, tend_h, hin)) : 0.0;
    if (S.tape_hpi) S.tape_hpi[i] = hpi;
    if constexpr (SPLIT)
      S.hpw[i] = hpi;
    else
      cell_limiter<T, NC>(m, S, L, c, k, i, hin, hpi);
  }
}

template <int T, int NW, int OC, int SPLIT, int LANES = 1>
__global__ void MPASO_BOUNDS(OC) k_sw_tend(DMesh m, DStat st, Stage S, int L) {
  stage_prologue();
  tend_item<T, NW, SPLIT, LANES>(m, st, S, L, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// Limiter kernel of the four-launch schedule: bounds, upwind tendency and
// R+- of every cell from the fluxes k_sw_tend<.., SPLIT = 1> wrote.
template <int T, int NC, int OC>
__global__ void MPASO_BOUNDS(OC) k_sw_limit(DMesh m, Stage S, int L) {
  stage_prologue();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nC * L) return;
  const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
  cell_limiter<T, NC>(m, S, L, c, k, i, S.h_in[i], S.hpw[i]);
}

// Diagnostics of a state (u, h): at cells kdiv = ke - nu div, whose edge
// difference / dcEdge is the kinetic-energy gradient of tend_u
// (apps/sw/tasks/solve.cc:228-231) plus the divergence part of del2
// momentum; vorticity and pv at vertices.  CellDiag accumulates the edge sums
// of one cell (ke, the divergence numerator) slot by slot.  (Folding g (h + b)
// into the same cell function would save two more instructions per edge but
// leaves an absolute error floor of ulp(g h) / dcEdge in tend_u, which breaks
// the relative parity bar for slow flows.)
struct CellDiag {
  const DStat &st;
  const Stage &S;
  const double *u;
  int L, k;
  double ke = 0.0, dv = 0.0;
  __device__ void operator()(int64_t s, int e, bool valid) {
    const double ue = u[(int64_t)e * L + k];
    const double kn = fma(st.kw[e], ue * ue, ke);
    ke = valid ? kn : ke;
    if (S.visc) dv = fma(st.sdv[s], ue, dv);  // sdv is 0 in pad slots
  }
  __device__ void finish(const DMesh &m, int c, int64_t i) const {
    double b = ke * m.invAreaCell[c];
    // sdv = edgeSignOnCell dv is inward-positive: div = -dv / area, -nu div = nu dv / area
    if (S.visc) b = fma(st.nuInva[c], dv, b);
    S.bern[i] = b;
  }
};

template <int NC>
__device__ __forceinline__ void cell_diag(const DMesh &m, const DStat &st, const Stage &S, int L,
                                          int c, int k, int64_t i, const double *u) {
  CellDiag d{st, S, u, L, k};
  for_slots<NC>(m.nEoC[c], [&](int j, bool ok) {
    const int64_t s = (int64_t)j * m.nC + c;
    d(s, m.eoc[s], ok);
  });
  d.finish(m, c, i);
}

__device__ __forceinline__ void vertex_diag(const DMesh &m, const DStat &st, const Stage &S, int L,
                                            int v, int k, int64_t i, const double *u,
                                            const double *h) {
  double circ = 0.0, hs = 0.0;
#pragma unroll
  for (int j = 0; j < kVertexDegree; ++j) {
    const int64_t s = (int64_t)j * m.nV + v;
    circ = fma(st.sdc[s], u[(int64_t)m.eov[s] * L + k], circ);
    hs = fma(m.kite[s], h[(int64_t)m.cov[s] * L + k], hs);
  }
  S.vort[i] = circ * m.invAreaTriangle[v];
  // (f + circ/A) / (hs/A) = (f A + circ) / hs
  const double pv = fma(m.fVertex[v], m.areaTriangle[v], circ) * rcp_nr(hs);
  S.pv[i] = pv;
  if (S.tape_pv) S.tape_pv[i] = pv, S.tape_hs[i] = hs;
}

// ------------------------------------------------------ K3: cells + vertices
template <int T, int NC>
__device__ __forceinline__ void final_item(const DMesh &m, const DStat &st, const Stage &S, int L, int64_t i) {
  const int64_t nCL = (int64_t)m.nC * L;
  const double *u_next = S.stage == 3 ? S.u_new : S.u_out;
  const double *h_next = S.stage == 3 ? S.h_new : S.h_out;
  if (i < nCL) {
    const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
    if constexpr (T > 0) {
      const double hn = h_next[i];
      // one pass over the cell's edges: tracer tendency and the next state's diagnostics
      CellDiag d{st, S, u_next, L, k};
      double tend[T];
      cell_tracer_tend<T, NC>(m, S, L, c, k, i, tend, d);
      d.finish(m, c, i);
      const double rh = rcp_nr(hn);
      const double hpv = S.h_prev[i];
#pragma unroll
      for (int t = 0; t < T; ++t) {
        // thickness-weighted tracer RK (apps/sw/tasks/solve.cc:162, 300-302, 337, 354)
        const double hp_tp = hpv * S.tr_prev[i * T + t];
        switch (S.stage) {
          case 0:
            S.tr_out[i * T + t] = fma(S.w_sub, tend[t], hp_tp) * rh;
            S.trh_acc[i * T + t] = fma(S.w_acc, tend[t], hp_tp);
            break;
          case 3:
            S.tr_new[i * T + t] = fma(S.w_acc, tend[t], S.trh_acc[i * T + t]) * rh;
            break;
          default:
            S.tr_out[i * T + t] = fma(S.w_sub, tend[t], hp_tp) * rh;
            S.trh_acc[i * T + t] = fma(S.w_acc, tend[t], S.trh_acc[i * T + t]);
        }
      }
    } else {
      cell_diag<NC>(m, st, S, L, c, k, i, u_next);
    }
    return;
  }
  i -= nCL;
  if (i >= (int64_t)m.nV * L) return;
  const int v = (int)(i / L), k = (int)(i - (int64_t)v * L);
  vertex_diag(m, st, S, L, v, k, i, u_next, h_next);
}

template <int T, int NC, int OC>
__global__ void MPASO_BOUNDS(OC) k_sw_final(DMesh m, DStat st, Stage S, int L) {
  stage_prologue();
  final_item<T, NC>(m, st, S, L, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// Initial diagnostics (apps/sw/run.cc:88-92).
// NC = 6: the cell loops unrolled for meshes of at most hexagons (as k_sw_final's unrolled variant)
template <int NC>
__global__ void __launch_bounds__(TPB) k_sw_diag(DMesh m, DStat st, Stage S, int L) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nCL = (int64_t)m.nC * L;
  if (i < nCL) {
    const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
    cell_diag<NC>(m, st, S, L, c, k, i, S.u_in);
    return;
  }
  i -= nCL;
  if (i >= (int64_t)m.nV * L) return;
  const int v = (int)(i / L), k = (int)(i - (int64_t)v * L);
  vertex_diag(m, st, S, L, v, k, i, S.u_in, S.h_in);
}

// ------------------------------------------------- persistent RK4 steps
// The whole run in one cooperative launch: every block of a grid the SMs hold
// at once loops over the steps, the RK stages and the three phases of a stage
// (the work of K1, K2, K3 above, grid-stride over the union of all members'
// entities), with a grid barrier between phases.  Loads of values an earlier
// phase wrote are plain (coherent) loads.
struct StageSet {
  Stage s[4];
};

// Grid barrier state: count[0] counts arrivals, count[1] is the error flag.
// Every wait is bounded: after `spin` polls it sets the flag and gives up,
// and a waiting block gives up as soon as it sees the flag, so the launch
// always ends.  `extra` arrivals beyond the grid are waited for too: 0 in use,
// > 0 only to make the waits run out on purpose (the test of the bound).
struct GridBar {
  unsigned int *count;
  long long spin;
  unsigned int extra;
};

__device__ bool grid_barrier(const GridBar &b, unsigned int &phase) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int *cnt = b.count;
    const unsigned int target = (phase + 1) * (gridDim.x + b.extra);
    __threadfence();  // this block's writes before the arrival
    atomicAdd(b.count, 1u);
    long long polls = 0;
    while (cnt[0] < target) {
      if (cnt[1] || ++polls > b.spin) {
        atomicExch(b.count + 1, 1u);
        break;
      }
      __nanosleep(64);
    }
    __threadfence();  // the other blocks' writes after it
  }
  __syncthreads();
  ++phase;
  return ((volatile unsigned int *)b.count)[1] == 0;
}

template <int T, int NW, int NC>
__global__ void __launch_bounds__(TPB) k_sw_persistent(DMesh m, DStat st, StageSet P, int L, int nsteps,
                                                       GridBar b) {
  unsigned int phase = 0;
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, nt = (int64_t)gridDim.x * blockDim.x;
  const int64_t n1 = (int64_t)m.nE * L, n2 = ((int64_t)m.nE + m.nC) * L, n3 = ((int64_t)m.nC + m.nV) * L;
  for (int step = 0; step < nsteps; ++step)
    for (int rk = 0; rk < 4; ++rk) {
      const Stage &S = P.s[rk];
      for (int64_t i = tid; i < n1; i += nt) edge_pre_item<T, NW, false>(m, st, S, L, i);
      if (!grid_barrier(b, phase)) return;
      for (int64_t i = tid; i < n2; i += nt) tend_item<T, NW, 0>(m, st, S, L, i);
      if (!grid_barrier(b, phase)) return;
      for (int64_t i = tid; i < n3; i += nt) final_item<T, NC>(m, st, S, L, i);
      if (!grid_barrier(b, phase)) return;
    }
}

// Derived statics of a state.
struct StatOut {
  double *sdv, *sdvi, *kw, *sdc, *dhs, *kd, *kdh, *dvh, *woe8;
  double2 *cpm2, *cpm1;
  double *nuInva, *nuDv;
};

__global__ void k_build_stat(DMesh m, double kappa, double nu, StatOut o) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < (int64_t)m.maxEoC * m.nC) {
    const int c = (int)(i % m.nC), j = (int)(i / m.nC);
    const double s = j < m.nEoC[c] ? m.eocSign[i] * m.dvEdge[m.eoc[i]] : 0.0;
    o.sdv[i] = s;
    o.sdvi[i] = 0.5 * s * m.invAreaCell[c];
  }
  if (i < m.nC) o.nuInva[i] = nu * m.invAreaCell[i];
  if (i < m.nE) {
    o.kw[i] = 0.25 * m.dcEdge[i] * m.dvEdge[i];
    const int2 c = m.coe[i];
    o.dhs[i] = m.bottomDepth[c.y] - m.bottomDepth[c.x];
    const double kd = m.meshScalingDel2[i] * kappa * m.dvEdge[i] * m.invDcEdge[i];
    o.kd[i] = kd;
    o.kdh[i] = 0.5 * kd;
    o.dvh[i] = 0.5 * m.dvEdge[i];
    o.nuDv[i] = nu * m.invDvEdge[i];
  }
  if (i < (int64_t)m.maxEoE * m.nE) o.woe8[i] = 0.125 * m.woe[i];
  if (i < (int64_t)m.maxAdv * m.nE) {
    o.cpm1[i] = make_double2(m.advCp[i], m.advCm[i]);
    o.cpm2[i] = make_double2(0.5 * m.advCp[i], 0.5 * m.advCm[i]);
  }
  if (i < (int64_t)kVertexDegree * m.nV) o.sdc[i] = m.eovSign[i] * m.dcEdge[m.eov[i]];
}

// Smallest index of a NaN or infinity in x[0, n) (exponent bits all set;
// integer pipe only), or first left as it was.
__global__ void k_first_nonfinite(const double *x, int64_t n, unsigned long long *first) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if ((__double_as_longlong(x[i]) & 0x7ff0000000000000LL) == 0x7ff0000000000000LL)
      atomicMin(first, (unsigned long long)i);
}

}  // namespace

// ------------------------------------------------------------ state context
SwState::~SwState() {
  if (graph) cudaGraphExecDestroy(graph);
  if (xg) cudaGraphExecDestroy(xg);
  for (auto &x : x_side)
    if (x) cudaStreamDestroy(x);
  for (auto &e : x_ev)
    if (e) cudaEventDestroy(e);
  if (out_stream) cudaStreamSynchronize(out_stream);
  for (int b = 0; b < 2; ++b) {
    if (out_buf[b]) cudaFree(out_buf[b]);
    if (out_read[b]) cudaEventDestroy(out_read[b]);
    if (out_done[b]) cudaEventDestroy(out_done[b]);
  }
  if (out_ready) cudaEventDestroy(out_ready);
  if (out_stream) cudaStreamDestroy(out_stream);
  if (io_stage) cudaFree(io_stage);
  if (aux) cudaFree(aux);
  if (pbar) cudaFree(pbar);
  if (tune_l2) {  // hand the persisting L2 lines back
    cudaCtxResetPersistingL2Cache();
    cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0);
  }
  free_adjoint(*this);
  if (arena) cudaFree(arena);
}

void alloc_arena(SwState &s, std::vector<std::pair<double **, int64_t>> &bufs) {
  size_t total = 0;
  for (auto &b : bufs) total += ((size_t)std::max<int64_t>(b.second, 1) * 8 + 255) & ~size_t(255);
  if (cudaMalloc(&s.arena, total) != cudaSuccess) {
    cudaGetLastError();
    fail(MPASO_ERR_ALLOC, "device allocation of the state failed (" + std::to_string(total) + " bytes)");
  }
  s.arena_bytes = total;
  MPASO_CUDA(cudaMemsetAsync(s.arena, 0, total, s.stream));
  char *p = (char *)s.arena;
  for (auto &b : bufs) {
    *b.first = (double *)p;
    p += ((size_t)std::max<int64_t>(b.second, 1) * 8 + 255) & ~size_t(255);
  }
}

void build_stat(SwState &s) {
  const DMesh &m = s.mesh->ctx.d;
  const int64_t nmax = std::max<int64_t>(std::max<int64_t>(m.nE, 3LL * m.nV), (int64_t)m.maxEoC * m.nC);
  const int64_t nmax2 = std::max<int64_t>(nmax, std::max<int64_t>((int64_t)m.maxEoE * m.nE,
                                                                  (int64_t)m.maxAdv * m.nE));
  StatOut o{(double *)s.st.sdv, (double *)s.st.sdvi, (double *)s.st.kw, (double *)s.st.sdc,
            (double *)s.st.dhs, (double *)s.st.kd, (double *)s.st.kdh, (double *)s.st.dvh,
            (double *)s.st.woe8, (double2 *)s.st.cpm2, (double2 *)s.st.cpm1, (double *)s.st.nuInva,
            (double *)s.st.nuDv};
  k_build_stat<<<blocks_for(nmax2, TPB), TPB, 0, s.stream>>>(m, s.p.kappa, s.p.nu, o);
  MPASO_CUDA(cudaGetLastError());
}

// The derived statics of a state, as (pointer, doubles) arena entries.
void stat_buffers(SwState &s, std::vector<std::pair<double **, int64_t>> &bufs) {
  const DMesh &m = s.mesh->ctx.d;
  const int64_t nC = m.nC, nE = m.nE, nV = m.nV;
  DStat &t = s.st;
  auto P = [](const double *&p) { return (double **)&p; };
  bufs.insert(bufs.end(), {{P(t.sdv), (int64_t)m.maxEoC * nC}, {P(t.sdvi), (int64_t)m.maxEoC * nC},
                           {P(t.kw), nE}, {P(t.sdc), 3 * nV}, {P(t.dhs), nE}, {P(t.kd), nE},
                           {P(t.kdh), nE}, {P(t.dvh), nE}, {P(t.woe8), (int64_t)m.maxEoE * nE},
                           {(double **)&t.cpm2, 2LL * m.maxAdv * nE},
                           {(double **)&t.cpm1, 2LL * m.maxAdv * nE}, {P(t.nuInva), nC}, {P(t.nuDv), nE}});
}

namespace {

Stage make_stage(SwState &s, int rk, double dt) {
  const double rk_w[4] = {dt / 6, dt / 3, dt / 3, dt / 6};  // apps/sw/run.cc:23-24
  const double rk_sub[4] = {dt / 2, dt / 2, dt, 0};
  Stage S{};
  S.stage = rk, S.w_sub = rk_sub[rk], S.w_acc = rk_w[rk], S.dt = dt, S.g = s.p.gravity, S.nu = s.p.nu;
  S.fct = s.p.fct, S.hmix = s.p.hmix, S.visc = s.p.nu != 0.0, S.pin_u = s.p.pin_u, S.centred = !s.p.fct;
  // buffer rotation: prev = 0, acc = 2, stage inputs 0 -> 1 -> 3 -> 1, new -> 0
  static const int uin[4] = {0, 1, 3, 1}, uout[4] = {1, 3, 1, -1};
  S.u_in = s.U[uin[rk]], S.h_in = s.H[uin[rk]];
  S.u_prev = s.U[0], S.h_prev = s.H[0], S.tr_prev = s.TR0;
  S.u_out = uout[rk] >= 0 ? s.U[uout[rk]] : nullptr;
  S.h_out = uout[rk] >= 0 ? s.H[uout[rk]] : nullptr;
  double *trs[4] = {s.TR0, s.TRA, s.TRB, s.TRA};
  S.tr_in = trs[rk];
  S.tr_out = rk < 3 ? trs[rk + 1] : nullptr;
  S.u_acc = s.U[2], S.h_acc = s.H[2], S.trh_acc = s.TRH;
  S.u_new = s.U[0], S.h_new = s.H[0], S.tr_new = s.TR0;
  S.pv = s.pv, S.vort = s.vort, S.bern = s.bern;
  S.FG = s.FG, S.pve = s.pve, S.A = s.A, S.LO = s.LO, S.DF = s.DF;
  S.R2 = s.R2, S.tLO = s.tLO, S.hpw = s.HPW;
  return S;
}

// Launch of a stage kernel, with the state's L2 persistence window attached
// when `win` and programmatic dependent launch when the state enables it
// (both travel into captured graphs with the launch).
template <class... A>
void launch_ex(void (*kern)(A...), int64_t n, int b, bool win, const SwState &s, cudaStream_t st,
               DMesh m, DStat d, Stage S, int L) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks_for(n, b));
  cfg.blockDim = dim3(b);
  cfg.stream = st;
  cudaLaunchAttribute at[2];
  unsigned na = 0;
  if (win) {
    at[na].id = cudaLaunchAttributeAccessPolicyWindow;
    at[na++].val.accessPolicyWindow = s.l2win;
  }
  if (s.tune_pdl) {
    at[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[na++].val.programmaticStreamSerializationAllowed = 1;
  }
  cfg.attrs = na ? at : nullptr;
  cfg.numAttrs = na;
  MPASO_CUDA(cudaLaunchKernelEx(&cfg, kern, m, d, S, L));
}

// Blocks of `b` threads of `kern` that one SM holds at once (cached per
// kernel and block size: the query is not free and launches repeat).
template <class K> int resident_blocks(K kern, int b) {
  static std::mutex mu;
  static std::map<std::pair<const void *, int>, int> cache;
  const auto key = std::make_pair((const void *)kern, b);
  std::lock_guard<std::mutex> g(mu);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  int nb = 0;
  MPASO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, b, 0));
  return cache[key] = std::max(nb, 1);
}

template <int T, int OC>
void launch_k1(const SwState &s, const Stage &S, bool unroll, int b, cudaStream_t st) {
  const DMesh &m = s.mesh->ctx.d;
  const int64_t n = (int64_t)m.nE * s.L;
  const bool win = s.tune_l2 == 1;
  auto kern = unroll ? k_sw_edge_pre<T, 10, OC> : k_sw_edge_pre<T, 0, OC>;
  // the grid-stride kernel runs on exactly the threads the SMs hold at once
  const int64_t nres = std::min<int64_t>(n, (int64_t)s.mesh->ctx.sms * resident_blocks(kern, b) * b);
  launch_ex(kern, nres, b, win, s, st, m, s.st, S, s.L);
}

template <int T, int OC, int SPLIT, int LANES>
void launch_k2_lanes(const SwState &s, const Stage &S, bool unroll, int b, cudaStream_t st) {
  const DMesh &m = s.mesh->ctx.d;
  const int64_t n = ((int64_t)m.nE * LANES + m.nC) * s.L;
  const bool win = s.tune_l2 == 2;
  if (unroll)
    launch_ex(k_sw_tend<T, 10, OC, SPLIT, LANES>, n, b, win, s, st, m, s.st, S, s.L);
  else
    launch_ex(k_sw_tend<T, 0, OC, SPLIT, LANES>, n, b, win, s, st, m, s.st, S, s.L);
}

template <int T, int OC, int SPLIT>
void launch_k2(const SwState &s, const Stage &S, bool unroll, int b, cudaStream_t st) {
  const DMesh &m = s.mesh->ctx.d;
  // several lanes per edge: the three-launch schedule with at most one tracer
  if constexpr (!SPLIT && T <= kLanesMaxT) {
    if (s.tune_lanes == 2) return launch_k2_lanes<T, OC, 0, 2>(s, S, unroll, b, st);
    if (s.tune_lanes == 4) return launch_k2_lanes<T, OC, 0, 4>(s, S, unroll, b, st);
  }
  launch_k2_lanes<T, OC, SPLIT, 1>(s, S, unroll, b, st);
  if constexpr (SPLIT && T > 0) {
    const int64_t nc = (int64_t)m.nC * s.L;
    if (unroll)
      launch_pdl(k_sw_limit<T, 6, OC>, nc, b, s.tune_pdl, st, m, S, s.L);
    else
      launch_pdl(k_sw_limit<T, 0, OC>, nc, b, s.tune_pdl, st, m, S, s.L);
  }
}

template <int T, int OC>
void launch_k3(const SwState &s, const Stage &S, bool unroll, int b, cudaStream_t st) {
  const DMesh &m = s.mesh->ctx.d;
  const int64_t n = ((int64_t)m.nC + m.nV) * s.L;
  if (unroll)
    launch_ex(k_sw_final<T, 6, OC>, n, b, false, s, st, m, s.st, S, s.L);
  else
    launch_ex(k_sw_final<T, 0, OC>, n, b, false, s, st, m, s.st, S, s.L);
}

template <int T> void launch_stage_T(SwState &s, const Stage &S, cudaStream_t st) {
  const DMesh &m = s.mesh->ctx.d;
  cudaEvent_t *ev = s.prof_events;
  // 10-slot edge stencils (K1, K2 edges) and at most 6 edges per cell (K2, K3 cells)
  const bool w10 = m.maxEoE == 10 && (m.maxAdv == 10 || !s.p.fct || T == 0), c6 = m.maxEoC <= 6;
  constexpr int OC1 = T <= kOccMaxT ? 1 : 0;  // no capped variants compiled beyond kOccMaxT
  const bool split = T > 0 && s.tune_split;    // four-launch schedule
  const bool u1 = w10 && s.tune_unroll[0], u2 = w10 && c6 && s.tune_unroll[1];
  if (split) {  // K1 does the thickness flux part only (the T = 0 kernel)
    if (s.tune_occ[0])
      launch_k1<0, 1>(s, S, u1, s.tune_tpb[0], st);
    else
      launch_k1<0, 0>(s, S, u1, s.tune_tpb[0], st);
  } else if (OC1 && s.tune_occ[0]) {
    launch_k1<T, OC1>(s, S, u1, s.tune_tpb[0], st);
  } else {
    launch_k1<T, 0>(s, S, u1, s.tune_tpb[0], st);
  }
  if (ev) prof_mark(ev[0], st);
  if (split) {
    if (OC1 && s.tune_occ[1])
      launch_k2<T, OC1, 1>(s, S, u2, s.tune_tpb[1], st);
    else
      launch_k2<T, 0, 1>(s, S, u2, s.tune_tpb[1], st);
  } else if (OC1 && s.tune_occ[1]) {
    launch_k2<T, OC1, 0>(s, S, u2, s.tune_tpb[1], st);
  } else {
    launch_k2<T, 0, 0>(s, S, u2, s.tune_tpb[1], st);
  }
  if (ev) prof_mark(ev[1], st);
  if (s.k2_mark) MPASO_CUDA(cudaEventRecord(s.k2_mark, st));
  if (OC1 && s.tune_occ[2])
    launch_k3<T, OC1>(s, S, c6 && s.tune_unroll[2], s.tune_tpb[2], st);
  else
    launch_k3<T, 0>(s, S, c6 && s.tune_unroll[2], s.tune_tpb[2], st);
  if (ev) prof_mark(ev[2], st);
}

void launch_stage(SwState &s, const Stage &S, cudaStream_t st) {
  switch (s.T) {
    case 0: launch_stage_T<0>(s, S, st); break;
    case 1: launch_stage_T<1>(s, S, st); break;
    case 2: launch_stage_T<2>(s, S, st); break;
    case 3: launch_stage_T<3>(s, S, st); break;
    case 4: launch_stage_T<4>(s, S, st); break;
    case 5: launch_stage_T<5>(s, S, st); break;
    case 6: launch_stage_T<6>(s, S, st); break;
    case 7: launch_stage_T<7>(s, S, st); break;
    case 8: launch_stage_T<8>(s, S, st); break;
    default: fail(MPASO_ERR_ARG, "ntr out of range");
  }
}

void ensure_diag(SwState &s, cudaStream_t st) {
  if (s.diag_valid) return;
  const DMesh &m = s.mesh->ctx.d;
  Stage S = make_stage(s, 0, 0.0);
  if (m.maxEoC <= 6)
    k_sw_diag<6><<<blocks_for(((int64_t)m.nC + m.nV) * s.L, TPB), TPB, 0, st>>>(m, s.st, S, s.L);
  else
    k_sw_diag<0><<<blocks_for(((int64_t)m.nC + m.nV) * s.L, TPB), TPB, 0, st>>>(m, s.st, S, s.L);
  MPASO_CUDA(cudaGetLastError());
  s.diag_valid = true;
}

void sw_steps(SwState &s, double dt, int nsteps, cudaStream_t st) {
  ensure_diag(s, st);
  for (int n = 0; n < nsteps; ++n)
    for (int rk = 0; rk < 4; ++rk) launch_stage(s, make_stage(s, rk, dt), st);
  MPASO_CUDA(cudaGetLastError());
}

template <int T, int NW, int NC>
void launch_persistent_T(SwState &s, const StageSet &P, int nsteps, GridBar b) {
  const DMesh &m = s.mesh->ctx.d;
  auto kern = k_sw_persistent<T, NW, NC>;
  int per_sm = 0;
  MPASO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TPB, 0));
  require(per_sm > 0, MPASO_ERR_CUDA, "persistent kernel does not fit an SM");
  const int64_t need = blocks_for(((int64_t)m.nE + m.nC) * s.L, TPB);
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)per_sm * s.mesh->ctx.sms, need));
  DMesh mm = m;
  DStat dd = s.st;
  StageSet pp = P;
  int L = s.L;
  void *args[] = {&mm, &dd, &pp, &L, &nsteps, &b};
  MPASO_CUDA(cudaLaunchCooperativeKernel((const void *)kern, dim3(grid), dim3(TPB), args, 0, s.stream));
}

template <int T> void launch_persistent(SwState &s, const StageSet &P, int nsteps, GridBar b) {
  const DMesh &m = s.mesh->ctx.d;
  const bool w10 = m.maxEoE == 10 && (m.maxAdv == 10 || !s.p.fct || T == 0), c6 = m.maxEoC <= 6;
  if (w10 && c6)
    launch_persistent_T<T, 10, 6>(s, P, nsteps, b);
  else
    launch_persistent_T<T, 0, 0>(s, P, nsteps, b);
}

// nsteps RK4 steps in one persistent launch; MPASO_ERR_TIMEOUT when a grid
// barrier gave up (the state is then partly advanced).
void sw_steps_persistent(SwState &s, double dt, int nsteps, long long spin, unsigned int extra) {
  require(s.p.app == MPASO_APP_SW, MPASO_ERR_ARG, "the persistent step is the sw app's");
  require(nsteps >= 0, MPASO_ERR_ARG, "nsteps < 0");
  if (nsteps == 0) return;
  ensure_diag(s, s.stream);
  if (!s.pbar) {
    if (cudaMalloc(&s.pbar, 2 * sizeof(unsigned int)) != cudaSuccess) {
      cudaGetLastError();
      s.pbar = nullptr;
      fail(MPASO_ERR_ALLOC, "device allocation of the grid barrier failed");
    }
  }
  MPASO_CUDA(cudaMemsetAsync(s.pbar, 0, 2 * sizeof(unsigned int), s.stream));
  StageSet P;
  for (int rk = 0; rk < 4; ++rk) P.s[rk] = make_stage(s, rk, dt);
  GridBar b{s.pbar, spin > 0 ? spin : (1LL << 26), extra};
  switch (s.T) {
    case 0: launch_persistent<0>(s, P, nsteps, b); break;
    case 1: launch_persistent<1>(s, P, nsteps, b); break;
    case 2: launch_persistent<2>(s, P, nsteps, b); break;
    case 3: launch_persistent<3>(s, P, nsteps, b); break;
    default: fail(MPASO_ERR_ARG, "the persistent step supports up to 3 tracers");
  }
  unsigned int flag[2] = {0, 0};
  MPASO_CUDA(cudaMemcpyAsync(flag, s.pbar, sizeof(flag), cudaMemcpyDeviceToHost, s.stream));
  MPASO_CUDA(cudaStreamSynchronize(s.stream));
  require(flag[1] == 0, MPASO_ERR_TIMEOUT, "a grid barrier of the persistent step gave up waiting");
}

}  // namespace

// Entry points of the ocean path (ocean.cu).
void ocean_create(SwState &s);
void ocean_steps(SwState &s, double dt, int nsteps, cudaStream_t st);
void ocean_prepare(SwState &s, double dt, cudaStream_t st);
void ocean_recompute(SwState &s, double dt, cudaStream_t st);
void ocean_one_stage(SwState &s, int rk, double dt, cudaStream_t st);
int ocean_launches_per_step(const SwState &s);

void sw_create(SwState &s) {
  const DMesh &m = s.mesh->ctx.d;
  const int64_t L = s.L, T = s.T;
  const int64_t nC = m.nC, nE = m.nE, nV = m.nV;
  std::vector<std::pair<double **, int64_t>> bufs = {
      {&s.U[0], nE * L}, {&s.U[1], nE * L}, {&s.U[2], nE * L}, {&s.U[3], nE * L},
      {&s.H[0], nC * L}, {&s.H[1], nC * L}, {&s.H[2], nC * L}, {&s.H[3], nC * L},
      {&s.TR0, nC * L * T}, {&s.TRA, nC * L * T}, {&s.TRB, nC * L * T}, {&s.TRH, nC * L * T},
      {&s.pv, nV * L}, {&s.vort, nV * L}, {&s.bern, nC * L},
      {(double **)&s.FG, 2 * nE * L}, {&s.pve, nE * L}, {&s.A, nE * L * T}, {&s.LO, nE * L * T},
      {&s.DF, nE * L * T}, {(double **)&s.R2, 2 * nC * L * T}, {&s.tLO, nC * L * T},
      {&s.HPW, T > 0 ? nC * L : 0}};
  stat_buffers(s, bufs);
  alloc_arena(s, bufs);
  build_stat(s);
}

// One RK stage of (h, u) only, on explicit buffers (the adjoint's taping
// recompute).  Tracers are passive in the sw app, so they are left out.
// tape_pv / tape_hs (may be null) receive pv and the kite-summed thickness of
// the stage's output state.
void sw_stage_ptrs(SwState &s, int rk, double dt, const double *u_in, const double *h_in,
                   const double *u_prev, const double *h_prev, double *u_out, double *h_out,
                   double *u_acc, double *h_acc, double *u_new, double *h_new, double *tape_pv,
                   double *tape_hs, double *tape_s1, cudaStream_t st) {
  Stage S = make_stage(s, rk, dt);
  S.u_in = u_in, S.h_in = h_in, S.u_prev = u_prev, S.h_prev = h_prev;
  S.u_out = u_out, S.h_out = h_out, S.u_acc = u_acc, S.h_acc = h_acc, S.u_new = u_new, S.h_new = h_new;
  S.fct = 0, S.hmix = 0;
  S.tape_pv = tape_pv, S.tape_hs = tape_hs, S.tape_s1 = tape_s1;
  launch_stage_T<0>(s, S, st);
}

// A stage with the state's weights and buffers, for callers that redirect
// some of its pointers (the adjoint's taping recompute with tracers).
Stage sw_make_stage(SwState &s, int rk, double dt) { return make_stage(s, rk, dt); }
void sw_launch_stage(SwState &s, const Stage &S, cudaStream_t st) { launch_stage(s, S, st); }

// Diagnostics (pv, vorticity, ke, divergence) of an explicit (u, h); pv and the
// kite-summed thickness also go to tape_pv / tape_hs when given.
void sw_diag_ptrs(SwState &s, const double *u, const double *h, double *tape_pv, double *tape_hs,
                  cudaStream_t st) {
  const DMesh &m = s.mesh->ctx.d;
  Stage S = make_stage(s, 0, 0.0);
  S.u_in = u, S.h_in = h;
  S.tape_pv = tape_pv, S.tape_hs = tape_hs;
  if (m.maxEoC <= 6)
    k_sw_diag<6><<<blocks_for(((int64_t)m.nC + m.nV) * s.L, TPB), TPB, 0, st>>>(m, s.st, S, s.L);
  else
    k_sw_diag<0><<<blocks_for(((int64_t)m.nC + m.nV) * s.L, TPB), TPB, 0, st>>>(m, s.st, S, s.L);
}

void sw_steps_pub(SwState &s, double dt, int nsteps, cudaStream_t st) { sw_steps(s, dt, nsteps, st); }

}  // namespace mpaso

using namespace mpaso;

namespace {

void field_geom(SwState &s, int field, int &entity, int64_t &row, double *&buf) {
  switch (field) {
    case MPASO_FIELD_H: entity = MPASO_CELLS, row = s.L, buf = s.H[0]; break;
    case MPASO_FIELD_U: entity = MPASO_EDGES, row = s.L, buf = s.U[0]; break;
    case MPASO_FIELD_TRACERS: entity = MPASO_CELLS, row = (int64_t)s.L * s.T, buf = s.TR0; break;
    case MPASO_FIELD_LAYER_THICKNESS_EDGE:
      require(s.p.app == MPASO_APP_OCEAN, MPASO_ERR_ARG, "layerThicknessEdge is an ocean field");
      entity = MPASO_EDGES, row = s.L, buf = s.HE;
      break;
    case MPASO_FIELD_VORTICITY:
    case MPASO_FIELD_PV_VERTEX:
      require(s.p.app == MPASO_APP_SW, MPASO_ERR_ARG, "vorticity / pv_vertex are sw diagnostics");
      ensure_diag(s, s.stream);  // diagnostics of the current state (kept current by the steps)
      entity = MPASO_VERTICES, row = s.L, buf = field == MPASO_FIELD_VORTICITY ? s.vort : s.pv;
      break;
    default: fail(MPASO_ERR_ARG, "unknown field id");
  }
  require(row > 0, MPASO_ERR_ARG, "field has no data (ntr = 0?)");
}

void run_steps(SwState &s, double dt, int nsteps, cudaStream_t st) {
  if (s.p.app == MPASO_APP_OCEAN)
    ocean_steps(s, dt, nsteps, st);
  else
    sw_steps(s, dt, nsteps, st);
}

// Device time (ms per launch) of the three stage kernels over nsteps RK4
// steps; advances the state.  One step is captured as a graph with an event
// node before the first kernel and after every kernel of each stage, and the
// graph is replayed nsteps times: the kernels run as the step graph runs them
// (no host round trip between launches), and the intervals between the event
// nodes add up to the step.
void time_stage_kernels(SwState &S, double dt, int nsteps, double ms[3]) {
  const bool oc = S.p.app == MPASO_APP_OCEAN;
  constexpr int nk = 3, nev = 4 * nk + 1;
  if (oc)
    ocean_prepare(S, dt, S.stream);
  else
    ensure_diag(S, S.stream);
  cudaEvent_t ev[nev] = {};
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  double acc[nk] = {0, 0, 0};
  auto release = [&] {
    S.prof_events = nullptr;
    if (ge) cudaGraphExecDestroy(ge);
    if (g) cudaGraphDestroy(g);
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
  };
  try {
    for (auto &e : ev) MPASO_CUDA(cudaEventCreate(&e));
    MPASO_CUDA(cudaStreamBeginCapture(S.stream, cudaStreamCaptureModeThreadLocal));
    try {
      MPASO_CUDA(cudaEventRecordWithFlags(ev[0], S.stream, cudaEventRecordExternal));
      for (int rk = 0; rk < 4; ++rk) {
        S.prof_events = ev + 1 + nk * rk;
        if (oc)
          ocean_one_stage(S, rk, dt, S.stream);
        else
          launch_stage(S, make_stage(S, rk, dt), S.stream);
      }
      S.prof_events = nullptr;
    } catch (...) {
      cudaStreamEndCapture(S.stream, &g);
      cudaGetLastError();
      throw;
    }
    MPASO_CUDA(cudaStreamEndCapture(S.stream, &g));
    MPASO_CUDA(cudaGraphInstantiate(&ge, g, 0));
    for (int n = 0; n < nsteps; ++n) {
      MPASO_CUDA(cudaGraphLaunch(ge, S.stream));
      MPASO_CUDA(cudaEventSynchronize(ev[nev - 1]));
      for (int j = 0; j < nev - 1; ++j) {
        float t = 0.f;
        MPASO_CUDA(cudaEventElapsedTime(&t, ev[j], ev[j + 1]));
        acc[j % nk] += t;
      }
    }
  } catch (...) {
    release();
    throw;
  }
  release();
  for (int k = 0; k < nk; ++k) ms[k] = acc[k] / (4.0 * nsteps);
}

// Device time (ms) of one uninterrupted RK4 step (no events between launches,
// so launch overlap shows), averaged over nsteps; advances the state.
double time_whole_steps(SwState &S, double dt, int nsteps) {
  cudaEvent_t a = nullptr, b = nullptr;
  float ms = 0.f;
  try {
    MPASO_CUDA(cudaEventCreate(&a));
    MPASO_CUDA(cudaEventCreate(&b));
    if (S.p.app == MPASO_APP_OCEAN)
      ocean_prepare(S, dt, S.stream);
    else
      ensure_diag(S, S.stream);
    MPASO_CUDA(cudaEventRecord(a, S.stream));
    run_steps(S, dt, nsteps, S.stream);
    MPASO_CUDA(cudaEventRecord(b, S.stream));
    MPASO_CUDA(cudaEventSynchronize(b));
    MPASO_CUDA(cudaEventElapsedTime(&ms, a, b));
  } catch (...) {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    throw;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / nsteps;
}

// A captured step graph bakes in the launch shapes; drop it when they change.
void drop_graph(SwState &S) {
  if (S.graph) {
    MPASO_CUDA(cudaGraphExecDestroy(S.graph));
    S.graph = nullptr;
  }
  if (S.xg) {
    MPASO_CUDA(cudaGraphExecDestroy(S.xg));
    S.xg = nullptr;
  }
  drop_adjoint_graph(S);
}

// Whether kernel k of the stage has a compile-time-unrolled variant on this mesh.
bool has_unrolled(const SwState &S, int k) {
  const DMesh &m = S.mesh->ctx.d;
  const bool c6 = m.maxEoC <= 6;
  if (S.p.app == MPASO_APP_OCEAN) return k == 0 ? m.maxAdv == 10 : c6;
  const bool w10 = m.maxEoE == 10 && (m.maxAdv == 10 || !S.p.fct || S.T == 0);
  return k == 0 ? w10 : k == 1 ? w10 && c6 : c6;
}

// Whether the register-capped (full occupancy) variants exist for this state.
bool has_capped(const SwState &S) { return S.p.app == MPASO_APP_SW && S.T <= kOccMaxT; }

// The static array an L2 window choice makes persistent, and its bytes.
std::pair<const void *, size_t> l2_target(const SwState &S, int which) {
  const DMesh &m = S.mesh->ctx.d;
  if (S.p.app != MPASO_APP_SW) return {nullptr, 0};
  if (which == 1 && S.p.fct && S.T > 0) return {S.st.cpm2, (size_t)m.maxAdv * m.nE * sizeof(double2)};
  if (which == 2) return {S.st.woe8, (size_t)m.maxEoE * m.nE * sizeof(double)};
  return {nullptr, 0};
}

// Sets the state's L2 persistence choice: reserves the device's persisting
// L2 (up to its maximum) and builds the access-policy window the chosen
// kernel's launches carry.  `which` = 0 releases it.
void set_l2_window(SwState &S, int which) {
  const int dev = S.mesh->ctx.device;
  const auto t = l2_target(S, which);
  if (!t.first) which = 0;
  if (S.tune_l2 && !which) {
    MPASO_CUDA(cudaCtxResetPersistingL2Cache());
    MPASO_CUDA(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0));
  }
  S.tune_l2 = which;
  S.l2win = cudaAccessPolicyWindow{};
  if (!which) return;
  int maxp = 0, maxw = 0;
  MPASO_CUDA(cudaDeviceGetAttribute(&maxp, cudaDevAttrMaxPersistingL2CacheSize, dev));
  MPASO_CUDA(cudaDeviceGetAttribute(&maxw, cudaDevAttrMaxAccessPolicyWindowSize, dev));
  require(maxp > 0 && maxw > 0, MPASO_ERR_ARG, "device has no persisting L2");
  const size_t bytes = std::min(t.second, (size_t)maxw);
  const size_t aside = std::min(bytes, (size_t)maxp);
  MPASO_CUDA(cudaCtxResetPersistingL2Cache());
  MPASO_CUDA(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, aside));
  S.l2win.base_ptr = const_cast<void *>(t.first);
  S.l2win.num_bytes = bytes;
  S.l2win.hitRatio = (float)std::min(1.0, (double)aside / (double)bytes);
  S.l2win.hitProp = cudaAccessPropertyPersisting;
  S.l2win.missProp = cudaAccessPropertyStreaming;
}

void get_config(const SwState &S, int32_t *config) {
  for (int k = 0; k < 3; ++k)
    config[k] = S.tune_unroll[k], config[3 + k] = S.tune_tpb[k], config[6 + k] = S.tune_occ[k];
  config[9] = S.tune_l2;
  config[10] = S.tune_pdl;
  config[11] = S.tune_split;
}

// Whether the state may run its TRiSK loop with several lanes per edge.
bool has_lanes(const SwState &S) { return S.p.app == MPASO_APP_SW && S.T <= kLanesMaxT; }

constexpr int kTpbChoices[3] = {64, 128, 256};

void step_graph(SwState &S, double dt, int nsteps);

// Device staging for host-memory exchanges (reference order), grown on
// demand and kept with the state, so repeated calls allocate nothing.
double *ensure_io(SwState &S, size_t bytes) {
  if (S.io_bytes < bytes) {
    if (S.io_stage) {
      MPASO_CUDA(cudaStreamSynchronize(S.stream));
      MPASO_CUDA(cudaFree(S.io_stage));
    }
    if (S.xg) {  // the captured host exchange holds the old staging addresses
      MPASO_CUDA(cudaGraphExecDestroy(S.xg));
      S.xg = nullptr;
    }
    S.io_stage = nullptr, S.io_bytes = 0;
    if (cudaMalloc((void **)&S.io_stage, bytes) != cudaSuccess) {
      cudaGetLastError();
      fail(MPASO_ERR_ALLOC, "device allocation of the host-exchange staging failed");
    }
    S.io_bytes = bytes;
  }
  return S.io_stage;
}

}  // namespace

extern "C" {

int mpaso_state_create(mpaso_mesh m, const mpaso_params *p, mpaso_state *out) {
  return guarded("mpaso_state_create", [&] {
    require(m && p && out, MPASO_ERR_ARG, "null argument");
    require(p->nlev >= 1 && p->nlev <= 4096, MPASO_ERR_ARG, "nlev out of range");
    require(p->ntr >= 0 && p->ntr <= kMaxTracers, MPASO_ERR_ARG, "ntr out of range (max 8)");
    require(p->app == MPASO_APP_SW || p->app == MPASO_APP_OCEAN, MPASO_ERR_ARG, "unknown app");
    if (p->fct) {
      require(m->ctx.has_fct, MPASO_ERR_ARG, "fct requested but the mesh has no FCT statics");
      require(m->ctx.d.fctLev == p->nlev, MPASO_ERR_ARG, "FCT statics built for another level count");
      std::vector<int> mlc(m->ctx.d.nC);
      MPASO_CUDA(cudaMemcpy(mlc.data(), m->ctx.d.maxLevelCell, mlc.size() * sizeof(int), cudaMemcpyDeviceToHost));
      for (int x : mlc)
        require(x == p->nlev, MPASO_ERR_ARG, "fused path needs maxLevelCell == nlev in every cell");
    }
    if (p->app == MPASO_APP_OCEAN) require(p->ntr >= 1, MPASO_ERR_ARG, "ocean app needs tracers");
    MPASO_CUDA(cudaSetDevice(m->ctx.device));
    auto *h = new mpaso_state_s();
    try {
      SwState &s = h->s;
      s.mesh = m, s.p = *p, s.L = p->nlev, s.T = p->ntr;
      MPASO_CUDA(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking));
      if (p->app == MPASO_APP_OCEAN)
        ocean_create(s);
      else
        sw_create(s);
      MPASO_CUDA(cudaStreamSynchronize(s.stream));
    } catch (...) {
      if (h->s.stream) cudaStreamDestroy(h->s.stream);
      delete h;
      throw;
    }
    m->refs.fetch_add(1);  // released by mpaso_state_destroy
    *out = h;
  });
}

int mpaso_state_destroy(mpaso_state s) {
  return guarded("mpaso_state_destroy", [&] {
    if (!s) return;
    mpaso_mesh m = s->s.mesh;  // alive: the state holds a reference
    cudaSetDevice(m->ctx.device);
    cudaStreamSynchronize(s->s.stream);
    cudaStream_t st = s->s.stream;
    delete s;
    cudaStreamDestroy(st);
    cudaGetLastError();  // teardown is best effort: leave no error pending for later calls
    release_mesh(m);
  });
}

int mpaso_state_set(mpaso_state s, int32_t field, const double *data) {
  return guarded("mpaso_state_set", [&] {
    require(s && data, MPASO_ERR_ARG, "null argument");
    SwState &S = s->s;
    MPASO_CUDA(cudaSetDevice(S.mesh->ctx.device));
    require(field != MPASO_FIELD_VORTICITY && field != MPASO_FIELD_PV_VERTEX, MPASO_ERR_ARG,
            "diagnostic fields are read-only");
    int entity;
    int64_t row;
    double *buf;
    field_geom(S, field, entity, row, buf);
    MeshCtx &ctx = S.mesh->ctx;
    const int64_t n = entity == MPASO_CELLS ? ctx.d.nC : entity == MPASO_EDGES ? ctx.d.nE : ctx.d.nV;
    const double *src = data;
    if (!is_device_pointer(data)) {
      double *stage = ensure_io(S, (size_t)n * row * 8);
      MPASO_CUDA(cudaMemcpyAsync(stage, data, (size_t)n * row * 8, cudaMemcpyHostToDevice, S.stream));
      src = stage;
    }
    k_gather_rows_pub(src, buf, ctx.d_perm[entity], n, (int)row, S.stream);
    MPASO_CUDA(cudaStreamSynchronize(S.stream));
    S.diag_valid = false;
    S.prep_dt = 0.0;
  });
}

int mpaso_state_snapshot(mpaso_state s, int32_t field, double *data) {
  return guarded("mpaso_state_snapshot", [&] {
    require(s && data, MPASO_ERR_ARG, "null argument");
    SwState &S = s->s;
    MPASO_CUDA(cudaSetDevice(S.mesh->ctx.device));
    int entity;
    int64_t row;
    double *buf;
    field_geom(S, field, entity, row, buf);
    MeshCtx &ctx = S.mesh->ctx;
    const int64_t n = entity == MPASO_CELLS ? ctx.d.nC : entity == MPASO_EDGES ? ctx.d.nE : ctx.d.nV;
    const size_t bytes = (size_t)n * row * sizeof(double);
    if (!S.out_stream) {
      MPASO_CUDA(cudaStreamCreateWithFlags(&S.out_stream, cudaStreamNonBlocking));
      MPASO_CUDA(cudaEventCreateWithFlags(&S.out_ready, cudaEventDisableTiming));
      for (int b = 0; b < 2; ++b) {
        MPASO_CUDA(cudaEventCreateWithFlags(&S.out_read[b], cudaEventDisableTiming));
        MPASO_CUDA(cudaEventCreateWithFlags(&S.out_done[b], cudaEventDisableTiming));
      }
    }
    if (S.out_bytes < bytes) {  // (re)size both buffers once every earlier copy has ended
      MPASO_CUDA(cudaStreamSynchronize(S.out_stream));
      for (auto &p : S.out_buf) {
        if (p) MPASO_CUDA(cudaFree(p));
        p = nullptr;
      }
      S.out_bytes = 0;
      for (auto &p : S.out_buf)
        if (cudaMalloc((void **)&p, bytes) != cudaSuccess) {
          cudaGetLastError();
          fail(MPASO_ERR_ALLOC, "device allocation of the snapshot buffers failed");
        }
      S.out_bytes = bytes;
    }
    const int b = S.out_next;
    S.out_next ^= 1;
    // the field as it stands after the work already queued on the state's stream
    MPASO_CUDA(cudaEventRecord(S.out_ready, S.stream));
    MPASO_CUDA(cudaStreamWaitEvent(S.out_stream, S.out_ready, 0));
    // the buffer's previous copy to the host must be over before it is refilled
    k_scatter_rows_pub(buf, S.out_buf[b], ctx.d_perm[entity], n, (int)row, S.out_stream);
    MPASO_CUDA(cudaEventRecord(S.out_read[b], S.out_stream));
    // later steps may overwrite the field only once the permutation has read it
    MPASO_CUDA(cudaStreamWaitEvent(S.stream, S.out_read[b], 0));
    MPASO_CUDA(cudaMemcpyAsync(data, S.out_buf[b], bytes, cudaMemcpyDeviceToHost, S.out_stream));
    MPASO_CUDA(cudaEventRecord(S.out_done[b], S.out_stream));
  });
}

int mpaso_state_snapshot_wait(mpaso_state s) {
  return guarded("mpaso_state_snapshot_wait", [&] {
    require(s != nullptr, MPASO_ERR_ARG, "null state");
    if (s->s.out_stream) MPASO_CUDA(cudaStreamSynchronize(s->s.out_stream));
  });
}

int mpaso_state_get(mpaso_state s, int32_t field, double *data) {
  return guarded("mpaso_state_get", [&] {
    require(s && data, MPASO_ERR_ARG, "null argument");
    SwState &S = s->s;
    MPASO_CUDA(cudaSetDevice(S.mesh->ctx.device));
    int entity;
    int64_t row;
    double *buf;
    field_geom(S, field, entity, row, buf);
    MeshCtx &ctx = S.mesh->ctx;
    const int64_t n = entity == MPASO_CELLS ? ctx.d.nC : entity == MPASO_EDGES ? ctx.d.nE : ctx.d.nV;
    const bool dev = is_device_pointer(data);
    double *dst = dev ? data : ensure_io(S, (size_t)n * row * 8);
    k_scatter_rows_pub(buf, dst, ctx.d_perm[entity], n, (int)row, S.stream);
    if (!dev) MPASO_CUDA(cudaMemcpyAsync(data, dst, (size_t)n * row * 8, cudaMemcpyDeviceToHost, S.stream));
    MPASO_CUDA(cudaStreamSynchronize(S.stream));
  });
}

int mpaso_state_check_finite(mpaso_state s) {
  return guarded("mpaso_state_check_finite", [&] {
    require(s != nullptr, MPASO_ERR_ARG, "null state");
    SwState &S = s->s;
    MeshCtx &ctx = S.mesh->ctx;
    MPASO_CUDA(cudaSetDevice(ctx.device));
    struct F {
      int id;
      const char *name;
    };
    std::vector<F> fields = {{MPASO_FIELD_H, "layer thickness"}, {MPASO_FIELD_U, "normal velocity"}};
    if (S.T > 0) fields.push_back({MPASO_FIELD_TRACERS, "tracer"});
    if (S.p.app == MPASO_APP_OCEAN) fields.push_back({MPASO_FIELD_LAYER_THICKNESS_EDGE, "edge layer thickness"});
    auto *first = reinterpret_cast<unsigned long long *>(ensure_io(S, fields.size() * 8));
    MPASO_CUDA(cudaMemsetAsync(first, 0xff, fields.size() * 8, S.stream));
    std::vector<int64_t> rows(fields.size());
    std::vector<int> ents(fields.size());
    for (size_t f = 0; f < fields.size(); ++f) {
      double *buf;
      field_geom(S, fields[f].id, ents[f], rows[f], buf);
      const int64_t n = (ents[f] == MPASO_CELLS ? ctx.d.nC : ctx.d.nE) * rows[f];
      k_first_nonfinite<<<152 * 8, 256, 0, S.stream>>>(buf, n, first + f);  // 8 blocks per SM
    }
    MPASO_CUDA(cudaGetLastError());
    std::vector<unsigned long long> h(fields.size());
    MPASO_CUDA(cudaMemcpyAsync(h.data(), first, fields.size() * 8, cudaMemcpyDeviceToHost, S.stream));
    MPASO_CUDA(cudaStreamSynchronize(S.stream));
    for (size_t f = 0; f < fields.size(); ++f) {
      if (h[f] == ~0ull) continue;
      // device index -> entity in file order, level (and tracer)
      const int64_t e = (int64_t)(h[f] / (unsigned long long)rows[f]), comp = (int64_t)(h[f] % rows[f]);
      const int32_t old = ctx.perm[ents[f]][e];
      std::string msg = std::string("non-finite ") + fields[f].name + " at " +
                        (ents[f] == MPASO_CELLS ? "cell " : "edge ") + std::to_string(old) + " level ";
      if (fields[f].id == MPASO_FIELD_TRACERS)
        msg += std::to_string(comp / S.T) + " tracer " + std::to_string(comp % S.T);
      else
        msg += std::to_string(comp);
      fail(MPASO_ERR_NUMERIC, msg);
    }
  });
}

int mpaso_rk4_step(mpaso_state s, double dt, int32_t nsteps) {
  return guarded("mpaso_rk4_step", [&] {
    require(s != nullptr && nsteps >= 0, MPASO_ERR_ARG, "bad argument");
    MPASO_CUDA(cudaSetDevice(s->s.mesh->ctx.device));
    run_steps(s->s, dt, nsteps, s->s.stream);
  });
}

int mpaso_rk4_step_graph(mpaso_state s, double dt, int32_t nsteps) {
  return guarded("mpaso_rk4_step_graph", [&] {
    require(s != nullptr && nsteps >= 0, MPASO_ERR_ARG, "bad argument");
    MPASO_CUDA(cudaSetDevice(s->s.mesh->ctx.device));
    step_graph(s->s, dt, nsteps);
  });
}

namespace {
// The host-buffer exchange of mpaso_rk4_step_host[_async]; `wait` = return
// after the results are in the host buffers, else right after the launch
// (page-locked buffers only).
void step_host(mpaso_state s, double dt, int32_t nsteps, double *h, double *u, double *tracers, bool wait) {
  {
    require(s && h && u && nsteps >= 0, MPASO_ERR_ARG, "bad argument");
    SwState &S = s->s;
    MeshCtx &ctx = S.mesh->ctx;
    MPASO_CUDA(cudaSetDevice(ctx.device));
    const int64_t nC = ctx.d.nC, nE = ctx.d.nE, L = S.L;
    const bool tr = tracers != nullptr && S.T > 0;
    const int64_t nh = nC * L, nu = nE * L, nt = tr ? nC * L * S.T : 0;
    const cudaStream_t st = S.stream;
    const size_t bytes = (size_t)(nh + nu + nt) * sizeof(double);
    double *dh = ensure_io(S, bytes), *du = dh + nh, *dtr = du + nu;
    // Page-locked buffers: the whole exchange (copies in, permutations, steps,
    // copies out) is one graph, captured once per buffer set, dt and nsteps.
    // Page-locked buffers mapped into the device's address space (the usual
    // case) also get device aliases: the exchange kernels then move and
    // permute each field in one pass over the host link.
    bool locked = true, mapped = true;
    double *alias[3] = {nullptr, nullptr, nullptr};
    {
      const void *ptrs[3] = {h, u, tr ? tracers : h};
      for (int f = 0; f < 3; ++f) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, ptrs[f]) != cudaSuccess || a.type != cudaMemoryTypeHost) locked = false;
        else alias[f] = (double *)a.devicePointer;
        cudaGetLastError();
        mapped = mapped && alias[f] != nullptr;
      }
    }
    require(wait || locked, MPASO_ERR_ARG, "the asynchronous exchange needs page-locked host buffers");
    const XKey key{h, u, tr ? tracers : nullptr, dt, nsteps};
    if (locked && S.xg && S.xkey == key) {
      MPASO_CUDA(cudaGraphLaunch(S.xg, st));
      if (wait) MPASO_CUDA(cudaStreamSynchronize(st));
      return;
    }
    if (S.xg) {
      MPASO_CUDA(cudaGraphExecDestroy(S.xg));
      S.xg = nullptr;
    }
    if (locked && !S.x_side[0]) {
      for (auto &x : S.x_side) MPASO_CUDA(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
      for (auto &e : S.x_ev) MPASO_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    if (locked) MPASO_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    // Pageable buffers: one copy per field each way through the staging
    // buffer and the permutation kernels.  Page-locked ones: see above (a
    // kernel that gathered from mapped host memory in context order was slower
    // than the copy engines; walking the host side in its own order is not).
    try {
    if (!locked) {
      MPASO_CUDA(cudaMemcpyAsync(dh, h, nh * sizeof(double), cudaMemcpyHostToDevice, st));
      MPASO_CUDA(cudaMemcpyAsync(du, u, nu * sizeof(double), cudaMemcpyHostToDevice, st));
      if (tr) MPASO_CUDA(cudaMemcpyAsync(dtr, tracers, nt * sizeof(double), cudaMemcpyHostToDevice, st));
      k_gather_rows_pub(dh, S.H[0], ctx.d_perm[MPASO_CELLS], nC, (int)L, st);
      k_gather_rows_pub(du, S.U[0], ctx.d_perm[MPASO_EDGES], nE, (int)L, st);
      if (tr) k_gather_rows_pub(dtr, S.TR0, ctx.d_perm[MPASO_CELLS], nC, (int)(L * S.T), st);
      S.diag_valid = false;
      S.prep_dt = 0.0;
      step_graph(S, dt, nsteps);
      k_scatter_rows_pub(S.H[0], dh, ctx.d_perm[MPASO_CELLS], nC, (int)L, st);
      k_scatter_rows_pub(S.U[0], du, ctx.d_perm[MPASO_EDGES], nE, (int)L, st);
      if (tr) k_scatter_rows_pub(S.TR0, dtr, ctx.d_perm[MPASO_CELLS], nC, (int)(L * S.T), st);
      MPASO_CUDA(cudaMemcpyAsync(h, dh, nh * sizeof(double), cudaMemcpyDeviceToHost, st));
      MPASO_CUDA(cudaMemcpyAsync(u, du, nu * sizeof(double), cudaMemcpyDeviceToHost, st));
      if (tr) MPASO_CUDA(cudaMemcpyAsync(tracers, dtr, nt * sizeof(double), cudaMemcpyDeviceToHost, st));
    } else {
      // Captured as a DAG over the state stream and two side streams: each field's
      // permutation starts when its own copy lands; the diagnostics wait for h and
      // u only, the steps for the tracers too; h and u go back out as soon as the
      // last stage's tendency kernel has written them, under that stage's tracer
      // kernel, and the tracers after it.
      const cudaStream_t su = S.x_side[0], sx = S.x_side[1];
      cudaEvent_t *E = S.x_ev;
      const int32_t *ic = ctx.d_iperm[MPASO_CELLS], *ie = ctx.d_iperm[MPASO_EDGES];
      MPASO_CUDA(cudaEventRecord(E[0], st));
      MPASO_CUDA(cudaStreamWaitEvent(su, E[0], 0));
      MPASO_CUDA(cudaStreamWaitEvent(sx, E[0], 0));
      if (mapped) {  // one pass per field; the tracers after h and u, under the diagnostics
        host_rows_pub(true, alias[0], S.H[0], ic, nC, (int)L, ctx.sms, st);
        host_rows_pub(true, alias[1], S.U[0], ie, nE, (int)L, ctx.sms, su);
        MPASO_CUDA(cudaEventRecord(E[1], su));
        if (tr) {
          MPASO_CUDA(cudaStreamWaitEvent(sx, E[1], 0));
          host_rows_pub(true, alias[2], S.TR0, ic, nC, (int)(L * S.T), ctx.sms, sx);
        }
      } else {
        MPASO_CUDA(cudaMemcpyAsync(dh, h, nh * sizeof(double), cudaMemcpyHostToDevice, st));
        k_gather_rows_pub(dh, S.H[0], ctx.d_perm[MPASO_CELLS], nC, (int)L, st);
        MPASO_CUDA(cudaMemcpyAsync(du, u, nu * sizeof(double), cudaMemcpyHostToDevice, su));
        k_gather_rows_pub(du, S.U[0], ctx.d_perm[MPASO_EDGES], nE, (int)L, su);
        MPASO_CUDA(cudaEventRecord(E[1], su));
        if (tr) {
          MPASO_CUDA(cudaMemcpyAsync(dtr, tracers, nt * sizeof(double), cudaMemcpyHostToDevice, sx));
          k_gather_rows_pub(dtr, S.TR0, ctx.d_perm[MPASO_CELLS], nC, (int)(L * S.T), sx);
        }
      }
      MPASO_CUDA(cudaEventRecord(E[2], sx));
      MPASO_CUDA(cudaStreamWaitEvent(st, E[1], 0));
      const bool sw = S.p.app == MPASO_APP_SW;
      if (sw) {
        S.diag_valid = false;
        ensure_diag(S, st);
      } else {
        ocean_recompute(S, dt, st);
      }
      MPASO_CUDA(cudaStreamWaitEvent(st, E[2], 0));
      if (sw && nsteps > 0) {
        for (int n = 0; n < nsteps; ++n)
          for (int rk = 0; rk < 4; ++rk) {
            if (n == nsteps - 1 && rk == 3) S.k2_mark = E[3];
            launch_stage(S, make_stage(S, rk, dt), st);
            S.k2_mark = nullptr;
          }
      } else {
        run_steps(S, dt, nsteps, st);
        MPASO_CUDA(cudaEventRecord(E[3], st));
      }
      MPASO_CUDA(cudaEventRecord(E[5], st));
      MPASO_CUDA(cudaStreamWaitEvent(su, E[3], 0));
      MPASO_CUDA(cudaStreamWaitEvent(sx, E[3], 0));
      if (mapped) {
        host_rows_pub(false, S.U[0], alias[1], ie, nE, (int)L, ctx.sms, su);
        host_rows_pub(false, S.H[0], alias[0], ic, nC, (int)L, ctx.sms, sx);
        if (tr) {
          MPASO_CUDA(cudaStreamWaitEvent(sx, E[5], 0));
          host_rows_pub(false, S.TR0, alias[2], ic, nC, (int)(L * S.T), ctx.sms, sx);
        }
      } else {
        k_scatter_rows_pub(S.U[0], du, ctx.d_perm[MPASO_EDGES], nE, (int)L, su);
        MPASO_CUDA(cudaMemcpyAsync(u, du, nu * sizeof(double), cudaMemcpyDeviceToHost, su));
        k_scatter_rows_pub(S.H[0], dh, ctx.d_perm[MPASO_CELLS], nC, (int)L, sx);
        MPASO_CUDA(cudaMemcpyAsync(h, dh, nh * sizeof(double), cudaMemcpyDeviceToHost, sx));
        if (tr) {
          MPASO_CUDA(cudaStreamWaitEvent(sx, E[5], 0));
          k_scatter_rows_pub(S.TR0, dtr, ctx.d_perm[MPASO_CELLS], nC, (int)(L * S.T), sx);
          MPASO_CUDA(cudaMemcpyAsync(tracers, dtr, nt * sizeof(double), cudaMemcpyDeviceToHost, sx));
        }
      }
      MPASO_CUDA(cudaEventRecord(E[4], su));
      MPASO_CUDA(cudaEventRecord(E[6], sx));
      MPASO_CUDA(cudaStreamWaitEvent(st, E[4], 0));  // join the side streams before the capture ends
      MPASO_CUDA(cudaStreamWaitEvent(st, E[6], 0));
    }
    } catch (...) {
      S.k2_mark = nullptr;
      if (locked) {
        cudaGraph_t g;
        cudaStreamEndCapture(st, &g);
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
      }
      throw;
    }
    if (locked) {
      cudaGraph_t g;
      MPASO_CUDA(cudaStreamEndCapture(st, &g));
      const cudaError_t e = cudaGraphInstantiate(&S.xg, g, 0);
      cudaGraphDestroy(g);
      MPASO_CUDA(e);
      S.xkey = key;
      MPASO_CUDA(cudaGraphLaunch(S.xg, st));
    }
    if (wait) MPASO_CUDA(cudaStreamSynchronize(st));
  }
}
}  // namespace

int mpaso_rk4_step_host(mpaso_state s, double dt, int32_t nsteps, double *h, double *u,
                        double *tracers) {
  return guarded("mpaso_rk4_step_host", [&] { step_host(s, dt, nsteps, h, u, tracers, true); });
}

int mpaso_rk4_step_host_async(mpaso_state s, double dt, int32_t nsteps, double *h, double *u,
                              double *tracers) {
  return guarded("mpaso_rk4_step_host_async", [&] { step_host(s, dt, nsteps, h, u, tracers, false); });
}

}  // extern "C"

namespace {
// Graph-replayed RK4 steps (the body of mpaso_rk4_step_graph).
void step_graph(SwState &S, double dt, int nsteps) {
  {
    if (S.p.app == MPASO_APP_SW)
      ensure_diag(S, S.stream);
    else
      ocean_prepare(S, dt, S.stream);
    if (!S.graph || S.graph_dt != dt) {
      if (S.graph) {
        MPASO_CUDA(cudaGraphExecDestroy(S.graph));
        S.graph = nullptr;
      }
      cudaGraph_t g;
      MPASO_CUDA(cudaStreamBeginCapture(S.stream, cudaStreamCaptureModeThreadLocal));
      try {
        run_steps(S, dt, 1, S.stream);
      } catch (...) {
        cudaStreamEndCapture(S.stream, &g);
        cudaGetLastError();
        throw;
      }
      MPASO_CUDA(cudaStreamEndCapture(S.stream, &g));
      MPASO_CUDA(cudaGraphInstantiate(&S.graph, g, 0));
      MPASO_CUDA(cudaGraphDestroy(g));
      S.graph_dt = dt;
    }
    for (int n = 0; n < nsteps; ++n) MPASO_CUDA(cudaGraphLaunch(S.graph, S.stream));
  }
}
}  // namespace

namespace mpaso {
void sw_steps_graph(SwState &s, double dt, int nsteps) { step_graph(s, dt, nsteps); }
}  // namespace mpaso

extern "C" {

int mpaso_state_profile(mpaso_state s, double dt, int32_t nsteps, double *ms_per_launch,
                        int32_t *nkinds, char *names, int32_t names_len) {
  return guarded("mpaso_state_profile", [&] {
    require(s && ms_per_launch && nkinds && nsteps > 0, MPASO_ERR_ARG, "bad argument");
    SwState &S = s->s;
    MPASO_CUDA(cudaSetDevice(S.mesh->ctx.device));
    const bool oc = S.p.app == MPASO_APP_OCEAN;
    const char *kinds = oc ? "oc_edges,oc_cells,oc_final" : "sw_edge_pre,sw_tend,sw_final";
    time_stage_kernels(S, dt, nsteps, ms_per_launch);
    *nkinds = 3;
    if (names && names_len > 0) {
      std::strncpy(names, kinds, (size_t)names_len - 1);
      names[names_len - 1] = 0;
    }
  });
}

int mpaso_rk4_step_persistent(mpaso_state s, double dt, int32_t nsteps, int64_t spin_limit,
                              int32_t extra_arrivals) {
  return guarded("mpaso_rk4_step_persistent", [&] {
    require(s != nullptr, MPASO_ERR_ARG, "null state");
    require(extra_arrivals >= 0, MPASO_ERR_ARG, "extra_arrivals < 0");
    SwState &S = s->s;
    MPASO_CUDA(cudaSetDevice(S.mesh->ctx.device));
    sw_steps_persistent(S, dt, nsteps, spin_limit, (unsigned int)extra_arrivals);
  });
}

int mpaso_state_sync(mpaso_state s) {
  return guarded("mpaso_state_sync", [&] {
    require(s != nullptr, MPASO_ERR_ARG, "null state");
    MPASO_CUDA(cudaStreamSynchronize(s->s.stream));
  });
}

int mpaso_state_stream(mpaso_state s, void **stream) {
  return guarded("mpaso_state_stream", [&] {
    require(s && stream, MPASO_ERR_ARG, "null argument");
    *stream = (void *)s->s.stream;
  });
}

int mpaso_state_launches_per_step(mpaso_state s, int32_t *n) {
  return guarded("mpaso_state_launches_per_step", [&] {
    require(s && n, MPASO_ERR_ARG, "null argument");
    *n = s->s.p.app == MPASO_APP_OCEAN ? ocean_launches_per_step(s->s) : 12;
  });
}

int mpaso_state_device_bytes(mpaso_state s, int64_t *bytes) {
  return guarded("mpaso_state_device_bytes", [&] {
    require(s && bytes, MPASO_ERR_ARG, "null argument");
    *bytes = (int64_t)s->s.arena_bytes;
  });
}

int mpaso_state_launch_config(mpaso_state s, int32_t *config) {
  return guarded("mpaso_state_launch_config", [&] {
    require(s && config, MPASO_ERR_ARG, "null argument");
    get_config(s->s, config);
  });
}

int mpaso_state_set_launch_config(mpaso_state s, const int32_t *config) {
  return guarded("mpaso_state_set_launch_config", [&] {
    require(s && config, MPASO_ERR_ARG, "null argument");
    for (int k = 0; k < 3; ++k) {
      require(config[k] == 0 || config[k] == 1, MPASO_ERR_ARG, "unroll flag must be 0 or 1");
      const int b = config[3 + k];
      require(b == 64 || b == 128 || b == 256, MPASO_ERR_ARG, "threads per block must be 64, 128 or 256");
      require(config[6 + k] == 0 || config[6 + k] == 1, MPASO_ERR_ARG, "occupancy flag must be 0 or 1");
    }
    require(config[9] >= 0 && config[9] <= 2, MPASO_ERR_ARG, "L2 window choice must be 0, 1 or 2");
    require(config[10] == 0 || config[10] == 1, MPASO_ERR_ARG, "launch overlap flag must be 0 or 1");
    require(config[11] == 0 || config[11] == 1, MPASO_ERR_ARG, "schedule flag must be 0 or 1");
    SwState &S = s->s;
    MPASO_CUDA(cudaSetDevice(S.mesh->ctx.device));
    MPASO_CUDA(cudaStreamSynchronize(S.stream));
    drop_graph(S);
    for (int k = 0; k < 3; ++k)
      S.tune_unroll[k] = config[k], S.tune_tpb[k] = config[3 + k], S.tune_occ[k] = config[6 + k];
    set_l2_window(S, config[9]);
    S.tune_pdl = config[10];
    S.tune_split = S.p.app == MPASO_APP_SW && S.T > 0 ? config[11] : 0;
  });
}

int mpaso_state_launch_config_ex(mpaso_state s, int32_t *config, int32_t n) {
  return guarded("mpaso_state_launch_config_ex", [&] {
    require(s && config && n >= 12, MPASO_ERR_ARG, "config needs at least 12 ints");
    get_config(s->s, config);
    if (n > 12) config[12] = s->s.tune_lanes;
    for (int k = 13; k < n; ++k) config[k] = 0;
  });
}

int mpaso_state_set_launch_config_ex(mpaso_state s, const int32_t *config, int32_t n) {
  return guarded("mpaso_state_set_launch_config_ex", [&] {
    require(s && config && n >= 12, MPASO_ERR_ARG, "config needs at least 12 ints");
    const int lanes = n > 12 ? config[12] : 1;
    require(lanes == 1 || lanes == 2 || lanes == 4, MPASO_ERR_ARG, "lanes per edge must be 1, 2 or 4");
    require(lanes == 1 || has_lanes(s->s), MPASO_ERR_ARG,
            "several lanes per edge need the sw app with at most one tracer");
    const int rc = mpaso_state_set_launch_config(s, config);
    if (rc != MPASO_OK) fail(rc, mpaso_last_error());
    s->s.tune_lanes = lanes;
  });
}

int mpaso_state_autotune(mpaso_state s, double dt, int32_t nsteps, int32_t *config) {
  return guarded("mpaso_state_autotune", [&] {
    require(s && nsteps > 0 && dt > 0.0, MPASO_ERR_ARG, "bad argument");
    SwState &S = s->s;
    MPASO_CUDA(cudaSetDevice(S.mesh->ctx.device));
    MPASO_CUDA(cudaStreamSynchronize(S.stream));
    const DMesh &m = S.mesh->ctx.d;
    // Every candidate starts from the same prognostic state, which is put
    // back at the end: (h, u, tracers) are the only fields a step reads that
    // it also overwrites.
    const size_t nh = (size_t)m.nC * S.L, nu = (size_t)m.nE * S.L, nt = (size_t)m.nC * S.L * S.T;
    double *keep = nullptr;
    MPASO_CUDA(cudaMalloc((void **)&keep, (nh + nu + nt) * sizeof(double)));
    auto save_restore = [&](bool save) {
      const std::pair<double *, size_t> f[3] = {{S.H[0], nh}, {S.U[0], nu}, {S.TR0, nt}};
      size_t off = 0;
      for (const auto &x : f) {
        if (x.second) {
          double *a = save ? keep + off : x.first;
          const double *b = save ? x.first : keep + off;
          MPASO_CUDA(cudaMemcpyAsync(a, b, x.second * sizeof(double), cudaMemcpyDeviceToDevice, S.stream));
        }
        off += x.second;
      }
      S.diag_valid = false;
    };
    try {
      drop_graph(S);
      save_restore(true);
      double ms[3];
      time_stage_kernels(S, dt, 1, ms);  // warm-up
      for (int k = 0; k < 3; ++k) {
        double best = 1e300;
        int best_u = S.tune_unroll[k], best_b = S.tune_tpb[k], best_o = S.tune_occ[k], best_l = S.tune_lanes;
        for (int lanes : {1, 2, 4}) {
          if (lanes > 1 && (k != 1 || !has_lanes(S))) continue;
          S.tune_lanes = lanes;
          for (int u = has_unrolled(S, k) ? 1 : 0; u >= 0; --u)
            for (int o = 0; o <= (has_capped(S) ? 1 : 0); ++o)
              for (int b : kTpbChoices) {
                S.tune_unroll[k] = u, S.tune_tpb[k] = b, S.tune_occ[k] = o;
                // one untimed step first: a variant's first launch loads its code
                save_restore(false);
                time_stage_kernels(S, dt, 1, ms);
                save_restore(false);
                time_stage_kernels(S, dt, nsteps, ms);
                if (ms[k] < best) best = ms[k], best_u = u, best_b = b, best_o = o, best_l = lanes;
              }
        }
        S.tune_unroll[k] = best_u, S.tune_tpb[k] = best_b, S.tune_occ[k] = best_o;
        if (k == 1) S.tune_lanes = best_l;
      }
      // L2 persistence changes every kernel's hit rate: judged on the whole stage
      double best = 1e300;
      int best_l2 = 0;
      for (int w = 0; w <= 2; ++w) {
        if (w && !l2_target(S, w).first) continue;
        set_l2_window(S, w);
        save_restore(false);
        time_stage_kernels(S, dt, 1, ms);
        save_restore(false);
        time_stage_kernels(S, dt, nsteps, ms);
        const double tot = ms[0] + ms[1] + ms[2];
        if (tot < 0.98 * best) best = tot, best_l2 = w;  // keep the simpler choice unless clearly faster
      }
      set_l2_window(S, best_l2);
      // four-launch schedule (sw with tracers), judged on the whole stage
      if (S.p.app == MPASO_APP_SW && S.T > 0) {
        double tot[2];
        for (int sp = 0; sp <= 1; ++sp) {
          S.tune_split = sp;
          save_restore(false);
          time_stage_kernels(S, dt, 1, ms);
          save_restore(false);
          time_stage_kernels(S, dt, nsteps, ms);
          tot[sp] = ms[0] + ms[1] + ms[2];
        }
        S.tune_split = tot[1] < 0.98 * tot[0] ? 1 : 0;
      }
      // programmatic dependent launch (sw stage kernels), judged on uninterrupted steps
      if (S.p.app == MPASO_APP_SW) {
        double t[2];
        for (int pdl = 0; pdl <= 1; ++pdl) {
          S.tune_pdl = pdl;
          save_restore(false);
          time_whole_steps(S, dt, 1);
          save_restore(false);
          t[pdl] = time_whole_steps(S, dt, nsteps);
        }
        S.tune_pdl = t[0] < 0.98 * t[1] ? 0 : 1;
      }
      save_restore(false);
      MPASO_CUDA(cudaStreamSynchronize(S.stream));
    } catch (...) {
      cudaStreamSynchronize(S.stream);
      cudaFree(keep);
      throw;
    }
    MPASO_CUDA(cudaFree(keep));
    if (config) get_config(S, config);
  });
}

}  // extern "C"

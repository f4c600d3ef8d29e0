// Hand-written adjoint (vector-Jacobian product) of the fused sw RK4 step for
// (h, u), with uniform checkpointing.
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
#include <cstring>

#include "rk4.cuh"

namespace mpaso {

struct AdjBuffers {
  void *arena = nullptr;
  size_t bytes = 0;
  int N = 0, k = 0, nck = 0, cap_ck = 0, cap_k = 0;
  double dt = 0.0;
  bool have_forward = false;
  double *ck_u = nullptr, *ck_h = nullptr;  // checkpoints [nck][nE L], [nck][nC L]
  double *tp_u = nullptr, *tp_h = nullptr;  // stage-state tape [4k + 1][...]
  double *uacc = nullptr, *hacc = nullptr;
  double *tp_pv = nullptr, *tp_hs = nullptr;  // pv, kite-summed h of every tape slot [4k + 1][nV L]
  double *pve = nullptr;
  double2 *FP = nullptr;  // {F, P} per edge, gathered together by B1
  double *lam_u = nullptr, *lam_h = nullptr, *acc_u = nullptr, *acc_h = nullptr;
  double *lk_u = nullptr, *lk_h = nullptr, *mu_u = nullptr, *mu_h = nullptr;
  double *lhe = nullptr, *lpve = nullptr, *lke = nullptr, *ldiv = nullptr, *lcirc = nullptr, *lhs = nullptr;
  // the whole reverse sweep, captured once per (N, k, dt) and replayed
  cudaGraphExec_t rev = nullptr;
  int rev_N = 0, rev_k = 0;
  double rev_dt = 0.0;
};

void drop_adjoint_graph(SwState &s) {
  if (s.adj && s.adj->rev) {
    cudaGraphExecDestroy(s.adj->rev);
    s.adj->rev = nullptr;
  }
}

void free_adjoint(SwState &s) {
  if (s.adj) {
    drop_adjoint_graph(s);
    if (s.adj->arena) cudaFree(s.adj->arena);
    delete s.adj;
    s.adj = nullptr;
  }
}

namespace {

constexpr int TPB = 256;

struct AdjArgs {
  const double *u, *h;                        // stage state
  const double *pv, *hs;                      // taped pv, kite-summed h of the stage state
  double *pve;                                // edge pv of the stage state
  double2 *FP;                                // {F = u he, P = lk_u pve} per edge
  const double *un, *hn, *pvn;                // state of the next stage to reverse (prep)
  int prep;                                   // B3 prepares FP, pve of that stage
  double *lk_u, *lk_h;                        // cotangent of the stage tendency (in), next one (out)
  double *mu_u, *mu_h;                        // J^T lk
  double *lhe, *lpve, *lke, *ldiv, *lcirc, *lhs;
  double *lam_u, *lam_h, *acc_u, *acc_h;
  int rk, visc;
  double dt, g, nu;
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
template <int NW>
__global__ void __launch_bounds__(TPB) k_adj_b1(DMesh m, AdjArgs a, int L) {
  stage_prologue();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nE * L) return;
  const int e = (int)(i / L), k = (int)(i - (int64_t)e * L);
  double s1 = 0.0, t1 = 0.0, t2 = 0.0;
  const int ne = NW > 0 ? NW : m.maxEoE;
#pragma unroll
  for (int j = 0; j < ne; ++j) {
    const int64_t s = (int64_t)j * m.nE + e;
    const int64_t io = (int64_t)m.eoe[s] * L + k;
    const double wt = m.woeT[s];
    const double2 fp = a.FP[io];
    s1 = fma(m.woe[s], fp.x, s1);
    t1 = fma(wt, a.lk_u[io], t1);
    t2 = fma(wt, fp.y, t2);
  }
  const int2 c = m.coe[e];
  const int64_t i1 = (int64_t)c.x * L + k, i2 = (int64_t)c.y * L + k;
  const double he = 0.5 * (a.h[i1] + a.h[i2]);
  const double Fe = a.FP[i].x, pve = a.pve[i], ue = a.u[i];
  const double dth = a.lk_h[i2] * m.invAreaCell[c.y] - a.lk_h[i1] * m.invAreaCell[c.x];
  const double lF = fma(0.5, fma(pve, t1, t2), m.dvEdge[e] * dth);
  a.lpve[i] = 0.5 * fma(a.lk_u[i], s1, Fe * t1);
  a.mu_u[i] = lF * he;
  a.lhe[i] = lF * ue;
}

// B2 (cells + vertices): gradient terms, h_e -> h, pv -> (circ, hs).
__global__ void __launch_bounds__(TPB) k_adj_b2(DMesh m, AdjArgs a, int L) {
  stage_prologue();
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nCL = (int64_t)m.nC * L;
  if (i < nCL) {
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
    a.mu_h[i] = fma(0.5, sl, -a.g * G);
    a.lke[i] = -G;
    if (a.visc) a.ldiv[i] = a.nu * G;
    return;
  }
  i -= nCL;
  if (i >= (int64_t)m.nV * L) return;
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

// RK4 cotangent bookkeeping for one element once mu is complete.
__device__ __forceinline__ double combine(const AdjArgs &a, int64_t i, double mu, double *lam, double *acc,
                                          double *lk) {
  const double dt = a.dt;
  double l;
  switch (a.rk) {
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
__global__ void __launch_bounds__(TPB) k_adj_b3(DMesh m, DStat st, AdjArgs a, int L) {
  stage_prologue();
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nCL = (int64_t)m.nC * L;
  if (i < nCL) {
    const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
    double mh = a.mu_h[i];
    for (int j = 0; j < m.maxEoC; ++j) {
      const int64_t s = (int64_t)j * m.nC + c;
      mh = fma(m.kiteR[s], a.lhs[(int64_t)m.vocR[s] * L + k], mh);
    }
    combine(a, i, mh, a.lam_h, a.acc_h, a.lk_h);
    return;
  }
  i -= nCL;
  if (i >= (int64_t)m.nE * L) return;
  const int e = (int)(i / L), k = (int)(i - (int64_t)e * L);
  const int2 c = m.coe[e];
  const int2 v = m.voe[e];
  const int64_t i1 = (int64_t)c.x * L + k, i2 = (int64_t)c.y * L + k;
  const double ia1 = m.invAreaCell[c.x], ia2 = m.invAreaCell[c.y];
  double mu = a.mu_u[i];
  mu = fma(m.dcEdge[e], a.lcirc[(int64_t)v.y * L + k] - a.lcirc[(int64_t)v.x * L + k], mu);
  mu = fma(2.0 * a.u[i] * st.kw[e], fma(a.lke[i1], ia1, a.lke[i2] * ia2), mu);
  if (a.visc) mu = fma(-m.dvEdge[e], fma(a.ldiv[i2], ia2, -a.ldiv[i1] * ia1), mu);
  const double lk = combine(a, i, mu, a.lam_u, a.acc_u, a.lk_u);
  // the next stage's B1 inputs (B1 of this stage has completed)
  if (a.prep) prep_edge(m, a, L, e, k, i, a.un, a.hn, a.pvn, lk);
}

__global__ void k_adj_init(int64_t n, const double *lam, double *lk, double c) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) lk[i] = c * lam[i];
}

void ensure_buffers(SwState &s, int N, int k) {
  const DMesh &m = s.mesh->ctx.d;
  const int64_t L = s.L, eu = (int64_t)m.nE * L, ch = (int64_t)m.nC * L, vv = (int64_t)m.nV * L;
  const int nck = (N + k - 1) / k + 1;
  AdjBuffers *A = s.adj;
  if (A && A->cap_ck >= nck && A->cap_k >= k) return;
  free_adjoint(s);
  A = s.adj = new AdjBuffers();
  std::vector<std::pair<double **, int64_t>> bufs = {
      {&A->ck_u, nck * eu}, {&A->ck_h, nck * ch}, {&A->tp_u, (4LL * k + 1) * eu},
      {&A->tp_h, (4LL * k + 1) * ch}, {&A->uacc, eu}, {&A->hacc, ch}, {&A->tp_pv, (4LL * k + 1) * vv},
      {&A->tp_hs, (4LL * k + 1) * vv},
      {(double **)&A->FP, 2 * eu}, {&A->pve, eu}, {&A->lam_u, eu}, {&A->lam_h, ch}, {&A->acc_u, eu},
      {&A->acc_h, ch}, {&A->lk_u, eu}, {&A->lk_h, ch}, {&A->mu_u, eu}, {&A->mu_h, ch}, {&A->lhe, eu},
      {&A->lpve, eu}, {&A->lke, ch}, {&A->ldiv, ch}, {&A->lcirc, vv}, {&A->lhs, vv}};
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
  A->cap_ck = nck;
  A->cap_k = k;
}

// Reverse of the stage whose input state is tape slot j; `first`: no B3 before
// it prepared its edge quantities; `prep_next`: prepare those of slot j - 1.
void stage_vjp(SwState &s, AdjBuffers &A, int rk, int j, bool first, bool prep_next, cudaStream_t st) {
  const DMesh &m = s.mesh->ctx.d;
  const int L = s.L;
  const int64_t nE = (int64_t)m.nE * L, nC = (int64_t)m.nC * L, nV = (int64_t)m.nV * L;
  AdjArgs a{};
  a.u = A.tp_u + (size_t)j * nE, a.h = A.tp_h + (size_t)j * nC;
  a.pv = A.tp_pv + (size_t)j * nV, a.hs = A.tp_hs + (size_t)j * nV;
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
  if (first) launch_pdl(k_adj_prep, nE, TPB, pdl, st, m, a, L);
  if (m.maxEoE == 10)
    launch_pdl(k_adj_b1<10>, nE, TPB, pdl, st, m, a, L);
  else
    launch_pdl(k_adj_b1<0>, nE, TPB, pdl, st, m, a, L);
  launch_pdl(k_adj_b2, nC + nV, TPB, pdl, st, m, a, L);
  launch_pdl(k_adj_b3, nC + nE, TPB, pdl, st, m, s.st, a, L);
}

void forward(SwState &s, double dt, int N, int k) {
  require(s.p.app == MPASO_APP_SW, MPASO_ERR_ARG, "the adjoint covers the sw app");
  require(!s.p.pin_u, MPASO_ERR_ARG, "the adjoint does not support a pinned wind (test case 1)");
  require(N >= 1 && k >= 1, MPASO_ERR_ARG, "nsteps and ckpt_every must be >= 1");
  ensure_buffers(s, N, k);
  AdjBuffers &A = *s.adj;
  const DMesh &m = s.mesh->ctx.d;
  const size_t eu = (size_t)m.nE * s.L * 8, ch = (size_t)m.nC * s.L * 8;
  A.N = N, A.k = k, A.dt = dt, A.nck = (N + k - 1) / k;
  MPASO_CUDA(cudaMemcpyAsync(A.ck_u, s.U[0], eu, cudaMemcpyDeviceToDevice, s.stream));
  MPASO_CUDA(cudaMemcpyAsync(A.ck_h, s.H[0], ch, cudaMemcpyDeviceToDevice, s.stream));
  for (int done = 0, c = 1; done < N; ++c) {
    const int n = std::min(k, N - done);
    sw_steps_graph(s, dt, n);
    done += n;
    if (done < N) {
      MPASO_CUDA(cudaMemcpyAsync(A.ck_u + (size_t)c * m.nE * s.L, s.U[0], eu, cudaMemcpyDeviceToDevice, s.stream));
      MPASO_CUDA(cudaMemcpyAsync(A.ck_h + (size_t)c * m.nC * s.L, s.H[0], ch, cudaMemcpyDeviceToDevice, s.stream));
    }
  }
  A.have_forward = true;
}

void reverse_body(SwState &s) {
  AdjBuffers &A = *s.adj;
  const DMesh &m = s.mesh->ctx.d;
  const int64_t eu = (int64_t)m.nE * s.L, ch = (int64_t)m.nC * s.L;
  const cudaStream_t st = s.stream;
  k_adj_init<<<blocks_for(eu, TPB), TPB, 0, st>>>(eu, A.lam_u, A.lk_u, A.dt / 6);
  k_adj_init<<<blocks_for(ch, TPB), TPB, 0, st>>>(ch, A.lam_h, A.lk_h, A.dt / 6);
  for (int seg = A.nck - 1; seg >= 0; --seg) {
    const int s0 = seg * A.k, n = std::min(A.k, A.N - s0);
    // taping recompute of the segment: slot 4t + rk holds the input of stage rk of step s0 + t
    MPASO_CUDA(cudaMemcpyAsync(A.tp_u, A.ck_u + (size_t)seg * eu, eu * 8, cudaMemcpyDeviceToDevice, st));
    MPASO_CUDA(cudaMemcpyAsync(A.tp_h, A.ck_h + (size_t)seg * ch, ch * 8, cudaMemcpyDeviceToDevice, st));
    const int64_t vv = (int64_t)m.nV * s.L;
    sw_diag_ptrs(s, A.tp_u, A.tp_h, A.tp_pv, A.tp_hs, st);
    for (int t = 0; t < n; ++t) {
      double *yu = A.tp_u + (size_t)4 * t * eu, *yh = A.tp_h + (size_t)4 * t * ch;
      for (int rk = 0; rk < 4; ++rk) {
        double *iu = yu + (size_t)rk * eu, *ih = yh + (size_t)rk * ch;
        double *ou = yu + (size_t)(rk + 1) * eu, *oh = yh + (size_t)(rk + 1) * ch;
        const size_t next = (size_t)(4 * t + rk + 1) * vv;  // tape slot of the stage's output
        sw_stage_ptrs(s, rk, A.dt, iu, ih, yu, yh, rk < 3 ? ou : nullptr, rk < 3 ? oh : nullptr, A.uacc,
                      A.hacc, rk == 3 ? ou : nullptr, rk == 3 ? oh : nullptr, A.tp_pv + next,
                      A.tp_hs + next, st);
      }
    }
    for (int t = n - 1; t >= 0; --t)
      for (int rk = 3; rk >= 0; --rk) {
        const int j = 4 * t + rk;
        stage_vjp(s, A, rk, j, t == n - 1 && rk == 3, j > 0, st);
      }
  }
  MPASO_CUDA(cudaGetLastError());
}

// The reverse sweep is ~800 launches per segment of small kernels: captured
// once as a graph for the current (N, k, dt) and buffers, then replayed.
void reverse(SwState &s) {
  AdjBuffers &A = *s.adj;
  if (A.rev && (A.rev_N != A.N || A.rev_k != A.k || A.rev_dt != A.dt)) drop_adjoint_graph(s);
  if (!A.rev) {
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
    A.rev_N = A.N, A.rev_k = A.k, A.rev_dt = A.dt;
  }
  MPASO_CUDA(cudaGraphLaunch(A.rev, s.stream));
  s.diag_valid = false;
}

void to_internal(SwState &s, const double *src, double *dst, int entity) {
  MeshCtx &ctx = s.mesh->ctx;
  const int64_t n = entity == MPASO_CELLS ? ctx.d.nC : ctx.d.nE;
  const double *p = src;
  double *stage = nullptr;
  if (!is_device_pointer(src)) {
    MPASO_CUDA(cudaMallocAsync((void **)&stage, (size_t)n * s.L * 8, s.stream));
    MPASO_CUDA(cudaMemcpyAsync(stage, src, (size_t)n * s.L * 8, cudaMemcpyHostToDevice, s.stream));
    p = stage;
  }
  k_gather_rows_pub(p, dst, ctx.d_perm[entity], n, s.L, s.stream);
  if (stage) MPASO_CUDA(cudaFreeAsync(stage, s.stream));
}

void from_internal(SwState &s, const double *src, double *dst, int entity) {
  MeshCtx &ctx = s.mesh->ctx;
  const int64_t n = entity == MPASO_CELLS ? ctx.d.nC : ctx.d.nE;
  const bool dev = is_device_pointer(dst);
  double *out = dst;
  if (!dev) MPASO_CUDA(cudaMallocAsync((void **)&out, (size_t)n * s.L * 8, s.stream));
  k_scatter_rows_pub(src, out, ctx.d_perm[entity], n, s.L, s.stream);
  if (!dev) {
    MPASO_CUDA(cudaMemcpyAsync(dst, out, (size_t)n * s.L * 8, cudaMemcpyDeviceToHost, s.stream));
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
    require(S.adj && S.adj->have_forward, MPASO_ERR_ARG, "mpaso_rk4_vjp needs a preceding mpaso_rk4_forward");
    MPASO_CUDA(cudaSetDevice(S.mesh->ctx.device));
    to_internal(S, gu, S.adj->lam_u, MPASO_EDGES);
    to_internal(S, gh, S.adj->lam_h, MPASO_CELLS);
    reverse(S);
    from_internal(S, S.adj->lam_u, gu0, MPASO_EDGES);
    from_internal(S, S.adj->lam_h, gh0, MPASO_CELLS);
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

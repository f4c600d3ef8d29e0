// Per-task kernels: one GPU kernel set per reference task, same signature and
// semantics, operating on the context's renumbered HBM layout.
//
// Each kernel evaluates every output element with the same sequence of IEEE
// operations as the reference loop it cites (this file is compiled with
// -fmad=false, so no multiply-add is fused), and scatter loops of the
// reference become gathers over the reverse connectivity in the order the
// scatter visited them.  Results therefore agree bit for bit with the
// reference tasks.  One thread per (entity, level); tracers loop inside.
#include "task_io.cuh"

namespace mpaso {
namespace {

constexpr int TPB = 256;

// ---------------------------------------------------------------- sw tasks
// apps/sw/tasks/solve.cc:31-39 (h_edge), :41-60 (circulation, vorticity),
// :62-77 (ke), :81-92 (h_vertex, pv_vertex).
__global__ void k_sw_diag_a(DMesh m, int L, const double *__restrict__ h, const double *__restrict__ u,
                            double *h_edge, double *h_vertex, double *circulation, double *vorticity,
                            double *ke, double *pv_vertex) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nEL = (int64_t)m.nE * L, nVL = (int64_t)m.nV * L, nCL = (int64_t)m.nC * L;
  if (i < nEL) {
    const int e = (int)(i / L), k = (int)(i - (int64_t)e * L);
    const int2 c = m.coe[e];
    h_edge[i] = 0.5 * (h[(int64_t)c.x * L + k] + h[(int64_t)c.y * L + k]);
    return;
  }
  i -= nEL;
  if (i < nVL) {
    const int v = (int)(i / L), k = (int)(i - (int64_t)v * L);
    double circ = 0.0;
    for (int j = 0; j < kVertexDegree; ++j) {  // edges in ascending reference order
      const int e = m.eov[(int64_t)j * m.nV + v];
      const double t = m.dcEdge[e] * u[(int64_t)e * L + k];
      circ = (m.eovSign[(int64_t)j * m.nV + v] < 0.0) ? circ - t : circ + t;
    }
    circulation[i] = circ;
    const double vort = circ / m.areaTriangle[v];
    vorticity[i] = vort;
    double hv = 0.0;
    for (int j = 0; j < kVertexDegree; ++j)
      hv += h[(int64_t)m.cov[(int64_t)j * m.nV + v] * L + k] * m.kite[(int64_t)j * m.nV + v];
    hv /= m.areaTriangle[v];
    h_vertex[i] = hv;
    pv_vertex[i] = (m.fVertex[v] + vort) / hv;
    return;
  }
  i -= nVL;
  if (i < nCL) {
    const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
    double s = 0.0;
    const int n = m.nEoC[c];
    for (int j = 0; j < n; ++j) {
      const int e = m.eoc[(int64_t)j * m.nC + c];
      const double ue = u[(int64_t)e * L + k];
      s += 0.25 * m.dcEdge[e] * m.dvEdge[e] * (ue * ue);
    }
    ke[i] = s / m.areaCell[c];
  }
}

// apps/sw/tasks/solve.cc:95-106: pv_edge(e) = 0 + 0.5 pv(v) over the edge's two vertices.
__global__ void k_sw_diag_b(DMesh m, int L, const double *__restrict__ pv_vertex, double *pv_edge) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nE * L) return;
  const int e = (int)(i / L), k = (int)(i - (int64_t)e * L);
  const int2 v = m.voe[e];
  const double a = 0.5 * pv_vertex[(int64_t)v.x * L + k], b = 0.5 * pv_vertex[(int64_t)v.y * L + k];
  pv_edge[i] = (0.0 + a) + b;  // two terms: order-free
}

// apps/sw/tasks/solve.cc:169-234
__global__ void k_sw_tend(DMesh m, int L, double g, const double *__restrict__ h_edge,
                          const double *__restrict__ h, const double *__restrict__ u,
                          const double *__restrict__ ke, const double *__restrict__ pv_edge,
                          double *tend_h, double *tend_u) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nEL = (int64_t)m.nE * L, nCL = (int64_t)m.nC * L;
  if (i < nEL) {
    const int e = (int)(i / L), k = (int)(i - (int64_t)e * L);
    const int2 c = m.coe[e];
    const int n = m.nEoE[e];
    const double pve = pv_edge[i];
    double q = 0;
    for (int j = 0; j < n; ++j) {
      const int eo = m.eoe[(int64_t)j * m.nE + e];
      const double workpv = 0.5 * (pve + pv_edge[(int64_t)eo * L + k]);
      q = q + m.woe[(int64_t)j * m.nE + e] * u[(int64_t)eo * L + k] * workpv * h_edge[(int64_t)eo * L + k];
    }
    const int64_t i1 = (int64_t)c.x * L + k, i2 = (int64_t)c.y * L + k;
    tend_u[i] = q - (ke[i2] - ke[i1] + g * (h[i2] + m.bottomDepth[c.y] - h[i1] - m.bottomDepth[c.x])) /
                        m.dcEdge[e];
    return;
  }
  i -= nEL;
  if (i < nCL) {
    const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
    double t = 0;
    const int n = m.nEoC[c];
    for (int j = 0; j < n; ++j) {  // scatter order: ascending reference edge id
      const int e = m.eocAsc[(int64_t)j * m.nC + c];
      const double flux = u[(int64_t)e * L + k] * m.dvEdge[e] * h_edge[(int64_t)e * L + k];
      t = (m.eocAscSign[(int64_t)j * m.nC + c] < 0.0) ? t - flux : t + flux;
    }
    tend_h[i] = t / m.areaCell[c];
  }
}

// apps/sw/tasks/solve.cc:237-270
__global__ void k_sw_scalar_tend(DMesh m, int L, int T, const double *__restrict__ h_edge,
                                 const double *__restrict__ u, const double *__restrict__ tr,
                                 double *tend) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nC * L) return;
  const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
  const int n = m.nEoC[c];
  for (int t = 0; t < T; ++t) {
    double acc = 0.0;
    for (int j = 0; j < n; ++j) {
      const int e = m.eocAsc[(int64_t)j * m.nC + c];
      const int2 cc = m.coe[e];
      const double tr_edge = 0.5 * (tr[((int64_t)cc.x * L + k) * T + t] + tr[((int64_t)cc.y * L + k) * T + t]);
      const double flux = u[(int64_t)e * L + k] * m.dvEdge[e] * h_edge[(int64_t)e * L + k] * tr_edge;
      acc = (m.eocAscSign[(int64_t)j * m.nC + c] < 0.0) ? acc - flux / m.areaCell[c]
                                                         : acc + flux / m.areaCell[c];
    }
    tend[i * T + t] = acc;
  }
}

// Elementwise sw tasks (no connectivity): apps/sw/tasks/solve.cc:273-367.
__global__ void k_sw_substep(int64_t nEL, int64_t nCL, int T, double *u_p, const double *u_o,
                             const double *u_t, double *h_p, const double *h_o, const double *h_t,
                             double *tr_p, const double *tr_o, const double *tr_t, double w, int pin_u) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < nEL) u_p[i] = pin_u ? u_o[i] : u_o[i] + w * u_t[i];
  if (i < nCL) {
    const double hp = h_o[i] + w * h_t[i];
    h_p[i] = hp;
    for (int t = 0; t < T; ++t) tr_p[i * T + t] = (h_o[i] * tr_o[i * T + t] + w * tr_t[i * T + t]) / hp;
  }
}

__global__ void k_sw_accumulate(int64_t nEL, int64_t nCL, int T, double *u_n, const double *u_t,
                                double *h_n, const double *h_t, double *tr_n, const double *tr_t,
                                double w) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < nEL) u_n[i] += w * u_t[i];
  if (i < nCL) {
    h_n[i] += w * h_t[i];
    for (int t = 0; t < T; ++t) tr_n[i * T + t] += w * tr_t[i * T + t];
  }
}

__global__ void k_sw_finalize(int64_t nEL, int64_t nCL, int T, const double *u_o, double *u_n,
                              const double *h_n, double *tr_n, int pin_u) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < nCL)
    for (int t = 0; t < T; ++t) tr_n[i * T + t] /= h_n[i];
  if (pin_u && i < nEL) u_n[i] = u_o[i];
}

// ---------------------------------------------------------------- ocean tasks
__global__ void k_oc_ntf(int64_t n, const double *hE, const double *u, double *ntf) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) ntf[i] = u[i] * hE[i];  // apps/ocean/tasks/solve.cc:49-54
}

// apps/ocean/tasks/solve.cc:60-97
__global__ void k_oc_provisional(DMesh m, int L, const double *__restrict__ h,
                                 const double *__restrict__ ntf, double *hProv, double *hProvInv,
                                 double *hNewInv, double dt) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nC * L) return;
  const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
  if (k >= m.maxLevelCell[c]) return;
  const double dtInvAreaCell = dt / m.areaCell[c];
  double hp = h[i];
  const int n = m.nEoC[c];
  for (int j = 0; j < n; ++j) {
    const int e = m.eoc[(int64_t)j * m.nC + c];
    const double sf = dtInvAreaCell * m.dvEdge[e] * m.eocSign[(int64_t)j * m.nC + c];
    hp += sf * ntf[(int64_t)e * L + k];
  }
  hProv[i] = hp;
  hProvInv[i] = 1.0 / hp;
  hNewInv[i] = 1.0 / hp;
}

// apps/ocean/tasks/solve.cc:99-118
__global__ void k_oc_low_order(DMesh m, int L, int T, const double *__restrict__ ntf,
                               const double *__restrict__ tr, double *lo) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nE * L) return;
  const int e = (int)(i / L), k = (int)(i - (int64_t)e * L);
  const int2 c = m.coe[e];
  const double f = ntf[i];
  const double ntf1 = (0.0 < f) ? f : 0.0;  // std::max(0.0, f)
  const double ntf2 = (f < 0.0) ? f : 0.0;  // std::min(0.0, f)
  for (int t = 0; t < T; ++t)
    lo[i * T + t] = m.dvEdge[e] * (ntf1 * tr[((int64_t)c.x * L + k) * T + t] +
                                   ntf2 * tr[((int64_t)c.y * L + k) * T + t]);
}

// apps/ocean/tasks/solve.cc:120-167 (coef3rdOrder = 0.25, :11)
__global__ void k_oc_high_order(DMesh m, int L, int T, const double *__restrict__ ntf,
                                const double *__restrict__ tr, double *ho) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nE * L) return;
  const int e = (int)(i / L), k = (int)(i - (int64_t)e * L);
  const double f = ntf[i];
  const double wgt = f * (double)m.hoMask[(int64_t)e * m.fctLev + k];
  const double sgn = (f < 0.0) ? -1.0 : (f > 0. ? 1.0 : 0.0);
  double flx[kMaxTracers];
  for (int t = 0; t < T; ++t) flx[t] = 0.0;
  const int n = m.nAdv[e];
  for (int a = 0; a < n; ++a) {
    const int cell = m.advCells[(int64_t)a * m.nE + e];
    const double coef1 = m.advCoef[(int64_t)a * m.nE + e];
    const double coef3 = m.advCoef3[(int64_t)a * m.nE + e] * 0.25;
    if (k < m.maxLevelCell[cell]) {
      const double wf = wgt * (coef1 + coef3 * sgn);
      for (int t = 0; t < T; ++t) flx[t] += tr[((int64_t)cell * L + k) * T + t] * wf;
    }
  }
  for (int t = 0; t < T; ++t) ho[i * T + t] = flx[t];
}

// apps/ocean/tasks/solve.cc:194-229: bounds (cells) and anti-diffusive flux (edges).
__global__ void k_oc_fct_a(DMesh m, int L, int T, const double *__restrict__ ntf,
                           const double *__restrict__ lo, const double *__restrict__ tr, double *ho,
                           double *flxIn, double *flxOut, double *trMax, double *trMin) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nCL = (int64_t)m.nC * L, nEL = (int64_t)m.nE * L;
  if (i < nCL) {
    const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
    const int mlc = m.maxLevelCell[c];
    if (k < mlc) {
      const int n = m.nEoC[c];
      for (int t = 0; t < T; ++t) {
        double mx = tr[i * T + t], mn = mx;
        for (int j = 0; j < n; ++j) {
          const int c2 = m.coc[(int64_t)j * m.nC + c];
          if (k < min(mlc, m.maxLevelCell[c2])) {
            const double x = tr[((int64_t)c2 * L + k) * T + t];
            mx = (mx < x) ? x : mx;  // std::max
            mn = (x < mn) ? x : mn;  // std::min
          }
        }
        trMax[i * T + t] = mx;
        trMin[i * T + t] = mn;
        flxIn[i * T + t] = 0.0;
        flxOut[i * T + t] = 0.0;
      }
    }
    return;
  }
  i -= nCL;
  if (i < nEL) {
    const int e = (int)(i / L), k = (int)(i - (int64_t)e * L);
    if (k >= m.maxLevelEdgeTop[e]) return;
    const int2 c = m.coe[e];
    const double tw = (double)((m.hoMask[(int64_t)e * m.fctLev + k] + 1) & 1) * (m.dvEdge[e] * 0.5) * ntf[i];
    for (int t = 0; t < T; ++t) {
      double x = ho[i * T + t];
      x += tw * (tr[((int64_t)c.x * L + k) * T + t] + tr[((int64_t)c.y * L + k) * T + t]);
      x -= lo[i * T + t];
      ho[i * T + t] = x;
    }
  }
}

// apps/ocean/tasks/solve.cc:232-267: per-cell sums and limiter factors.
__global__ void k_oc_fct_b(DMesh m, int L, int T, const double *__restrict__ hProvInv,
                           const double *__restrict__ h, const double *__restrict__ lo,
                           const double *__restrict__ tr, const double *__restrict__ ho,
                           double *flxIn, double *flxOut, double *tend,
                           const double *__restrict__ trMax, const double *__restrict__ trMin,
                           double dt) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nC * L) return;
  const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
  const double eps = 1.e-10;
  const double invAreaCell1 = 1.0 / m.areaCell[c];
  const int n = m.nEoC[c];
  for (int t = 0; t < T; ++t) {
    double td = tend[i * T + t], fin = flxIn[i * T + t], fout = flxOut[i * T + t];
    for (int j = 0; j < n; ++j) {
      const int e = m.eoc[(int64_t)j * m.nC + c];
      if (k < m.maxLevelEdgeTop[e]) {
        const double sf = m.eocSign[(int64_t)j * m.nC + c] * invAreaCell1;
        td += sf * lo[((int64_t)e * L + k) * T + t];
        const double x = sf * ho[((int64_t)e * L + k) * T + t];
        fin += (0.0 < x) ? x : 0.0;
        fout += (x < 0.0) ? x : 0.0;
      }
    }
    tend[i * T + t] = td;
    if (k < m.maxLevelCell[c]) {
      const double hpi = hProvInv[i];
      const double up = (tr[i * T + t] * h[i] + dt * td) * hpi;
      const double mxn = up + dt * fin * hpi;
      const double mnn = up + dt * fout * hpi;
      double sfac = (trMax[i * T + t] - up) / (mxn - up + eps);
      sfac = (0.0 < sfac) ? sfac : 0.0;
      flxIn[i * T + t] = (sfac < 1.0) ? sfac : 1.0;
      sfac = (up - trMin[i * T + t]) / (up - mnn + eps);
      sfac = (0.0 < sfac) ? sfac : 0.0;
      flxOut[i * T + t] = (sfac < 1.0) ? sfac : 1.0;
    } else {
      flxIn[i * T + t] = fin;
      flxOut[i * T + t] = fout;
    }
  }
}

// apps/ocean/tasks/solve.cc:270-282: rescale anti-diffusive fluxes.
__global__ void k_oc_fct_c(DMesh m, int L, int T, const double *__restrict__ flxIn,
                           const double *__restrict__ flxOut, double *ho) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nE * L) return;
  const int e = (int)(i / L), k = (int)(i - (int64_t)e * L);
  if (k >= m.maxLevelEdgeTop[e]) return;
  const int2 c = m.coe[e];
  for (int t = 0; t < T; ++t) {
    const double x = ho[i * T + t];
    const int64_t i1 = ((int64_t)c.x * L + k) * T + t, i2 = ((int64_t)c.y * L + k) * T + t;
    const double a = flxIn[i2] < flxOut[i1] ? flxIn[i2] : flxOut[i1];
    const double b = flxOut[i2] < flxIn[i1] ? flxOut[i2] : flxIn[i1];
    ho[i * T + t] = ((0.0 < x) ? x : 0.0) * a + ((x < 0.0) ? x : 0.0) * b;
  }
}

// apps/ocean/tasks/solve.cc:287-326
__global__ void k_oc_accumulate_fct(DMesh m, int L, int T, const double *__restrict__ hProvInv,
                                    const double *__restrict__ h, const double *__restrict__ ho,
                                    const double *__restrict__ tr, double *trProv, double *tend,
                                    double dt) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nC * L) return;
  const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
  const double invAreaCell1 = 1.0 / m.areaCell[c];
  const int n = m.nEoC[c];
  for (int t = 0; t < T; ++t) {
    double td = tend[i * T + t];
    for (int j = 0; j < n; ++j) {
      const int e = m.eoc[(int64_t)j * m.nC + c];
      if (k < m.maxLevelEdgeTop[e])
        td += m.eocSign[(int64_t)j * m.nC + c] * invAreaCell1 * ho[((int64_t)e * L + k) * T + t];
    }
    tend[i * T + t] = td;
    if (k < m.maxLevelCell[c]) trProv[i * T + t] = (tr[i * T + t] * h[i] + dt * td) * hProvInv[i];
  }
}

// apps/ocean/tasks/solve.cc:328-366
__global__ void k_oc_hmix(DMesh m, int L, int T, const double *__restrict__ hE,
                          const double *__restrict__ tr, double *tend, double coef) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)m.nC * L) return;
  const int c = (int)(i / L), k = (int)(i - (int64_t)c * L);
  const double invArea = 1.0 / m.areaCell[c];
  const int n = m.nEoC[c];
  for (int t = 0; t < T; ++t) {
    double td = tend[i * T + t];
    for (int j = 0; j < n; ++j) {
      const int e = m.eoc[(int64_t)j * m.nC + c];
      if (k < m.maxLevelEdgeTop[e]) {
        const int2 cc = m.coe[e];
        const double rho = m.meshScalingDel2[e] * coef * m.dvEdge[e] / m.dcEdge[e];
        const double ttf = tr[((int64_t)cc.y * L + k) * T + t] - tr[((int64_t)cc.x * L + k) * T + t];
        const double flux = hE[(int64_t)e * L + k] * ttf * rho;
        td -= m.eocSign[(int64_t)j * m.nC + c] * flux * invArea;
      }
    }
    tend[i * T + t] = td;
  }
}

// apps/ocean/tasks/solve.cc:368-399
__global__ void k_oc_step_forward(int64_t n, const double *tend, const double *tr, double *trNew,
                                  double *trPrev, double w, double wsub) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  trNew[i] += w * tend[i];
  trPrev[i] = tr[i] + wsub * tend[i];
}

void check_levels(int L, int T) {
  require(L >= 1 && L <= 4096, MPASO_ERR_ARG, "nlev out of range");
  require(T >= 0 && T <= kMaxTracers, MPASO_ERR_ARG, "ntr out of range (max 8)");
}

void require_fct(TaskIO &io, int L) {
  require(io.ctx().has_fct, MPASO_ERR_ARG, "mesh context was created without FCT statics");
  require(io.dm().fctLev == L, MPASO_ERR_ARG, "nlev differs from the FCT statics' level count");
}

cudaStream_t plain_stream(mpaso_mesh m, void *stream) {
  require(m != nullptr, MPASO_ERR_ARG, "null mesh context");
  MPASO_CUDA(cudaSetDevice(m->ctx.device));
  return stream ? (cudaStream_t)stream : m->ctx.stream;
}

// Elementwise tasks need no renumbering: they run on the caller's arrays
// directly when all are device memory, else on staged copies.
struct Flat {
  std::vector<std::pair<double *, size_t>> args;  // user ptr, doubles
  std::vector<bool> out;
  std::vector<double *> dev;
  bool host = false;
  cudaStream_t s;
  mpaso_mesh m;
  void add(const double *p, size_t n, bool o) {
    require(p != nullptr, MPASO_ERR_ARG, "null field pointer");
    args.push_back({const_cast<double *>(p), n});
    out.push_back(o);
    host |= !is_device_pointer(p);
  }
  void stage() {
    dev.resize(args.size());
    if (!host) {
      for (size_t a = 0; a < args.size(); ++a) dev[a] = args[a].first;
      return;
    }
    size_t total = 0;
    for (auto &a : args) total += (a.second * sizeof(double) + 255) & ~size_t(255);
    char *base = (char *)m->ctx.ensure_scratch(total);
    for (size_t a = 0; a < args.size(); ++a) {
      dev[a] = (double *)base;
      base += (args[a].second * sizeof(double) + 255) & ~size_t(255);
      const cudaMemcpyKind kind = is_device_pointer(args[a].first) ? cudaMemcpyDeviceToDevice
                                                                    : cudaMemcpyHostToDevice;
      MPASO_CUDA(cudaMemcpyAsync(dev[a], args[a].first, args[a].second * sizeof(double), kind, s));
    }
  }
  void finish() {
    MPASO_CUDA(cudaGetLastError());
    if (!host) return;
    for (size_t a = 0; a < args.size(); ++a)
      if (out[a]) {
        const cudaMemcpyKind kind = is_device_pointer(args[a].first) ? cudaMemcpyDeviceToDevice
                                                                      : cudaMemcpyDeviceToHost;
        MPASO_CUDA(cudaMemcpyAsync(args[a].first, dev[a], args[a].second * sizeof(double), kind, s));
      }
    MPASO_CUDA(cudaStreamSynchronize(s));
  }
};

}  // namespace

// Launches the compute_tend kernel on arrays already in the context's
// numbering (used by the allocation-free entry point in noalloc.cu).
void launch_task_sw_tend(const DMesh &d, int L, double g, const double *h_edge, const double *h,
                         const double *u, const double *ke, const double *pv_edge, double *tend_h,
                         double *tend_u, cudaStream_t s) {
  const int64_t n = ((int64_t)d.nE + d.nC) * L;
  k_sw_tend<<<blocks_for(n, TPB), TPB, 0, s>>>(d, L, g, h_edge, h, u, ke, pv_edge, tend_h, tend_u);
}

}  // namespace mpaso

using namespace mpaso;

extern "C" {

int mpaso_sw_compute_solve_diagnostics(mpaso_mesh m, int32_t nlev, const double *h,
                                       const double *u, double *h_edge, double *h_vertex,
                                       double *circulation, double *vorticity, double *ke,
                                       double *pv_edge, double *pv_vertex, void *stream) {
  return guarded("mpaso_sw_compute_solve_diagnostics", [&] {
    check_levels(nlev, 0);
    TaskIO io(m, stream);
    const int L = nlev;
    const int ih = io.in(h, MPASO_CELLS, L), iu = io.in(u, MPASO_EDGES, L);
    const int ohe = io.out(h_edge, MPASO_EDGES, L), ohv = io.out(h_vertex, MPASO_VERTICES, L);
    const int oci = io.out(circulation, MPASO_VERTICES, L), ovo = io.out(vorticity, MPASO_VERTICES, L);
    const int oke = io.out(ke, MPASO_CELLS, L), ope = io.out(pv_edge, MPASO_EDGES, L);
    const int opv = io.out(pv_vertex, MPASO_VERTICES, L);
    io.stage();
    const DMesh &d = io.dm();
    const int64_t n = ((int64_t)d.nE + d.nV + d.nC) * L;
    k_sw_diag_a<<<blocks_for(n, TPB), TPB, 0, io.stream()>>>(d, L, io.ptr(ih), io.ptr(iu), io.ptr(ohe),
                                                             io.ptr(ohv), io.ptr(oci), io.ptr(ovo),
                                                             io.ptr(oke), io.ptr(opv));
    k_sw_diag_b<<<blocks_for((int64_t)d.nE * L, TPB), TPB, 0, io.stream()>>>(d, L, io.ptr(opv), io.ptr(ope));
    io.finish();
  });
}

int mpaso_sw_compute_tend(mpaso_mesh m, int32_t nlev, const double *h_edge, const double *h,
                          const double *u, const double *ke, const double *pv_edge,
                          double *tend_h, double *tend_u, void *stream) {
  return guarded("mpaso_sw_compute_tend", [&] {
    check_levels(nlev, 0);
    TaskIO io(m, stream);
    const int L = nlev;
    const int ihe = io.in(h_edge, MPASO_EDGES, L), ih = io.in(h, MPASO_CELLS, L);
    const int iu = io.in(u, MPASO_EDGES, L), ike = io.in(ke, MPASO_CELLS, L);
    const int ipe = io.in(pv_edge, MPASO_EDGES, L);
    const int oth = io.out(tend_h, MPASO_CELLS, L), otu = io.out(tend_u, MPASO_EDGES, L);
    io.stage();
    const DMesh &d = io.dm();
    const int64_t n = ((int64_t)d.nE + d.nC) * L;
    k_sw_tend<<<blocks_for(n, TPB), TPB, 0, io.stream()>>>(d, L, io.ctx().gravity, io.ptr(ihe), io.ptr(ih),
                                                           io.ptr(iu), io.ptr(ike), io.ptr(ipe),
                                                           io.ptr(oth), io.ptr(otu));
    io.finish();
  });
}

int mpaso_sw_compute_scalar_tend(mpaso_mesh m, int32_t nlev, int32_t ntr, const double *h_edge,
                                 const double *u, const double *tracers, double *tracer_tend,
                                 void *stream) {
  return guarded("mpaso_sw_compute_scalar_tend", [&] {
    check_levels(nlev, ntr);
    TaskIO io(m, stream);
    const int L = nlev, T = ntr;
    const int ihe = io.in(h_edge, MPASO_EDGES, L), iu = io.in(u, MPASO_EDGES, L);
    const int itr = io.in(tracers, MPASO_CELLS, L * T);
    const int ot = io.out(tracer_tend, MPASO_CELLS, L * T);
    io.stage();
    const DMesh &d = io.dm();
    k_sw_scalar_tend<<<blocks_for((int64_t)d.nC * L, TPB), TPB, 0, io.stream()>>>(
        d, L, T, io.ptr(ihe), io.ptr(iu), io.ptr(itr), io.ptr(ot));
    io.finish();
  });
}

int mpaso_sw_compute_substep(mpaso_mesh m, int32_t nlev, int32_t ntr, double *u_provis,
                             const double *u_old, const double *u_tend, double *h_provis,
                             const double *h_old, const double *h_tend, double *tracers_provis,
                             const double *tracers_old, const double *tracers_tend,
                             double rkweight, int32_t pin_u, void *stream) {
  return guarded("mpaso_sw_compute_substep", [&] {
    check_levels(nlev, ntr);
    Flat f;
    f.s = plain_stream(m, stream), f.m = m;
    const size_t nEL = (size_t)m->ctx.d.nE * nlev, nCL = (size_t)m->ctx.d.nC * nlev;
    f.add(u_provis, nEL, true), f.add(u_old, nEL, false), f.add(u_tend, nEL, false);
    f.add(h_provis, nCL, true), f.add(h_old, nCL, false), f.add(h_tend, nCL, false);
    f.add(tracers_provis, nCL * ntr, true), f.add(tracers_old, nCL * ntr, false);
    f.add(tracers_tend, nCL * ntr, false);
    f.stage();
    k_sw_substep<<<blocks_for((int64_t)std::max(nEL, nCL), TPB), TPB, 0, f.s>>>(
        nEL, nCL, ntr, f.dev[0], f.dev[1], f.dev[2], f.dev[3], f.dev[4], f.dev[5], f.dev[6],
        f.dev[7], f.dev[8], rkweight, pin_u);
    f.finish();
  });
}

int mpaso_sw_accumulate_update(mpaso_mesh m, int32_t nlev, int32_t ntr, double *u_new,
                               const double *u_tend, double *h_new, const double *h_tend,
                               double *tracers_new, const double *tracers_tend, double rkweight,
                               void *stream) {
  return guarded("mpaso_sw_accumulate_update", [&] {
    check_levels(nlev, ntr);
    Flat f;
    f.s = plain_stream(m, stream), f.m = m;
    const size_t nEL = (size_t)m->ctx.d.nE * nlev, nCL = (size_t)m->ctx.d.nC * nlev;
    f.add(u_new, nEL, true), f.add(u_tend, nEL, false), f.add(h_new, nCL, true);
    f.add(h_tend, nCL, false), f.add(tracers_new, nCL * ntr, true), f.add(tracers_tend, nCL * ntr, false);
    f.stage();
    k_sw_accumulate<<<blocks_for((int64_t)std::max(nEL, nCL), TPB), TPB, 0, f.s>>>(
        nEL, nCL, ntr, f.dev[0], f.dev[1], f.dev[2], f.dev[3], f.dev[4], f.dev[5], rkweight);
    f.finish();
  });
}

int mpaso_sw_finalize_timestep(mpaso_mesh m, int32_t nlev, int32_t ntr, const double *u_old,
                               double *u_new, const double *h_new, double *tracers_new,
                               int32_t pin_u, void *stream) {
  return guarded("mpaso_sw_finalize_timestep", [&] {
    check_levels(nlev, ntr);
    Flat f;
    f.s = plain_stream(m, stream), f.m = m;
    const size_t nEL = (size_t)m->ctx.d.nE * nlev, nCL = (size_t)m->ctx.d.nC * nlev;
    f.add(u_old, nEL, false), f.add(u_new, nEL, true), f.add(h_new, nCL, false);
    f.add(tracers_new, nCL * ntr, true);
    f.stage();
    k_sw_finalize<<<blocks_for((int64_t)std::max(nEL, nCL), TPB), TPB, 0, f.s>>>(
        nEL, nCL, ntr, f.dev[0], f.dev[1], f.dev[2], f.dev[3], pin_u);
    f.finish();
  });
}

int mpaso_oc_calc_normal_thickness_flux(mpaso_mesh m, int32_t nlev,
                                        const double *layerThicknessEdge,
                                        const double *normalVelocity,
                                        double *normalThicknessFlux, void *stream) {
  return guarded("mpaso_oc_calc_normal_thickness_flux", [&] {
    check_levels(nlev, 0);
    Flat f;
    f.s = plain_stream(m, stream), f.m = m;
    const size_t nEL = (size_t)m->ctx.d.nE * nlev;
    f.add(layerThicknessEdge, nEL, false), f.add(normalVelocity, nEL, false);
    f.add(normalThicknessFlux, nEL, true);
    f.stage();
    k_oc_ntf<<<blocks_for((int64_t)nEL, TPB), TPB, 0, f.s>>>(nEL, f.dev[0], f.dev[1], f.dev[2]);
    f.finish();
  });
}

int mpaso_oc_calc_provisional_layer_thicknesses(mpaso_mesh m, int32_t nlev,
                                                const double *layerThickness,
                                                const double *normalThicknessFlux,
                                                double *hProv, double *hProvInv, double *hNewInv,
                                                double dt, void *stream) {
  return guarded("mpaso_oc_calc_provisional_layer_thicknesses", [&] {
    check_levels(nlev, 0);
    TaskIO io(m, stream);
    require(io.ctx().has_fct || true, MPASO_ERR_ARG, "");
    const int L = nlev;
    const int ih = io.in(layerThickness, MPASO_CELLS, L), intf = io.in(normalThicknessFlux, MPASO_EDGES, L);
    const int op = io.out(hProv, MPASO_CELLS, L), opi = io.out(hProvInv, MPASO_CELLS, L);
    const int oni = io.out(hNewInv, MPASO_CELLS, L);
    io.stage();
    const DMesh &d = io.dm();
    k_oc_provisional<<<blocks_for((int64_t)d.nC * L, TPB), TPB, 0, io.stream()>>>(
        d, L, io.ptr(ih), io.ptr(intf), io.ptr(op), io.ptr(opi), io.ptr(oni), dt);
    io.finish();
  });
}

int mpaso_oc_calc_horiz_tracer_advection_flux_mono_low_order(
    mpaso_mesh m, int32_t nlev, int32_t ntr, const double *normalThicknessFlux,
    const double *tracers, double *lowOrderFlux, void *stream) {
  return guarded("mpaso_oc_calc_horiz_tracer_advection_flux_mono_low_order", [&] {
    check_levels(nlev, ntr);
    TaskIO io(m, stream);
    const int L = nlev, T = ntr;
    const int intf = io.in(normalThicknessFlux, MPASO_EDGES, L), itr = io.in(tracers, MPASO_CELLS, L * T);
    const int olo = io.out(lowOrderFlux, MPASO_EDGES, L * T);
    io.stage();
    const DMesh &d = io.dm();
    k_oc_low_order<<<blocks_for((int64_t)d.nE * L, TPB), TPB, 0, io.stream()>>>(d, L, T, io.ptr(intf),
                                                                                 io.ptr(itr), io.ptr(olo));
    io.finish();
  });
}

int mpaso_oc_calc_horiz_tracer_advection_flux_mono_high_order(
    mpaso_mesh m, int32_t nlev, int32_t ntr, const double *normalThicknessFlux,
    const double *tracers, double *highOrderFlux, void *stream) {
  return guarded("mpaso_oc_calc_horiz_tracer_advection_flux_mono_high_order", [&] {
    check_levels(nlev, ntr);
    TaskIO io(m, stream);
    require_fct(io, nlev);
    const int L = nlev, T = ntr;
    const int intf = io.in(normalThicknessFlux, MPASO_EDGES, L), itr = io.in(tracers, MPASO_CELLS, L * T);
    const int oho = io.out(highOrderFlux, MPASO_EDGES, L * T);
    io.stage();
    const DMesh &d = io.dm();
    k_oc_high_order<<<blocks_for((int64_t)d.nE * L, TPB), TPB, 0, io.stream()>>>(d, L, T, io.ptr(intf),
                                                                                  io.ptr(itr), io.ptr(oho));
    io.finish();
  });
}

int mpaso_oc_correct_and_rescale_high_order_mono_horiz_flux(
    mpaso_mesh m, int32_t nlev, int32_t ntr, const double *hProvInv, const double *layerThickness,
    const double *normalThicknessFlux, const double *lowOrderFlux, const double *tracers,
    double *highOrderFlux, double *flxIn, double *flxOut, double *tend, double *tracerMax,
    double *tracerMin, double dt, void *stream) {
  return guarded("mpaso_oc_correct_and_rescale_high_order_mono_horiz_flux", [&] {
    check_levels(nlev, ntr);
    TaskIO io(m, stream);
    require_fct(io, nlev);
    const int L = nlev, T = ntr;
    const int ihpi = io.in(hProvInv, MPASO_CELLS, L), ih = io.in(layerThickness, MPASO_CELLS, L);
    const int intf = io.in(normalThicknessFlux, MPASO_EDGES, L);
    const int ilo = io.in(lowOrderFlux, MPASO_EDGES, L * T), itr = io.in(tracers, MPASO_CELLS, L * T);
    const int oho = io.out(highOrderFlux, MPASO_EDGES, L * T);
    const int ofi = io.out(flxIn, MPASO_CELLS, L * T), ofo = io.out(flxOut, MPASO_CELLS, L * T);
    const int ote = io.out(tend, MPASO_CELLS, L * T);
    const int omx = io.out(tracerMax, MPASO_CELLS, L * T), omn = io.out(tracerMin, MPASO_CELLS, L * T);
    io.stage();
    const DMesh &d = io.dm();
    const cudaStream_t s = io.stream();
    k_oc_fct_a<<<blocks_for(((int64_t)d.nC + d.nE) * L, TPB), TPB, 0, s>>>(
        d, L, T, io.ptr(intf), io.ptr(ilo), io.ptr(itr), io.ptr(oho), io.ptr(ofi), io.ptr(ofo),
        io.ptr(omx), io.ptr(omn));
    k_oc_fct_b<<<blocks_for((int64_t)d.nC * L, TPB), TPB, 0, s>>>(
        d, L, T, io.ptr(ihpi), io.ptr(ih), io.ptr(ilo), io.ptr(itr), io.ptr(oho), io.ptr(ofi),
        io.ptr(ofo), io.ptr(ote), io.ptr(omx), io.ptr(omn), dt);
    k_oc_fct_c<<<blocks_for((int64_t)d.nE * L, TPB), TPB, 0, s>>>(d, L, T, io.ptr(ofi), io.ptr(ofo),
                                                                   io.ptr(oho));
    io.finish();
  });
}

int mpaso_oc_accumulate_horiz_tracer_advection_tend_mono_FCT(
    mpaso_mesh m, int32_t nlev, int32_t ntr, const double *hProvInv, const double *layerThickness,
    const double *highOrderFlux, const double *tracers, double *tracersProv, double *tend,
    double dt, void *stream) {
  return guarded("mpaso_oc_accumulate_horiz_tracer_advection_tend_mono_FCT", [&] {
    check_levels(nlev, ntr);
    TaskIO io(m, stream);
    require_fct(io, nlev);
    const int L = nlev, T = ntr;
    const int ihpi = io.in(hProvInv, MPASO_CELLS, L), ih = io.in(layerThickness, MPASO_CELLS, L);
    const int iho = io.in(highOrderFlux, MPASO_EDGES, L * T), itr = io.in(tracers, MPASO_CELLS, L * T);
    const int otp = io.out(tracersProv, MPASO_CELLS, L * T), ote = io.out(tend, MPASO_CELLS, L * T);
    io.stage();
    const DMesh &d = io.dm();
    k_oc_accumulate_fct<<<blocks_for((int64_t)d.nC * L, TPB), TPB, 0, io.stream()>>>(
        d, L, T, io.ptr(ihpi), io.ptr(ih), io.ptr(iho), io.ptr(itr), io.ptr(otp), io.ptr(ote), dt);
    io.finish();
  });
}

int mpaso_oc_tracer_hmix_del2_tend(mpaso_mesh m, int32_t nlev, int32_t ntr,
                                   const double *layerThicknessEdge, const double *tracers,
                                   double *tend, double coef, void *stream) {
  return guarded("mpaso_oc_tracer_hmix_del2_tend", [&] {
    check_levels(nlev, ntr);
    TaskIO io(m, stream);
    const int L = nlev, T = ntr;
    const int ihe = io.in(layerThicknessEdge, MPASO_EDGES, L), itr = io.in(tracers, MPASO_CELLS, L * T);
    const int ote = io.out(tend, MPASO_CELLS, L * T);
    io.stage();
    const DMesh &d = io.dm();
    k_oc_hmix<<<blocks_for((int64_t)d.nC * L, TPB), TPB, 0, io.stream()>>>(d, L, T, io.ptr(ihe),
                                                                            io.ptr(itr), io.ptr(ote), coef);
    io.finish();
  });
}

int mpaso_oc_step_tracers_forward(mpaso_mesh m, int32_t nlev, int32_t ntr, const double *tend,
                                  const double *tracers, double *tracersNew, double *tracersPrev,
                                  double rk_weight, double rk_subweight, void *stream) {
  return guarded("mpaso_oc_step_tracers_forward", [&] {
    check_levels(nlev, ntr);
    Flat f;
    f.s = plain_stream(m, stream), f.m = m;
    const size_t n = (size_t)m->ctx.d.nC * nlev * ntr;
    f.add(tend, n, false), f.add(tracers, n, false), f.add(tracersNew, n, true), f.add(tracersPrev, n, true);
    f.stage();
    k_oc_step_forward<<<blocks_for((int64_t)n, TPB), TPB, 0, f.s>>>(n, f.dev[0], f.dev[1], f.dev[2],
                                                                    f.dev[3], rk_weight, rk_subweight);
    f.finish();
  });
}

}  // extern "C"

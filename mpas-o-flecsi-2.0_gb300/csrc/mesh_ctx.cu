// Mesh context: builds the device-resident mesh from the reference's
// connectivity (mpasoflecsi/specialization/mesh.cc:67-116 semantics),
// renumbers it along a Hilbert curve, and uploads slot-major arrays to HBM.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>

#include "device.cuh"

namespace mpaso {

MeshCtx::~MeshCtx() {
  if (arena) cudaFree(arena);
  if (scratch) cudaFree(scratch);
  if (geo) cudaFree(geo);
  for (auto &p : d_perm)
    if (p) cudaFree(p);
  for (auto &p : d_iperm)
    if (p) cudaFree(p);
  if (stream) cudaStreamDestroy(stream);
}

void *MeshCtx::ensure_scratch(size_t bytes) {
  if (bytes <= scratch_bytes) return scratch;
  if (scratch) {
    MPASO_CUDA(cudaStreamSynchronize(stream));
    MPASO_CUDA(cudaFree(scratch));
    scratch = nullptr;
    scratch_bytes = 0;
  }
  const size_t want = std::max(bytes, scratch_bytes * 3 / 2);
  if (cudaMalloc(&scratch, want) != cudaSuccess) {
    cudaGetLastError();
    fail(MPASO_ERR_ALLOC, "device scratch allocation of " + std::to_string(want) + " bytes failed");
  }
  scratch_bytes = want;
  return scratch;
}

namespace {

struct Crs {
  std::vector<int64_t> off;
  std::vector<int32_t> idx;
  int64_t n() const { return (int64_t)off.size() - 1; }
  int64_t len(int64_t i) const { return off[i + 1] - off[i]; }
  int32_t at(int64_t i, int64_t j) const { return idx[off[i] + j]; }
};

Crs copy_crs(const int64_t *off, const int32_t *idx, int64_t n, int64_t n_to, const char *name) {
  require(off && idx, MPASO_ERR_ARG, std::string("missing connectivity ") + name);
  Crs c;
  c.off.assign(off, off + n + 1);
  require(c.off[0] == 0, MPASO_ERR_MESH, std::string(name) + ": offsets must start at 0");
  for (int64_t i = 0; i < n; ++i)
    if (c.off[i + 1] < c.off[i]) fail(MPASO_ERR_MESH, std::string(name) + ": offsets decrease");
  c.idx.assign(idx, idx + c.off[n]);
  for (int32_t v : c.idx)
    if (v < 0 || v >= n_to) fail(MPASO_ERR_MESH, std::string(name) + ": index out of range");
  return c;
}

// v2c[c2v[c][v]].push_back(c) -- mpasoflecsi/specialization/mesh.cc:108-116.
Crs transpose(const Crs &a, int64_t n_to) {
  Crs t;
  t.off.assign(n_to + 1, 0);
  for (int32_t v : a.idx) t.off[v + 1]++;
  for (int64_t i = 0; i < n_to; ++i) t.off[i + 1] += t.off[i];
  t.idx.resize(a.idx.size());
  std::vector<int64_t> fill(t.off.begin(), t.off.end() - 1);
  for (int64_t i = 0; i < a.n(); ++i)
    for (int64_t j = a.off[i]; j < a.off[i + 1]; ++j) t.idx[fill[a.idx[j]]++] = (int32_t)i;
  return t;
}

// Device arena: sub-allocations aligned to 256 B inside one cudaMalloc.  It
// keeps pointers to the host vectors, which must stay alive until upload();
// each is copied once, straight into its slice.
struct Arena {
  struct Item {
    const void *src;
    size_t bytes;
    size_t off;
    const void **dst;
  };
  std::vector<Item> items;
  size_t total = 0;
  template <class T> void add(const std::vector<T> &v, const T **dst) {
    items.push_back({v.data(), v.size() * sizeof(T), total, (const void **)dst});
    total += (v.size() * sizeof(T) + 255) & ~size_t(255);
  }
  void upload(MeshCtx &ctx) {
    if (cudaMalloc(&ctx.arena, std::max<size_t>(total, 256)) != cudaSuccess) {
      cudaGetLastError();
      fail(MPASO_ERR_ALLOC, "device allocation of the mesh context failed");
    }
    ctx.arena_bytes = total;
    for (auto &it : items)
      if (it.bytes) MPASO_CUDA(cudaMemcpy((char *)ctx.arena + it.off, it.src, it.bytes, cudaMemcpyHostToDevice));
    for (auto &it : items) *it.dst = (const char *)ctx.arena + it.off;
  }
};

// `mcells` (optional, ensembles): first cell of each member plus the total;
// members are then renumbered each within its own block, with its own
// bounding box, so a member keeps the order it would have alone.
void build(MeshCtx &ctx, const mpaso_mesh_desc &d, const std::vector<int64_t> *mcells = nullptr) {
  const int64_t nC = d.nCells, nE = d.nEdges, nV = d.nVertices;
  require(nC > 0 && nE > 0 && nV > 0 && nE < (1LL << 30), MPASO_ERR_ARG, "bad entity counts");
  require(d.areaCell && d.dvEdge && d.dcEdge && d.areaTriangle && d.kiteAreasOnVertex && d.fVertex &&
              d.weightsOnEdge,
          MPASO_ERR_ARG, "missing geometry field");
  const Crs c2v = copy_crs(d.c2v_off, d.c2v, nC, nV, "c2v");
  const Crs c2e = copy_crs(d.c2e_off, d.c2e, nC, nE, "c2e");
  const Crs c2c = copy_crs(d.c2c_off, d.c2c, nC, nC, "c2c");
  const Crs e2v = copy_crs(d.e2v_off, d.e2v, nE, nV, "e2v");
  const Crs e2e = copy_crs(d.e2e_off, d.e2e, nE, nE, "e2e");
  const Crs v2c = transpose(c2v, nV), e2c = transpose(c2e, nE), v2e = transpose(e2v, nV);
  for (int64_t e = 0; e < nE; ++e) {
    require(e2c.len(e) == 2, MPASO_ERR_MESH, "every edge needs exactly two cells");
    require(e2v.len(e) == 2, MPASO_ERR_MESH, "every edge needs exactly two vertices");
    require(e2e.len(e) <= kMaxEdges2, MPASO_ERR_MESH, "edgesOnEdge longer than maxEdges2");
  }
  for (int64_t v = 0; v < nV; ++v) {
    require(v2c.len(v) == kVertexDegree, MPASO_ERR_MESH, "every vertex needs three cells");
    require(v2e.len(v) == kVertexDegree, MPASO_ERR_MESH, "every vertex needs three edges");
  }
  int maxEoC = 0, maxEoE = 0;
  for (int64_t c = 0; c < nC; ++c) {
    require(c2e.len(c) <= kMaxEdges && c2e.len(c) >= 1, MPASO_ERR_MESH, "edgesOnCell length");
    require(c2c.len(c) == c2e.len(c), MPASO_ERR_MESH, "cellsOnCell / edgesOnCell length mismatch");
    maxEoC = std::max(maxEoC, (int)c2e.len(c));
  }
  for (int64_t e = 0; e < nE; ++e) maxEoE = std::max(maxEoE, (int)e2e.len(e));

  // ---- permutation ----
  // reorder: 0 keep the numbering; 1 cells along a Hilbert curve, edges and
  // vertices after the lowest new id of their cells; 2 cells, edges and
  // vertices each along the Hilbert curve of their own position (edge:
  // midpoint of its cells, vertex: centroid of its cells); 3 cells in Morton
  // (Z) order, edges and vertices as in 1.  Each ensemble member is ordered
  // inside its own block.
  require(d.reorder >= 0 && d.reorder <= 3, MPASO_ERR_ARG, "reorder must be 0..3");
  std::vector<int32_t> pc(nC), pe(nE), pv(nV);
  std::iota(pc.begin(), pc.end(), 0);
  std::iota(pe.begin(), pe.end(), 0);
  std::iota(pv.begin(), pv.end(), 0);
  std::vector<int32_t> member(nC, 0);
  struct Box {
    double lo[3], hi[3];
    int dims, bits;
  };
  std::vector<Box> boxes;
  const double *xyz[3] = {d.xCell, d.yCell, d.zCell};
  auto quant = [&](const Box &B, const double *p, uint32_t q[3]) {
    for (int a = 0; a < 3; ++a) q[a] = 0;
    for (int a = 0; a < B.dims; ++a) {
      const double span = B.hi[a] > B.lo[a] ? B.hi[a] - B.lo[a] : 1.0;
      const double t = std::min(1.0, std::max(0.0, (p[a] - B.lo[a]) / span));
      q[a] = (uint32_t)(t * (double)((1u << B.bits) - 1));
    }
  };
  auto cell_pos = [&](int64_t c, double p[3]) {
    for (int a = 0; a < 3; ++a) p[a] = xyz[a] ? xyz[a][c] : 0.0;
  };
  if (d.reorder) {
    require(d.xCell && d.yCell, MPASO_ERR_ARG, "reorder needs xCell/yCell(/zCell)");
    const std::vector<int64_t> whole = {0, nC};
    const std::vector<int64_t> &blk = mcells ? *mcells : whole;
    std::vector<uint64_t> key(nC);
    boxes.resize(blk.size() - 1);
    parallel_for((int64_t)blk.size() - 1, [&](int64_t b) {
      const int64_t c0 = blk[b], c1 = blk[b + 1];
      Box B{{1e300, 1e300, 1e300}, {-1e300, -1e300, -1e300}, 2, 30};
      for (int a = 0; a < 3; ++a)
        if (xyz[a])
          for (int64_t c = c0; c < c1; ++c) B.lo[a] = std::min(B.lo[a], xyz[a][c]), B.hi[a] = std::max(B.hi[a], xyz[a][c]);
      // a member whose z is absent or constant (a plane) is ordered in 2-D
      B.dims = (d.zCell && B.hi[2] > B.lo[2]) ? 3 : 2;
      B.bits = B.dims == 3 ? 20 : 30;
      boxes[b] = B;
      for (int64_t c = c0; c < c1; ++c) {
        double p[3];
        uint32_t q[3];
        cell_pos(c, p);
        quant(B, p, q);
        key[c] = d.reorder == 3 ? morton_key(q, B.dims, B.bits) : hilbert_key(q, B.dims, B.bits);
        member[c] = (int32_t)b;
      }
    }, 1);
    // (member, key, id) tuples sorted once: the unique id as the last key
    // gives the order a stable sort by (member, key) gives
    struct CK {
      int32_t m, id;
      uint64_t k;
    };
    std::vector<CK> ck(nC);
    parallel_for(nC, [&](int64_t c) { ck[c] = CK{member[c], (int32_t)c, key[c]}; });
    std::sort(ck.begin(), ck.end(), [](const CK &a, const CK &b) {
      return a.m != b.m ? a.m < b.m : a.k != b.k ? a.k < b.k : a.id < b.id;
    });
    for (int64_t k = 0; k < nC; ++k) pc[k] = ck[k].id;
  }
  std::vector<int32_t> ic(nC);
  for (int64_t k = 0; k < nC; ++k) ic[pc[k]] = (int32_t)k;
  if (d.reorder == 2) {  // edges and vertices on their own curves, inside their member's block
    auto own_key = [&](const int32_t *cells, int n) {
      double p[3] = {0, 0, 0}, q[3];
      for (int j = 0; j < n; ++j) {
        cell_pos(cells[j], q);
        for (int a = 0; a < 3; ++a) p[a] += q[a] / n;
      }
      uint32_t u[3];
      const Box &B = boxes[member[cells[0]]];
      quant(B, p, u);
      return std::make_pair(member[cells[0]], hilbert_key(u, B.dims, B.bits));
    };
    std::vector<std::pair<int32_t, uint64_t>> ek(nE), vk(nV);
    for (int64_t e = 0; e < nE; ++e) {
      const int32_t cs[2] = {e2c.at(e, 0), e2c.at(e, 1)};
      ek[e] = own_key(cs, 2);
    }
    for (int64_t v = 0; v < nV; ++v) {
      int32_t cs[kVertexDegree];
      for (int j = 0; j < kVertexDegree; ++j) cs[j] = v2c.at(v, j);
      vk[v] = own_key(cs, kVertexDegree);
    }
    std::stable_sort(pe.begin(), pe.end(), [&](int32_t a, int32_t b) { return ek[a] < ek[b]; });
    std::stable_sort(pv.begin(), pv.end(), [&](int32_t a, int32_t b) { return vk[a] < vk[b]; });
  } else if (d.reorder) {
    // edges by (lower, higher) new id of their cells, vertices by the lowest
    // new id of theirs; keys computed once, ties by the old id (= a stable sort)
    std::vector<std::pair<uint64_t, int32_t>> ek(nE);
    parallel_for(nE, [&](int64_t e) {
      const uint32_t a = (uint32_t)ic[e2c.at(e, 0)], b = (uint32_t)ic[e2c.at(e, 1)];
      ek[e] = {((uint64_t)std::min(a, b) << 32) | std::max(a, b), (int32_t)e};
    });
    std::sort(ek.begin(), ek.end());
    for (int64_t k = 0; k < nE; ++k) pe[k] = ek[k].second;
    std::vector<std::pair<uint64_t, int32_t>> vk(nV);
    parallel_for(nV, [&](int64_t v) {
      int32_t m = INT32_MAX;
      for (int j = 0; j < kVertexDegree; ++j) m = std::min(m, ic[v2c.at(v, j)]);
      vk[v] = {(uint64_t)(uint32_t)m, (int32_t)v};
    });
    std::sort(vk.begin(), vk.end());
    for (int64_t k = 0; k < nV; ++k) pv[k] = vk[k].second;
  }
  std::vector<int32_t> ie(nE), iv(nV);
  for (int64_t k = 0; k < nE; ++k) ie[pe[k]] = (int32_t)k;
  for (int64_t k = 0; k < nV; ++k) iv[pv[k]] = (int32_t)k;

  // ---- cells ----
  Arena A;
  DMesh &m = ctx.d;
  m.nC = (int)nC, m.nE = (int)nE, m.nV = (int)nV, m.maxEoC = maxEoC, m.maxEoE = maxEoE;
  std::vector<int> nEoC(nC), eoc((size_t)maxEoC * nC), eocAsc((size_t)maxEoC * nC), coc((size_t)maxEoC * nC);
  std::vector<int> nbr((size_t)maxEoC * nC);
  std::vector<double> eocSign((size_t)maxEoC * nC, 0.0), eocAscSign((size_t)maxEoC * nC, 0.0);
  std::vector<double> area(nC), invArea(nC), hs(nC, 0.0);
  std::vector<int> mlc(nC, 1);
  const Crs c2eAsc = transpose(e2c, nC);  // edges of each cell, ascending reference id
  parallel_for(nC, [&](int64_t k) {
    const int32_t c = pc[k];
    const int n = (int)c2e.len(c);
    nEoC[k] = n;
    for (int j = 0; j < maxEoC; ++j) {
      const size_t s = (size_t)j * nC + k;
      if (j < n) {
        const int32_t e = c2e.at(c, j);
        eoc[s] = ie[e];
        coc[s] = ic[c2c.at(c, j)];
        const bool first = c == e2c.at(e, 0);
        nbr[s] = (int)(((uint32_t)ic[first ? e2c.at(e, 1) : e2c.at(e, 0)] << 1) | (first ? 1u : 0u));
        eocSign[s] = d.edgeSignOnCell ? d.edgeSignOnCell[(size_t)c * kMaxEdges + j]
                                      : (c == e2c.at(e, 0) ? -1.0 : 1.0);
        const int32_t ea = c2eAsc.at(c, j);
        eocAsc[s] = ie[ea];
        eocAscSign[s] = (c == e2c.at(ea, 0)) ? -1.0 : 1.0;
      } else {  // pad: repeat slot 0 with a zero sign
        eoc[s] = ie[c2e.at(c, 0)];
        coc[s] = k;
        nbr[s] = (int)((uint32_t)k << 1);
        eocAsc[s] = ie[c2e.at(c, 0)];
      }
    }
    area[k] = d.areaCell[c];
    invArea[k] = 1.0 / d.areaCell[c];
    if (d.bottomDepth) hs[k] = d.bottomDepth[c];
    if (d.maxLevelCell) mlc[k] = d.maxLevelCell[c];
  });
  A.add(nEoC, &m.nEoC), A.add(eoc, &m.eoc), A.add(eocSign, &m.eocSign), A.add(eocAsc, &m.eocAsc);
  A.add(eocAscSign, &m.eocAscSign), A.add(coc, &m.coc), A.add(nbr, &m.nbr), A.add(area, &m.areaCell);
  A.add(invArea, &m.invAreaCell), A.add(hs, &m.bottomDepth), A.add(mlc, &m.maxLevelCell);

  // ---- edges ----
  std::vector<int2> coe(nE), voe(nE);
  std::vector<double> dv(nE), dc(nE), idc(nE), idv(nE), msd(nE, 1.0);
  std::vector<int> nEoE(nE), eoe((size_t)std::max(maxEoE, 1) * nE), mlet(nE, 1);
  std::vector<double> woe((size_t)std::max(maxEoE, 1) * nE, 0.0);
  parallel_for(nE, [&](int64_t k) {
    const int32_t e = pe[k];
    coe[k] = make_int2(ic[e2c.at(e, 0)], ic[e2c.at(e, 1)]);
    voe[k] = make_int2(iv[e2v.at(e, 0)], iv[e2v.at(e, 1)]);
    dv[k] = d.dvEdge[e], dc[k] = d.dcEdge[e];
    idc[k] = 1.0 / d.dcEdge[e], idv[k] = 1.0 / d.dvEdge[e];
    const int n = (int)e2e.len(e);
    nEoE[k] = n;
    for (int j = 0; j < maxEoE; ++j) {
      const size_t s = (size_t)j * nE + k;
      if (j < n) {
        eoe[s] = ie[e2e.at(e, j)];
        woe[s] = d.weightsOnEdge[(size_t)e * kMaxEdges2 + j];
      } else {
        eoe[s] = (int)k;  // pad: own edge with zero weight
      }
    }
    if (d.maxLevelEdgeTop) mlet[k] = d.maxLevelEdgeTop[e];
    if (d.meshScalingDel2) msd[k] = d.meshScalingDel2[e];
  });
  A.add(coe, &m.coe), A.add(voe, &m.voe), A.add(dv, &m.dvEdge), A.add(dc, &m.dcEdge);
  A.add(idc, &m.invDcEdge), A.add(idv, &m.invDvEdge), A.add(nEoE, &m.nEoE), A.add(eoe, &m.eoe);
  A.add(woe, &m.woe), A.add(mlet, &m.maxLevelEdgeTop), A.add(msd, &m.meshScalingDel2);

  // ---- FCT statics ----
  ctx.has_fct = d.nAdvCellsForEdge && d.advCellsForEdge && d.advCoef && d.advCoef_3rd &&
                d.highOrderAdvMask && d.fct_nlev > 0;
  int maxAdv = 1;
  if (ctx.has_fct)
    for (int64_t e = 0; e < nE; ++e) {
      require(d.nAdvCellsForEdge[e] >= 0 && d.nAdvCellsForEdge[e] <= kMaxEdges2, MPASO_ERR_MESH,
              "nAdvCellsForEdge out of range");
      maxAdv = std::max(maxAdv, (int)d.nAdvCellsForEdge[e]);
    }
  m.maxAdv = maxAdv;
  m.fctLev = ctx.has_fct ? d.fct_nlev : 1;
  std::vector<int> nAdv(nE, 0), advCells((size_t)maxAdv * nE, 0), mask((size_t)nE * m.fctLev, 1);
  std::vector<double> ac((size_t)maxAdv * nE, 0.0), a3((size_t)maxAdv * nE, 0.0);
  std::vector<double> cp((size_t)maxAdv * nE, 0.0), cm((size_t)maxAdv * nE, 0.0);
  if (ctx.has_fct) {
    parallel_for(nE, [&](int64_t k) {
      const int32_t e = pe[k];
      const int n = d.nAdvCellsForEdge[e];
      nAdv[k] = n;
      for (int j = 0; j < maxAdv; ++j) {
        const size_t s = (size_t)j * nE + k;
        if (j < n) {
          const int32_t cc = d.advCellsForEdge[(size_t)e * kMaxEdges2 + j];
          require(cc >= 0 && cc < nC, MPASO_ERR_MESH, "advCellsForEdge out of range");
          advCells[s] = ic[cc];
          const double c1 = d.advCoef[(size_t)e * kMaxEdges2 + j];
          const double c3 = d.advCoef_3rd[(size_t)e * kMaxEdges2 + j] * 0.25;  // coef3rdOrder
          ac[s] = c1, a3[s] = d.advCoef_3rd[(size_t)e * kMaxEdges2 + j];
          cp[s] = c1 + c3, cm[s] = c1 - c3;
        } else {
          advCells[s] = coe[k].x;
        }
      }
      for (int l = 0; l < m.fctLev; ++l) mask[(size_t)k * m.fctLev + l] = d.highOrderAdvMask[(size_t)e * m.fctLev + l];
    });
  }
  A.add(nAdv, &m.nAdv), A.add(advCells, &m.advCells), A.add(ac, &m.advCoef), A.add(a3, &m.advCoef3);
  A.add(cp, &m.advCp), A.add(cm, &m.advCm), A.add(mask, &m.hoMask);

  // ---- vertices ----
  std::vector<int> cov((size_t)kVertexDegree * nV), eov((size_t)kVertexDegree * nV);
  std::vector<double> kite((size_t)kVertexDegree * nV), eovSign((size_t)kVertexDegree * nV);
  std::vector<double> aT(nV), iaT(nV), fV(nV);
  parallel_for(nV, [&](int64_t k) {
    const int32_t v = pv[k];
    for (int j = 0; j < kVertexDegree; ++j) {
      const size_t s = (size_t)j * nV + k;
      cov[s] = ic[v2c.at(v, j)];
      kite[s] = d.kiteAreasOnVertex[(size_t)v * kVertexDegree + j];
      const int32_t e = v2e.at(v, j);
      eov[s] = ie[e];
      eovSign[s] = (e2v.at(e, 0) == v) ? -1.0 : 1.0;
    }
    aT[k] = d.areaTriangle[v], iaT[k] = 1.0 / d.areaTriangle[v], fV[k] = d.fVertex[v];
  });
  A.add(cov, &m.cov), A.add(kite, &m.kite), A.add(eov, &m.eov), A.add(eovSign, &m.eovSign);
  A.add(aT, &m.areaTriangle), A.add(iaT, &m.invAreaTriangle), A.add(fV, &m.fVertex);

  // ---- reverse connectivity (adjoint): transposed TRiSK weights, cell -> (vertex, kite) ----
  // e' in edgesOnEdge(e) <=> e in edgesOnEdge(e') (both share a cell), so the
  // transposed stencil of e is its own stencil with the partner's weight.
  std::vector<double> woeT((size_t)std::max(maxEoE, 1) * nE, 0.0);
  parallel_for(nE, [&](int64_t k) {
    for (int j = 0; j < nEoE[k]; ++j) {
      const int eo = eoe[(size_t)j * nE + k];
      int p = 0;
      while (p < nEoE[eo] && eoe[(size_t)p * nE + eo] != (int)k) ++p;
      require(p < nEoE[eo], MPASO_ERR_MESH, "edgesOnEdge is not symmetric");
      woeT[(size_t)j * nE + k] = woe[(size_t)p * nE + eo];
    }
  });
  std::vector<int> vocR((size_t)maxEoC * nC, 0);
  std::vector<double> kiteR((size_t)maxEoC * nC, 0.0);
  std::vector<int> fillc(nC, 0);
  for (int64_t v = 0; v < nV; ++v)
    for (int j = 0; j < kVertexDegree; ++j) {
      const int c = cov[(size_t)j * nV + v];
      require(fillc[c] < maxEoC, MPASO_ERR_MESH, "cell with more vertices than edges");
      vocR[(size_t)fillc[c] * nC + c] = (int)v;
      kiteR[(size_t)fillc[c] * nC + c] = kite[(size_t)j * nV + v];
      fillc[c]++;
    }
  for (int64_t c = 0; c < nC; ++c)
    for (int j = fillc[c]; j < maxEoC; ++j) vocR[(size_t)j * nC + c] = vocR[c];
  A.add(woeT, &m.woeT), A.add(vocR, &m.vocR), A.add(kiteR, &m.kiteR);
  // cell -> entries of the advection stencils that read the cell: the edge
  // (ascending; -1 pads at the end of each column) and the coefficient pair
  // {advCoef + 0.25 advCoef_3rd, advCoef - 0.25 advCoef_3rd} of the cell there
  // (counted CSR, filled in ascending edge order).  Ensemble members own
  // disjoint blocks of cells and of edges, so members fill in parallel; the
  // edge blocks are found from the members of the edges' cells, which do not
  // decrease along the edge numbering (one block when they would).
  std::vector<int64_t> eblk = {0, nE};
  if (mcells && mcells->size() > 2) {
    const std::vector<int64_t> &mc = *mcells;
    auto member_of = [&](int64_t k) {
      return std::upper_bound(mc.begin(), mc.end(), (int64_t)coe[k].x) - mc.begin() - 1;
    };
    std::vector<int64_t> b = {0};
    bool mono = true;
    for (int64_t k = 1; k < nE && mono; ++k) {
      const auto a = member_of(k - 1), c = member_of(k);
      if (c < a) mono = false;
      if (c != a) b.push_back(k);
    }
    b.push_back(nE);
    if (mono) eblk = b;
  }
  const int64_t nblk = (int64_t)eblk.size() - 1;
  std::vector<int> revN(ctx.has_fct ? nC : 0, 0);
  if (ctx.has_fct)
    parallel_for(nblk, [&](int64_t b) {
      for (int64_t k = eblk[b]; k < eblk[b + 1]; ++k)
        for (int j = 0; j < nAdv[k]; ++j) revN[advCells[(size_t)j * nE + k]]++;
    }, 1);
  int maxAdvR = 1;
  for (int r : revN) maxAdvR = std::max(maxAdvR, r);
  std::vector<int> advRe((size_t)maxAdvR * nC, -1);
  std::vector<double> advRc((size_t)2 * maxAdvR * nC, 0.0);
  std::fill(revN.begin(), revN.end(), 0);
  if (ctx.has_fct)
    parallel_for(nblk, [&](int64_t b) {
      for (int64_t k = eblk[b]; k < eblk[b + 1]; ++k)
        for (int j = 0; j < nAdv[k]; ++j) {
          const size_t sa = (size_t)j * nE + k;
          const int c = advCells[sa];
          const size_t o = (size_t)revN[c]++ * nC + c;
          advRe[o] = (int)k;
          advRc[2 * o] = cp[sa], advRc[2 * o + 1] = cm[sa];
        }
    }, 1);
  m.maxAdvR = maxAdvR;
  A.add(advRe, &m.advRe), A.add(advRc, (const double **)&m.advRc);
  // cellsOnCell with the cell itself and repeated neighbours replaced by -1
  std::vector<int> cocU((size_t)maxEoC * nC, -1);
  parallel_for(nC, [&](int64_t c) {
    for (int j = 0; j < nEoC[c]; ++j) {
      const int o = coc[(size_t)j * nC + c];
      bool dup = o == (int)c;
      for (int p = 0; p < j && !dup; ++p) dup = coc[(size_t)p * nC + c] == o;
      if (!dup) cocU[(size_t)j * nC + c] = o;
    }
  });
  A.add(cocU, &m.cocU);

  A.upload(ctx);
  ctx.perm[0] = pc, ctx.perm[1] = pe, ctx.perm[2] = pv;
  ctx.iperm[0] = ic, ctx.iperm[1] = ie, ctx.iperm[2] = iv;
  for (int t = 0; t < 3; ++t) {
    const size_t bytes = ctx.perm[t].size() * sizeof(int32_t);
    MPASO_CUDA(cudaMalloc(&ctx.d_perm[t], bytes));
    MPASO_CUDA(cudaMemcpy(ctx.d_perm[t], ctx.perm[t].data(), bytes, cudaMemcpyHostToDevice));
    MPASO_CUDA(cudaMalloc(&ctx.d_iperm[t], bytes));
    MPASO_CUDA(cudaMemcpy(ctx.d_iperm[t], ctx.iperm[t].data(), bytes, cudaMemcpyHostToDevice));
  }
}

// Disjoint union of member descriptions: fields concatenated in member
// order, connectivity and advection-cell indices shifted by each member's
// first cell / edge / vertex.  The vectors in `keep` own the arrays `u`
// points at.
struct Union {
  // uninitialised host buffers: their pages are first touched by the
  // parallel member copies, not by a zero fill on one thread
  template <class T> struct Buf {
    std::unique_ptr<T[]> p;
    T *alloc(size_t n) {
      p.reset(new T[std::max<size_t>(n, 1)]);
      return p.get();
    }
  };
  mpaso_mesh_desc u{};
  std::vector<Buf<int64_t>> offs;
  std::vector<Buf<int32_t>> ints;
  std::vector<Buf<double>> dbls;
  std::vector<int64_t> mcells, medges, mverts;
};

void make_union(Union &U, const mpaso_mesh_desc *m, int n) {
  require(n >= 1, MPASO_ERR_ARG, "an ensemble needs at least one member");
  const bool fct = m[0].advCoef != nullptr;
  U.mcells = {0}, U.medges = {0}, U.mverts = {0};
  for (int i = 0; i < n; ++i) {
    require(m[i].nCells > 0 && m[i].nEdges > 0 && m[i].nVertices > 0, MPASO_ERR_ARG, "bad member sizes");
    require((m[i].advCoef != nullptr) == fct, MPASO_ERR_ARG, "either every member has FCT statics or none");
    require(!fct || m[i].fct_nlev == m[0].fct_nlev, MPASO_ERR_ARG, "members' FCT statics differ in levels");
    require((m[i].reorder != 0) == (m[0].reorder != 0), MPASO_ERR_ARG, "members disagree on reorder");
    U.mcells.push_back(U.mcells.back() + m[i].nCells);
    U.medges.push_back(U.medges.back() + m[i].nEdges);
    U.mverts.push_back(U.mverts.back() + m[i].nVertices);
  }
  mpaso_mesh_desc &u = U.u;
  u.nCells = U.mcells.back(), u.nEdges = U.medges.back(), u.nVertices = U.mverts.back();
  require(u.nEdges < (1LL << 30), MPASO_ERR_ARG, "ensemble too large");
  // connectivity: (offsets member, index member, rows of member, target offsets)
  struct C {
    const int64_t *mpaso_mesh_desc::*off;
    const int32_t *mpaso_mesh_desc::*idx;
    const std::vector<int64_t> *rows, *to;
  };
  const C cs[5] = {{&mpaso_mesh_desc::c2v_off, &mpaso_mesh_desc::c2v, &U.mcells, &U.mverts},
                   {&mpaso_mesh_desc::c2e_off, &mpaso_mesh_desc::c2e, &U.mcells, &U.medges},
                   {&mpaso_mesh_desc::c2c_off, &mpaso_mesh_desc::c2c, &U.mcells, &U.mcells},
                   {&mpaso_mesh_desc::e2v_off, &mpaso_mesh_desc::e2v, &U.medges, &U.mverts},
                   {&mpaso_mesh_desc::e2e_off, &mpaso_mesh_desc::e2e, &U.medges, &U.medges}};
  // every union array is sized once and each member copies into its own
  // slice, members in parallel
  for (const C &c : cs) {
    std::vector<int64_t> ibase(n + 1, 0);
    for (int i = 0; i < n; ++i) {
      const int64_t *o = m[i].*c.off;
      require(o && m[i].*c.idx, MPASO_ERR_ARG, "member connectivity missing");
      ibase[i + 1] = ibase[i] + o[(*c.rows)[i + 1] - (*c.rows)[i]];
    }
    U.offs.emplace_back();
    U.ints.emplace_back();
    int64_t *off = U.offs.back().alloc((size_t)c.rows->back() + 1);
    int32_t *idx = U.ints.back().alloc((size_t)ibase[n]);
    off[0] = 0;
    parallel_for(n, [&](int64_t i) {
      const int64_t *o = m[i].*c.off;
      const int32_t *x = m[i].*c.idx;
      const int64_t r0 = (*c.rows)[i], rows = (*c.rows)[i + 1] - r0, shift = (*c.to)[i], base = ibase[i];
      for (int64_t r = 0; r < rows; ++r) off[r0 + r + 1] = base + o[r + 1];
      for (int64_t k = 0; k < o[rows]; ++k) idx[base + k] = (int32_t)(x[k] + shift);
    }, 1);
    u.*c.off = off;
    u.*c.idx = idx;
  }
  // per-entity fields: (member, values per entity, entity rows, default when NULL)
  auto cat = [&](const double *mpaso_mesh_desc::*f, int per, const std::vector<int64_t> &rows,
                 bool may_be_null) -> const double * {
    for (int i = 0; i < n; ++i) require(m[i].*f || may_be_null, MPASO_ERR_ARG, "member geometry field missing");
    U.dbls.emplace_back();
    double *v = U.dbls.back().alloc((size_t)rows.back() * per);
    parallel_for(n, [&](int64_t i) {
      const double *x = m[i].*f;
      double *y = v + rows[i] * per;
      const int64_t cnt = (rows[i + 1] - rows[i]) * per;
      if (x)
        std::copy(x, x + cnt, y);
      else
        std::fill(y, y + cnt, 0.0);
    }, 1);
    return v;
  };
  auto cati = [&](const int32_t *mpaso_mesh_desc::*f, int per, const std::vector<int64_t> &rows) -> const int32_t * {
    for (int i = 0; i < n; ++i) require(m[i].*f, MPASO_ERR_ARG, "member FCT field missing");
    U.ints.emplace_back();
    int32_t *v = U.ints.back().alloc((size_t)rows.back() * per);
    parallel_for(n, [&](int64_t i) {
      const int32_t *x = m[i].*f;
      std::copy(x, x + (rows[i + 1] - rows[i]) * per, v + rows[i] * per);
    }, 1);
    return v;
  };
  u.areaCell = cat(&mpaso_mesh_desc::areaCell, 1, U.mcells, false);
  u.dvEdge = cat(&mpaso_mesh_desc::dvEdge, 1, U.medges, false);
  u.dcEdge = cat(&mpaso_mesh_desc::dcEdge, 1, U.medges, false);
  u.areaTriangle = cat(&mpaso_mesh_desc::areaTriangle, 1, U.mverts, false);
  u.kiteAreasOnVertex = cat(&mpaso_mesh_desc::kiteAreasOnVertex, 3, U.mverts, false);
  u.fVertex = cat(&mpaso_mesh_desc::fVertex, 1, U.mverts, false);
  u.weightsOnEdge = cat(&mpaso_mesh_desc::weightsOnEdge, kMaxEdges2, U.medges, false);
  u.bottomDepth = cat(&mpaso_mesh_desc::bottomDepth, 1, U.mcells, true);
  u.reorder = m[0].reorder;
  if (u.reorder) {
    u.xCell = cat(&mpaso_mesh_desc::xCell, 1, U.mcells, false);
    u.yCell = cat(&mpaso_mesh_desc::yCell, 1, U.mcells, false);
    u.zCell = cat(&mpaso_mesh_desc::zCell, 1, U.mcells, true);
  }
  if (fct) {
    const int L = m[0].fct_nlev;
    u.fct_nlev = L;
    u.maxLevelCell = cati(&mpaso_mesh_desc::maxLevelCell, 1, U.mcells);
    u.maxLevelEdgeTop = cati(&mpaso_mesh_desc::maxLevelEdgeTop, 1, U.medges);
    u.nAdvCellsForEdge = cati(&mpaso_mesh_desc::nAdvCellsForEdge, 1, U.medges);
    u.highOrderAdvMask = cati(&mpaso_mesh_desc::highOrderAdvMask, L, U.medges);
    // advection cells: the first nAdv entries of each row shift by the member's first cell
    for (int i = 0; i < n; ++i)
      require(m[i].advCellsForEdge && m[i].nAdvCellsForEdge, MPASO_ERR_ARG, "member FCT field missing");
    U.ints.emplace_back();
    int32_t *adv = U.ints.back().alloc((size_t)u.nEdges * kMaxEdges2);
    parallel_for(n, [&](int64_t i) {
      int32_t *y = adv + U.medges[i] * kMaxEdges2;
      for (int64_t e = 0; e < m[i].nEdges; ++e)
        for (int j = 0; j < kMaxEdges2; ++j) {
          const int32_t x = m[i].advCellsForEdge[e * kMaxEdges2 + j];
          y[e * kMaxEdges2 + j] = j < m[i].nAdvCellsForEdge[e] ? (int32_t)(x + U.mcells[i]) : x;
        }
    }, 1);
    u.advCellsForEdge = adv;
    u.edgeSignOnCell = cat(&mpaso_mesh_desc::edgeSignOnCell, kMaxEdges, U.mcells, false);
    u.advCoef = cat(&mpaso_mesh_desc::advCoef, kMaxEdges2, U.medges, false);
    u.advCoef_3rd = cat(&mpaso_mesh_desc::advCoef_3rd, kMaxEdges2, U.medges, false);
    u.meshScalingDel2 = cat(&mpaso_mesh_desc::meshScalingDel2, 1, U.medges, false);
  }
}

}  // namespace
}  // namespace mpaso

extern "C" {

int mpaso_mesh_create_ensemble(const mpaso_mesh_desc *members, int32_t n, int device, mpaso_mesh *out) {
  return mpaso::guarded("mpaso_mesh_create_ensemble", [&] {
    mpaso::require(members && out && n >= 1, MPASO_ERR_ARG, "bad argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      mpaso::fail(MPASO_ERR_NODEVICE, "no CUDA device");
    }
    if (device < 0) MPASO_CUDA(cudaGetDevice(&device));
    mpaso::require(device < ndev, MPASO_ERR_ARG, "device index out of range");
    MPASO_CUDA(cudaSetDevice(device));
    mpaso::Union U;
    mpaso::make_union(U, members, n);
    auto *h = new mpaso_mesh_s();
    try {
      h->ctx.device = device;
      MPASO_CUDA(cudaDeviceGetAttribute(&h->ctx.sms, cudaDevAttrMultiProcessorCount, device));
      MPASO_CUDA(cudaStreamCreateWithFlags(&h->ctx.stream, cudaStreamNonBlocking));
      mpaso::build(h->ctx, U.u, &U.mcells);
      for (int i = 0; i <= n; ++i)
        h->ctx.members.insert(h->ctx.members.end(), {U.mcells[i], U.medges[i], U.mverts[i]});
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

int mpaso_mesh_members(mpaso_mesh m, int32_t *n, int64_t *offsets) {
  return mpaso::guarded("mpaso_mesh_members", [&] {
    mpaso::require(m && n, MPASO_ERR_ARG, "null argument");
    const auto &mb = m->ctx.members;
    if (mb.empty()) {  // a plain mesh is an ensemble of one
      *n = 1;
      if (offsets) {
        const int64_t v[6] = {0, 0, 0, m->ctx.d.nC, m->ctx.d.nE, m->ctx.d.nV};
        std::memcpy(offsets, v, sizeof v);
      }
      return;
    }
    *n = (int32_t)(mb.size() / 3 - 1);
    if (offsets) std::memcpy(offsets, mb.data(), mb.size() * sizeof(int64_t));
  });
}

int mpaso_device_count(int32_t *n) {
  return mpaso::guarded("mpaso_device_count", [&] {
    mpaso::require(n != nullptr, MPASO_ERR_ARG, "null output");
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) {
      cudaGetLastError();
      c = 0;
    }
    *n = c;
  });
}

const char *mpaso_build_info(void) {
  return "libmpaso: FP64 MPAS-O-FleCSI RK4 tendency path for sm_103a (GB300)";
}

int mpaso_mesh_create(const mpaso_mesh_desc *desc, int device, mpaso_mesh *out) {
  return mpaso::guarded("mpaso_mesh_create", [&] {
    mpaso::require(desc != nullptr && out != nullptr, MPASO_ERR_ARG, "null argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      mpaso::fail(MPASO_ERR_NODEVICE, "no CUDA device");
    }
    if (device < 0) MPASO_CUDA(cudaGetDevice(&device));
    mpaso::require(device < ndev, MPASO_ERR_ARG, "device index out of range");
    MPASO_CUDA(cudaSetDevice(device));
    auto *h = new mpaso_mesh_s();
    try {
      h->ctx.device = device;
      MPASO_CUDA(cudaDeviceGetAttribute(&h->ctx.sms, cudaDevAttrMultiProcessorCount, device));
      MPASO_CUDA(cudaStreamCreateWithFlags(&h->ctx.stream, cudaStreamNonBlocking));
      mpaso::build(h->ctx, *desc);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

int mpaso_mesh_destroy(mpaso_mesh m) {
  return mpaso::guarded("mpaso_mesh_destroy", [&] {
    if (m) mpaso::release_mesh(m);
  });
}

int mpaso_mesh_permutation(mpaso_mesh m, int32_t entity, int32_t *new_to_old) {
  return mpaso::guarded("mpaso_mesh_permutation", [&] {
    mpaso::require(m && new_to_old && entity >= 0 && entity < 3, MPASO_ERR_ARG, "bad argument");
    const auto &p = m->ctx.perm[entity];
    std::memcpy(new_to_old, p.data(), p.size() * sizeof(int32_t));
  });
}

int mpaso_mesh_set_gravity(mpaso_mesh m, double gravity) {
  return mpaso::guarded("mpaso_mesh_set_gravity", [&] {
    mpaso::require(m != nullptr, MPASO_ERR_ARG, "null mesh");
    m->ctx.gravity = gravity;
  });
}

int mpaso_mesh_device_bytes(mpaso_mesh m, int64_t *bytes) {
  return mpaso::guarded("mpaso_mesh_device_bytes", [&] {
    mpaso::require(m && bytes, MPASO_ERR_ARG, "null argument");
    const mpaso::DMesh &d = m->ctx.d;
    // the arena, the per-task scratch and both permutations of each entity
    *bytes = (int64_t)(m->ctx.arena_bytes + m->ctx.scratch_bytes) + 2 * 4 * (d.nC + d.nE + d.nV);
  });
}

}  // extern "C"

// MPAS Voronoi mesh generation (host).  Builds every mesh dataset that the
// reference reads (mpasoflecsi/tasks/io.cc:14-63, specialization/
// definition.hh:1055-1106) from a triangulation of the cell generators:
//
//   vertices = triangles (circumcentres), edges = triangle sides (their duals),
//   cells    = generators.
//
// Orientation conventions (the ones the reference's task code assumes, see
// apps/sw/tasks/solve.cc:191-233 and apps/ocean/tasks/init_functions.cc:75-78):
//   - cellsOnEdge = (c1, c2) with c1 < c2; the edge normal n points c1 -> c2;
//   - verticesOnEdge = (v1, v2) with the tangent k x n pointing v1 -> v2;
//   - edgesOnCell / cellsOnCell / verticesOnCell counter-clockwise, cellsOnCell[j]
//     across edgesOnCell[j], verticesOnCell[j] between edgesOnCell[j] and [j+1];
//   - cellsOnVertex, edgesOnVertex ascending, kiteAreasOnVertex paired with
//     cellsOnVertex;
//   - edgesOnEdge = edges of c1 counter-clockwise after e, then edges of c2
//     counter-clockwise after e, with TRiSK weightsOnEdge (Thuburn, Ringler,
//     Skamarock & Klemp, J. Comput. Phys. 228 (2009); Ringler et al.,
//     J. Comput. Phys. 229 (2010)) so that sum_j W[e][j] u[eoe_j] is the
//     velocity component along k x n_e.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <numeric>
#include <unordered_map>
#include <vector>

#include "common.hh"

namespace mpaso {
namespace {

constexpr int kMaxEdges = 8;
constexpr int kMaxEdges2 = 16;
constexpr int kVertexDegree = 3;

struct V3 {
  double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 unit(V3 a) { return (1.0 / norm(a)) * a; }

// Great-circle angle between unit vectors (robust for small angles).
inline double arc(V3 a, V3 b) { return std::atan2(norm(cross(a, b)), dot(a, b)); }

// Area of the spherical triangle abc on the unit sphere (Van Oosterom &
// Strackee 1983 formula, tan(E/2) = |a.(b x c)| / (1 + a.b + b.c + c.a)).
inline double sph_tri_area(V3 a, V3 b, V3 c) {
  const double num = std::fabs(dot(a, cross(b, c)));
  const double den = 1.0 + dot(a, b) + dot(b, c) + dot(c, a);
  return 2.0 * std::atan2(num, den);
}

}  // namespace

struct GenMesh {
  bool sphere = false;
  double radius = 1.0, Lx = 0.0, Ly = 0.0, omega = 0.0, f0 = 0.0;
  int nC = 0, nE = 0, nV = 0;
  std::vector<V3> pc, pe, pv;  // sphere: unit vectors; plane: metres, z = 0
  std::vector<std::array<int, 3>> tri;  // vertex -> its three cells (CCW)
  std::vector<int32_t> nEdgesOnCell, edgesOnCell, cellsOnCell, verticesOnCell;
  std::vector<int32_t> cellsOnEdge, verticesOnEdge, nEdgesOnEdge, edgesOnEdge;
  std::vector<int32_t> cellsOnVertex, edgesOnVertex;
  std::vector<double> areaCell, areaTriangle, kiteAreasOnVertex, dcEdge, dvEdge, angleEdge,
      weightsOnEdge;
  std::vector<double> xCell, yCell, zCell, xEdge, yEdge, zEdge, xVertex, yVertex, zVertex;
  std::vector<double> latCell, lonCell, latEdge, lonEdge, latVertex, lonVertex;
  std::vector<double> fCell, fEdge, fVertex, meshDensity;

  // Displacement from a to b: plain difference on the sphere, minimum image
  // on the periodic plane.
  V3 rel(V3 a, V3 b) const {
    V3 d = b - a;
    if (!sphere) {
      d.x -= Lx * std::nearbyint(d.x / Lx);
      d.y -= Ly * std::nearbyint(d.y / Ly);
      d.z = 0.0;
    }
    return d;
  }
  V3 wrap(V3 p) const {
    if (sphere) return p;
    p.x -= Lx * std::floor(p.x / Lx);
    p.y -= Ly * std::floor(p.y / Ly);
    return p;
  }
  double dist(V3 a, V3 b) const { return sphere ? radius * arc(a, b) : norm(rel(a, b)); }

  V3 circumcentre(int a, int b, int c) const {
    if (sphere) {
      V3 n = unit(cross(pc[b] - pc[a], pc[c] - pc[a]));
      if (dot(n, pc[a] + pc[b] + pc[c]) < 0) n = -1.0 * n;
      return n;
    }
    const V3 B = rel(pc[a], pc[b]), C = rel(pc[a], pc[c]);
    const double d = 2.0 * (B.x * C.y - B.y * C.x);
    const double b2 = B.x * B.x + B.y * B.y, c2 = C.x * C.x + C.y * C.y;
    const V3 u = {(C.y * b2 - B.y * c2) / d, (B.x * c2 - C.x * b2) / d, 0.0};
    return wrap(pc[a] + u);
  }

  // Area of the kite (cell centre P, edge point E1, vertex V, edge point E2).
  double kite_area(V3 P, V3 E1, V3 V, V3 E2) const {
    if (sphere) return radius * radius * (sph_tri_area(P, E1, V) + sph_tri_area(P, V, E2));
    const V3 a = rel(P, E1), b = rel(P, V), c = rel(P, E2);
    // Shoelace over (0, a, b, c).
    return 0.5 * std::fabs(a.x * b.y - a.y * b.x + b.x * c.y - b.y * c.x);
  }

  void build();
};

void GenMesh::build() {
  nC = (int)pc.size();
  nV = (int)tri.size();
  // ---- edges: one per unordered pair of cells sharing a triangle side ----
  std::unordered_map<uint64_t, int> emap;
  emap.reserve((size_t)nV * 2);
  cellsOnEdge.clear();
  verticesOnEdge.clear();
  auto key = [](int a, int b) { return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b; };
  for (int t = 0; t < nV; ++t) {
    for (int k = 0; k < 3; ++k) {
      const int a = tri[t][k], b = tri[t][(k + 1) % 3];
      require(a != b, MPASO_ERR_MESH, "degenerate triangle");
      const int c1 = std::min(a, b), c2 = std::max(a, b);
      auto it = emap.find(key(c1, c2));
      int e;
      if (it == emap.end()) {
        e = (int)cellsOnEdge.size() / 2;
        emap.emplace(key(c1, c2), e);
        cellsOnEdge.push_back(c1);
        cellsOnEdge.push_back(c2);
        verticesOnEdge.push_back(-1);
        verticesOnEdge.push_back(-1);
      } else {
        e = it->second;
      }
      // Triangle t holds the directed side a -> b counter-clockwise, so it lies
      // on the left of a -> b.  The left of c1 -> c2 is the +k x n side: v2.
      const int slot = (a == c1) ? 1 : 0;
      require(verticesOnEdge[2 * e + slot] < 0, MPASO_ERR_MESH, "non-manifold edge");
      verticesOnEdge[2 * e + slot] = t;
    }
  }
  nE = (int)cellsOnEdge.size() / 2;
  for (int e = 0; e < nE; ++e)
    require(verticesOnEdge[2 * e] >= 0 && verticesOnEdge[2 * e + 1] >= 0, MPASO_ERR_MESH,
            "open edge: triangulation is not closed");
  auto edge_of = [&](int a, int b) {
    auto it = emap.find(key(std::min(a, b), std::max(a, b)));
    require(it != emap.end(), MPASO_ERR_MESH, "missing edge");
    return it->second;
  };

  // ---- counter-clockwise cell neighbourhoods ----
  std::vector<std::vector<std::array<int, 3>>> around(nC);  // (b, c, t): b then c CCW
  for (int t = 0; t < nV; ++t)
    for (int k = 0; k < 3; ++k)
      around[tri[t][k]].push_back({tri[t][(k + 1) % 3], tri[t][(k + 2) % 3], t});
  nEdgesOnCell.assign(nC, 0);
  edgesOnCell.assign((size_t)nC * kMaxEdges, -1);
  cellsOnCell.assign((size_t)nC * kMaxEdges, -1);
  verticesOnCell.assign((size_t)nC * kMaxEdges, -1);
  for (int i = 0; i < nC; ++i) {
    auto &ar = around[i];
    const int n = (int)ar.size();
    require(n >= 3 && n <= kMaxEdges, MPASO_ERR_MESH, "cell with unsupported edge count");
    int b = ar[0][0];
    for (auto &x : ar) b = std::min(b, x[0]);  // start at the lowest neighbour
    for (int k = 0; k < n; ++k) {
      const std::array<int, 3> *nx = nullptr;
      for (auto &x : ar)
        if (x[0] == b) nx = &x;
      require(nx != nullptr, MPASO_ERR_MESH, "broken cell fan");
      cellsOnCell[(size_t)i * kMaxEdges + k] = b;
      edgesOnCell[(size_t)i * kMaxEdges + k] = edge_of(i, b);
      verticesOnCell[(size_t)i * kMaxEdges + k] = (*nx)[2];
      b = (*nx)[1];
    }
    require(b == cellsOnCell[(size_t)i * kMaxEdges], MPASO_ERR_MESH, "cell fan does not close");
    nEdgesOnCell[i] = n;
  }

  // ---- positions ----
  pv.resize(nV);
  for (int t = 0; t < nV; ++t) pv[t] = circumcentre(tri[t][0], tri[t][1], tri[t][2]);
  pe.resize(nE);
  for (int e = 0; e < nE; ++e) {
    const V3 a = pc[cellsOnEdge[2 * e]], b = pc[cellsOnEdge[2 * e + 1]];
    pe[e] = sphere ? unit(a + b) : wrap(a + 0.5 * rel(a, b));
  }

  // ---- lengths ----
  dcEdge.resize(nE);
  dvEdge.resize(nE);
  for (int e = 0; e < nE; ++e) {
    dcEdge[e] = dist(pc[cellsOnEdge[2 * e]], pc[cellsOnEdge[2 * e + 1]]);
    dvEdge[e] = dist(pv[verticesOnEdge[2 * e]], pv[verticesOnEdge[2 * e + 1]]);
  }

  // ---- kites and areas ----
  std::vector<double> kite_ck((size_t)nC * kMaxEdges, 0.0);
  areaCell.assign(nC, 0.0);
  for (int i = 0; i < nC; ++i) {
    const int n = nEdgesOnCell[i];
    double s = 0.0;
    for (int k = 0; k < n; ++k) {
      const int e1 = edgesOnCell[(size_t)i * kMaxEdges + k];
      const int e2 = edgesOnCell[(size_t)i * kMaxEdges + (k + 1) % n];
      const int v = verticesOnCell[(size_t)i * kMaxEdges + k];
      const double ka = kite_area(pc[i], pe[e1], pv[v], pe[e2]);
      kite_ck[(size_t)i * kMaxEdges + k] = ka;
      s += ka;
    }
    areaCell[i] = s;
  }
  cellsOnVertex.assign((size_t)nV * kVertexDegree, -1);
  edgesOnVertex.assign((size_t)nV * kVertexDegree, -1);
  kiteAreasOnVertex.assign((size_t)nV * kVertexDegree, 0.0);
  for (int t = 0; t < nV; ++t) {
    std::array<int, 3> c = tri[t];
    std::sort(c.begin(), c.end());
    std::array<int, 3> es = {edge_of(tri[t][0], tri[t][1]), edge_of(tri[t][1], tri[t][2]),
                             edge_of(tri[t][2], tri[t][0])};
    std::sort(es.begin(), es.end());
    for (int j = 0; j < 3; ++j) {
      cellsOnVertex[(size_t)t * 3 + j] = c[j];
      edgesOnVertex[(size_t)t * 3 + j] = es[j];
    }
  }
  for (int i = 0; i < nC; ++i)
    for (int k = 0; k < nEdgesOnCell[i]; ++k) {
      const int v = verticesOnCell[(size_t)i * kMaxEdges + k];
      int j = 0;
      while (j < 3 && cellsOnVertex[(size_t)v * 3 + j] != i) ++j;
      require(j < 3, MPASO_ERR_MESH, "vertex/cell mismatch");
      kiteAreasOnVertex[(size_t)v * 3 + j] = kite_ck[(size_t)i * kMaxEdges + k];
    }
  areaTriangle.assign(nV, 0.0);
  for (int t = 0; t < nV; ++t)
    areaTriangle[t] = kiteAreasOnVertex[(size_t)t * 3] + kiteAreasOnVertex[(size_t)t * 3 + 1] +
                      kiteAreasOnVertex[(size_t)t * 3 + 2];

  // ---- edgesOnEdge + TRiSK weights ----
  nEdgesOnEdge.assign(nE, 0);
  edgesOnEdge.assign((size_t)nE * kMaxEdges2, -1);
  weightsOnEdge.assign((size_t)nE * kMaxEdges2, 0.0);
  for (int e = 0; e < nE; ++e) {
    int cnt = 0;
    for (int side = 0; side < 2; ++side) {
      const int c = cellsOnEdge[2 * e + side];
      const double sgn = side == 0 ? 1.0 : -1.0;  // k x n_out(c) = +t_e for c1, -t_e for c2
      const int n = nEdgesOnCell[c];
      int j = 0;
      while (j < n && edgesOnCell[(size_t)c * kMaxEdges + j] != e) ++j;
      require(j < n, MPASO_ERR_MESH, "edge not on its cell");
      double R = 0.0;
      for (int k = 1; k < n; ++k) {
        const int pos = (j + k) % n, vpos = (j + k - 1) % n;
        R += kite_ck[(size_t)c * kMaxEdges + vpos] / areaCell[c];
        const int ep = edgesOnCell[(size_t)c * kMaxEdges + pos];
        const double s_out = (cellsOnEdge[2 * ep] == c) ? 1.0 : -1.0;
        edgesOnEdge[(size_t)e * kMaxEdges2 + cnt] = ep;
        weightsOnEdge[(size_t)e * kMaxEdges2 + cnt] =
            sgn * (0.5 - R) * s_out * dvEdge[ep] / dcEdge[e];
        ++cnt;
      }
    }
    nEdgesOnEdge[e] = cnt;
  }

  // ---- coordinates, angles, Coriolis ----
  auto put = [&](const std::vector<V3> &p, std::vector<double> &x, std::vector<double> &y,
                 std::vector<double> &z, std::vector<double> &lat, std::vector<double> &lon,
                 std::vector<double> &f) {
    const size_t n = p.size();
    x.resize(n), y.resize(n), z.resize(n), lat.resize(n), lon.resize(n), f.resize(n);
    for (size_t i = 0; i < n; ++i) {
      if (sphere) {
        x[i] = radius * p[i].x, y[i] = radius * p[i].y, z[i] = radius * p[i].z;
        lat[i] = std::asin(std::max(-1.0, std::min(1.0, p[i].z)));
        double lo = std::atan2(p[i].y, p[i].x);
        if (lo < 0) lo += 2.0 * M_PI;
        lon[i] = lo;
        f[i] = 2.0 * omega * std::sin(lat[i]);
      } else {
        x[i] = p[i].x, y[i] = p[i].y, z[i] = 0.0, lat[i] = 0.0, lon[i] = 0.0, f[i] = f0;
      }
    }
  };
  put(pc, xCell, yCell, zCell, latCell, lonCell, fCell);
  put(pe, xEdge, yEdge, zEdge, latEdge, lonEdge, fEdge);
  put(pv, xVertex, yVertex, zVertex, latVertex, lonVertex, fVertex);
  angleEdge.resize(nE);
  for (int e = 0; e < nE; ++e) {
    V3 d = rel(pc[cellsOnEdge[2 * e]], pc[cellsOnEdge[2 * e + 1]]);
    if (sphere) {
      const V3 E = pe[e];
      d = d - dot(d, E) * E;
      V3 east = {-E.y, E.x, 0.0};
      if (norm(east) < 1e-14) east = {1.0, 0.0, 0.0};
      east = unit(east);
      const V3 north = cross(E, east);
      angleEdge[e] = std::atan2(dot(d, north), dot(d, east));
    } else {
      angleEdge[e] = std::atan2(d.y, d.x);
    }
  }
  meshDensity.assign(nC, 1.0);
}

namespace {

GenMesh *make_icosa(int level, double radius, double omega) {
  require(level >= 0 && level <= 10, MPASO_ERR_ARG, "icosahedral level must be in [0, 10]");
  require(radius > 0, MPASO_ERR_ARG, "radius must be positive");
  auto *m = new GenMesh();
  m->sphere = true;
  m->radius = radius;
  m->omega = omega;
  const double phi = (1.0 + std::sqrt(5.0)) / 2.0;
  std::vector<V3> p = {{-1, phi, 0}, {1, phi, 0}, {-1, -phi, 0}, {1, -phi, 0},
                       {0, -1, phi}, {0, 1, phi}, {0, -1, -phi}, {0, 1, -phi},
                       {phi, 0, -1}, {phi, 0, 1}, {-phi, 0, -1}, {-phi, 0, 1}};
  // Fixed generic rotation (Euler z-y-z 0.3, 0.7, 1.1 rad): keeps every
  // generator, edge point and vertex off the coordinate planes.
  const double a1 = 0.3, a2 = 0.7, a3 = 1.1;
  auto rotz = [](V3 v, double a) {
    return V3{std::cos(a) * v.x - std::sin(a) * v.y, std::sin(a) * v.x + std::cos(a) * v.y, v.z};
  };
  auto roty = [](V3 v, double a) {
    return V3{std::cos(a) * v.x + std::sin(a) * v.z, v.y, -std::sin(a) * v.x + std::cos(a) * v.z};
  };
  for (auto &v : p) v = unit(rotz(roty(rotz(v, a1), a2), a3));
  std::vector<std::array<int, 3>> f = {
      {0, 11, 5}, {0, 5, 1},  {0, 1, 7},   {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
      {11, 10, 2}, {10, 7, 6}, {7, 1, 8},  {3, 9, 4},  {3, 4, 2},   {3, 2, 6}, {3, 6, 8},
      {3, 8, 9},  {4, 9, 5},  {2, 4, 11},  {6, 2, 10}, {8, 6, 7},   {9, 8, 1}};
  for (auto &t : f)
    if (dot(cross(p[t[1]] - p[t[0]], p[t[2]] - p[t[0]]), p[t[0]] + p[t[1]] + p[t[2]]) < 0)
      std::swap(t[1], t[2]);
  for (int l = 0; l < level; ++l) {
    std::unordered_map<uint64_t, int> mid;
    mid.reserve(f.size() * 2);
    auto midpoint = [&](int a, int b) {
      const uint64_t k = ((uint64_t)std::min(a, b) << 32) | (uint32_t)std::max(a, b);
      auto it = mid.find(k);
      if (it != mid.end()) return it->second;
      p.push_back(unit(p[a] + p[b]));
      const int id = (int)p.size() - 1;
      mid.emplace(k, id);
      return id;
    };
    std::vector<std::array<int, 3>> g;
    g.reserve(f.size() * 4);
    for (auto &t : f) {
      const int ab = midpoint(t[0], t[1]), bc = midpoint(t[1], t[2]), ca = midpoint(t[2], t[0]);
      g.push_back({t[0], ab, ca});
      g.push_back({t[1], bc, ab});
      g.push_back({t[2], ca, bc});
      g.push_back({ab, bc, ca});
    }
    f.swap(g);
  }
  m->pc = p;
  m->tri = f;
  m->build();
  return m;
}

GenMesh *make_hex(int nx, int ny, double dc, double f0) {
  require(nx >= 4 && ny >= 4 && (ny % 2) == 0, MPASO_ERR_ARG,
          "planar hex mesh needs nx >= 4, ny >= 4 and ny even");
  require(dc > 0, MPASO_ERR_ARG, "dc must be positive");
  auto *m = new GenMesh();
  m->sphere = false;
  m->f0 = f0;
  const double dy = dc * std::sqrt(3.0) / 2.0;
  m->Lx = nx * dc;
  m->Ly = ny * dy;
  m->pc.resize((size_t)nx * ny);
  auto id = [nx, ny](int i, int j) { return ((j % ny + ny) % ny) * nx + ((i % nx + nx) % nx); };
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
      m->pc[id(i, j)] = {(i + 0.5 * (j & 1)) * dc, j * dy, 0.0};
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      // Up-right / up-left neighbours in the offset-row layout.
      const int ur = (j & 1) ? id(i + 1, j + 1) : id(i, j + 1);
      const int ul = (j & 1) ? id(i, j + 1) : id(i - 1, j + 1);
      m->tri.push_back({id(i, j), id(i + 1, j), ur});
      m->tri.push_back({id(i, j), ur, ul});
    }
  m->build();
  return m;
}

// Rebuild `in` with cells in Hilbert order and triangles (vertices) ordered by
// their lowest new cell; edges then follow in first-encounter order.
GenMesh *reorder(const GenMesh &in, int32_t *pc_out, int32_t *pe_out, int32_t *pv_out) {
  const int nC = in.nC;
  std::vector<uint64_t> keys(nC);
  for (int i = 0; i < nC; ++i) {
    uint32_t q[3];
    if (in.sphere) {
      const int bits = 20;
      const double s = (double)((1u << bits) - 1);
      q[0] = (uint32_t)((in.pc[i].x + 1.0) * 0.5 * s);
      q[1] = (uint32_t)((in.pc[i].y + 1.0) * 0.5 * s);
      q[2] = (uint32_t)((in.pc[i].z + 1.0) * 0.5 * s);
      keys[i] = hilbert_key(q, 3, bits);
    } else {
      const int bits = 24;
      const double s = (double)((1u << bits) - 1);
      q[0] = (uint32_t)(in.pc[i].x / in.Lx * s);
      q[1] = (uint32_t)(in.pc[i].y / in.Ly * s);
      keys[i] = hilbert_key(q, 2, bits);
    }
  }
  std::vector<int> order(nC);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return keys[a] < keys[b]; });
  std::vector<int> newc(nC);
  for (int k = 0; k < nC; ++k) newc[order[k]] = k;
  auto *m = new GenMesh();
  m->sphere = in.sphere, m->radius = in.radius, m->Lx = in.Lx, m->Ly = in.Ly;
  m->omega = in.omega, m->f0 = in.f0;
  m->pc.resize(nC);
  for (int k = 0; k < nC; ++k) m->pc[k] = in.pc[order[k]];
  const int nV = in.nV;
  std::vector<std::array<int, 3>> t2(nV);
  std::vector<std::pair<std::array<int, 3>, int>> tk(nV);
  for (int t = 0; t < nV; ++t) {
    std::array<int, 3> c = {newc[in.tri[t][0]], newc[in.tri[t][1]], newc[in.tri[t][2]]};
    // rotate so the lowest cell leads (keeps CCW order)
    int lo = 0;
    for (int k = 1; k < 3; ++k)
      if (c[k] < c[lo]) lo = k;
    t2[t] = {c[lo], c[(lo + 1) % 3], c[(lo + 2) % 3]};
    std::array<int, 3> s = t2[t];
    std::sort(s.begin(), s.end());
    tk[t] = {s, t};
  }
  std::stable_sort(tk.begin(), tk.end(),
                   [](const auto &a, const auto &b) { return a.first < b.first; });
  m->tri.resize(nV);
  for (int k = 0; k < nV; ++k) m->tri[k] = t2[tk[k].second];
  m->build();
  if (pc_out)
    for (int k = 0; k < nC; ++k) pc_out[k] = order[k];
  if (pv_out)
    for (int k = 0; k < nV; ++k) pv_out[k] = tk[k].second;
  if (pe_out) {
    std::unordered_map<uint64_t, int> old;
    old.reserve((size_t)in.nE * 2);
    for (int e = 0; e < in.nE; ++e)
      old.emplace(((uint64_t)in.cellsOnEdge[2 * e] << 32) | (uint32_t)in.cellsOnEdge[2 * e + 1], e);
    for (int e = 0; e < m->nE; ++e) {
      int a = order[m->cellsOnEdge[2 * e]], b = order[m->cellsOnEdge[2 * e + 1]];
      if (a > b) std::swap(a, b);
      pe_out[e] = old.at(((uint64_t)a << 32) | (uint32_t)b);
    }
  }
  return m;
}

struct FieldRef {
  int dtype;
  int64_t rows, cols;
  const void *data;
  bool one_based;
};

bool lookup(const GenMesh &m, const std::string &n, FieldRef &r) {
  auto I = [&](const std::vector<int32_t> &v, int64_t rows, int64_t cols, bool ob) {
    r = {MPASO_DTYPE_INT32, rows, cols, v.data(), ob};
    return true;
  };
  auto D = [&](const std::vector<double> &v, int64_t rows, int64_t cols) {
    r = {MPASO_DTYPE_FLOAT64, rows, cols, v.data(), false};
    return true;
  };
  const int64_t C = m.nC, E = m.nE, V = m.nV;
  if (n == "nEdgesOnCell") return I(m.nEdgesOnCell, C, 1, false);
  if (n == "edgesOnCell") return I(m.edgesOnCell, C, kMaxEdges, true);
  if (n == "cellsOnCell") return I(m.cellsOnCell, C, kMaxEdges, true);
  if (n == "verticesOnCell") return I(m.verticesOnCell, C, kMaxEdges, true);
  if (n == "cellsOnEdge") return I(m.cellsOnEdge, E, 2, true);
  if (n == "verticesOnEdge") return I(m.verticesOnEdge, E, 2, true);
  if (n == "nEdgesOnEdge") return I(m.nEdgesOnEdge, E, 1, false);
  if (n == "edgesOnEdge") return I(m.edgesOnEdge, E, kMaxEdges2, true);
  if (n == "cellsOnVertex") return I(m.cellsOnVertex, V, kVertexDegree, true);
  if (n == "edgesOnVertex") return I(m.edgesOnVertex, V, kVertexDegree, true);
  if (n == "areaCell") return D(m.areaCell, C, 1);
  if (n == "areaTriangle") return D(m.areaTriangle, V, 1);
  if (n == "kiteAreasOnVertex") return D(m.kiteAreasOnVertex, V, kVertexDegree);
  if (n == "dcEdge") return D(m.dcEdge, E, 1);
  if (n == "dvEdge") return D(m.dvEdge, E, 1);
  if (n == "angleEdge") return D(m.angleEdge, E, 1);
  if (n == "weightsOnEdge") return D(m.weightsOnEdge, E, kMaxEdges2);
  if (n == "xCell") return D(m.xCell, C, 1);
  if (n == "yCell") return D(m.yCell, C, 1);
  if (n == "zCell") return D(m.zCell, C, 1);
  if (n == "xEdge") return D(m.xEdge, E, 1);
  if (n == "yEdge") return D(m.yEdge, E, 1);
  if (n == "zEdge") return D(m.zEdge, E, 1);
  if (n == "xVertex") return D(m.xVertex, V, 1);
  if (n == "yVertex") return D(m.yVertex, V, 1);
  if (n == "zVertex") return D(m.zVertex, V, 1);
  if (n == "latCell") return D(m.latCell, C, 1);
  if (n == "lonCell") return D(m.lonCell, C, 1);
  if (n == "latEdge") return D(m.latEdge, E, 1);
  if (n == "lonEdge") return D(m.lonEdge, E, 1);
  if (n == "latVertex") return D(m.latVertex, V, 1);
  if (n == "lonVertex") return D(m.lonVertex, V, 1);
  if (n == "fCell") return D(m.fCell, C, 1);
  if (n == "fEdge") return D(m.fEdge, E, 1);
  if (n == "fVertex") return D(m.fVertex, V, 1);
  if (n == "meshDensity") return D(m.meshDensity, C, 1);
  return false;
}

const char *kNames =
    "nEdgesOnCell,edgesOnCell,cellsOnCell,verticesOnCell,cellsOnEdge,verticesOnEdge,"
    "nEdgesOnEdge,edgesOnEdge,cellsOnVertex,edgesOnVertex,areaCell,areaTriangle,"
    "kiteAreasOnVertex,dcEdge,dvEdge,angleEdge,weightsOnEdge,xCell,yCell,zCell,xEdge,yEdge,"
    "zEdge,xVertex,yVertex,zVertex,latCell,lonCell,latEdge,lonEdge,latVertex,lonVertex,fCell,"
    "fEdge,fVertex,meshDensity";

}  // namespace
}  // namespace mpaso

struct mpaso_genmesh_s {
  mpaso::GenMesh *m;
};

extern "C" {

int mpaso_genmesh_icosa(int level, double radius, double omega, mpaso_genmesh *out) {
  return mpaso::guarded("mpaso_genmesh_icosa", [&] {
    mpaso::require(out != nullptr, MPASO_ERR_ARG, "null output handle");
    *out = new mpaso_genmesh_s{mpaso::make_icosa(level, radius, omega)};
  });
}

int mpaso_genmesh_hex(int nx, int ny, double dc, double f0, mpaso_genmesh *out) {
  return mpaso::guarded("mpaso_genmesh_hex", [&] {
    mpaso::require(out != nullptr, MPASO_ERR_ARG, "null output handle");
    *out = new mpaso_genmesh_s{mpaso::make_hex(nx, ny, dc, f0)};
  });
}

int mpaso_genmesh_reorder_sfc(mpaso_genmesh in, mpaso_genmesh *out, int32_t *perm_cell,
                              int32_t *perm_edge, int32_t *perm_vertex) {
  return mpaso::guarded("mpaso_genmesh_reorder_sfc", [&] {
    mpaso::require(in && in->m && out, MPASO_ERR_ARG, "null handle");
    *out = new mpaso_genmesh_s{mpaso::reorder(*in->m, perm_cell, perm_edge, perm_vertex)};
  });
}

int mpaso_genmesh_dims(mpaso_genmesh m, int64_t dims[3], int32_t flags[1], double geom[3]) {
  return mpaso::guarded("mpaso_genmesh_dims", [&] {
    mpaso::require(m && m->m && dims, MPASO_ERR_ARG, "null handle");
    dims[0] = m->m->nC, dims[1] = m->m->nE, dims[2] = m->m->nV;
    if (flags) flags[0] = m->m->sphere ? 1 : 0;
    if (geom) geom[0] = m->m->radius, geom[1] = m->m->Lx, geom[2] = m->m->Ly;
  });
}

int mpaso_genmesh_field(mpaso_genmesh m, const char *name, int32_t *dtype, int64_t *rows,
                        int64_t *cols) {
  return mpaso::guarded("mpaso_genmesh_field", [&] {
    mpaso::require(m && m->m && name, MPASO_ERR_ARG, "null argument");
    mpaso::FieldRef r;
    if (!mpaso::lookup(*m->m, name, r))
      mpaso::fail(MPASO_ERR_NOTFOUND, std::string("unknown dataset ") + name);
    if (dtype) *dtype = r.dtype;
    if (rows) *rows = r.rows;
    if (cols) *cols = r.cols;
  });
}

int mpaso_genmesh_copy(mpaso_genmesh m, const char *name, void *dst) {
  return mpaso::guarded("mpaso_genmesh_copy", [&] {
    mpaso::require(m && m->m && name && dst, MPASO_ERR_ARG, "null argument");
    mpaso::FieldRef r;
    if (!mpaso::lookup(*m->m, name, r))
      mpaso::fail(MPASO_ERR_NOTFOUND, std::string("unknown dataset ") + name);
    const int64_t n = r.rows * r.cols;
    if (r.dtype == MPASO_DTYPE_FLOAT64) {
      std::memcpy(dst, r.data, (size_t)n * sizeof(double));
    } else {
      const int32_t *s = (const int32_t *)r.data;
      int32_t *d = (int32_t *)dst;
      // MPAS file convention: 1-based ids, 0 = unused slot.
      for (int64_t i = 0; i < n; ++i) d[i] = r.one_based ? s[i] + 1 : s[i];
    }
  });
}

const char *mpaso_genmesh_names(void) { return mpaso::kNames; }

void mpaso_genmesh_free(mpaso_genmesh m) {
  if (m) {
    delete m->m;
    delete m;
  }
}

}  // extern "C"

// Internal device-side definitions of libmpaso: the mesh context as it lives
// in HBM, launch helpers, and FP64 helpers that keep work off the FP64 pipe.
//
// Layout: every entity is renumbered along a Hilbert curve (cells) and by
// lowest adjacent cell (edges, vertices).  Per-entity fields keep the
// reference's per-entity rows ([n][L], [n][L][T]) in the new numbering.
// Ragged connectivity is stored slot-major ([slot][n]) so that a warp reading
// slot j of 32 consecutive entities issues one coalesced load.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <string>
#include <vector>

#include "common.hh"
#include "mpaso.h"

namespace mpaso {

constexpr int kMaxEdges = 8;     // mpasoflecsi/common/constants.hh:11
constexpr int kMaxEdges2 = 16;   // constants.hh:12
constexpr int kVertexDegree = 3; // constants.hh:14
constexpr int kMaxTracers = 8;

#define MPASO_CUDA(call)                                                               \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      ::mpaso::fail(MPASO_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Device view of a mesh context (all pointers are device memory).
struct DMesh {
  int nC, nE, nV;
  int maxEoC, maxEoE, maxAdv, fctLev;
  // ---- cells ----
  const int *nEoC;            // [nC]
  const int *eoc;             // [maxEoC][nC] edgesOnCell, file order
  const double *eocSign;      // [maxEoC][nC] edgeSignOnCell (-1: c is cells(e)[0]), file order
  const int *eocAsc;          // [maxEoC][nC] edges of c by ascending reference edge id
  const double *eocAscSign;   // [maxEoC][nC] sign for eocAsc (-1: c is cells(e)[0])
  const int *coc;             // [maxEoC][nC] cellsOnCell, file order
  // [maxEoC][nC] the cell across eoc[j][c], shifted left one bit, | 1 where c
  // is cells(e)[0] of that edge (pads: own index, bit 0)
  const int *nbr;
  const double *areaCell, *invAreaCell, *bottomDepth;
  const int *maxLevelCell;    // [nC]
  // ---- edges ----
  const int2 *coe;            // [nE] cells(e): ascending reference ids (transposed c2e)
  const int2 *voe;            // [nE] vertices(e): file order
  const double *dvEdge, *dcEdge, *invDcEdge, *invDvEdge;
  const int *nEoE;            // [nE]
  const int *eoe;             // [maxEoE][nE] edgesOnEdge, file order
  const double *woe;          // [maxEoE][nE] weightsOnEdge
  const int *maxLevelEdgeTop; // [nE]
  const int *nAdv;            // [nE]
  const int *advCells;        // [maxAdv][nE]
  const double *advCoef, *advCoef3;  // [maxAdv][nE] reference coefficients
  const double *advCp, *advCm;       // [maxAdv][nE] advCoef +/- 0.25 advCoef_3rd
  const int *hoMask;          // [nE][fctLev] highOrderAdvMask
  const double *meshScalingDel2;
  // ---- vertices ----
  const int *cov;             // [3][nV] cells(v): ascending reference ids (transposed c2v)
  const double *kite;         // [3][nV] kiteAreasOnVertex, paired with cov by slot
  const int *eov;             // [3][nV] edges(v): ascending reference ids (transposed e2v)
  const double *eovSign;      // [3][nV] -1: v is vertices(e)[0], +1: vertices(e)[1]
  const double *areaTriangle, *invAreaTriangle, *fVertex;
  // ---- reverse connectivity for the adjoint (gathers instead of scatters) ----
  const double *woeT;         // [maxEoE][nE] weight of e in the stencil of eoe[j][e] (0 in pads)
  const int *vocR;            // [maxEoC][nC] vertices of c (pads repeat slot 0)
  const double *kiteR;        // [maxEoC][nC] kite of c at vocR[j][c] (0 in pads)
  // [maxAdvR][nC] every advection stencil entry that reads the cell
  // (advCells[slot][edge] == c): the edge (ascending, -1 pads last) and the
  // cell's coefficient pair there {advCp, advCm}
  const int *advRe;
  const double2 *advRc;
  int maxAdvR;
  const int *cocU;            // [maxEoC][nC] cellsOnCell, -1 for the cell itself and repeats
};

// Host-side mesh context.
struct MeshCtx {
  int device = 0;
  int sms = 152;  // streaming multiprocessors of `device` (set when the context is built)
  cudaStream_t stream = nullptr;
  double gravity = 9.80616;  // mpasoflecsi/common/constants.hh:30-31
  bool has_fct = false;
  DMesh d{};
  std::vector<int32_t> perm[3];   // new -> reference id
  std::vector<int32_t> iperm[3];  // reference id -> new
  int32_t *d_perm[3] = {nullptr, nullptr, nullptr};  // device copies of perm
  int32_t *d_iperm[3] = {nullptr, nullptr, nullptr};  // device copies of iperm
  void *arena = nullptr;
  size_t arena_bytes = 0;
  // growable scratch for the per-task entries
  void *scratch = nullptr;
  size_t scratch_bytes = 0;
  void *ensure_scratch(size_t bytes);
  // ensemble contexts: first cell / edge / vertex of each member (n + 1 rows)
  std::vector<int64_t> members;
  // geometry of the test-case initialisers (mpaso_mesh_set_geometry): latCell,
  // lonCell, latVertex, lonVertex, latEdge, lonEdge, angleEdge, xCell, yCell,
  // zCell back to back in the context numbering; null until set
  double *geo = nullptr;
  ~MeshCtx();
};

// ------------------------------------------------------------------ launch
inline int blocks_for(int64_t n, int threads) { return (int)((n + threads - 1) / threads); }

// --------------------------------------------------- FP64 helpers (INT pipe)
// GB300 issues FP64 at a small fraction of its integer rate, so selects,
// min/max, sign tests and sign flips on doubles are done on bit patterns.
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ double bitsd(long long b) { return __longlong_as_double(b); }

// std::max(0.0, x) for non-NaN x (returns +0.0 for x <= 0).
__device__ __forceinline__ double dpos(double x) {
  const long long b = dbits(x);
  return bitsd(b > 0 ? b : 0LL);
}
// std::min(0.0, x) for non-NaN x.
__device__ __forceinline__ double dneg(double x) {
  const long long b = dbits(x);
  return bitsd(b < 0 ? b : 0LL);
}
// Signed-magnitude -> two's-complement order key: a < b  <=>  key(a) < key(b)
// for non-NaN values (treats -0 < +0).
__device__ __forceinline__ long long dkey(double x) {
  const long long b = dbits(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
// std::min / std::max semantics (b wins only when strictly smaller / larger).
__device__ __forceinline__ double dmin(double a, double b) { return dkey(b) < dkey(a) ? b : a; }
__device__ __forceinline__ double dmax(double a, double b) { return dkey(a) < dkey(b) ? b : a; }
// min(1, max(0, x)) for non-NaN x.
__device__ __forceinline__ double dclamp01(double x) {
  const long long b = dbits(x);
  const long long p = b > 0 ? b : 0LL;
  return bitsd(p > 0x3ff0000000000000LL ? 0x3ff0000000000000LL : p);
}
// x * s for s in {-1, +1} given as the sign bit mask (0 or 1<<63).
__device__ __forceinline__ double dflip(double x, long long signmask) {
  return bitsd(dbits(x) ^ signmask);
}
__device__ __forceinline__ bool dgt0(double x) { return dbits(x) > 0; }
__device__ __forceinline__ bool dlt0(double x) { return dbits(x) < 0 && dbits(x) != (long long)0x8000000000000000ULL; }

}  // namespace mpaso

// A mesh context is shared by the states made on it: mpaso_mesh_destroy drops
// the caller's reference and the context is freed with the last reference,
// so states and their mesh may be destroyed in either order.
struct mpaso_mesh_s {
  mpaso::MeshCtx ctx;
  std::atomic<int> refs{1};
};

namespace mpaso {
// Drops one reference; frees the context (on its device) with the last one.
inline void release_mesh(mpaso_mesh_s *m) {
  if (m->refs.fetch_sub(1) != 1) return;
  cudaSetDevice(m->ctx.device);
  cudaStreamSynchronize(m->ctx.stream);
  delete m;
  cudaGetLastError();  // teardown is best effort: leave no error pending for later calls
}
}  // namespace mpaso

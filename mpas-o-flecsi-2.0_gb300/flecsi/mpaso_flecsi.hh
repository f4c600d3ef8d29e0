// FleCSI-side wrapper library: the reference's task functions with their
// exact signatures, whose bodies call libmpaso's C ABI.  Built inside a FleCSI
// build of the reference in place of apps/sw/tasks/solve.cc and
// apps/ocean/tasks/solve.cc (sw_tasks.cc, ocean_tasks.cc here), it leaves every
// flecsi::execute<...> call site of apps/sw/run.cc and apps/ocean/run.cc as it
// is.  A task receives accessors over FleCSI's own storage (one vltensor /
// vltracer per entity, contiguous) and hands their raw pointers over; host
// memory (FleCSI's MPI backend) is copied to the device and back by each call.
//
// The device mesh context holds what the tasks do not pass (connectivity,
// geometry, FCT statics): make_mesh_context() builds it once from the mesh
// specialization after read_fields (apps/sw/initialize.cc:41-61), and
// mesh_context() is what the task bodies use.
//
// Single-color runs only.  The specialization partitions the mesh into one
// color per process (mpasoflecsi/specialization/mesh.cc:31); with more than
// one, a color's local connectivity holds partition-edge cells whose stencils
// reach into ghosts, and the device context has no halo exchange.
// make_mesh_context() refuses such runs.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "flecsi/execution.hh"
#include "mpaso.h"

namespace mpaso_flecsi {

// Failure of a libmpaso call; a FleCSI build reports it through flog_assert.
[[noreturn]] inline void fail(const std::string &what) { throw std::runtime_error("libmpaso: " + what); }

inline void ok(int rc) {
  if (rc != MPASO_OK) fail(mpaso_last_error());
}

inline mpaso_mesh &mesh_context() {
  static mpaso_mesh m = nullptr;
  return m;
}

inline mpaso_mesh context() {
  if (!mesh_context()) fail("no device mesh context: call mpaso_flecsi::make_mesh_context first");
  return mesh_context();
}

// Raw pointer to an accessor's storage: span().data() where the accessor has
// span() (FleCSI 2), &a(0) otherwise.
template <class A, class = void> struct has_span : std::false_type {};
template <class A> struct has_span<A, std::void_t<decltype(std::declval<A &>().span())>> : std::true_type {};

template <class A> auto raw(A a) {
  if constexpr (has_span<A>::value) {
    using E = std::remove_reference_t<decltype(*a.span().data())>;
    return reinterpret_cast<std::conditional_t<std::is_const_v<E>, const double *, double *>>(a.span().data());
  } else {
    return reinterpret_cast<double *>(&a(0));
  }
}

// Builds the device mesh context from the mesh specialization (reference ids,
// file order of c2v/c2e/c2c/e2v/e2e as the specialization holds them) and the
// static fields; fct (optional) carries the FCT statics of the ocean app.
struct FctStatics {
  int32_t nlev = 0;
  const int32_t *maxLevelCell = nullptr, *maxLevelEdgeTop = nullptr, *nAdvCellsForEdge = nullptr;
  const int32_t *advCellsForEdge = nullptr, *highOrderAdvMask = nullptr;
  const double *edgeSignOnCell = nullptr, *advCoef = nullptr, *advCoef_3rd = nullptr, *meshScalingDel2 = nullptr;
};

template <class Mesh, class DA>
void make_mesh_context(Mesh &m, DA areaCell, DA dvEdge, DA dcEdge, DA areaTriangle, const double *kiteAreasOnVertex,
                       DA fVertex, const double *weightsOnEdge, const double *bottomDepth, DA xCell, DA yCell,
                       DA zCell, const FctStatics *fct = nullptr, int device = -1) {
  if (flecsi::processes() != 1)
    fail("the device mesh context supports single-color runs only (" + std::to_string(flecsi::processes()) +
         " colors): the per-task wrappers have no halo exchange");
  std::vector<int64_t> off[5];
  std::vector<int32_t> idx[5];  // c2v, c2e, c2c, e2v, e2e
  for (auto &o : off) o.push_back(0);
  for (auto c : m.cells()) {
    for (auto v : m.vertices(c)) idx[0].push_back((int32_t)v);
    for (auto e : m.edges(c)) idx[1].push_back((int32_t)e);
    for (auto n : m.cells(c)) idx[2].push_back((int32_t)n);
    for (int k = 0; k < 3; ++k) off[k].push_back((int64_t)idx[k].size());
  }
  for (auto e : m.edges()) {
    for (auto v : m.vertices(e)) idx[3].push_back((int32_t)v);
    for (auto o : m.edges(e)) idx[4].push_back((int32_t)o);
    for (int k = 3; k < 5; ++k) off[k].push_back((int64_t)idx[k].size());
  }
  mpaso_mesh_desc d{};
  d.nCells = (int64_t)m.cells().size(), d.nEdges = (int64_t)m.edges().size();
  d.nVertices = (int64_t)m.vertices().size();
  d.c2v_off = off[0].data(), d.c2v = idx[0].data(), d.c2e_off = off[1].data(), d.c2e = idx[1].data();
  d.c2c_off = off[2].data(), d.c2c = idx[2].data(), d.e2v_off = off[3].data(), d.e2v = idx[3].data();
  d.e2e_off = off[4].data(), d.e2e = idx[4].data();
  d.areaCell = raw(areaCell), d.dvEdge = raw(dvEdge), d.dcEdge = raw(dcEdge), d.areaTriangle = raw(areaTriangle);
  d.kiteAreasOnVertex = kiteAreasOnVertex, d.fVertex = raw(fVertex), d.weightsOnEdge = weightsOnEdge;
  d.bottomDepth = bottomDepth, d.xCell = raw(xCell), d.yCell = raw(yCell), d.zCell = raw(zCell);
  d.reorder = 1;
  if (fct) {
    d.fct_nlev = fct->nlev, d.maxLevelCell = fct->maxLevelCell, d.maxLevelEdgeTop = fct->maxLevelEdgeTop;
    d.nAdvCellsForEdge = fct->nAdvCellsForEdge, d.advCellsForEdge = fct->advCellsForEdge;
    d.highOrderAdvMask = fct->highOrderAdvMask, d.edgeSignOnCell = fct->edgeSignOnCell;
    d.advCoef = fct->advCoef, d.advCoef_3rd = fct->advCoef_3rd, d.meshScalingDel2 = fct->meshScalingDel2;
  }
  if (mesh_context()) {
    mpaso_mesh_destroy(mesh_context());
    mesh_context() = nullptr;
  }
  ok(mpaso_mesh_create(&d, device, &mesh_context()));
}

}  // namespace mpaso_flecsi

// TEST INFRASTRUCTURE ONLY.  Builds the device mesh context through the FleCSI
// wrapper library (mpas-o-flecsi-2.0_gb300/flecsi/mpaso_flecsi.hh) from the
// header shim's mesh view and accessors, as a FleCSI build of the reference
// would after read_fields.  Linked by oracle/build.py with the wrapper task
// bodies (in place of the reference's solve.cc files), the reference's own
// driver logic (ref_driver.cc) and libmpaso, where the reference checkout
// exists.
#include <cstring>
#include <stdexcept>
#include <string>

#include "apps/sw/state.hh"
#include "mpaso_flecsi.hh"
#include "oracle.h"

namespace {
template <class T> flecsi::accessor_t<T, flecsi::ro, flecsi::ro> view(const T *p) { return {const_cast<T *>(p)}; }
}  // namespace

// xyz: the cell centres (x, y, z; nC each) the context orders the mesh by.
extern "C" int flw_make_context(const orc_mesh *om, const orc_static *s, const double *xyz, int32_t fct, char *err,
                                int errlen) {
  try {
    mpas::mesh::view v;
    v.nC = (std::size_t)om->nC, v.nE = (std::size_t)om->nE, v.nV = (std::size_t)om->nV;
    mpas::mesh::crs *dst[ORC_NCNX] = {&v.c2v, &v.c2e, &v.c2c, &v.e2v, &v.e2e, &v.v2c, &v.e2c, &v.v2e};
    for (int k = 0; k < ORC_NCNX; ++k) *dst[k] = {om->off[k], om->idx[k]};
    const double *x = xyz, *y = xyz + om->nC, *z = xyz + 2 * om->nC;
    // the FCT / del2 statics of the ocean tasks, as a FleCSI build passes them
    // from its state (apps/ocean/state.hh:68-101)
    mpaso_flecsi::FctStatics f;
    f.nlev = (int32_t)mpas::nVertLevels;
    f.maxLevelCell = s->maxLevelCell, f.maxLevelEdgeTop = s->maxLevelEdgeTop;
    f.nAdvCellsForEdge = s->nAdvCellsForEdge, f.advCellsForEdge = s->advCellsForEdge;
    f.highOrderAdvMask = s->highOrderAdvMask, f.edgeSignOnCell = s->edgeSignOnCell;
    f.advCoef = s->advCoef, f.advCoef_3rd = s->advCoef_3rd, f.meshScalingDel2 = s->meshScalingDel2;
    mpaso_flecsi::make_mesh_context(v, view(s->areaCell), view(s->dvEdge), view(s->dcEdge), view(s->areaTriangle),
                                    s->kiteAreasOnVertex, view(s->fVertex), s->weightsOnEdge, s->bottomDepth,
                                    view(x), view(y), view(z), fct ? &f : nullptr);
    return 0;
  } catch (const std::exception &e) {
    std::strncpy(err, e.what(), (size_t)errlen - 1);
    err[errlen - 1] = '\0';
    return 1;
  }
}

// Releases the device mesh context the wrappers use.
extern "C" void flw_destroy_context(void) {
  if (mpaso_flecsi::mesh_context()) {
    mpaso_mesh_destroy(mpaso_flecsi::mesh_context());
    mpaso_flecsi::mesh_context() = nullptr;
  }
}

// Sets the process (color) count the shim reports, for the refusal check.
extern "C" void flw_set_processes(int n) { flecsi::process_count = (std::size_t)n; }

// Oracle shim (test infrastructure only): the output-field descriptors named by
// apps/sw/state.hh:66-70; the HDF5 machinery behind them is not needed.
#pragma once
#include "mpasoflecsi/common/types.hh"

namespace mpas { namespace io { namespace desc {
struct thickness {};
struct topography {};
struct vorticity {};
struct pv_vertex {};
struct tracers {};
}}}  // namespace mpas::io::desc

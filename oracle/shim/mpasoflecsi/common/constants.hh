// Oracle shim (test infrastructure only): replaces mpasoflecsi/common/
// constants.hh so the vertical level count, tracer count and gravity can be
// chosen per oracle build (-DMPASO_REF_NVL, -DMPASO_REF_NTR,
// -DMPASO_REF_GRAVITY).  The sizes and physical constants otherwise carry the
// reference's values (mpasoflecsi/common/constants.hh:11-34).
#pragma once
#include <cstddef>

#ifndef MPASO_REF_NVL
#define MPASO_REF_NVL 5
#endif
#ifndef MPASO_REF_NTR
#define MPASO_REF_NTR 5
#endif
#ifndef MPASO_REF_GRAVITY
#define MPASO_REF_GRAVITY 9.80616
#endif

namespace mpas {
static constexpr std::size_t maxEdges = 8;
static constexpr std::size_t maxEdges2 = maxEdges * 2;
static constexpr std::size_t nAdvectionCells = maxEdges2;
static constexpr std::size_t vertexDegree = 3;
static constexpr std::size_t nVertLevels = MPASO_REF_NVL;
static constexpr std::size_t maxTracers = MPASO_REF_NTR;
static constexpr std::size_t deuce = 2;
}  // namespace mpas

namespace mpas_constants {
static constexpr double a = 6371000.0;
static constexpr double pi = 3.141592653589793;
static constexpr double gravity = MPASO_REF_GRAVITY;
static constexpr double omega = 7.29212e-5;
static constexpr double rho_sw = 1026.0;
}  // namespace mpas_constants

// Oracle shim (test infrastructure only): per-entity tensor types with the
// same std::array layouts as mpasoflecsi/common/types.hh:16-49, built on the
// shim's FleCSI accessors.  Also supplies the `real_t` the reference's
// apps/sw/tasks/solve.cc:220,223 uses without declaring it.
#pragma once
#include <array>
#include <complex>

#include "flecsi/data.hh"
#include "mpasoflecsi/common/constants.hh"

namespace mpas {

#ifdef MPASO_REF_COMPLEX_STEP
// Complex-step build (oracle/ref_cstep.cc): state fields carry x + i eps dx,
// so the reference tasks' own arithmetic carries the tangent in the
// imaginary part.  compute_error (not on the step) reduces into a double.
using real_t = std::complex<double>;
inline double &operator+=(double &a, const std::complex<double> &b) { return a += b.real(); }
#else
using real_t = double;
#endif

template <class T, int... II> struct tensor;
template <class T, int... II> using tensor_t = typename tensor<T, II...>::type;
template <class T> struct tensor<T> { using type = T; };
template <class T, int I, int... II> struct tensor<T, I, II...> {
  using type = std::array<tensor_t<T, II...>, I>;
};

template <class T> using vdtensor = std::array<T, vertexDegree>;
// Per-level state: in the complex-step build every per-level double (the
// reference spells some state accessors vltensor<double>) becomes real_t.
template <class T> struct level_scalar { using type = T; };
template <> struct level_scalar<double> { using type = real_t; };
template <class T> using vltensor = std::array<typename level_scalar<T>::type, nVertLevels>;
using vlreal = vltensor<real_t>;
using vltracer = tensor_t<real_t, nVertLevels, maxTracers>;
template <class T> using metensor = std::array<T, maxEdges>;
template <class T> using me2tensor = std::array<T, maxEdges2>;
using derivtensor = tensor_t<double, maxEdges2, 2>;

template <class T, flecsi::partition_privilege_t P1, flecsi::partition_privilege_t P2>
using acc = typename flecsi::template field<T>::template accessor<P1, P2>;

using flecsi::na;
using flecsi::ro;
using flecsi::rw;
using flecsi::wo;

template <class... T> struct type_list {};

}  // namespace mpas

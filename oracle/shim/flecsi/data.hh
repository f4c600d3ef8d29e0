// Oracle shim (test infrastructure only): FleCSI data model stand-ins.
// field<T>::accessor<P1,P2> is a plain indexable view over caller memory laid
// out exactly as FleCSI stores a field (one T per entity, AoS).
#pragma once
// FleCSI's headers pull these in; the reference's sources rely on that.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <iostream>
#include <map>
#include <vector>
#include <cstdint>
#include <initializer_list>
#include <istream>
#include <ostream>
#include <string>
#include <utility>

#include "flecsi/flog.hh"

namespace flecsi {

enum partition_privilege_t { na, ro, wo, rw };

namespace util {
using id = std::uint32_t;
}

namespace topo {
// Typed entity id: converts to an index, compares through that conversion.
template <int Space> struct id {
  std::size_t v;
  constexpr operator std::size_t() const { return v; }
};
}  // namespace topo

template <class T, partition_privilege_t P1, partition_privilege_t P2> struct accessor_t {
  T *data = nullptr;
  T &operator()(std::size_t i) const { return data[i]; }
};

template <class T> struct field {
  template <partition_privilege_t P1, partition_privilege_t P2>
  using accessor = accessor_t<T, P1, P2>;
  template <class Topo, int Space> struct definition {
    constexpr definition() {}
  };
};

}  // namespace flecsi

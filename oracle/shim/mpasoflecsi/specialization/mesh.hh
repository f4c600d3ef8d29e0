// Oracle shim (test infrastructure only): the `mpas::mesh` topology interface
// the reference's tasks use (mpasoflecsi/specialization/mesh.hh:20-75), over
// CRS connectivity supplied by the oracle driver.  The driver builds c2v, c2e,
// c2c, e2v, e2e in file order and v2c, e2c, v2e by transposition, as
// mpasoflecsi/specialization/mesh.cc:67-116 does.
#pragma once
#include <cstddef>
#include <cstdint>

#include "flecsi/data.hh"
#include "mpasoflecsi/common/types.hh"

namespace mpas {

struct mesh {
  enum index_space { vertices, edges, cells };

  struct crs {
    const std::int64_t *off = nullptr;
    const std::int32_t *idx = nullptr;
  };

  template <int S> struct id_iter {
    const std::int32_t *p;
    flecsi::topo::id<S> operator*() const { return {(std::size_t)*p}; }
    id_iter &operator++() { ++p; return *this; }
    bool operator!=(const id_iter &o) const { return p != o.p; }
  };
  template <int S> struct ragged {
    const std::int32_t *p;
    std::size_t n;
    std::size_t size() const { return n; }
    flecsi::topo::id<S> operator[](std::size_t i) const { return {(std::size_t)p[i]}; }
    id_iter<S> begin() const { return {p}; }
    id_iter<S> end() const { return {p + n}; }
  };
  template <int S> struct count_iter {
    std::size_t i;
    flecsi::topo::id<S> operator*() const { return {i}; }
    count_iter &operator++() { ++i; return *this; }
    bool operator!=(const count_iter &o) const { return i != o.i; }
  };
  template <int S> struct range {
    std::size_t n;
    std::size_t size() const { return n; }
    flecsi::topo::id<S> operator[](std::size_t i) const { return {i}; }
    count_iter<S> begin() const { return {0}; }
    count_iter<S> end() const { return {n}; }
  };

  static constexpr int kC = cells, kE = edges, kV = vertices;

  struct view {
    std::size_t nC = 0, nE = 0, nV = 0;
    crs c2v, c2e, c2c, e2v, e2e, v2c, e2c, v2e;

    template <int S> static ragged<S> row(const crs &c, std::size_t i) {
      return {c.idx + c.off[i], (std::size_t)(c.off[i + 1] - c.off[i])};
    }
    range<kC> cells() const { return {nC}; }
    range<kE> edges() const { return {nE}; }
    range<kV> vertices() const { return {nV}; }
    ragged<kC> cells(flecsi::topo::id<kC> c) const { return row<kC>(c2c, c); }
    ragged<kC> cells(flecsi::topo::id<kE> e) const { return row<kC>(e2c, e); }
    ragged<kC> cells(flecsi::topo::id<kV> v) const { return row<kC>(v2c, v); }
    ragged<kE> edges(flecsi::topo::id<kC> c) const { return row<kE>(c2e, c); }
    ragged<kE> edges(flecsi::topo::id<kE> e) const { return row<kE>(e2e, e); }
    ragged<kE> edges(flecsi::topo::id<kV> v) const { return row<kE>(v2e, v); }
    ragged<kV> vertices(flecsi::topo::id<kC> c) const { return row<kV>(c2v, c); }
    ragged<kV> vertices(flecsi::topo::id<kE> e) const { return row<kV>(e2v, e); }
  };

  template <flecsi::partition_privilege_t P1, flecsi::partition_privilege_t P2>
  using accessor = view;

  struct slot {};
  struct cslot {};
};

}  // namespace mpas

// Oracle shim (test infrastructure only): program_option stand-in.  The
// drivers set option values directly (the reference reads them from the CLI).
#pragma once
#include <cstddef>
#include <initializer_list>
#include <utility>

#include "flecsi/data.hh"

namespace flecsi {

// Processes, i.e. colors (the specialization makes one color per process,
// mpasoflecsi/specialization/mesh.cc:31).  One in every oracle run; a test
// probe sets more to check the wrappers' refusal of multi-color runs.
inline std::size_t process_count = 1;
inline std::size_t processes() { return process_count; }

struct option_default_t {};
inline constexpr option_default_t option_default{};

template <class T> struct program_option {
  T v{};
  program_option(const char *, const char *, int) {}
  program_option(const char *, const char *, const char *,
                 std::initializer_list<std::pair<option_default_t, T>> init) {
    for (auto &p : init) v = p.second;
  }
  T value() const { return v; }
  void set(T x) { v = x; }
  friend bool operator==(const program_option &o, const T &x) { return o.v == x; }
};

}  // namespace flecsi

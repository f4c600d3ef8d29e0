// Oracle shim (test infrastructure only): stands in for FleCSI's flog so the
// reference's task sources compile unmodified.  flog(...) output is discarded;
// flog_assert / flog_fatal throw, and the oracle drivers turn that into a
// nonzero status.
#pragma once
#include <sstream>
#include <stdexcept>
#include <string>

namespace flecsi_shim {
struct null_stream {
  template <class T> null_stream &operator<<(const T &) { return *this; }
  null_stream &operator<<(std::ostream &(*)(std::ostream &)) { return *this; }
};
}  // namespace flecsi_shim

#define flog(level) (flecsi_shim::null_stream())
#define flog_assert(cond, msg)                                      \
  do {                                                              \
    if (!(cond)) {                                                  \
      std::ostringstream flog_os_;                                  \
      flog_os_ << msg;                                              \
      throw std::runtime_error("flog_assert: " + flog_os_.str());   \
    }                                                               \
  } while (0)
#define flog_fatal(msg)                                             \
  do {                                                              \
    std::ostringstream flog_os_;                                    \
    flog_os_ << msg;                                                \
    throw std::runtime_error("flog_fatal: " + flog_os_.str());      \
  } while (0)

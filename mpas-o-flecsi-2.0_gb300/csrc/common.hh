// Shared host-side helpers of libmpaso: error reporting across the C ABI and
// the space-filling-curve keys used to renumber meshes.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>

#include "mpaso_mesh.h"

namespace mpaso {

// Exception carrying an MPASO_ERR_* code; converted to a return status at the
// C ABI so that no exception ever crosses it.
struct error : std::runtime_error {
  int code;
  error(int c, const std::string &msg) : std::runtime_error(msg), code(c) {}
};

void set_last_error(const std::string &msg);

[[noreturn]] inline void fail(int code, const std::string &msg) { throw error(code, msg); }

inline void require(bool ok, int code, const std::string &msg) {
  if (!ok) fail(code, msg);
}

// Runs `body` and maps exceptions to MPASO_ERR_* codes + the thread-local message.
template <class F> int guarded(const char *where, F &&body) {
  try {
    body();
    return MPASO_OK;
  } catch (const error &e) {
    set_last_error(std::string(where) + ": " + e.what());
    return e.code;
  } catch (const std::bad_alloc &) {
    set_last_error(std::string(where) + ": host allocation failed");
    return MPASO_ERR_ALLOC;
  } catch (const std::exception &e) {
    set_last_error(std::string(where) + ": " + e.what());
    return MPASO_ERR_MESH;
  }
}

// Hilbert index of a point with `dims` (2 or 3) coordinates, each quantised to
// `bits` bits.  Transpose-form algorithm of J. Skilling, "Programming the
// Hilbert curve", AIP Conf. Proc. 707 (2004).
uint64_t hilbert_key(const uint32_t *coords, int dims, int bits);
// Morton (Z-order) index: the coordinates' bits interleaved, most significant first.
uint64_t morton_key(const uint32_t *coords, int dims, int bits);

}  // namespace mpaso

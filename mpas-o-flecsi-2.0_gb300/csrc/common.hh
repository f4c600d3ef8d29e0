// Shared host-side helpers of libmpaso: error reporting across the C ABI and
// the space-filling-curve keys used to renumber meshes.
#pragma once

#include <algorithm>
#include <cstdint>
#include <exception>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include <nvtx3/nvToolsExt.h>

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
// The message is only turned into a std::string on failure: checks inside
// per-element loops cost a compare, not an allocation.
inline void require(bool ok, int code, const char *msg) {
  if (!ok) fail(code, msg);
}

// f(i) for i in [0, n) on the host's threads, in contiguous ranges of at
// least `grain` iterations (one thread when n is small).  For loops whose
// iterations write disjoint outputs; an exception in any range is rethrown
// on the calling thread after every range has finished.
template <class F> void parallel_for(int64_t n, F &&f, int64_t grain = 1 << 14) {
  const int64_t hw = std::max<int64_t>(1, (int64_t)std::thread::hardware_concurrency());
  const int64_t nt = std::min<int64_t>(hw, (n + grain - 1) / std::max<int64_t>(grain, 1));
  if (nt <= 1) {
    for (int64_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::exception_ptr ep;
  std::mutex mu;
  std::vector<std::thread> th;
  th.reserve(nt);
  for (int64_t t = 0; t < nt; ++t)
    th.emplace_back([&, t] {
      try {
        for (int64_t i = n * t / nt, e = n * (t + 1) / nt; i < e; ++i) f(i);
      } catch (...) {
        std::lock_guard<std::mutex> g(mu);
        if (!ep) ep = std::current_exception();
      }
    });
  for (auto &x : th) x.join();
  if (ep) std::rethrow_exception(ep);
}

// Runs `body` and maps exceptions to MPASO_ERR_* codes + the thread-local
// message.  Every C-ABI call is an NVTX range named after the entry point
// (seen by Nsight tools and `ncu --nvtx`; a pointer check when none is attached).
template <class F> int guarded(const char *where, F &&body) {
  nvtxRangePushA(where);
  struct Pop {
    ~Pop() { nvtxRangePop(); }
  } pop;
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

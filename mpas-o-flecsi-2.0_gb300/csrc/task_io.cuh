// Staging of per-task arguments: reference-numbered host or device arrays are
// gathered into the context's Hilbert numbering before a task kernel runs and
// scattered back afterwards.
#pragma once

#include "device.cuh"

namespace mpaso {

__global__ void k_gather_rows(const double *__restrict__ src, double *__restrict__ dst,
                              const int32_t *__restrict__ perm, int64_t n, int row);
__global__ void k_scatter_rows(const double *__restrict__ src, double *__restrict__ dst,
                               const int32_t *__restrict__ perm, int64_t n, int row);

bool is_device_pointer(const void *p);
// One pass between a page-locked host array (reference order, through its
// device alias) and a device array (context order): import (host -> device)
// or export; iperm maps reference ids to context ids.
void host_rows_pub(bool import, const double *src, double *dst, const int32_t *iperm, int64_t n, int row,
                   int sms, cudaStream_t s);
void k_gather_rows_pub(const double *src, double *dst, const int32_t *perm, int64_t n, int row,
                       cudaStream_t s);
void k_scatter_rows_pub(const double *src, double *dst, const int32_t *perm, int64_t n, int row,
                        cudaStream_t s);

class TaskIO {
 public:
  TaskIO(mpaso_mesh m, void *stream);
  ~TaskIO();
  // Registers an argument; returns its slot.  `entity` = MPASO_CELLS/EDGES/VERTICES,
  // `row` = doubles per entity.  Outputs are copied in as well, so entries a task
  // leaves untouched keep their values (FleCSI storage semantics).
  int in(const double *p, int entity, int row) { return add(p, entity, row, false); }
  int out(double *p, int entity, int row) { return add(p, entity, row, true); }
  void stage();                  // copies + gathers into the internal layout
  double *ptr(int slot) const { return args_[slot].internal; }
  void finish();                 // scatters outputs back, syncs for host memory
  cudaStream_t stream() const { return stream_; }
  MeshCtx &ctx() { return m_->ctx; }
  const DMesh &dm() const { return m_->ctx.d; }

 private:
  struct Arg {
    double *user;
    int entity, row;
    bool output, host;
    double *internal = nullptr, *raw = nullptr;
  };
  int add(const double *p, int entity, int row, bool output);
  int64_t count(int entity) const;
  mpaso_mesh m_;
  cudaStream_t stream_;
  std::vector<Arg> args_;
  bool any_host_ = false;
};

}  // namespace mpaso

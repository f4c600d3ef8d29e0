// Staging of per-task arguments between the reference numbering and the
// context's Hilbert numbering.
#include "task_io.cuh"

namespace mpaso {

__global__ void k_gather_rows(const double *__restrict__ src, double *__restrict__ dst,
                              const int32_t *__restrict__ perm, int64_t n, int row) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n * row) return;
  const int64_t e = i / row, r = i - e * row;
  dst[i] = src[(int64_t)perm[e] * row + r];
}

__global__ void k_scatter_rows(const double *__restrict__ src, double *__restrict__ dst,
                               const int32_t *__restrict__ perm, int64_t n, int row) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n * row) return;
  const int64_t e = i / row, r = i - e * row;
  dst[(int64_t)perm[e] * row + r] = src[i];
}

// Rows between page-locked host memory (reference order, read or written
// through its device alias) and device memory (context order), in one pass:
// the host side is walked in order, 16 bytes a thread where both sides allow
// (coalesced over the host link), and the device side is scattered through
// iperm (reference id -> context id).  import: dst[iperm[j]] = src[j];
// export: dst[j] = src[iperm[j]] (rows of `row` doubles).
template <bool IMPORT>
__global__ void k_host_rows(const double *__restrict__ src, double *__restrict__ dst,
                            const int32_t *__restrict__ iperm, int64_t n, int row, bool pairs) {
  const int64_t total = n * row, stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  auto dev = [&](int64_t i) {
    const int64_t j = i / row, r = i - j * row;
    return (int64_t)iperm[j] * row + r;
  };
  if (pairs) {  // total even, host side 16-byte aligned
    for (int64_t p = t0; p < total / 2; p += stride) {
      const int64_t i = 2 * p;
      if constexpr (IMPORT) {
        const double2 v = reinterpret_cast<const double2 *>(src)[p];
        dst[dev(i)] = v.x;
        dst[dev(i + 1)] = v.y;
      } else {
        reinterpret_cast<double2 *>(dst)[p] = make_double2(src[dev(i)], src[dev(i + 1)]);
      }
    }
  } else {
    for (int64_t i = t0; i < total; i += stride) {
      if constexpr (IMPORT)
        dst[dev(i)] = src[i];
      else
        dst[i] = src[dev(i)];
    }
  }
}

void host_rows_pub(bool import, const double *src, double *dst, const int32_t *iperm, int64_t n, int row,
                   int sms, cudaStream_t s) {
  const int64_t total = n * row;
  const double *host = import ? src : dst;
  const bool pairs = total % 2 == 0 && ((uintptr_t)host & 15) == 0;
  const int64_t work = pairs ? total / 2 : total;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(blocks_for(work, 256), (int64_t)sms * 8));
  if (import)
    k_host_rows<true><<<blocks, 256, 0, s>>>(src, dst, iperm, n, row, pairs);
  else
    k_host_rows<false><<<blocks, 256, 0, s>>>(src, dst, iperm, n, row, pairs);
  MPASO_CUDA(cudaGetLastError());
}

void k_gather_rows_pub(const double *src, double *dst, const int32_t *perm, int64_t n, int row,
                       cudaStream_t s) {
  k_gather_rows<<<blocks_for(n * row, 256), 256, 0, s>>>(src, dst, perm, n, row);
  MPASO_CUDA(cudaGetLastError());
}

void k_scatter_rows_pub(const double *src, double *dst, const int32_t *perm, int64_t n, int row,
                        cudaStream_t s) {
  k_scatter_rows<<<blocks_for(n * row, 256), 256, 0, s>>>(src, dst, perm, n, row);
  MPASO_CUDA(cudaGetLastError());
}

bool is_device_pointer(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

TaskIO::TaskIO(mpaso_mesh m, void *stream) : m_(m) {
  require(m != nullptr, MPASO_ERR_ARG, "null mesh context");
  MPASO_CUDA(cudaSetDevice(m->ctx.device));
  stream_ = stream ? (cudaStream_t)stream : m->ctx.stream;
}

TaskIO::~TaskIO() = default;

int64_t TaskIO::count(int entity) const {
  const DMesh &d = m_->ctx.d;
  return entity == MPASO_CELLS ? d.nC : entity == MPASO_EDGES ? d.nE : d.nV;
}

int TaskIO::add(const double *p, int entity, int row, bool output) {
  require(p != nullptr, MPASO_ERR_ARG, "null field pointer");
  require(row >= 1, MPASO_ERR_ARG, "bad row length");
  Arg a{const_cast<double *>(p), entity, row, output, !is_device_pointer(p)};
  any_host_ |= a.host;
  args_.push_back(a);
  return (int)args_.size() - 1;
}

void TaskIO::stage() {
  size_t total = 0;
  for (auto &a : args_) {
    const size_t bytes = ((size_t)count(a.entity) * a.row * sizeof(double) + 255) & ~size_t(255);
    total += a.host ? 2 * bytes : bytes;
  }
  char *base = (char *)m_->ctx.ensure_scratch(total);
  size_t off = 0;
  for (auto &a : args_) {
    const int64_t n = count(a.entity);
    const size_t bytes = ((size_t)n * a.row * sizeof(double) + 255) & ~size_t(255);
    a.internal = (double *)(base + off);
    off += bytes;
    const double *src = a.user;
    if (a.host) {
      a.raw = (double *)(base + off);
      off += bytes;
      MPASO_CUDA(cudaMemcpyAsync(a.raw, a.user, (size_t)n * a.row * sizeof(double),
                                 cudaMemcpyHostToDevice, stream_));
      src = a.raw;
    }
    k_gather_rows<<<blocks_for(n * a.row, 256), 256, 0, stream_>>>(src, a.internal,
                                                                  m_->ctx.d_perm[a.entity], n, a.row);
  }
  MPASO_CUDA(cudaGetLastError());
}

void TaskIO::finish() {
  for (auto &a : args_) {
    if (!a.output) continue;
    const int64_t n = count(a.entity);
    double *dst = a.host ? a.raw : a.user;
    k_scatter_rows<<<blocks_for(n * a.row, 256), 256, 0, stream_>>>(a.internal, dst,
                                                                   m_->ctx.d_perm[a.entity], n, a.row);
    if (a.host)
      MPASO_CUDA(cudaMemcpyAsync(a.user, a.raw, (size_t)n * a.row * sizeof(double),
                                 cudaMemcpyDeviceToHost, stream_));
  }
  MPASO_CUDA(cudaGetLastError());
  if (any_host_) MPASO_CUDA(cudaStreamSynchronize(stream_));
}

}  // namespace mpaso

// Allocation-free variant of the compute_tend task entry.
//
// Who needs it: callers that must not allocate device memory while they run --
// a task body executing inside a runtime that owns and pools all device memory
// (a Legion/FleCSI task, an MPI rank sharing the GPU under a fixed memory
// budget), code running under a strict no-cudaMalloc policy because
// cudaMalloc/cudaFree can synchronize the whole device and stall other work,
// or a process that has already handed nearly all HBM to a pool.  The regular
// mpaso_sw_compute_tend stages its arguments through a scratch buffer that the
// mesh context grows with cudaMalloc on demand; this variant stages them
// through one fixed array compiled into the library instead.
//
// The array is a file-scope __device__ buffer of kScratchDoubles doubles
// (32 MiB).  Every GPU that loads the library holds it until the process
// exits.  Host code cannot use the symbol itself as a device address, so each
// call (with the context's device current) asks the runtime for the address
// with cudaGetSymbolAddress -- a cheap lookup -- and keeps it per device.  A
// call made while its stream is being captured uses the kept address instead
// (the lookup may load the module, which a capture does not allow), so make
// the first call on each device before any stream capture.  Looking the
// address up again on every uncaptured call keeps it right after a
// cudaDeviceReset, which reloads the module and may move the array.  All calls
// share the one array: calls whose GPU work overlaps (different streams,
// different host threads) race on it.
#include <mutex>

#include "task_io.cuh"

namespace mpaso {

void launch_task_sw_tend(const DMesh &d, int L, double g, const double *h_edge, const double *h,
                         const double *u, const double *ke, const double *pv_edge, double *tend_h,
                         double *tend_u, cudaStream_t s);

namespace {

constexpr size_t kScratchDoubles = size_t(4) << 20;  // 32 MiB
static __device__ __align__(256) double g_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_addr[kMaxDevices] = {};

// Device address of g_scratch on `device` (which must be current): looked up
// afresh unless `s` is capturing, in which case the address kept from the
// last uncaptured call on this device is used.
double *scratch_address(int device, cudaStream_t s) {
  require(device >= 0 && device < kMaxDevices, MPASO_ERR_ARG, "device index out of range");
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  MPASO_CUDA(cudaStreamIsCapturing(s, &cs));
  std::lock_guard<std::mutex> lock(g_mu);
  if (cs != cudaStreamCaptureStatusNone) {
    require(g_addr[device] != nullptr, MPASO_ERR_ARG,
            "the first allocation-free call on a device must come before any stream capture");
    return g_addr[device];
  }
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
  if (e != cudaSuccess || p == nullptr) {
    cudaGetLastError();
    fail(MPASO_ERR_CUDA, std::string("cudaGetSymbolAddress of the static scratch failed: ") +
                             cudaGetErrorString(e));
  }
  g_addr[device] = (double *)p;
  return g_addr[device];
}

}  // namespace
}  // namespace mpaso

using namespace mpaso;

extern "C" int mpaso_sw_compute_tend_noalloc(mpaso_mesh m, int32_t nlev, const double *h_edge,
                                             const double *h, const double *u, const double *ke,
                                             const double *pv_edge, double *tend_h,
                                             double *tend_u, void *stream) {
  return guarded("mpaso_sw_compute_tend_noalloc", [&] {
    require(m != nullptr, MPASO_ERR_ARG, "null mesh context");
    require(nlev >= 1 && nlev <= 4096, MPASO_ERR_ARG, "nlev out of range");
    const double *ins[5] = {h_edge, h, u, ke, pv_edge};
    for (const double *p : ins)
      require(p && is_device_pointer(p), MPASO_ERR_ARG,
              "every input must be a device pointer (this entry stages nothing through host memory)");
    require(tend_h && tend_u && is_device_pointer(tend_h) && is_device_pointer(tend_u), MPASO_ERR_ARG,
            "outputs must be device pointers");
    MeshCtx &ctx = m->ctx;
    const DMesh &d = ctx.d;
    const int64_t L = nlev, nC = d.nC, nE = d.nE;
    // staging of 3 edge inputs, 2 cell inputs and the 2 outputs, in the context numbering
    const int64_t need = (3 * nE + 2 * nC + nC + nE) * L;
    if ((size_t)need > kScratchDoubles)
      fail(MPASO_ERR_ARG, "mesh too large for the allocation-free entry: needs " + std::to_string(need) +
                              " doubles of staging, the static scratch holds " +
                              std::to_string(kScratchDoubles) + " ((4 nEdges + 3 nCells) * nlev must fit)");
    MPASO_CUDA(cudaSetDevice(ctx.device));
    const cudaStream_t s = stream ? (cudaStream_t)stream : ctx.stream;
    double *base = scratch_address(ctx.device, s);
    double *s_he = base, *s_u = s_he + nE * L, *s_pve = s_u + nE * L, *s_h = s_pve + nE * L;
    double *s_ke = s_h + nC * L, *s_th = s_ke + nC * L, *s_tu = s_th + nC * L;
    // Every scratch element read below is written earlier in this call (the
    // gathers fill the inputs, the kernel writes all of tend_h and tend_u), so
    // nothing has to be cleared between calls.
    k_gather_rows_pub(h_edge, s_he, ctx.d_perm[MPASO_EDGES], nE, (int)L, s);
    k_gather_rows_pub(u, s_u, ctx.d_perm[MPASO_EDGES], nE, (int)L, s);
    k_gather_rows_pub(pv_edge, s_pve, ctx.d_perm[MPASO_EDGES], nE, (int)L, s);
    k_gather_rows_pub(h, s_h, ctx.d_perm[MPASO_CELLS], nC, (int)L, s);
    k_gather_rows_pub(ke, s_ke, ctx.d_perm[MPASO_CELLS], nC, (int)L, s);
    launch_task_sw_tend(d, (int)L, ctx.gravity, s_he, s_h, s_u, s_ke, s_pve, s_th, s_tu, s);
    MPASO_CUDA(cudaGetLastError());
    k_scatter_rows_pub(s_th, tend_h, ctx.d_perm[MPASO_CELLS], nC, (int)L, s);
    k_scatter_rows_pub(s_tu, tend_u, ctx.d_perm[MPASO_EDGES], nE, (int)L, s);
  });
}

// FP64 issue-rate probe: the ceiling the fused RK4 kernels run against on
// GB300 (FP64 is a small fraction of the FP32 rate there).  Independent DFMA
// chains per thread, grid sized to fill every SM; finite loop, no memory
// traffic except one store per thread.
#include "device.cuh"

namespace mpaso {
namespace {
constexpr int kIters = 2048;
__global__ void k_dfma_chains(double *out, double a, double b) {
  double x[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) x[j] = threadIdx.x + j;
#pragma unroll 4
  for (int i = 0; i < kIters; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = fma(x[j], a, b);
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += x[j];
  out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = s;
}
}  // namespace
}  // namespace mpaso

extern "C" int mpaso_probe_fp64(int device, double *dfma_per_s) {
  return mpaso::guarded("mpaso_probe_fp64", [&] {
    mpaso::require(dfma_per_s != nullptr, MPASO_ERR_ARG, "null output");
    MPASO_CUDA(cudaSetDevice(device));
    int sms = 0;
    MPASO_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    const int blocks = sms * 8, threads = 256;
    double *buf = nullptr;
    MPASO_CUDA(cudaMalloc(&buf, (size_t)blocks * threads * sizeof(double)));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0);
      mpaso::k_dfma_chains<<<blocks, threads>>>(buf, 0.999999, 1e-9);
      cudaEventRecord(e1);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) best = ms < best ? ms : best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const cudaError_t err = cudaGetLastError();
    cudaFree(buf);
    if (err != cudaSuccess) mpaso::fail(MPASO_ERR_CUDA, cudaGetErrorString(err));
    *dfma_per_s = (double)blocks * threads * mpaso::kIters * 8 / (best * 1e-3);
  });
}

// fma_peak.cu -- the FP64 and FP32 fused multiply-add rates of the current
// GPU, measured with CUDA events: the denominators of the tracer's
// FP64-pipe and FP32-pipe roofline fractions.  Nothing on the ray-tracing
// path is a contraction, so the tensor-core peak is not the bound; the FMA
// pipes are.  Every thread runs kChains independent FMA chains (enough
// independent work to hide the pipes' latency) over a grid of several
// resident blocks per SM; the result is stored so that no chain is dead.
// Changes no device setting: the rate is at whatever clock the GPU runs.
#include <cuda_runtime.h>

#include "robast_gb.h"
#include "device_state.cuh"

namespace rbg {

constexpr int kChains = 8;
constexpr int kPeakThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kPeakThreads) fma_peak_kernel(int iters, T a, T b, T* out) {
  T v[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) v[c] = (T)(threadIdx.x + c) * (T)1e-3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
#pragma unroll
      for (int c = 0; c < kChains; ++c) v[c] = fma(v[c], a, b);
    }
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += v[c];
  out[blockIdx.x * (size_t)blockDim.x + threadIdx.x] = s;
}

template <typename T>
int fma_rate(int iters, double* flops_per_s, cudaStream_t st) {
  const int blocks = sm_count() * 8;
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * (size_t)blocks * kPeakThreads) != cudaSuccess) return RBG_ERR_NOMEM;
  cudaEvent_t e0, e1;
  int rc = RBG_OK;
  if (cudaEventCreate(&e0) != cudaSuccess) {
    cudaFree(out);
    return RBG_ERR_CUDA;
  }
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    cudaFree(out);
    return RBG_ERR_CUDA;
  }
  // a' = a * (1 - 2^-20) + 2^-21 stays near 0.5: no overflow or denormals
  const T a = (T)(1.0 - 1.0 / 1048576.0), b = (T)(1.0 / 2097152.0);
  float best = 0.f;
  for (int rep = 0; rep < 3 && rc == RBG_OK; ++rep) {
    float ms = 0.f;
    if (cudaEventRecord(e0, st) != cudaSuccess) rc = RBG_ERR_CUDA;
    fma_peak_kernel<T><<<blocks, kPeakThreads, 0, st>>>(iters, a, b, out);
    if (cudaGetLastError() != cudaSuccess || cudaEventRecord(e1, st) != cudaSuccess ||
        cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
      rc = RBG_ERR_CUDA;
    if (rc == RBG_OK && rep > 0 && (best == 0.f || ms < best)) best = ms;  // the first launch warms up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (rc != RBG_OK) return rc;
  const double fmas = (double)blocks * kPeakThreads * iters * 16.0 * kChains;
  *flops_per_s = best > 0.f ? 2.0 * fmas / (best * 1e-3) : 0.0;
  return RBG_OK;
}

}  // namespace rbg

extern "C" int rbg_measure_fma_peak(int32_t bits, double* flops_per_s, void* stream) {
  if (!flops_per_s) return RBG_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (bits == 64) return rbg::fma_rate<double>(512, flops_per_s, st);
  if (bits == 32) return rbg::fma_rate<float>(8192, flops_per_s, st);
  return RBG_ERR_ARG;
}

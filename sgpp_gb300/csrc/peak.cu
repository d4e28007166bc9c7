// Vector FMA throughput probe (roofline denominator for the FP32 / FP64 hat kernels).
#include <cuda_runtime.h>

#include <string>

#include "../../include/sgmev_tools.h"

namespace sgmev {
extern thread_local std::string g_last_error;
}

namespace {

constexpr int kChains = 8;

template <typename T>
__global__ void __launch_bounds__(256) fma_chain_kernel(T* sink, int iters, T a, T b) {
  T c[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) c[i] = static_cast<T>(threadIdx.x) * T(1e-3) + T(i);
  for (int k = 0; k < iters; ++k) {
#pragma unroll
    for (int i = 0; i < kChains; ++i) c[i] = fma(c[i], a, b);
  }
  T s = T(0);
#pragma unroll
  for (int i = 0; i < kChains; ++i) s += c[i];
  if (s == T(-1234.5)) sink[blockIdx.x] = s;  // keeps the chains alive; never true
}

template <typename T>
int measure(double* fps) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  T* sink = nullptr;
  if (cudaMalloc(&sink, sizeof(T) * 65536) != cudaSuccess) return SGMEV_ERR_OOM;
  const int blocks = sms * 8;
  const int threads = 256;
  const int iters = sizeof(T) == 4 ? 8192 : 512;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0);
    fma_chain_kernel<T><<<blocks, threads>>>(sink, iters, T(0.999999), T(1e-7));
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;  // first launch is a warm-up
  }
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (e != cudaSuccess) {
    sgmev::g_last_error = cudaGetErrorString(e);
    return SGMEV_ERR_CUDA;
  }
  const double flops = 2.0 * blocks * threads * static_cast<double>(iters) * kChains;
  *fps = flops / (best * 1e-3);
  return SGMEV_OK;
}

}  // namespace

extern "C" SGMEV_API int sgmev_fma_peak(int precision, double* flops_per_second,
                                        int* sm_clock_khz) {
  if (!flops_per_second) return SGMEV_ERR_INVALID;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    sgmev::g_last_error = "no CUDA device is visible";
    return SGMEV_ERR_NO_DEVICE;
  }
  if (sm_clock_khz) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(sm_clock_khz, cudaDevAttrClockRate, dev);
  }
  if (precision == SGMEV_FP32) return measure<float>(flops_per_second);
  if (precision == SGMEV_FP64) return measure<double>(flops_per_second);
  sgmev::g_last_error = "precision must be SGMEV_FP64 or SGMEV_FP32";
  return SGMEV_ERR_INVALID;
}

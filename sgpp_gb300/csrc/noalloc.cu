// B^T v for callers that must not allocate GPU memory (sgmev_mult_transpose_noalloc).
//
// Some callers cannot let a library call cudaMalloc: a host application whose own memory
// manager owns the device's memory budget and hands out every buffer itself, or a
// latency-critical loop in which the implicit device synchronisation of cudaMalloc / cudaFree
// is not acceptable. For them this entry point takes every input and output as a device
// pointer the caller already owns and keeps its only scratch — the per-split partial sums of
// the multTranspose tile kernel — in the fixed-size file-scope array below, which every GPU
// that loads this library holds until the process exits.
//
// The array is shared by all calls: two calls whose kernels overlap on the GPU (different
// streams, or different host threads) race on it and corrupt each other's results; callers
// serialise such calls. Each call writes every partial it later reads, so nothing needs
// clearing between calls.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "../../include/sgmev.h"
#include "kernels.cuh"

namespace sgmev {
extern thread_local std::string g_last_error;
}

namespace {

// 2^21 doubles = 16 MiB of partial sums: n_grid x splits <= 2^21 (so n_grid <= 2,097,152).
constexpr int64_t kScratchDoubles = int64_t(1) << 21;
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_ptr[kMaxDevices] = {nullptr};  // device address of the array, per device

constexpr int kBlock = 128;
constexpr int kRG = 2;   // grid points per thread
constexpr int kDT = 64;  // data points per shared-memory tile
constexpr int kMaxTemplDim = 16;
constexpr int kMaxDim = 64;

int fail(int code, const std::string& msg) {
  sgmev::g_last_error = msg;
  return code;
}

int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Same arithmetic as mult_transpose_kernel<double>, reading the reference's row-major layouts
// directly (level/index [n x DIM], data [m x DIM]) with bounds checks instead of padding.
template <int DIM>
__global__ void __launch_bounds__(kBlock) noalloc_multt_kernel(
    const double* __restrict__ level_pow2, const double* __restrict__ index, int64_t n,
    const double* __restrict__ data, const double* __restrict__ v, int64_t m, int64_t chunk,
    double* __restrict__ part) {
  __shared__ double s_x[kDT * DIM];  // row-major tile: contiguous in global memory
  __shared__ double s_v[kDT];
  const int64_t g0 = static_cast<int64_t>(blockIdx.x) * (kBlock * kRG) + threadIdx.x;
  double2 l[kRG][DIM];
#pragma unroll
  for (int k = 0; k < kRG; ++k) {
    const int64_t g = g0 + k * kBlock;
#pragma unroll
    for (int t = 0; t < DIM; ++t)
      l[k][t] = g < n ? make_double2(level_pow2[g * DIM + t], index[g * DIM + t])
                      : make_double2(0.0, 2.0);  // outside the grid: hat 0
  }
  double acc[kRG];
#pragma unroll
  for (int k = 0; k < kRG; ++k) acc[k] = 0.0;
  const int64_t j_begin = static_cast<int64_t>(blockIdx.y) * chunk;
  const int64_t j_end = std::min<int64_t>(j_begin + chunk, m);
  for (int64_t jt = j_begin; jt < j_end; jt += kDT) {
    const int cnt = static_cast<int>(std::min<int64_t>(kDT, j_end - jt));
    __syncthreads();
    for (int k = threadIdx.x; k < kDT * DIM; k += kBlock)
      s_x[k] = k < cnt * DIM ? data[jt * DIM + k] : 0.0;  // x = 0 gives hat 0
    for (int k = threadIdx.x; k < kDT; k += kBlock) s_v[k] = k < cnt ? v[jt + k] : 0.0;
    __syncthreads();
    for (int j = 0; j < cnt; ++j) {
      double p[kRG];
#pragma unroll
      for (int k = 0; k < kRG; ++k) p[k] = sgmev::hat_first(s_x[j * DIM], l[k][0]);
#pragma unroll
      for (int t = 1; t < DIM; ++t) {
        const double xv = s_x[j * DIM + t];
#pragma unroll
        for (int k = 0; k < kRG; ++k) p[k] = sgmev::hat_next(p[k], xv, l[k][t]);
      }
      const double vj = s_v[j];
#pragma unroll
      for (int k = 0; k < kRG; ++k) acc[k] = fma(vj, p[k], acc[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < kRG; ++k) {
    const int64_t g = g0 + k * kBlock;
    if (g < n) part[static_cast<int64_t>(blockIdx.y) * n + g] = acc[k];
  }
}

// dimensions above the templated range: one grid point per thread, coordinates from global
__global__ void noalloc_multt_generic_kernel(const double* __restrict__ level_pow2,
                                             const double* __restrict__ index, int64_t n, int dim,
                                             const double* __restrict__ data,
                                             const double* __restrict__ v, int64_t m,
                                             int64_t chunk, double* __restrict__ part) {
  const int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const int64_t j_begin = static_cast<int64_t>(blockIdx.y) * chunk;
  const int64_t j_end = std::min<int64_t>(j_begin + chunk, m);
  double acc = 0.0;
  for (int64_t j = j_begin; j < j_end; ++j) {
    double p = sgmev::hat_first(data[j * dim], make_double2(level_pow2[g * dim], index[g * dim]));
    for (int t = 1; t < dim; ++t)
      p = sgmev::hat_next(p, data[j * dim + t],
                          make_double2(level_pow2[g * dim + t], index[g * dim + t]));
    acc = fma(v[j], p, acc);
  }
  part[static_cast<int64_t>(blockIdx.y) * n + g] = acc;
}

// result[g] = sum over splits in a fixed order
__global__ void noalloc_reduce_kernel(const double* __restrict__ part, int nsplit, int64_t n,
                                      double* __restrict__ result) {
  for (int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; g < n;
       g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < nsplit; ++k) s += part[k * n + g];
    result[g] = s;
  }
}

// Once per device, with that device current: the device address of the scratch array. In host
// code `g_noalloc_scratch` names a host-side stand-in, never the device memory itself.
int scratch_for_current_device(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(SGMEV_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(SGMEV_ERR_UNSUPPORTED, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(SGMEV_ERR_CUDA, std::string("cudaGetSymbolAddress(no-alloc scratch): ") +
                                      cudaGetErrorString(e));
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return SGMEV_OK;
}

template <int DIM>
void launch_dim(dim3 grid, cudaStream_t s, const double* lp, const double* ix, int64_t n,
                const double* data, const double* v, int64_t m, int64_t chunk, double* part) {
  noalloc_multt_kernel<DIM><<<grid, kBlock, 0, s>>>(lp, ix, n, data, v, m, chunk, part);
}

}  // namespace

extern "C" SGMEV_API int sgmev_mult_transpose_noalloc(int dim, int64_t n_grid,
                                                      const double* d_level_pow2,
                                                      const double* d_index, int64_t n_data,
                                                      const double* d_data,
                                                      const double* d_source, double* d_result,
                                                      void* stream) {
  if (dim < 1 || dim > kMaxDim) return fail(SGMEV_ERR_INVALID, "dim must be in [1, 64]");
  if (n_grid < 0 || n_data < 0) return fail(SGMEV_ERR_INVALID, "negative size");
  if (n_grid > kScratchDoubles)
    return fail(SGMEV_ERR_INVALID,
                "n_grid = " + std::to_string(n_grid) + " exceeds the no-alloc scratch capacity of " +
                    std::to_string(kScratchDoubles) + " grid points");
  if (n_grid == 0) return SGMEV_OK;
  if (!d_level_pow2 || !d_index || !d_result || (n_data > 0 && (!d_data || !d_source)))
    return fail(SGMEV_ERR_INVALID, "NULL device pointer");
  // an error another component left pending on this thread is drained here, so that the checks
  // after the launches below report only this call's own failures
  (void)cudaGetLastError();
  double* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc != SGMEV_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int devnum = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&devnum);
  if (e != cudaSuccess) return fail(SGMEV_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, devnum);
  if (e != cudaSuccess || sms < 1)
    return fail(SGMEV_ERR_CUDA, std::string("cudaDeviceGetAttribute(multiprocessor count): ") +
                                    cudaGetErrorString(e));

  const bool templ = dim <= kMaxTemplDim;
  const int64_t tiles = templ ? ceil_div(n_grid, kBlock * kRG) : ceil_div(n_grid, kBlock);
  // splits of the data axis: fill >= 4 CTAs per SM, within the scratch capacity
  int64_t nsplit = ceil_div(4 * int64_t(sms), tiles);
  nsplit = std::min<int64_t>(nsplit, kScratchDoubles / n_grid);
  nsplit = std::min<int64_t>(nsplit, std::max<int64_t>(1, ceil_div(n_data, kDT)));
  nsplit = std::max<int64_t>(nsplit, 1);
  const int64_t chunk = std::max<int64_t>(kDT, ceil_div(ceil_div(n_data, nsplit), kDT) * kDT);
  nsplit = std::max<int64_t>(1, ceil_div(n_data, chunk));
  dim3 grid(static_cast<unsigned>(tiles), static_cast<unsigned>(nsplit));
  if (templ) {
    switch (dim) {
#define F(D)                                                                                  \
  case D:                                                                                     \
    launch_dim<D>(grid, s, d_level_pow2, d_index, n_grid, d_data, d_source, n_data, chunk,    \
                  scratch);                                                                   \
    break;
      F(1) F(2) F(3) F(4) F(5) F(6) F(7) F(8) F(9) F(10) F(11) F(12) F(13) F(14) F(15) F(16)
#undef F
      default:
        break;
    }
  } else {
    noalloc_multt_generic_kernel<<<grid, kBlock, 0, s>>>(d_level_pow2, d_index, n_grid, dim,
                                                          d_data, d_source, n_data, chunk,
                                                          scratch);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return fail(SGMEV_ERR_CUDA, std::string("no-alloc multTranspose launch: ") + cudaGetErrorString(e));
  const unsigned rblocks =
      static_cast<unsigned>(std::min<int64_t>(8 * int64_t(sms), ceil_div(n_grid, 256)));
  noalloc_reduce_kernel<<<rblocks, 256, 0, s>>>(scratch, static_cast<int>(nsplit), n_grid,
                                                d_result);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return fail(SGMEV_ERR_CUDA, std::string("no-alloc reduction launch: ") + cudaGetErrorString(e));
  return SGMEV_OK;
}

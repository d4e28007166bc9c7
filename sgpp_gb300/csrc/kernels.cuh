// Dense streaming kernels for the d-dimensional piecewise-linear hat basis (sm_103a).
//
// The algorithm is the reference's STREAMING one — every (grid point, data point) pair is
// evaluated as a product of d one-dimensional hats (OperationMultiEvalStreaming_multImpl.cpp:
// 577-623, _multTransposeImpl.cpp:485-510, hat from LinearBasis.hpp:37-41) — laid out for the GPU:
//
//   data  xt[t * mpad + j]          dim-major, zero-padded to mpad (a hat is 0 at x = 0)
//   grid  li[g * DIM + t] = (2^l, i) interleaved pairs, padded rows (0, 2) evaluate to 0
//   mult  CTA = (data tile of BLOCK*R points) x (grid chunk); each thread keeps R data points
//         in registers, grid pairs stream through shared memory as broadcast reads
//   multT CTA = (grid tile of BLOCK*RG points) x (data chunk); each thread keeps RG grid points'
//         pairs in registers, data tiles stream through shared memory
// Each CTA writes its partial sums to part[split][...]; reduce_splits() adds the splits in a
// fixed order, so results are bitwise reproducible (no atomics).
//
// Per (pair, dim) the FP32 hat costs three FMA-pipe instructions:
//   t = fma(x, 2^l, -i);  h = sat(1 - |t|);  p *= h
// (the clamp max(., 0) folds into the saturating add because 1 - |t| <= 1).
// FP64 has no saturating add, so the update is written p = fma(-p, min(|t|, 1), p), which
// equals p * max(1 - |t|, 0) up to one rounding.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sgmev {

template <typename T>
struct Pair;
template <>
struct Pair<float> {
  using type = float2;
};
template <>
struct Pair<double> {
  using type = double2;
};

__device__ __forceinline__ float hat_first(float x, float2 li) {
  return __saturatef(1.0f - fabsf(fmaf(x, li.x, -li.y)));
}
__device__ __forceinline__ float hat_next(float p, float x, float2 li) {
  return p * __saturatef(1.0f - fabsf(fmaf(x, li.x, -li.y)));
}
__device__ __forceinline__ double hat_first(double x, double2 li) {
  return fmax(1.0 - fabs(fma(x, li.x, -li.y)), 0.0);
}
__device__ __forceinline__ double hat_next(double p, double x, double2 li) {
  const double u = fmin(fabs(fma(x, li.x, -li.y)), 1.0);
  return fma(-p, u, p);
}

// ---------------------------------------------------------------------------------------
// mult: part[split][j] = sum_{g in chunk(split)} alpha_g prod_t hat(x_jt; l_gt, i_gt)
// grid: (data tiles) x (grid chunks). chunk_len is a multiple of GT.
// ---------------------------------------------------------------------------------------
template <typename T, int DIM, int R, int BLOCK, int GT>
__global__ void __launch_bounds__(BLOCK) mult_kernel(const T* __restrict__ xt, int64_t mpad,
                                                     const typename Pair<T>::type* __restrict__ li,
                                                     const T* __restrict__ alpha, int64_t npad,
                                                     int64_t chunk_len, int64_t tile_offset,
                                                     T* __restrict__ part) {
  using T2 = typename Pair<T>::type;
  __shared__ T2 s_li[GT * DIM];
  __shared__ T s_a[GT];

  const int64_t tile = static_cast<int64_t>(blockIdx.x) + tile_offset;
  const int64_t j0 = tile * (BLOCK * R) + threadIdx.x;

  T x[R][DIM];
#pragma unroll
  for (int r = 0; r < R; ++r) {
#pragma unroll
    for (int t = 0; t < DIM; ++t) x[r][t] = xt[static_cast<int64_t>(t) * mpad + j0 + r * BLOCK];
  }
  T acc[R];
#pragma unroll
  for (int r = 0; r < R; ++r) acc[r] = T(0);

  const int64_t g_begin = static_cast<int64_t>(blockIdx.y) * chunk_len;
  int64_t g_end = g_begin + chunk_len;
  if (g_end > npad) g_end = npad;

  for (int64_t g0 = g_begin; g0 < g_end; g0 += GT) {
    __syncthreads();
    for (int k = threadIdx.x; k < GT * DIM; k += BLOCK) s_li[k] = li[g0 * DIM + k];
    for (int k = threadIdx.x; k < GT; k += BLOCK) s_a[k] = alpha[g0 + k];
    __syncthreads();
#pragma unroll 2
    for (int g = 0; g < GT; ++g) {
      T p[R];
      const T2 l0 = s_li[g * DIM];
#pragma unroll
      for (int r = 0; r < R; ++r) p[r] = hat_first(x[r][0], l0);
#pragma unroll
      for (int t = 1; t < DIM; ++t) {
        const T2 lt = s_li[g * DIM + t];
#pragma unroll
        for (int r = 0; r < R; ++r) p[r] = hat_next(p[r], x[r][t], lt);
      }
      const T a = s_a[g];
#pragma unroll
      for (int r = 0; r < R; ++r) acc[r] = fma(a, p[r], acc[r]);
    }
  }
  T* out = part + static_cast<int64_t>(blockIdx.y) * mpad;
#pragma unroll
  for (int r = 0; r < R; ++r) out[j0 + r * BLOCK] = acc[r];
}

// ---------------------------------------------------------------------------------------
// multT: part[split][g] = sum_{j in chunk(split)} v_j prod_t hat(x_jt; l_gt, i_gt)
// grid: (grid tiles of BLOCK*RG points) x (data chunks). chunk_len is a multiple of DT.
// ---------------------------------------------------------------------------------------
template <typename T, int DIM, int RG, int BLOCK, int DT>
__global__ void __launch_bounds__(BLOCK) mult_transpose_kernel(
    const T* __restrict__ xt, const T* __restrict__ v, int64_t mpad,
    const typename Pair<T>::type* __restrict__ li, int64_t npad, int64_t chunk_len,
    int64_t tile_offset, T* __restrict__ part) {
  using T2 = typename Pair<T>::type;
  __shared__ T s_x[DIM * DT];
  __shared__ T s_v[DT];

  const int64_t tile = static_cast<int64_t>(blockIdx.x) + tile_offset;
  const int64_t g0 = tile * (BLOCK * RG) + threadIdx.x;

  T2 l[RG][DIM];
#pragma unroll
  for (int k = 0; k < RG; ++k) {
#pragma unroll
    for (int t = 0; t < DIM; ++t) l[k][t] = li[(g0 + k * BLOCK) * DIM + t];
  }
  T acc[RG];
#pragma unroll
  for (int k = 0; k < RG; ++k) acc[k] = T(0);

  const int64_t j_begin = static_cast<int64_t>(blockIdx.y) * chunk_len;
  int64_t j_end = j_begin + chunk_len;
  if (j_end > mpad) j_end = mpad;

  for (int64_t jt = j_begin; jt < j_end; jt += DT) {
    __syncthreads();
#pragma unroll
    for (int t = 0; t < DIM; ++t) {
      for (int k = threadIdx.x; k < DT; k += BLOCK)
        s_x[t * DT + k] = xt[static_cast<int64_t>(t) * mpad + jt + k];
    }
    for (int k = threadIdx.x; k < DT; k += BLOCK) s_v[k] = v[jt + k];
    __syncthreads();
#pragma unroll 2
    for (int j = 0; j < DT; ++j) {
      T p[RG];
      const T x0 = s_x[j];
#pragma unroll
      for (int k = 0; k < RG; ++k) p[k] = hat_first(x0, l[k][0]);
#pragma unroll
      for (int t = 1; t < DIM; ++t) {
        const T xv = s_x[t * DT + j];
#pragma unroll
        for (int k = 0; k < RG; ++k) p[k] = hat_next(p[k], xv, l[k][t]);
      }
      const T vj = s_v[j];
#pragma unroll
      for (int k = 0; k < RG; ++k) acc[k] = fma(vj, p[k], acc[k]);
    }
  }
  T* out = part + static_cast<int64_t>(blockIdx.y) * npad;
#pragma unroll
  for (int k = 0; k < RG; ++k) out[g0 + k * BLOCK] = acc[k];
}

// ---------------------------------------------------------------------------------------
// Generic-dimension fallbacks (dim not instantiated above): one data point (mult) or one grid
// point (multT) per thread, coordinates re-read from global/L1. Correctness path for large d.
// ---------------------------------------------------------------------------------------
template <typename T>
__global__ void mult_generic_kernel(const T* __restrict__ xt, int64_t mpad, int dim,
                                    const typename Pair<T>::type* __restrict__ li,
                                    const T* __restrict__ alpha, int64_t npad, int64_t chunk_len,
                                    int64_t j_offset, int64_t j_count, T* __restrict__ part) {
  const int64_t j = j_offset + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= j_offset + j_count) return;
  const int64_t g_begin = static_cast<int64_t>(blockIdx.y) * chunk_len;
  int64_t g_end = g_begin + chunk_len;
  if (g_end > npad) g_end = npad;
  T acc = T(0);
  for (int64_t g = g_begin; g < g_end; ++g) {
    T p = hat_first(xt[j], li[g * dim]);
    for (int t = 1; t < dim; ++t) p = hat_next(p, xt[static_cast<int64_t>(t) * mpad + j], li[g * dim + t]);
    acc = fma(alpha[g], p, acc);
  }
  part[static_cast<int64_t>(blockIdx.y) * mpad + j] = acc;
}

template <typename T>
__global__ void mult_transpose_generic_kernel(const T* __restrict__ xt, const T* __restrict__ v,
                                              int64_t mpad, int dim,
                                              const typename Pair<T>::type* __restrict__ li,
                                              int64_t npad, int64_t chunk_len, int64_t g_offset,
                                              int64_t g_count, T* __restrict__ part) {
  const int64_t g = g_offset + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (g >= g_offset + g_count) return;
  const int64_t j_begin = static_cast<int64_t>(blockIdx.y) * chunk_len;
  int64_t j_end = j_begin + chunk_len;
  if (j_end > mpad) j_end = mpad;
  T acc = T(0);
  for (int64_t j = j_begin; j < j_end; ++j) {
    T p = hat_first(xt[j], li[g * dim]);
    for (int t = 1; t < dim; ++t) p = hat_next(p, xt[static_cast<int64_t>(t) * mpad + j], li[g * dim + t]);
    acc = fma(v[j], p, acc);
  }
  part[static_cast<int64_t>(blockIdx.y) * npad + g] = acc;
}

// ---------------------------------------------------------------------------------------
// Fixed-order reduction over splits: out[i] = sum_s part[s*stride + i] (+ scale * add[i]),
// accumulated in double. Indices in [n_valid, n_total) are written as zero (padding).
// ---------------------------------------------------------------------------------------
template <typename TP, typename TO>
__global__ void reduce_splits_kernel(const TP* __restrict__ part, int nsplit, int64_t stride,
                                     int64_t begin, int64_t n_valid, int64_t n_total,
                                     TO* __restrict__ out, const double* __restrict__ add,
                                     double scale) {
  for (int64_t i = begin + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
       i < n_total; i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double s = 0.0;
    if (i < n_valid) {
      for (int k = 0; k < nsplit; ++k) s += static_cast<double>(part[k * stride + i]);
      if (add) s = fma(scale, add[i], s);
    }
    out[i] = static_cast<TO>(s);
  }
}

// ---------------------------------------------------------------------------------------
// Staging and vector kernels
// ---------------------------------------------------------------------------------------
// rows [m x dim] row-major doubles -> dim-major, optional bounding box map, zero padding
__global__ void stage_data_kernel(const double* __restrict__ rows, int64_t m, int dim,
                                  int64_t mpad, const double* __restrict__ bb_left,
                                  const double* __restrict__ bb_width, double* __restrict__ xt64,
                                  float* __restrict__ xt32);

// (2^l, i) row-major doubles -> interleaved pairs, padded rows (0, 2)
__global__ void stage_grid_kernel(const double* __restrict__ level_pow2,
                                  const double* __restrict__ index, int64_t n, int dim,
                                  int64_t npad, double2* __restrict__ li64,
                                  float2* __restrict__ li32);

__global__ void convert_pad_kernel(const double* __restrict__ in, int64_t n, int64_t npad,
                                   double* __restrict__ out64, float* __restrict__ out32);

}  // namespace sgmev

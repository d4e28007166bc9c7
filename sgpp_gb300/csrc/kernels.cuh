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
//
// The modified linear basis of ModLinear grids (MOD = true; LinearModifiedBasis.hpp:40-58, as
// streamed by OperationMultiEvalModMaskStreaming_multImpl.cpp:83-122) uses the same kernels with
// a pair (L', c') per (grid point, dimension) and a factor 2^b per grid point (b = number of
// its boundary-adjacent dimensions, level >= 2 and i = 1 or 2^l - 1):
//   l = 1           (0, +0)                 h = 1
//   i = 1           (2^{l-1}, -0)           h = 2 (1 - 2^{l-1} x)            = 2 - 2^l x
//   i = 2^l - 1     (-2^{l-1}, -2^{l-1})    h = 2 (1 - 2^{l-1} (1 - x))      = 2^l x - i + 1
//   otherwise       (2^l, i)                h = max(1 - |2^l x - i|, 0)
// t = fma(x, L', -c'); a set sign bit of c' marks a boundary-adjacent function, which takes t
// itself instead of |t| (one bitwise and), so it extrapolates linearly beyond the cube's faces
// as the reference's mask evaluation does; the clamp at 0 stays. The factors 2^b are exact and
// are folded into alpha (mult) and into the sums (multT) inside the kernels.
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
// squared hats (diagonal of B^T B): p = prod_t hat_t^2
__device__ __forceinline__ float hat_first_sq(float x, float2 li) {
  const float h = hat_first(x, li);
  return h * h;
}
__device__ __forceinline__ float hat_next_sq(float p, float x, float2 li) {
  const float h = __saturatef(1.0f - fabsf(fmaf(x, li.x, -li.y)));
  return p * (h * h);
}
__device__ __forceinline__ double hat_first(double x, double2 li) {
  return fmax(1.0 - fabs(fma(x, li.x, -li.y)), 0.0);
}
__device__ __forceinline__ double hat_next(double p, double x, double2 li) {
  const double u = fmin(fabs(fma(x, li.x, -li.y)), 1.0);
  return fma(-p, u, p);
}

// ModLinear factors (MOD = true): d = |t| for interior functions, t for boundary-adjacent ones
__device__ __forceinline__ float mod_dist(float x, float2 li) {
  const float t = fmaf(x, li.x, -li.y);
  return __uint_as_float(__float_as_uint(t) & (__float_as_uint(li.y) | 0x7FFFFFFFu));
}
__device__ __forceinline__ double mod_dist(double x, double2 li) {
  const double t = fma(x, li.x, -li.y);
  const int hi = __double2hiint(t) & (__double2hiint(li.y) | 0x7FFFFFFF);
  return __hiloint2double(hi, __double2loint(t));
}
template <typename T, typename T2>
__device__ __forceinline__ T hat_first_mod(T x, T2 li) {
  return fmax(T(1) - mod_dist(x, li), T(0));
}
template <typename T, typename T2>
__device__ __forceinline__ T hat_next_mod(T p, T x, T2 li) {
  return fma(-p, fmin(mod_dist(x, li), T(1)), p);
}

// basis dispatch
template <bool MOD, typename T, typename T2>
__device__ __forceinline__ T h_first(T x, T2 li) {
  if constexpr (MOD) return hat_first_mod(x, li);
  else return hat_first(x, li);
}
template <bool MOD, typename T, typename T2>
__device__ __forceinline__ T h_next(T p, T x, T2 li) {
  if constexpr (MOD) return hat_next_mod(p, x, li);
  else return hat_next(p, x, li);
}
template <bool MOD, typename T, typename T2>
__device__ __forceinline__ T h_first_sq(T x, T2 li) {
  if constexpr (MOD) {
    const T h = hat_first_mod(x, li);
    return h * h;
  } else {
    return hat_first_sq(x, li);
  }
}
template <bool MOD, typename T, typename T2>
__device__ __forceinline__ T h_next_sq(T p, T x, T2 li) {
  if constexpr (MOD) {
    const T h = hat_first_mod(x, li);
    return p * (h * h);
  } else {
    return hat_next_sq(p, x, li);
  }
}

// ---------------------------------------------------------------------------------------
// mult: part[split][j] = sum_{g in chunk(split)} alpha_g prod_t hat(x_jt; l_gt, i_gt)
// grid: (data tiles) x (grid chunks). chunk_len is a multiple of GT.
// ---------------------------------------------------------------------------------------
template <typename T, int DIM, int R, int BLOCK, int GT, bool MOD = false>
__global__ void __launch_bounds__(BLOCK) mult_kernel(const T* __restrict__ xt, int64_t mpad,
                                                     const typename Pair<T>::type* __restrict__ li,
                                                     const T* __restrict__ alpha, int64_t npad,
                                                     int64_t chunk_len, int64_t tile_offset,
                                                     T* __restrict__ part,
                                                     const T* __restrict__ gscale = nullptr) {
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
    for (int k = threadIdx.x; k < GT; k += BLOCK)
      s_a[k] = MOD ? alpha[g0 + k] * gscale[g0 + k] : alpha[g0 + k];
    __syncthreads();
#pragma unroll 2
    for (int g = 0; g < GT; ++g) {
      T p[R];
      const T2 l0 = s_li[g * DIM];
#pragma unroll
      for (int r = 0; r < R; ++r) p[r] = h_first<MOD>(x[r][0], l0);
#pragma unroll
      for (int t = 1; t < DIM; ++t) {
        const T2 lt = s_li[g * DIM + t];
#pragma unroll
        for (int r = 0; r < R; ++r) p[r] = h_next<MOD>(p[r], x[r][t], lt);
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
template <typename T, int DIM, int RG, int BLOCK, int DT, bool SQ = false, bool MOD = false>
__global__ void __launch_bounds__(BLOCK) mult_transpose_kernel(
    const T* __restrict__ xt, const T* __restrict__ v, int64_t mpad,
    const typename Pair<T>::type* __restrict__ li, int64_t npad, int64_t chunk_len,
    int64_t tile_offset, T* __restrict__ part, const T* __restrict__ gscale = nullptr) {
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
      for (int k = 0; k < RG; ++k) {
        if constexpr (SQ) p[k] = h_first_sq<MOD>(x0, l[k][0]);
        else p[k] = h_first<MOD>(x0, l[k][0]);
      }
#pragma unroll
      for (int t = 1; t < DIM; ++t) {
        const T xv = s_x[t * DT + j];
#pragma unroll
        for (int k = 0; k < RG; ++k) {
          if constexpr (SQ) p[k] = h_next_sq<MOD>(p[k], xv, l[k][t]);
          else p[k] = h_next<MOD>(p[k], xv, l[k][t]);
        }
      }
      const T vj = s_v[j];
#pragma unroll
      for (int k = 0; k < RG; ++k) acc[k] = fma(vj, p[k], acc[k]);
    }
  }
  T* out = part + static_cast<int64_t>(blockIdx.y) * npad;
#pragma unroll
  for (int k = 0; k < RG; ++k) {
    if constexpr (MOD) {
      const T sc = gscale[g0 + k * BLOCK];
      out[g0 + k * BLOCK] = acc[k] * (SQ ? sc * sc : sc);
    } else {
      out[g0 + k * BLOCK] = acc[k];
    }
  }
}

// ---------------------------------------------------------------------------------------
// Generic-dimension fallbacks (dim not instantiated above): one data point (mult) or one grid
// point (multT) per thread, coordinates re-read from global/L1. Correctness path for large d.
// ---------------------------------------------------------------------------------------
template <typename T, bool MOD = false>
__global__ void mult_generic_kernel(const T* __restrict__ xt, int64_t mpad, int dim,
                                    const typename Pair<T>::type* __restrict__ li,
                                    const T* __restrict__ alpha, int64_t npad, int64_t chunk_len,
                                    int64_t j_offset, int64_t j_count, T* __restrict__ part,
                                    const T* __restrict__ gscale = nullptr) {
  const int64_t j = j_offset + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= j_offset + j_count) return;
  const int64_t g_begin = static_cast<int64_t>(blockIdx.y) * chunk_len;
  int64_t g_end = g_begin + chunk_len;
  if (g_end > npad) g_end = npad;
  T acc = T(0);
  for (int64_t g = g_begin; g < g_end; ++g) {
    T p = h_first<MOD>(xt[j], li[g * dim]);
    for (int t = 1; t < dim; ++t)
      p = h_next<MOD>(p, xt[static_cast<int64_t>(t) * mpad + j], li[g * dim + t]);
    acc = fma(MOD ? alpha[g] * gscale[g] : alpha[g], p, acc);
  }
  part[static_cast<int64_t>(blockIdx.y) * mpad + j] = acc;
}

template <typename T, bool SQ = false, bool MOD = false>
__global__ void mult_transpose_generic_kernel(const T* __restrict__ xt, const T* __restrict__ v,
                                              int64_t mpad, int dim,
                                              const typename Pair<T>::type* __restrict__ li,
                                              int64_t npad, int64_t chunk_len, int64_t g_offset,
                                              int64_t g_count, T* __restrict__ part,
                                              const T* __restrict__ gscale = nullptr) {
  const int64_t g = g_offset + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (g >= g_offset + g_count) return;
  const int64_t j_begin = static_cast<int64_t>(blockIdx.y) * chunk_len;
  int64_t j_end = j_begin + chunk_len;
  if (j_end > mpad) j_end = mpad;
  T acc = T(0);
  for (int64_t j = j_begin; j < j_end; ++j) {
    T p = h_first<MOD>(xt[j], li[g * dim]);
    if (SQ) p = p * p;
    for (int t = 1; t < dim; ++t) {
      const T h = h_first<MOD>(xt[static_cast<int64_t>(t) * mpad + j], li[g * dim + t]);
      p = p * (SQ ? h * h : h);
    }
    acc = fma(v[j], p, acc);
  }
  if constexpr (MOD) acc *= SQ ? gscale[g] * gscale[g] : gscale[g];
  part[static_cast<int64_t>(blockIdx.y) * npad + g] = acc;
}

// ---------------------------------------------------------------------------------------
// df64: FP64-accurate products on the FP32 pipes (float-float arithmetic).
//
// A data coordinate is the pair x = xh + xl (xh = float(x), xl = float(x - xh)); a grid point
// per dimension is the float4 (L, A, B, 0) = (2^l, 1 - i, 1 + i, 0), all exact in FP32 for
// l, log2(i) < 24. The hat is
//     h(x) = max(0, min(L x + A, B - L x))
// and within the support both branch values at xh, a = fma(xh, L, A) and b = fma(xh, -L, B),
// are exact FP32 numbers (Sterbenz's lemma: L xh lies within a factor two of i - 1, i or i + 1,
// and L xh itself is exact because L is a power of two). The low part of x moves the rising
// branch by +L xl and the falling one by -L xl, again exactly. The branch is chosen on the
// sign of (a - b) + 2 L xl (a - b is exact near the kink) and the clamp on the sign of the pair
// sum, so every one-dimensional hat is an exact float-float pair (hh, hl). Products use
// Dekker's two-product via FMA (Dekker 1971: p = a*b, e = fma(a, b, -p)); sums use Knuth's
// two-sum (Knuth, TAOCP vol. 2, 4.2.2). The relative error of one pair-product is ~2^-47, far
// below the 1e-12 parity bound.
// ---------------------------------------------------------------------------------------
struct ff {
  float h, l;
};

__device__ __forceinline__ ff hat_ff(float xh, float xl, float4 g) {
  const float a = fmaf(xh, g.x, g.y);
  const float b = fmaf(xh, -g.x, g.z);
  const float s = g.x * xl;
  const float c = fmaf(2.0f, s, a - b);
  const bool rise = c <= 0.0f;
  const float h = rise ? a : b;
  const float lo = rise ? s : -s;
  const bool pos = (h + lo) > 0.0f;
  return ff{pos ? h : 0.0f, pos ? lo : 0.0f};
}

// ModLinear grid constants (MOD = true) in the scaled form of the file header, as (L', A, B, 0)
// with h = max(0, min(L' x + A, B - L' x)) and a factor 2^b per grid point:
//   l = 1 (0, 1, 1);  i = 1 (2^{l-1}, kModOpen, 1);  i = 2^l - 1 (2^{l-1}, 1 - 2^{l-1}, kModOpen);
//   otherwise as the hat (2^l, 1 - i, 1 + i).
// kModOpen leaves one branch unbounded, so a boundary-adjacent function extrapolates beyond the
// cube's faces. Its value next to the face (1 - 2^{l-1} x near x = 0) is no longer an exact FP32
// number, so the branch value's rounding error is recovered with Knuth's two-sum (TAOCP vol. 2,
// 4.2.2) and carried in the low part: every factor stays an exact float-float pair up to one
// rounding of the low part.
constexpr float kModOpen = 18446744073709551616.0f;  // 2^64

__device__ __forceinline__ ff hat_ff_mod(float xh, float xl, float4 g) {
  const float y = xh * g.x;  // exact: g.x is 0 or a power of two
  const float a = y + g.y;
  const float b = g.z - y;
  const float s = g.x * xl;
  const bool rise = fmaf(2.0f, s, a - b) <= 0.0f;
  const float P = rise ? y : -y, Q = rise ? g.y : g.z;
  const float h = rise ? a : b;  // fl(P + Q)
  const float bb = h - P;
  const float err = (P - (h - bb)) + (Q - bb);  // P + Q = h + err exactly
  const float lo = err + (rise ? s : -s);
  const bool pos = (h + lo) > 0.0f;
  return ff{pos ? h : 0.0f, pos ? lo : 0.0f};
}

template <bool MOD>
__device__ __forceinline__ ff h_ff(float xh, float xl, float4 g) {
  if constexpr (MOD) return hat_ff_mod(xh, xl, g);
  else return hat_ff(xh, xl, g);
}

// (p.h + p.l) * (q.h + q.l), unnormalised; the l*l term is below the working precision
__device__ __forceinline__ ff mul_ff(ff p, ff q) {
  const float nh = p.h * q.h;
  const float e = fmaf(p.h, q.h, -nh);
  return ff{nh, fmaf(p.h, q.l, fmaf(p.l, q.h, e))};
}

// acc += q (two-sum on the high parts, low parts added)
__device__ __forceinline__ void add_ff(ff& acc, ff q) {
  const float s = acc.h + q.h;
  const float bb = s - acc.h;
  const float err = (acc.h - (s - bb)) + (q.h - bb);
  acc.l = acc.l + (q.l + err);
  acc.h = s;
}

// fast two-sum renormalisation (|acc.h| >= |acc.l| or acc.h == 0)
__device__ __forceinline__ void renorm_ff(ff& acc) {
  const float t = acc.h + acc.l;
  acc.l = acc.l - (t - acc.h);
  acc.h = t;
}

// mult in df64: part[split][j] = (hi, lo) of sum_{g in chunk} alpha_g prod_t hat(x_jt)
template <int DIM, int R, int BLOCK, int GT, bool MOD = false>
__global__ void __launch_bounds__(BLOCK) mult_df_kernel(
    const float* __restrict__ xh_t, const float* __restrict__ xl_t, int64_t mpad,
    const float4* __restrict__ gq, const float* __restrict__ ah_v, const float* __restrict__ al_v,
    int64_t npad, int64_t chunk_len, int64_t tile_offset, float2* __restrict__ part,
    const float* __restrict__ gscale = nullptr) {
  __shared__ float4 s_g[GT * DIM];
  __shared__ float2 s_a[GT];
  const int64_t tile = static_cast<int64_t>(blockIdx.x) + tile_offset;
  const int64_t j0 = tile * (BLOCK * R) + threadIdx.x;
  float xh[R][DIM], xl[R][DIM];
#pragma unroll
  for (int r = 0; r < R; ++r) {
#pragma unroll
    for (int t = 0; t < DIM; ++t) {
      xh[r][t] = xh_t[static_cast<int64_t>(t) * mpad + j0 + r * BLOCK];
      xl[r][t] = xl_t[static_cast<int64_t>(t) * mpad + j0 + r * BLOCK];
    }
  }
  ff acc[R];
#pragma unroll
  for (int r = 0; r < R; ++r) acc[r] = ff{0.0f, 0.0f};
  const int64_t g_begin = static_cast<int64_t>(blockIdx.y) * chunk_len;
  int64_t g_end = g_begin + chunk_len;
  if (g_end > npad) g_end = npad;
  for (int64_t g0 = g_begin; g0 < g_end; g0 += GT) {
    __syncthreads();
    for (int k = threadIdx.x; k < GT * DIM; k += BLOCK) s_g[k] = gq[g0 * DIM + k];
    for (int k = threadIdx.x; k < GT; k += BLOCK) {
      const float sc = MOD ? gscale[g0 + k] : 1.0f;
      s_a[k] = make_float2(ah_v[g0 + k] * sc, al_v[g0 + k] * sc);
    }
    __syncthreads();
    for (int g = 0; g < GT; ++g) {
      ff p[R];
      const float4 q0 = s_g[g * DIM];
#pragma unroll
      for (int r = 0; r < R; ++r) p[r] = h_ff<MOD>(xh[r][0], xl[r][0], q0);
#pragma unroll
      for (int t = 1; t < DIM; ++t) {
        const float4 qt = s_g[g * DIM + t];
#pragma unroll
        for (int r = 0; r < R; ++r) p[r] = mul_ff(p[r], h_ff<MOD>(xh[r][t], xl[r][t], qt));
      }
      const float2 a = s_a[g];
#pragma unroll
      for (int r = 0; r < R; ++r) add_ff(acc[r], mul_ff(p[r], ff{a.x, a.y}));
    }
#pragma unroll
    for (int r = 0; r < R; ++r) renorm_ff(acc[r]);
  }
  float2* out = part + static_cast<int64_t>(blockIdx.y) * mpad;
#pragma unroll
  for (int r = 0; r < R; ++r) out[j0 + r * BLOCK] = make_float2(acc[r].h, acc[r].l);
}

// multT in df64: part[split][g] = (hi, lo) of sum_{j in chunk} v_j prod_t hat(x_jt)
template <int DIM, int RG, int BLOCK, int DT, bool MOD = false>
__global__ void __launch_bounds__(BLOCK) mult_transpose_df_kernel(
    const float* __restrict__ xh_t, const float* __restrict__ xl_t, const float* __restrict__ vh,
    const float* __restrict__ vl, int64_t mpad, const float4* __restrict__ gq, int64_t npad,
    int64_t chunk_len, int64_t tile_offset, float2* __restrict__ part,
    const float* __restrict__ gscale = nullptr) {
  __shared__ float2 s_x[DIM * DT];
  __shared__ float2 s_v[DT];
  const int64_t tile = static_cast<int64_t>(blockIdx.x) + tile_offset;
  const int64_t g0 = tile * (BLOCK * RG) + threadIdx.x;
  float4 q[RG][DIM];
#pragma unroll
  for (int k = 0; k < RG; ++k) {
#pragma unroll
    for (int t = 0; t < DIM; ++t) q[k][t] = gq[(g0 + k * BLOCK) * DIM + t];
  }
  ff acc[RG];
#pragma unroll
  for (int k = 0; k < RG; ++k) acc[k] = ff{0.0f, 0.0f};
  const int64_t j_begin = static_cast<int64_t>(blockIdx.y) * chunk_len;
  int64_t j_end = j_begin + chunk_len;
  if (j_end > mpad) j_end = mpad;
  for (int64_t jt = j_begin; jt < j_end; jt += DT) {
    __syncthreads();
#pragma unroll
    for (int t = 0; t < DIM; ++t) {
      for (int k = threadIdx.x; k < DT; k += BLOCK) {
        const int64_t src = static_cast<int64_t>(t) * mpad + jt + k;
        s_x[t * DT + k] = make_float2(xh_t[src], xl_t[src]);
      }
    }
    for (int k = threadIdx.x; k < DT; k += BLOCK) s_v[k] = make_float2(vh[jt + k], vl[jt + k]);
    __syncthreads();
    for (int j = 0; j < DT; ++j) {
      ff p[RG];
      const float2 x0 = s_x[j];
#pragma unroll
      for (int k = 0; k < RG; ++k) p[k] = h_ff<MOD>(x0.x, x0.y, q[k][0]);
#pragma unroll
      for (int t = 1; t < DIM; ++t) {
        const float2 xv = s_x[t * DT + j];
#pragma unroll
        for (int k = 0; k < RG; ++k) p[k] = mul_ff(p[k], h_ff<MOD>(xv.x, xv.y, q[k][t]));
      }
      const float2 vj = s_v[j];
#pragma unroll
      for (int k = 0; k < RG; ++k) add_ff(acc[k], mul_ff(p[k], ff{vj.x, vj.y}));
    }
#pragma unroll
    for (int k = 0; k < RG; ++k) renorm_ff(acc[k]);
  }
  float2* out = part + static_cast<int64_t>(blockIdx.y) * npad;
#pragma unroll
  for (int k = 0; k < RG; ++k) {
    const float sc = MOD ? gscale[g0 + k * BLOCK] : 1.0f;
    out[g0 + k * BLOCK] = make_float2(acc[k].h * sc, acc[k].l * sc);
  }
}

// generic-dimension df64 fallbacks (one point per thread, coordinates from global/L1)
template <bool MOD = false>
__global__ void mult_df_generic_kernel(const float* __restrict__ xh_t, const float* __restrict__ xl_t,
                                       int64_t mpad, int dim, const float4* __restrict__ gq,
                                       const float* __restrict__ ah_v, const float* __restrict__ al_v,
                                       int64_t npad, int64_t chunk_len, int64_t j_offset,
                                       int64_t j_count, float2* __restrict__ part,
                                       const float* __restrict__ gscale = nullptr) {
  const int64_t j = j_offset + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= j_offset + j_count) return;
  const int64_t g_begin = static_cast<int64_t>(blockIdx.y) * chunk_len;
  int64_t g_end = g_begin + chunk_len;
  if (g_end > npad) g_end = npad;
  ff acc{0.0f, 0.0f};
  for (int64_t g = g_begin; g < g_end; ++g) {
    ff p = h_ff<MOD>(xh_t[j], xl_t[j], gq[g * dim]);
    for (int t = 1; t < dim; ++t) {
      const int64_t src = static_cast<int64_t>(t) * mpad + j;
      p = mul_ff(p, h_ff<MOD>(xh_t[src], xl_t[src], gq[g * dim + t]));
    }
    const float sc = MOD ? gscale[g] : 1.0f;
    add_ff(acc, mul_ff(p, ff{ah_v[g] * sc, al_v[g] * sc}));
    if ((g & 31) == 31) renorm_ff(acc);
  }
  renorm_ff(acc);
  part[static_cast<int64_t>(blockIdx.y) * mpad + j] = make_float2(acc.h, acc.l);
}

template <bool MOD = false>
__global__ void mult_transpose_df_generic_kernel(const float* __restrict__ xh_t,
                                                 const float* __restrict__ xl_t,
                                                 const float* __restrict__ vh,
                                                 const float* __restrict__ vl, int64_t mpad, int dim,
                                                 const float4* __restrict__ gq, int64_t npad,
                                                 int64_t chunk_len, int64_t g_offset,
                                                 int64_t g_count, float2* __restrict__ part,
                                                 const float* __restrict__ gscale = nullptr) {
  const int64_t g = g_offset + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (g >= g_offset + g_count) return;
  const int64_t j_begin = static_cast<int64_t>(blockIdx.y) * chunk_len;
  int64_t j_end = j_begin + chunk_len;
  if (j_end > mpad) j_end = mpad;
  ff acc{0.0f, 0.0f};
  for (int64_t j = j_begin; j < j_end; ++j) {
    ff p = h_ff<MOD>(xh_t[j], xl_t[j], gq[g * dim]);
    for (int t = 1; t < dim; ++t) {
      const int64_t src = static_cast<int64_t>(t) * mpad + j;
      p = mul_ff(p, h_ff<MOD>(xh_t[src], xl_t[src], gq[g * dim + t]));
    }
    add_ff(acc, mul_ff(p, ff{vh[j], vl[j]}));
    if ((j & 31) == 31) renorm_ff(acc);
  }
  renorm_ff(acc);
  const float sc = MOD ? gscale[g] : 1.0f;
  part[static_cast<int64_t>(blockIdx.y) * npad + g] = make_float2(acc.h * sc, acc.l * sc);
}

// ---------------------------------------------------------------------------------------
// Fixed-order reduction over splits: out[i] = sum_s part[s*stride + i] (+ scale * add[i]),
// accumulated in double. Indices in [n_valid, n_total) are written as zero (padding).
// ---------------------------------------------------------------------------------------
// float-float partials: value = hi + lo, accumulated in double
template <typename TP>
__device__ __forceinline__ double part_value(TP v) {
  return static_cast<double>(v);
}
template <>
__device__ __forceinline__ double part_value<float2>(float2 v) {
  return static_cast<double>(v.x) + static_cast<double>(v.y);
}

template <typename TO>
__device__ __forceinline__ void store_out(TO* out, int64_t i, double s) {
  out[i] = static_cast<TO>(s);
}
template <>
__device__ __forceinline__ void store_out<float2>(float2* out, int64_t i, double s) {
  const float h = static_cast<float>(s);
  out[i] = make_float2(h, static_cast<float>(s - static_cast<double>(h)));
}

template <typename TP, typename TO>
__global__ void reduce_splits_kernel(const TP* __restrict__ part, int nsplit, int64_t stride,
                                     int64_t begin, int64_t n_valid, int64_t n_total,
                                     TO* __restrict__ out, const double* __restrict__ add,
                                     double scale) {
  for (int64_t i = begin + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
       i < n_total; i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double s = 0.0;
    if (i < n_valid) {
      for (int k = 0; k < nsplit; ++k) s += part_value(part[k * stride + i]);
      if (add) s = fma(scale, add[i], s);
    }
    store_out(out, i, s);
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

// Device helpers shared by the subspace kernels (internal to libsgpp_gb300).
//
// Cell arithmetic: with S = 2^{l-1} and x in [0, 1), fma_rd(x, S, 2^23) = 2^23 + floor(x S)
// exactly (x S is exact, and [2^23, 2^24) has spacing 1), so the float's bit pattern is
// bits(2^23) + k and a position is base + sum_t bits(r_t) * stride_t, the magic offsets being
// folded into base.
//
// Active dimensions: the level-1 hat h1(x) = min(2x, 2 - 2x) (exact, > 0 inside (0, 1)) does not
// depend on the subspace, so a point carries H1 = prod_t h1(x_t) and r_t = 1 / h1(x_t), and a
// subspace with active dimensions A = {t : l_t > 1} costs |A| one-dimensional evaluations:
//     p = H1 * prod_{t in A} h_{l_t}(x_t) * r_t
// (the h1 factors cancel to rounding). A point with a coordinate outside (2^-100, 1) gets H1 = 0
// (its hats are 0, or below 2^-90 next to the origin) and coordinates 0.5, so every cell index
// stays inside its subspace.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sgmev {
namespace subk {

constexpr unsigned kMagicBits = 0x4B000000u;  // bits of 2^23
constexpr float kMagic = 8388608.0f;          // 2^23
constexpr float kTwoMagic = 16777216.0f;      // 2^24
constexpr float kActLow = 7.88860905e-31f;    // 2^-100
constexpr int kOwnTile = 256;                 // points per staged tile of the owner kernels

// whether a coordinate lies in the evaluated domain
__device__ __forceinline__ bool act_inside(float x) { return x > kActLow && x < 1.0f; }

// one-dimensional hat of level l (S = 2^{l-1}, L = 2^l) at x in [0, 1): returns h, sets rr to
// 2^23 + cell
__device__ __forceinline__ float hat_cell(float x, float S, float L, float& rr) {
  rr = __fmaf_rd(x, S, kMagic);
  const float nI = fmaf(rr, -2.0f, kTwoMagic - 1.0f);  // -(2k + 1), exact
  return __saturatef(1.0f - fabsf(fmaf(x, L, nI)));
}

// rows of a staged tile: (H1 * v, 0, (x_0, 1 / h1(x_0)), ..., (x_{d-1}, 1 / h1(x_{d-1})))
template <int DIM>
struct ActRow {
  static constexpr int W = (2 + 2 * DIM + 3) / 4 * 4;
};

// Stage kOwnTile points of `tile` into s_pt (all threads of the CTA take part; two barriers).
// v == nullptr stages H1 in place of H1 * v.
template <int DIM>
__device__ __forceinline__ void act_stage_tile(float* s_pt, int64_t tile,
                                               const float* __restrict__ xt, int64_t mpad,
                                               int64_t m, const float* __restrict__ v) {
  constexpr int W = ActRow<DIM>::W;
  const int64_t j0 = tile * kOwnTile;
  for (int k = threadIdx.x; k < kOwnTile * DIM; k += blockDim.x) {
    const int t = k / kOwnTile, jj = k - t * kOwnTile;
    s_pt[jj * W + 2 + 2 * t] = xt[static_cast<int64_t>(t) * mpad + j0 + jj];
  }
  __syncthreads();
  for (int jj = threadIdx.x; jj < kOwnTile; jj += blockDim.x) {
    float* row = s_pt + jj * W;
    const int64_t j = j0 + jj;
    bool inside = j < m;
#pragma unroll
    for (int t = 0; t < DIM; ++t) inside = inside && act_inside(row[2 + 2 * t]);
    float h1p = 1.0f;
#pragma unroll
    for (int t = 0; t < DIM; ++t) {
      const float x = inside ? row[2 + 2 * t] : 0.5f;
      const float h1 = fminf(2.0f * x, 2.0f - 2.0f * x);
      h1p *= h1;
      row[2 + 2 * t] = x;
      row[3 + 2 * t] = 1.0f / h1;
    }
    row[0] = inside ? (v ? h1p * v[j] : h1p) : 0.0f;
    row[1] = 0.0f;
  }
  __syncthreads();
}

// Per-thread descriptor of a subspace's active dimensions, held in registers for up to NA of them.
template <int NA>
struct ActDesc {
  int toff[NA > 0 ? NA : 1];  // float offset of (x_t, r_t) in a row
  float S[NA > 0 ? NA : 1], L[NA > 0 ? NA : 1];
  uint32_t st[NA > 0 ? NA : 1];

  __device__ __forceinline__ void load(const int4* __restrict__ q) {
#pragma unroll
    for (int a = 0; a < NA; ++a) {
      toff[a] = 2 + 2 * q[a].x;
      S[a] = __int_as_float(q[a].y);
      L[a] = __int_as_float(q[a].z);
      st[a] = static_cast<uint32_t>(q[a].w);
    }
  }

  // p = row[0] * prod_a h_a * r_a, c = cbase + sum_a bits(cell_a) * stride_a
  __device__ __forceinline__ float eval(const float* __restrict__ row, uint32_t cbase,
                                        uint32_t& c) const {
    float p = row[0];
    c = cbase;
#pragma unroll
    for (int a = 0; a < NA; ++a) {
      const float2 xr = *reinterpret_cast<const float2*>(row + toff[a]);
      float rr;
      const float h = hat_cell(xr.x, S[a], L[a], rr);
      p = (p * h) * xr.y;
      c += __float_as_uint(rr) * st[a];
    }
    return p;
  }
};

// the same for any number of active dimensions, read from the descriptor array each time
__device__ __forceinline__ float act_eval_dyn(const float* __restrict__ row,
                                              const int4* __restrict__ q, int na, uint32_t cbase,
                                              uint32_t& c) {
  float p = row[0];
  c = cbase;
  for (int a = 0; a < na; ++a) {
    const int4 d = q[a];
    const float2 xr = *reinterpret_cast<const float2*>(row + 2 + 2 * d.x);
    float rr;
    const float h = hat_cell(xr.x, __int_as_float(d.y), __int_as_float(d.z), rr);
    p = (p * h) * xr.y;
    c += __float_as_uint(rr) * static_cast<uint32_t>(d.w);
  }
  return p;
}

}  // namespace subk
}  // namespace sgmev

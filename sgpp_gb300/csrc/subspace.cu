// Subspace-skipping evaluation of the hat basis in FP32 (the reference's DEFAULT operator does
// the same on the CPU by hierarchical descent, base/src/sgpp/base/algorithm/AlgorithmEvaluation.hpp
// :129-179; SUBSPACELINEAR by flat subspace arrays, DatadrivenOpFactory.cpp:453-470).
//
// For a data point x and a subspace with level vector l, exactly one basis function can be
// non-zero: in dimension t its index is i_t = 2 k_t + 1 with k_t = floor(x_t 2^{l_t - 1}). So a
// product costs one evaluation per subspace instead of one per grid point. The kernels are
// branch-free per dimension: with S = 2^{l-1}, L = 2^l and xc = x clamped into [0, 1),
//     r  = fma_rd(xc, S, 2^23)            = 2^23 + floor(xc S) exactly (xc S is exact: S = 2^k,
//                                           and [2^23, 2^24) has spacing 1; rounded downwards)
//     t  = fma(x, L, fma(r, -2, 2^24 - 1)) = x L - (2k + 1),  h = sat(1 - |t|),  p *= h
//     flat += bits(r) * stride            (bits(2^23 + k) = bits(2^23) + k; the offset term is
//                                           folded into the subspace base)
// xc < 1 keeps k at most S - 1, and x outside [0, 1) selects an edge cell whose hat is 0.
//
//   mult        gather: result_j = sum_s asub[pos_s(x_j)] * prod_t h_t; asub in shared memory
//   multT       scatter: contributions v_j * prod_t h_t are rounded to 43-bit fixed point (one
//               power-of-two scale from max|v| and M), split into a high word and a 22-bit low
//               word, added into two shared-memory int32 accumulators, and flushed into a global
//               int64 vector after every 512-point tile (so no word sum can overflow); integer
//               addition is exact and associative, so the result is the same bit for bit
//               whatever the order of the atomic updates
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <type_traits>
#include <vector>

#include "devmem.h"
#include "kernels.cuh"
#include "subspace.h"
#include "subspace_common.cuh"

namespace sgmev {

namespace {

using namespace subk;

constexpr int kSDT = 64;                  // subspaces per shared-memory descriptor tile
constexpr float kBelowOne = 0.99999994f;      // largest float < 1

constexpr int kMulttThreads = 256, kMulttR = 2;

template <int DIM, int R>
struct Pt {
  float x[R][DIM];
  float xc[R][DIM];
};

template <int DIM, int R>
__device__ __forceinline__ void load_points(Pt<DIM, R>& pt, const float* __restrict__ xt,
                                            int64_t mpad, int64_t j0, int stride) {
#pragma unroll
  for (int r = 0; r < R; ++r) {
#pragma unroll
    for (int t = 0; t < DIM; ++t) {
      const float v = xt[static_cast<int64_t>(t) * mpad + j0 + r * stride];
      pt.x[r][t] = v;
      pt.xc[r][t] = fminf(fmaxf(v, 0.0f), kBelowOne);
    }
  }
}

// flat position and product of the one possibly non-zero basis function of subspace `s`
template <int DIM, int R>
__device__ __forceinline__ void eval_subspace(const Pt<DIM, R>& pt, const int4* __restrict__ d,
                                              uint32_t base, uint32_t last, uint32_t (&flat)[R],
                                              float (&p)[R]) {
#pragma unroll
  for (int r = 0; r < R; ++r) {
    flat[r] = base;
    p[r] = 1.0f;
  }
#pragma unroll
  for (int t = 0; t < DIM; ++t) {
    const int4 q = d[t];
    const float S = __int_as_float(q.x);
    const float L = __int_as_float(q.y);
    const uint32_t st = static_cast<uint32_t>(q.z);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const float rr = __fmaf_rd(pt.xc[r][t], S, kMagic);
      const float nI = fmaf(rr, -2.0f, kTwoMagic - 1.0f);
      const float tt = fmaf(pt.x[r][t], L, nI);
      p[r] *= __saturatef(1.0f - fabsf(tt));
      flat[r] += __float_as_uint(rr) * st;
    }
  }
  // the arithmetic above keeps flat inside the subspace; the clamp only guards the shared-memory
  // index against a corrupted descriptor
#pragma unroll
  for (int r = 0; r < R; ++r) flat[r] = min(flat[r], last);
}

// Active-dimension evaluation (FP32). Most subspaces have level 1 in most dimensions, and the
// level-1 hat h1(x) = min(2x, 2 - 2x) (exact, and > 0 inside (0, 1)) does not depend on the
// subspace. So a point carries H1 = prod_t h1(x_t) and r_t = 1 / h1(x_t), and a subspace with
// active dimensions A = {t : l_t > 1} costs |A| one-dimensional evaluations:
//     p = H1 * prod_{t in A} h_{l_t}(x_t) * r_t,      flat = base_A + sum_{t in A} bits(r) * stride_t
// (the h1 factors cancel to rounding). A point with a coordinate outside (2^-100, 1) gets H1 = 0
// (its hats are 0, or below 2^-90 next to the origin) and coordinates 0.5, so every cell index
// stays inside its subspace.
constexpr int kActThreads = 256, kActR = 2;  // the mult kernel: tiles of 512 points, 2 per thread
constexpr int kActUnrolled = 6;              // active-dimension counts with unrolled evaluation

// p_r *= prod_{a < na} h(x_{r, t_a}) / h1(x_{r, t_a}), flat_r += sum_a bits(cell) * stride_a, for the
// kActR points of this thread; xr points at the thread's (x, 1 / h1) pairs, dimension t at
// xr[t * kActR * kActThreads + r * kActThreads]
template <int NA>
__device__ __forceinline__ void act_eval(const int4* __restrict__ d, const float2* __restrict__ xr,
                                         int na, float (&p)[kActR], uint32_t (&flat)[kActR]) {
#pragma unroll
  for (int a = 0; a < (NA < 0 ? 1 : NA); ++a) {
    if (NA < 0 && a >= na) break;
    const int4 q = d[a];
    const float S = __int_as_float(q.y), L = __int_as_float(q.z);
    const uint32_t st = static_cast<uint32_t>(q.w);
    const float2* xt = xr + q.x * (kActR * kActThreads);
#pragma unroll
    for (int r = 0; r < kActR; ++r) {
      const float2 v = xt[r * kActThreads];
      const float rr = __fmaf_rd(v.x, S, kMagic);
      const float nI = fmaf(rr, -2.0f, kTwoMagic - 1.0f);
      const float h = __saturatef(1.0f - fabsf(fmaf(v.x, L, nI)));
      p[r] = (p[r] * h) * v.y;
      flat[r] += __float_as_uint(rr) * st;
    }
  }
  if (NA < 0) {  // more active dimensions than the unrolled cases: plain loop
    for (int a = 1; a < na; ++a) {
      const int4 q = d[a];
      const float S = __int_as_float(q.y), L = __int_as_float(q.z);
      const uint32_t st = static_cast<uint32_t>(q.w);
      const float2* xt = xr + q.x * (kActR * kActThreads);
#pragma unroll
      for (int r = 0; r < kActR; ++r) {
        const float2 v = xt[r * kActThreads];
        const float rr = __fmaf_rd(v.x, S, kMagic);
        const float nI = fmaf(rr, -2.0f, kTwoMagic - 1.0f);
        const float h = __saturatef(1.0f - fabsf(fmaf(v.x, L, nI)));
        p[r] = (p[r] * h) * v.y;
        flat[r] += __float_as_uint(rr) * st;
      }
    }
  }
}

// GA: alpha is read from global memory (through L1/L2) instead of being staged in shared memory,
// for grids with more positions than shared memory holds
template <int DIM, bool GA>
__global__ void __launch_bounds__(kActThreads, 2) sub_mult_act_kernel(
    const int4* __restrict__ act, const int4* __restrict__ sact, int n_sub,
    const float* __restrict__ asub, int total, const float* __restrict__ xt, int64_t mpad,
    int64_t m, int64_t tile_begin, int64_t n_tiles, float* __restrict__ out32,
    double* __restrict__ out64) {
  extern __shared__ __align__(16) unsigned char smem[];
  int4* s_act = reinterpret_cast<int4*>(smem);             // [kSDT * DIM] (t, S, L, stride)
  int4* s_info = s_act + kSDT * DIM;                        // [kSDT] (base, cells, -, n_active)
  float2* s_xr = reinterpret_cast<float2*>(s_info + kSDT);  // [DIM][kActR][kActThreads]
  float* s_stage = reinterpret_cast<float*>(s_xr + DIM * kActR * kActThreads);  // [total]
  const int tid = threadIdx.x;
  const float2* xr = s_xr + tid;
  if (!GA)
    for (int k = tid; k < total; k += kActThreads) s_stage[k] = asub[k];
  const float* s_a = GA ? asub : s_stage;
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t j0 = (tile_begin + tile) * (kActR * kActThreads) + tid;
    float h1p[kActR];
#pragma unroll
    for (int r = 0; r < kActR; ++r) {
      const int64_t j = j0 + r * kActThreads;
      float xv[DIM];
      bool inside = j < m;
#pragma unroll
      for (int t = 0; t < DIM; ++t) {
        xv[t] = xt[static_cast<int64_t>(t) * mpad + j];
        inside = inside && act_inside(xv[t]);
      }
      h1p[r] = inside ? 1.0f : 0.0f;
#pragma unroll
      for (int t = 0; t < DIM; ++t) {
        const float x = inside ? xv[t] : 0.5f;
        const float h1 = fminf(2.0f * x, 2.0f - 2.0f * x);
        h1p[r] *= h1;
        // thread-private slots: read back only by this thread
        s_xr[(t * kActR + r) * kActThreads + tid] = make_float2(x, 1.0f / h1);
      }
    }
    float acc[kActR];
#pragma unroll
    for (int r = 0; r < kActR; ++r) acc[r] = 0.0f;
    for (int s0 = 0; s0 < n_sub; s0 += kSDT) {
      const int cnt = min(kSDT, n_sub - s0);
      __syncthreads();
      for (int k = tid; k < cnt * DIM; k += kActThreads) s_act[k] = act[s0 * DIM + k];
      for (int k = tid; k < cnt; k += kActThreads) s_info[k] = sact[s0 + k];
      __syncthreads();
      for (int s = 0; s < cnt; ++s) {
        const int4 si = s_info[s];
        const int4* d = s_act + s * DIM;
        float p[kActR];
        uint32_t flat[kActR];
#pragma unroll
        for (int r = 0; r < kActR; ++r) {
          p[r] = h1p[r];
          flat[r] = static_cast<uint32_t>(si.x);
        }
        switch (si.w) {  // warp-uniform: every thread walks the same subspace
          case 0: break;
          case 1: act_eval<1>(d, xr, 1, p, flat); break;
          case 2: act_eval<2>(d, xr, 2, p, flat); break;
          case 3: act_eval<(DIM < 3 ? DIM : 3)>(d, xr, 3, p, flat); break;
          case 4: act_eval<(DIM < 4 ? DIM : 4)>(d, xr, 4, p, flat); break;
          case 5: act_eval<(DIM < 5 ? DIM : 5)>(d, xr, 5, p, flat); break;
          case kActUnrolled: act_eval<(DIM < kActUnrolled ? DIM : kActUnrolled)>(d, xr, kActUnrolled, p, flat); break;
          default: act_eval<-1>(d, xr, si.w, p, flat); break;
        }
#pragma unroll
        for (int r = 0; r < kActR; ++r)
          acc[r] = fmaf(s_a[min(flat[r], static_cast<uint32_t>(total - 1))], p[r], acc[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < kActR; ++r) {
      const int64_t j = j0 + r * kActThreads;
      const float v = j < m ? acc[r] : 0.0f;
      if (out32) out32[j] = v;
      if (out64) out64[j] = static_cast<double>(v);
    }
  }
}

// df64 (FP64-accurate) subspace mult. A point is the float-float value x = x_hi + x_lo
// (|x_lo| <= ulp(x_hi) / 2). Points with a coordinate outside the open interval (0, 1) see only zero
// hats (every Linear-grid hat vanishes there), so their result is 0 and their coordinates are
// replaced by 0.5 before the loop. For x in (0, 1) the cell and hat per dimension are
//     sl = L x_lo                          exact (L = 2^l)
//     t2 = fma_rd(x_hi, L, sl)             = the largest float <= x L (one rounding, downwards)
//     r  = fma_rd(t2, 0.5, 2^23)           = 2^23 + k, k = floor(x S) in [0, S - 1]
//     m  = fma(r, -2, 2^24)                = -2k exactly
//     a  = fma(x_hi, L, m), b = fma(x_hi, -L, 2 - m)
// floor(t2 / 2) = floor(x L / 2) because every even integer is a float, so rounding downwards
// cannot cross one. x lies in the closed cell [k/S, (k+1)/S], where the hat is
// min(x L - 2k, 2k + 2 - x L) >= 0; the smaller side is (a, sl) (rising) or (b, -sl) (falling), and
// its high part is exact (Sterbenz: x_hi L lies within a factor 2 of 2k resp. 2k + 2), as is
// a - b near the middle, so the sign test picks the side exactly and the float-float hat is exact.
// alpha is a float-float pair per position in shared memory.
constexpr int kDfThreads = 512, kDfR = 1;

template <int DIM, bool GA>
__global__ void __launch_bounds__(kDfThreads, 1) sub_mult_df_kernel(
    const int4* __restrict__ desc, const uint32_t* __restrict__ base, int n_sub,
    const float2* __restrict__ asub2, int total, const float* __restrict__ xh_t,
    const float* __restrict__ xl_t, int64_t mpad, int64_t m, int64_t tile_begin,
    int64_t n_tiles, double* __restrict__ out64) {
  extern __shared__ __align__(16) unsigned char smem[];
  int4* s_desc = reinterpret_cast<int4*>(smem);
  uint32_t* s_base = reinterpret_cast<uint32_t*>(s_desc + kSDT * DIM);
  float2* s_stage = reinterpret_cast<float2*>(s_base + kSDT);
  if (!GA)
    for (int k = threadIdx.x; k < total; k += kDfThreads) s_stage[k] = asub2[k];
  const float2* s_a = GA ? asub2 : s_stage;
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t j0 = (tile_begin + tile) * (kDfThreads * kDfR) + threadIdx.x;
    float xh[kDfR][DIM], xl[kDfR][DIM];
    bool inside[kDfR];
#pragma unroll
    for (int r = 0; r < kDfR; ++r) {
      inside[r] = true;
#pragma unroll
      for (int t = 0; t < DIM; ++t) {
        const int64_t src = static_cast<int64_t>(t) * mpad + j0 + r * kDfThreads;
        const float h = xh_t[src], l = xl_t[src];
        inside[r] = inside[r] && (h > 0.0f || (h == 0.0f && l > 0.0f)) &&
                    (h < 1.0f || (h == 1.0f && l < 0.0f));
        xh[r][t] = h;
        xl[r][t] = l;
      }
#pragma unroll
      for (int t = 0; t < DIM; ++t) {
        xh[r][t] = inside[r] ? xh[r][t] : 0.5f;
        xl[r][t] = inside[r] ? xl[r][t] : 0.0f;
      }
    }
    ff acc[kDfR];
#pragma unroll
    for (int r = 0; r < kDfR; ++r) acc[r] = ff{0.0f, 0.0f};
    for (int s0 = 0; s0 < n_sub; s0 += kSDT) {
      const int cnt = min(kSDT, n_sub - s0);
      __syncthreads();
      for (int k = threadIdx.x; k < cnt * DIM; k += kDfThreads) s_desc[k] = desc[s0 * DIM + k];
      for (int k = threadIdx.x; k < cnt; k += kDfThreads) s_base[k] = base[s0 + k];
      __syncthreads();
      for (int s = 0; s < cnt; ++s) {
        const int4* d = s_desc + s * DIM;
        uint32_t flat[kDfR];
        ff p[kDfR];
#pragma unroll
        for (int r = 0; r < kDfR; ++r) flat[r] = s_base[s];
#pragma unroll
        for (int t = 0; t < DIM; ++t) {
          const int4 q = d[t];
          const float L = __int_as_float(q.y);
          const uint32_t st = static_cast<uint32_t>(q.z);
#pragma unroll
          for (int r = 0; r < kDfR; ++r) {
            const float sl = L * xl[r][t];
            const float t2 = __fmaf_rd(xh[r][t], L, sl);
            const float rr = __fmaf_rd(t2, 0.5f, kMagic);
            const float m2k = fmaf(rr, -2.0f, kTwoMagic);
            const float a = fmaf(xh[r][t], L, m2k);
            const float b = fmaf(xh[r][t], -L, 2.0f - m2k);
            const bool rise = fmaf(2.0f, sl, a - b) <= 0.0f;
            const ff h{rise ? a : b, rise ? sl : -sl};
            p[r] = t == 0 ? h : mul_ff(p[r], h);
            flat[r] += __float_as_uint(rr) * st;
          }
        }
#pragma unroll
        for (int r = 0; r < kDfR; ++r) {
          const float2 a = s_a[min(flat[r], static_cast<uint32_t>(total - 1))];
          add_ff(acc[r], mul_ff(p[r], ff{a.x, a.y}));
        }
      }
#pragma unroll
      for (int r = 0; r < kDfR; ++r) renorm_ff(acc[r]);
    }
#pragma unroll
    for (int r = 0; r < kDfR; ++r) {
      const int64_t j = j0 + r * kDfThreads;
      out64[j] = (j < m && inside[r]) ? static_cast<double>(acc[r].h) + static_cast<double>(acc[r].l)
                                      : 0.0;
    }
  }
}

__global__ void scatter_alpha_df_kernel(const float* __restrict__ ah, const float* __restrict__ al,
                                        const int* __restrict__ pos, int64_t n,
                                        float2* __restrict__ asub2) {
  for (int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; g < n;
       g += static_cast<int64_t>(gridDim.x) * blockDim.x)
    asub2[pos[g]] = make_float2(ah[g], al[g]);
}

// fixed-point scale 2^k for contributions |v_j| * prod h <= max|v|: one contribution stays below
// 2^43 (so its high word over 512 points and its 22-bit low words over 512 points fit int32) and
// all M contributions stay below 2^62 (the global int64 sums)
__device__ __forceinline__ float fixed_scale(unsigned int maxbits, float m_total) {
  const float mv = __uint_as_float(maxbits);
  if (!(mv > 0.0f)) return 1.0f;
  int e1 = 0, e2 = 0;
  frexpf(mv, &e1);            // mv < 2^e1
  frexpf(mv * m_total, &e2);  // M mv < 2^e2
  const int k = min(43 - e1, 62 - e2);
  return ldexpf(1.0f, max(-126, min(k, 126)));
}

template <int DIM>
__global__ void __launch_bounds__(kMulttThreads) sub_multt_kernel(
    const int4* __restrict__ desc, const uint32_t* __restrict__ base, int n_sub, int total,
    const float* __restrict__ xt, int64_t mpad, int64_t m, int64_t n_tiles,
    const float* __restrict__ v, const unsigned int* __restrict__ maxbits, float m_total,
    unsigned long long* __restrict__ acc_g) {
  extern __shared__ __align__(16) unsigned char smem[];
  int4* s_desc = reinterpret_cast<int4*>(smem);
  uint32_t* s_base = reinterpret_cast<uint32_t*>(s_desc + kSDT * DIM);
  int* s_hi = reinterpret_cast<int*>(s_base + kSDT);
  int* s_lo = s_hi + total;
  for (int k = threadIdx.x; k < total; k += kMulttThreads) {
    s_hi[k] = 0;
    s_lo[k] = 0;
  }
  const float scale = fixed_scale(*maxbits, m_total);
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t j0 = tile * (kMulttThreads * kMulttR) + threadIdx.x;
    Pt<DIM, kMulttR> pt;
    load_points(pt, xt, mpad, j0, kMulttThreads);
    float vj[kMulttR];
#pragma unroll
    for (int r = 0; r < kMulttR; ++r) {
      const int64_t j = j0 + r * kMulttThreads;
      vj[r] = j < m ? v[j] * scale : 0.0f;
    }
    for (int s0 = 0; s0 < n_sub; s0 += kSDT) {
      const int cnt = min(kSDT, n_sub - s0);
      __syncthreads();
      for (int k = threadIdx.x; k < cnt * DIM; k += kMulttThreads) s_desc[k] = desc[s0 * DIM + k];
      for (int k = threadIdx.x; k < cnt; k += kMulttThreads) s_base[k] = base[s0 + k];
      __syncthreads();
      for (int s = 0; s < cnt; ++s) {
        uint32_t flat[kMulttR];
        float p[kMulttR];
        eval_subspace<DIM, kMulttR>(pt, s_desc + s * DIM, s_base[s],
                                    static_cast<uint32_t>(total - 1), flat, p);
#pragma unroll
        for (int r = 0; r < kMulttR; ++r) {
          const long long q = __float2ll_rn(vj[r] * p[r]);
          if (q != 0) {
            atomicAdd(&s_hi[flat[r]], static_cast<int>(q >> 22));
            atomicAdd(&s_lo[flat[r]], static_cast<int>(q & 0x3FFFFF));
          }
        }
      }
    }
    // flush this tile's sums (at most 512 contributions per word since the last flush)
    __syncthreads();
    for (int k = threadIdx.x; k < total; k += kMulttThreads) {
      const long long a = (static_cast<long long>(s_hi[k]) << 22) + s_lo[k];
      if (a != 0) atomicAdd(&acc_g[k], static_cast<unsigned long long>(a));
      s_hi[k] = 0;
      s_lo[k] = 0;
    }
  }
}

// Owner-computes multTranspose. Thread k of a pass owns subspace s = pass * blockDim + k and sums
// v_j * prod_t h_t(x_j) over the CTA's points into per-cell accumulators in shared memory, laid out
// [cell][thread] so that a warp's 32 updates hit 32 different banks. The points of a tile are
// staged in shared memory as rows (x_0 .. x_{d-1}, v) and read by all threads at once (broadcast).
// After each tile a thread adds its cells into the CTA's FP64 row of the partial matrix (its cells
// belong to it alone, so the update order is fixed); sum_rows_kernel adds the rows in CTA order.
// Every step has a fixed order, so the result is the same bit for bit from run to run.
// Points with a coordinate outside the open interval (0, 1) see only zero hats; the staging step
// gives them v = 0 and coordinates 0.5, which keeps the cell arithmetic inside the subspace with no
// clamp. FP32: the per-dimension product is the one of the mult kernel. DF: as sub_mult_df_kernel,
// with float-float per-tile sums.
constexpr int kOwnMaxThreads = 512;
constexpr size_t kOwnSmemBudget = 200 * 1024;  // shared memory of an owner-computes CTA
constexpr int kActOwnThreads = 512;  // FP32 owner kernel (128-thread CTAs measured slower)
constexpr int kActFlushTiles = 4;    // FP32 owner kernel: tiles summed in FP32 per flush

template <int DIM, bool DF>
struct OwnLayout {
  static constexpr int W = DF ? (2 * DIM + 2 + 3) / 4 * 4 : (DIM + 1 + 3) / 4 * 4;  // floats per row
  static constexpr int V = DF ? 2 * DIM : DIM;                                       // v column
  using Acc = typename std::conditional<DF, float2, float>::type;
};

// MOD (modified linear basis, data in [0, 1]): every real point is evaluated, faces included.
template <int DIM, bool DF, bool MOD = false>
__device__ __forceinline__ void own_stage_tile(float* s_pt, int64_t tile,
                                               const float* __restrict__ xh_t,
                                               const float* __restrict__ xl_t, int64_t mpad,
                                               int64_t m, const float* __restrict__ vh,
                                               const float* __restrict__ vl) {
  using Lay = OwnLayout<DIM, DF>;
  const int64_t j0 = tile * kOwnTile;
  for (int k = threadIdx.x; k < kOwnTile * DIM; k += blockDim.x) {
    const int t = k / kOwnTile, jj = k - t * kOwnTile;
    const int64_t src = static_cast<int64_t>(t) * mpad + j0 + jj;
    s_pt[jj * Lay::W + t] = xh_t[src];
    if constexpr (DF) s_pt[jj * Lay::W + DIM + t] = xl_t[src];
  }
  __syncthreads();
  for (int jj = threadIdx.x; jj < kOwnTile; jj += blockDim.x) {
    float* row = s_pt + jj * Lay::W;
    const int64_t j = j0 + jj;
    bool inside = j < m;
#pragma unroll
    for (int t = 0; t < DIM; ++t) {
      const float h = row[t];
      if constexpr (MOD) {
        (void)h;
      } else if constexpr (DF) {
        const float l = row[DIM + t];
        inside = inside && (h > 0.0f || (h == 0.0f && l > 0.0f)) &&
                 (h < 1.0f || (h == 1.0f && l < 0.0f));
      } else {
        inside = inside && h > 0.0f && h < 1.0f;
      }
    }
    if (!inside) {
#pragma unroll
      for (int t = 0; t < DIM; ++t) {
        row[t] = 0.5f;
        if constexpr (DF) row[DIM + t] = 0.0f;
      }
    }
    // vh == nullptr: the v column holds the inside flag (1 or 0), vl's column 0
    row[Lay::V] = inside ? (vh ? vh[j] : 1.0f) : 0.0f;
    if constexpr (DF) row[Lay::V + 1] = (inside && vl) ? vl[j] : 0.0f;
  }
  __syncthreads();
}

template <int DIM, bool DF>
__global__ void __launch_bounds__(kOwnMaxThreads, 1) sub_multt_own_kernel(
    const int4* __restrict__ desc, const int4* __restrict__ sinfo, int n_sub, int cmax,
    int total, const float* __restrict__ xh_t, const float* __restrict__ xl_t, int64_t mpad,
    int64_t m, const float* __restrict__ vh, const float* __restrict__ vl, int64_t n_tiles,
    double* __restrict__ rows) {
  using Lay = OwnLayout<DIM, DF>;
  using Acc = typename Lay::Acc;
  extern __shared__ __align__(16) unsigned char smem[];
  float* s_pt = reinterpret_cast<float*>(smem);                // [kOwnTile][W]
  Acc* s_acc = reinterpret_cast<Acc*>(s_pt + kOwnTile * Lay::W);  // [cmax][blockDim]
  double* row = rows + static_cast<int64_t>(blockIdx.x) * total;
  const int tid = threadIdx.x, nth = blockDim.x;
  for (int s0 = 0; s0 < n_sub; s0 += nth) {
    const int sid = s0 + tid;
    const bool active = sid < n_sub;
    const int4 info = active ? sinfo[sid] : make_int4(0, 0, 0, 0);  // (offset, cells, cbase, 0)
    float S[DIM], L[DIM];
    uint32_t st[DIM];
#pragma unroll
    for (int t = 0; t < DIM; ++t) {
      const int4 q = active ? desc[static_cast<int64_t>(sid) * DIM + t]
                            : make_int4(__float_as_int(1.0f), __float_as_int(2.0f), 0, 0);
      S[t] = __int_as_float(q.x);
      L[t] = __int_as_float(q.y);
      st[t] = static_cast<uint32_t>(q.z);
    }
    for (int c = 0; c < info.y; ++c) s_acc[c * nth + tid] = Acc{};
    bool first = true;
    for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
      __syncthreads();  // the previous tile's rows are no longer read
      own_stage_tile<DIM, DF>(s_pt, tile, xh_t, xl_t, mpad, m, vh, vl);
      if (active) {
        for (int jj = 0; jj < kOwnTile; ++jj) {
          const float4* r4 = reinterpret_cast<const float4*>(s_pt + jj * Lay::W);
          float rw[Lay::W];
#pragma unroll
          for (int k = 0; k < Lay::W / 4; ++k) {
            const float4 f = r4[k];
            rw[4 * k] = f.x;
            rw[4 * k + 1] = f.y;
            rw[4 * k + 2] = f.z;
            rw[4 * k + 3] = f.w;
          }
          uint32_t c = static_cast<uint32_t>(info.z);
          if constexpr (DF) {
            ff p{1.0f, 0.0f};
#pragma unroll
            for (int t = 0; t < DIM; ++t) {
              const float xh = rw[t], xl = rw[DIM + t];
              const float sl = L[t] * xl;
              const float t2 = __fmaf_rd(xh, L[t], sl);
              const float rr = __fmaf_rd(t2, 0.5f, kMagic);
              const float m2k = fmaf(rr, -2.0f, kTwoMagic);
              const float a = fmaf(xh, L[t], m2k);
              const float b = fmaf(xh, -L[t], 2.0f - m2k);
              const bool rise = fmaf(2.0f, sl, a - b) <= 0.0f;
              const ff h{rise ? a : b, rise ? sl : -sl};
              p = t == 0 ? h : mul_ff(p, h);
              c += __float_as_uint(rr) * st[t];
            }
            const ff q = mul_ff(p, ff{rw[Lay::V], rw[Lay::V + 1]});
            float2* slot = reinterpret_cast<float2*>(s_acc) + min(c, static_cast<uint32_t>(cmax - 1)) * nth + tid;
            ff a{slot->x, slot->y};
            add_ff(a, q);
            *slot = make_float2(a.h, a.l);
          } else {
            float p = 1.0f;
#pragma unroll
            for (int t = 0; t < DIM; ++t) {
              const float rr = __fmaf_rd(rw[t], S[t], kMagic);
              const float nI = fmaf(rr, -2.0f, kTwoMagic - 1.0f);
              const float h = __saturatef(1.0f - fabsf(fmaf(rw[t], L[t], nI)));
              p = t == 0 ? h : p * h;
              c += __float_as_uint(rr) * st[t];
            }
            float* slot = reinterpret_cast<float*>(s_acc) + min(c, static_cast<uint32_t>(cmax - 1)) * nth + tid;
            *slot = fmaf(rw[Lay::V], p, *slot);
          }
        }
        // this tile's sums into the CTA's FP64 row (cells of this subspace are this thread's)
        for (int c = 0; c < info.y; ++c) {
          Acc& a = s_acc[c * nth + tid];
          double v;
          if constexpr (DF) {
            v = static_cast<double>(a.x) + static_cast<double>(a.y);
          } else {
            v = static_cast<double>(a);
          }
          double* dst = row + info.x + c;
          *dst = first ? v : *dst + v;
          a = Acc{};
        }
      }
      first = false;
    }
    if (active && first)  // no tile for this CTA: its row holds zeros
      for (int c = 0; c < info.y; ++c) row[info.x + c] = 0.0;
  }
}

// Build of the materialised products (see subspace_mat.cu): thread k of a pass owns subspace
// s = pass * blockDim + k and writes, for every point of the CTA's tiles, the float-float product
// of its basis function (renormalised: hi = the FP32 rounding of the pair) and the cell index, in
// the layout P_hi[g][s], P_lo[g][s] (float4: points 4g .. 4g+3) and C[g][s] (a byte per point).
// The arithmetic is the one of the float-float kernels above, so the cells follow x_hi + x_lo.
// MOD: the modified linear basis (LinearModifiedBasis.hpp:40-58) for data in [0, 1]. A level-1
// factor is 1; the cell is clamped to [0, S - 1] (x = 1 lies in the last cell); in the first
// cell of a level >= 2 the function is the falling branch 2 - 2^l x throughout, in the last cell
// the rising branch 2^l x - 2^l + 2, elsewhere the hat. The falling branch next to x = 0 is not
// an exact FP32 number, so its rounding error is recovered with Knuth's two-sum (TAOCP vol. 2,
// 4.2.2) into the low part.
template <int DIM, bool MOD>
__global__ void __launch_bounds__(kOwnMaxThreads, 1) sub_mat_build_kernel(
    const int4* __restrict__ desc, const int4* __restrict__ sinfo, int n_sub, int s_pad,
    const float* __restrict__ xh_t, const float* __restrict__ xl_t, int64_t mpad, int64_t m,
    int64_t n_tiles, float4* __restrict__ phi, float4* __restrict__ plo, uint4* __restrict__ p16,
    uint32_t* __restrict__ cm, float p16_scale) {
  using Lay = OwnLayout<DIM, true>;
  extern __shared__ __align__(16) unsigned char smem[];
  float* s_pt = reinterpret_cast<float*>(smem);  // [kOwnTile][W]
  const int tid = threadIdx.x;
  constexpr int kGroupsPerTile = kOwnTile / 4;
  for (int s0 = 0; s0 < s_pad; s0 += blockDim.x) {
    const int sid = s0 + tid;
    const bool real = sid < n_sub;
    const int4 info = real ? sinfo[sid] : make_int4(0, 0, 0, 0);  // (offset, cells, cbase, 0)
    float L[DIM];
    uint32_t st[DIM];
#pragma unroll
    for (int t = 0; t < DIM; ++t) {
      const int4 q = real ? desc[static_cast<int64_t>(sid) * DIM + t]
                          : make_int4(__float_as_int(1.0f), __float_as_int(2.0f), 0, 0);
      L[t] = __int_as_float(q.y);
      st[t] = static_cast<uint32_t>(q.z);
    }
    for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
      __syncthreads();  // the previous tile's rows are no longer read
      own_stage_tile<DIM, true, MOD>(s_pt, tile, xh_t, xl_t, mpad, m, nullptr, nullptr);
      if (sid >= s_pad) continue;
      const int64_t at = tile * kGroupsPerTile * static_cast<int64_t>(s_pad) + sid;
      for (int g = 0; g < kGroupsPerTile; ++g) {
        float hv[4], lv[4];
        uint32_t cells = 0;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float* rw = s_pt + (4 * g + i) * Lay::W;
          uint32_t c = static_cast<uint32_t>(info.z);
          ff p{0.0f, 0.0f};
          if (real) {
            p = ff{1.0f, 0.0f};
#pragma unroll
            for (int t = 0; t < DIM; ++t) {
              const float xh = rw[t], xl = rw[DIM + t];
              const float sl = L[t] * xl;
              const float t2 = __fmaf_rd(xh, L[t], sl);
              float rr = __fmaf_rd(t2, 0.5f, kMagic);
              if constexpr (MOD) rr = fminf(fmaxf(rr, kMagic), kMagic + (0.5f * L[t] - 1.0f));
              const float m2k = fmaf(rr, -2.0f, kTwoMagic);
              const float a = fmaf(xh, L[t], m2k);
              const float b = fmaf(xh, -L[t], 2.0f - m2k);
              bool rise = fmaf(2.0f, sl, a - b) <= 0.0f;
              ff h{rise ? a : b, rise ? sl : -sl};
              if constexpr (MOD) {
                const uint32_t k = __float_as_uint(rr) - kMagicBits;
                const uint32_t last = static_cast<uint32_t>(0.5f * L[t]) - 1u;
                if (L[t] == 2.0f) {
                  h = ff{1.0f, 0.0f};
                } else {
                  if (k == 0u) rise = false;
                  else if (k == last) rise = true;
                  const float y = xh * L[t];  // exact
                  const float P = rise ? y : -y, Q = rise ? m2k : 2.0f - m2k;
                  const float hh = rise ? a : b;  // fl(P + Q)
                  const float bb = hh - P;
                  const float err = (P - (hh - bb)) + (Q - bb);
                  h = ff{hh, err + (rise ? sl : -sl)};
                }
              }
              p = t == 0 ? h : mul_ff(p, h);
              c += __float_as_uint(rr) * st[t];
            }
            const float in = rw[Lay::V];  // 1 inside the domain, 0 outside
            p = ff{p.h * in, p.l * in};
            const float sh = p.h + p.l;
            p = ff{sh, p.l - (sh - p.h)};
          } else {
            c = 0;
          }
          hv[i] = p.h;
          lv[i] = p.l;
          cells |= (c & 0xFFu) << (8 * i);
        }
        const int64_t k = at + static_cast<int64_t>(g) * s_pad;
        phi[k] = make_float4(hv[0], hv[1], hv[2], hv[3]);
        plo[k] = make_float4(lv[0], lv[1], lv[2], lv[3]);
        const __half2 h01 = __floats2half2_rn(hv[0] * p16_scale, hv[1] * p16_scale),
                      h23 = __floats2half2_rn(hv[2] * p16_scale, hv[3] * p16_scale);
        // FP16 copy by pairs of groups: group gg is half gg % 2 of pair gg / 2
        const int64_t gg = tile * kGroupsPerTile + g;
        reinterpret_cast<uint2*>(p16 + (gg >> 1) * s_pad + sid)[gg & 1] =
            make_uint2(*reinterpret_cast<const uint32_t*>(&h01),
                       *reinterpret_cast<const uint32_t*>(&h23));
        cm[k] = cells;
      }
    }
  }
}

template <int DIM>
cudaError_t launch_mat_build(const SubPlan& p, cudaStream_t s, const float* xh, const float* xl,
                             int64_t mpad, int64_t m, int num_sms) {
  using Lay = OwnLayout<DIM, true>;
  const size_t sm = sizeof(float) * kOwnTile * Lay::W;
  auto kern = p.mod ? sub_mat_build_kernel<DIM, true> : sub_mat_build_kernel<DIM, false>;
  cudaError_t e = set_smem_cap(kern, sm);
  if (e != cudaSuccess) return e;
  const int64_t nt = mpad / kOwnTile;
  const int nth = static_cast<int>(std::min<int64_t>(kOwnMaxThreads, p.s_pad));
  const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(nt, 2LL * num_sms));
  kern<<<static_cast<unsigned>(blocks), nth, sm, s>>>(p.desc, p.sinfo, p.n_sub,
                                                      static_cast<int>(p.s_pad), xh, xl, mpad, m,
                                                      nt, p.pmat, p.pmat_lo, p.pmat16,
                                                      static_cast<uint32_t*>(p.cmat),
                                                      std::ldexp(1.0f, p16_exp(p)));
  return cudaGetLastError();
}

// Owner-computes multTranspose with active-dimension evaluation (FP32): as sub_multt_own_kernel,
// with rows (H1 * v, 0, (x_0, 1 / h1(x_0)), ..., (x_{d-1}, 1 / h1(x_{d-1}))); a thread's active
// dimensions are held in registers for up to 4 of them (unrolled per count), else looped over.
// one tile of points for a subspace with NA active dimensions: s_acc[c * nth + tid] += p_j
template <int NA>
__device__ __forceinline__ void act_own_tile(const float* __restrict__ s_pt, int w,
                                             const int4* __restrict__ q, uint32_t cbase,
                                             int cmax, float* __restrict__ s_acc, int nth, int tid) {
  int toff[NA > 0 ? NA : 1];
  float S[NA > 0 ? NA : 1], L[NA > 0 ? NA : 1];
  uint32_t st[NA > 0 ? NA : 1];
#pragma unroll
  for (int a = 0; a < NA; ++a) {
    toff[a] = 2 + 2 * q[a].x;
    S[a] = __int_as_float(q[a].y);
    L[a] = __int_as_float(q[a].z);
    st[a] = static_cast<uint32_t>(q[a].w);
  }
  float* acc = s_acc + tid;
  for (int jj = 0; jj < kOwnTile; ++jj) {
    const float* r = s_pt + jj * w;
    float p = r[0];
    uint32_t c = cbase;
#pragma unroll
    for (int a = 0; a < NA; ++a) {
      const float2 xr = *reinterpret_cast<const float2*>(r + toff[a]);
      const float rr = __fmaf_rd(xr.x, S[a], kMagic);
      const float nI = fmaf(rr, -2.0f, kTwoMagic - 1.0f);
      const float h = __saturatef(1.0f - fabsf(fmaf(xr.x, L[a], nI)));
      p = (p * h) * xr.y;
      c += __float_as_uint(rr) * st[a];
    }
    acc[min(c, static_cast<uint32_t>(cmax - 1)) * nth] += p;
  }
}

// more active dimensions than the unrolled cases: a loop over them
__device__ __forceinline__ void act_own_tile_dyn(const float* __restrict__ s_pt, int w,
                                                 const int4* __restrict__ q, int na,
                                                 uint32_t cbase, int cmax,
                                                 float* __restrict__ s_acc, int nth, int tid) {
  float* acc = s_acc + tid;
  for (int jj = 0; jj < kOwnTile; ++jj) {
    const float* r = s_pt + jj * w;
    float p = r[0];
    uint32_t c = cbase;
    for (int a = 0; a < na; ++a) {
      const int4 d = q[a];
      const float2 xr = *reinterpret_cast<const float2*>(r + 2 + 2 * d.x);
      const float rr = __fmaf_rd(xr.x, __int_as_float(d.y), kMagic);
      const float nI = fmaf(rr, -2.0f, kTwoMagic - 1.0f);
      const float h = __saturatef(1.0f - fabsf(fmaf(xr.x, __int_as_float(d.z), nI)));
      p = (p * h) * xr.y;
      c += __float_as_uint(rr) * static_cast<uint32_t>(d.w);
    }
    acc[min(c, static_cast<uint32_t>(cmax - 1)) * nth] += p;
  }
}

template <int DIM>
__global__ void __launch_bounds__(kActOwnThreads, 2) sub_multt_act_kernel(
    const int4* __restrict__ act, const int4* __restrict__ sact, int n_sub, int cmax, int total,
    const float* __restrict__ xt, int64_t mpad, int64_t m, const float* __restrict__ v,
    int64_t n_tiles, double* __restrict__ rows) {
  constexpr int W = ActRow<DIM>::W;
  extern __shared__ __align__(16) unsigned char smem[];
  float* s_pt = reinterpret_cast<float*>(smem);   // [kOwnTile][W]
  float* s_acc = s_pt + kOwnTile * W;             // [cmax][blockDim]
  double* row = rows + static_cast<int64_t>(blockIdx.x) * total;
  const int tid = threadIdx.x, nth = blockDim.x;
  for (int s0 = 0; s0 < n_sub; s0 += nth) {
    const int sid = s0 + tid;
    const bool active = sid < n_sub;
    const int4 info = active ? sact[sid] : make_int4(0, 0, 0, 0);  // (base, cells, cbase, n_active)
    const uint32_t offset = static_cast<uint32_t>(info.x) - static_cast<uint32_t>(info.z);
    const uint32_t cbase = static_cast<uint32_t>(info.z);
    const int4* q = act + static_cast<int64_t>(active ? sid : 0) * DIM;
    for (int c = 0; c < info.y; ++c) s_acc[c * nth + tid] = 0.0f;
    bool first = true;
    int since = 0;  // tiles summed in s_acc since the last flush
    for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
      __syncthreads();  // the previous tile's rows are no longer read
      act_stage_tile<DIM>(s_pt, tile, xt, mpad, m, v);
      if (active) {
        // subspaces are sorted by their active-dimension count, so a warp mostly takes one case
        switch (info.w) {
          case 0: act_own_tile<0>(s_pt, W, q, cbase, cmax, s_acc, nth, tid); break;
          case 1: act_own_tile<1>(s_pt, W, q, cbase, cmax, s_acc, nth, tid); break;
          case 2: act_own_tile<(DIM < 2 ? DIM : 2)>(s_pt, W, q, cbase, cmax, s_acc, nth, tid); break;
          case 3: act_own_tile<(DIM < 3 ? DIM : 3)>(s_pt, W, q, cbase, cmax, s_acc, nth, tid); break;
          case 4: act_own_tile<(DIM < 4 ? DIM : 4)>(s_pt, W, q, cbase, cmax, s_acc, nth, tid); break;
          default: act_own_tile_dyn(s_pt, W, q, info.w, cbase, cmax, s_acc, nth, tid); break;
        }
      }
      ++since;
      // FP32 sums over kActFlushTiles tiles (1024 points), then into the FP64 row
      if (since == kActFlushTiles || tile + gridDim.x >= n_tiles) {
        if (active) {
          for (int c = 0; c < info.y; ++c) {
            float& a = s_acc[c * nth + tid];
            double* dst = row + offset + c;
            *dst = first ? static_cast<double>(a) : *dst + static_cast<double>(a);
            a = 0.0f;
          }
        }
        first = false;
        since = 0;
      }
    }
    if (active && first)
      for (int c = 0; c < info.y; ++c) row[offset + c] = 0.0;
  }
}

// sums[k] = sum over rows b in order of rows[b][k] (k < total)
// sums[k] = sum over rows b of rows[b][k] (k < total) in a fixed order: a block of 32 x 8 threads
// takes 32 positions; thread (x, y) adds rows y, y + 8, y + 16, ... in order (four loads in
// flight), and the 8 partial sums are then added in y order
constexpr int kSumRowGroups = 8;

__global__ void __launch_bounds__(32 * kSumRowGroups) sum_rows_kernel(
    const double* __restrict__ rows, int nrows, int64_t total, double* __restrict__ sums) {
  __shared__ double part[kSumRowGroups][32];
  const int64_t k = static_cast<int64_t>(blockIdx.x) * 32 + threadIdx.x;
  const int y = threadIdx.y;
  double a = 0.0;
  if (k < total) {
    int b = y;
    for (; b + 3 * kSumRowGroups < nrows; b += 4 * kSumRowGroups) {
      const double r0 = rows[static_cast<int64_t>(b) * total + k];
      const double r1 = rows[static_cast<int64_t>(b + kSumRowGroups) * total + k];
      const double r2 = rows[static_cast<int64_t>(b + 2 * kSumRowGroups) * total + k];
      const double r3 = rows[static_cast<int64_t>(b + 3 * kSumRowGroups) * total + k];
      a += r0;
      a += r1;
      a += r2;
      a += r3;
    }
    for (; b < nrows; b += kSumRowGroups) a += rows[static_cast<int64_t>(b) * total + k];
  }
  part[y][threadIdx.x] = a;
  __syncthreads();
  if (y == 0 && k < total) {
    double r = part[0][threadIdx.x];
    for (int g = 1; g < kSumRowGroups; ++g) r += part[g][threadIdx.x];
    sums[k] = r;
  }
}

// out[g] (g < n; zero in [n, npad)) = sums[pos[g]] (+ scale_add * add[g])
__global__ void gather_sums_kernel(const double* __restrict__ sums, const int* __restrict__ pos,
                                   int64_t n, int64_t npad, const double* __restrict__ add,
                                   double scale_add, double* __restrict__ out) {
  for (int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; g < npad;
       g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double r = 0.0;
    if (g < n) {
      r = sums[pos[g]];
      if (add) r = fma(scale_add, add[g], r);
    }
    out[g] = r;
  }
}

__global__ void maxabs_kernel(const float* __restrict__ v, int64_t m, unsigned int* __restrict__ out) {
  __shared__ float s[256];
  float mx = 0.0f;
  for (int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; j < m;
       j += static_cast<int64_t>(gridDim.x) * blockDim.x)
    mx = fmaxf(mx, fabsf(v[j]));
  s[threadIdx.x] = mx;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] = fmaxf(s[threadIdx.x], s[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicMax(out, __float_as_uint(s[0]));  // non-negative: bit order = value order
}

__global__ void scatter_alpha_kernel(const float* __restrict__ alpha, const int* __restrict__ pos,
                                     int64_t n, float* __restrict__ asub) {
  for (int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; g < n;
       g += static_cast<int64_t>(gridDim.x) * blockDim.x)
    asub[pos[g]] = alpha[g];
}

__global__ void gather_result_kernel(const unsigned long long* __restrict__ acc,
                                     const int* __restrict__ pos, int64_t n, int64_t npad,
                                     const unsigned int* __restrict__ maxbits, float m_total,
                                     const double* __restrict__ add, double scale_add,
                                     double* __restrict__ out) {
  const double inv = 1.0 / static_cast<double>(fixed_scale(*maxbits, m_total));
  for (int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; g < npad;
       g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double r = 0.0;
    if (g < n) {
      r = static_cast<double>(static_cast<long long>(acc[pos[g]])) * inv;
      if (add) r = fma(scale_add, add[g], r);
    }
    out[g] = r;
  }
}

size_t multt_smem(int dim, int64_t total) {
  return sizeof(int4) * kSDT * dim + sizeof(uint32_t) * kSDT + 2 * sizeof(int) * total;
}

int64_t multt_blocks(int64_t mpad, int num_sms) {
  const int64_t nt = mpad / (kMulttThreads * kMulttR);
  return std::max<int64_t>(1, std::min<int64_t>(nt, static_cast<int64_t>(num_sms) * 3));
}

template <int DIM>
cudaError_t launch_mult(const SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad,
                        int64_t m, float* out32, double* out64, int64_t t0, int64_t nt,
                        int num_sms) {
  const bool ga = p.total > kSubMaxPositions;
  const size_t sm = sizeof(int4) * (kSDT * DIM + kSDT) +
                    sizeof(float2) * DIM * kActR * kActThreads + (ga ? 0 : sizeof(float) * p.total);
  auto kern = ga ? sub_mult_act_kernel<DIM, true> : sub_mult_act_kernel<DIM, false>;
  cudaError_t e = set_smem_cap(kern, sm);
  if (e != cudaSuccess) return e;
  const int64_t blocks = std::min<int64_t>(nt, static_cast<int64_t>(num_sms) * 8);
  kern<<<static_cast<unsigned>(std::max<int64_t>(blocks, 1)), kActThreads, sm, s>>>(
      p.act, p.sact, p.n_sub, p.asub, static_cast<int>(p.total), xt, mpad, m, t0, nt, out32, out64);
  return cudaGetLastError();
}

template <int DIM>
cudaError_t launch_mult_df(const SubPlan& p, cudaStream_t s, const float* xh, const float* xl,
                           int64_t mpad, int64_t m, double* out64, int64_t t0, int64_t nt,
                           int num_sms) {
  const bool ga = p.total > kSubMaxPositions;
  const size_t sm = sizeof(int4) * kSDT * DIM + sizeof(uint32_t) * kSDT + (ga ? 0 : sizeof(float2) * p.total);
  auto kern = ga ? sub_mult_df_kernel<DIM, true> : sub_mult_df_kernel<DIM, false>;
  cudaError_t e = set_smem_cap(kern, sm);
  if (e != cudaSuccess) return e;
  const int64_t blocks = std::min<int64_t>(nt, static_cast<int64_t>(num_sms) * 8);
  kern<<<static_cast<unsigned>(std::max<int64_t>(blocks, 1)), kDfThreads, sm, s>>>(
      p.desc, p.base, p.n_sub, p.asub2, static_cast<int>(p.total), xh, xl, mpad, m, t0, nt, out64);
  return cudaGetLastError();
}

template <int DIM>
cudaError_t launch_multt(const SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad,
                         int64_t m, const float* v, int num_sms) {
  const size_t sm = multt_smem(DIM, p.total);
  cudaError_t e = set_smem_cap(sub_multt_kernel<DIM>, sm);
  if (e != cudaSuccess) return e;
  const int64_t nt = mpad / (kMulttThreads * kMulttR);
  const int64_t blocks = multt_blocks(mpad, num_sms);
  sub_multt_kernel<DIM><<<static_cast<unsigned>(blocks), kMulttThreads, sm, s>>>(
      p.desc, p.base, p.n_sub, static_cast<int>(p.total), xt, mpad, m, nt, v, p.maxbits,
      static_cast<float>(std::max<int64_t>(m, 1)), p.acc);
  return cudaGetLastError();
}

// threads (subspaces) per CTA of the owner-computes multTranspose: one per subspace up to the
// kernel's width, fewer when the per-thread cell sums (cmax of them) would overflow the shared
// memory budget next to the staged rows
int own_threads(const SubPlan& p, bool df) {
  const int64_t w = df ? (2 * p.dim + 2 + 3) / 4 * 4 : (2 + 2 * p.dim + 3) / 4 * 4;
  const int64_t rows = static_cast<int64_t>(sizeof(float)) * kOwnTile * w;
  const int64_t per = (df ? 8 : 4) * std::max(p.cmax, 1);
  const int64_t fit = (static_cast<int64_t>(kOwnSmemBudget) - rows) / per / 32 * 32;
  int64_t t = std::min<int64_t>(df ? kOwnMaxThreads : kActOwnThreads, (p.n_sub + 31) / 32 * 32);
  t = std::min<int64_t>(t, std::max<int64_t>(fit, 32));
  return static_cast<int>(t);
}

size_t own_smem(const SubPlan& p, int dim, bool df) {
  const int w = df ? (2 * dim + 2 + 3) / 4 * 4 : (dim + 1 + 3) / 4 * 4;
  return sizeof(float) * kOwnTile * w +
         (df ? sizeof(float2) : sizeof(float)) * static_cast<size_t>(p.cmax) * own_threads(p, df);
}

template <int DIM, bool DF>
cudaError_t launch_multt_own(const SubPlan& p, cudaStream_t s, const float* xh, const float* xl,
                             int64_t mpad, int64_t m, const float* vh, const float* vl,
                             int num_sms) {
  auto kern = sub_multt_own_kernel<DIM, DF>;
  const size_t sm = own_smem(p, DIM, DF);
  const int nth = own_threads(p, DF);
  cudaError_t e = set_smem_cap(kern, sm);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nth, sm);
  if (e != cudaSuccess) return e;
  const int64_t nt = mpad / kOwnTile;
  // a fixed grid for a given device and plan: the row count, and with it the summation order,
  // does not change between calls
  const int64_t rows = std::min<int64_t>(std::max(1, per_sm) * static_cast<int64_t>(num_sms), std::min<int64_t>(p.row_cap, std::max<int64_t>(nt, 1)));
  kern<<<static_cast<unsigned>(rows), nth, sm, s>>>(p.desc, p.sinfo, p.n_sub, p.cmax,
                                                    static_cast<int>(p.total), xh, xl, mpad, m, vh,
                                                    vl, nt, p.rows);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  sum_rows_kernel<<<static_cast<unsigned>((p.total + 31) / 32), dim3(32, kSumRowGroups), 0, s>>>(
      p.rows, static_cast<int>(rows), p.total, reinterpret_cast<double*>(p.acc));
  return cudaGetLastError();
}

size_t act_own_smem(const SubPlan& p, int dim) {
  return sizeof(float) * kOwnTile * ((2 + 2 * dim + 3) / 4 * 4) +
         sizeof(float) * static_cast<size_t>(p.cmax) * own_threads(p, false);
}

template <int DIM>
cudaError_t launch_multt_act(const SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad,
                             int64_t m, const float* v, int num_sms) {
  auto kern = sub_multt_act_kernel<DIM>;
  const size_t sm = act_own_smem(p, DIM);
  const int nth = own_threads(p, false);
  cudaError_t e = set_smem_cap(kern, sm);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nth, sm);
  if (e != cudaSuccess) return e;
  const int64_t nt = mpad / kOwnTile;
  const int64_t rows = std::min<int64_t>(std::max(1, per_sm) * static_cast<int64_t>(num_sms), std::min<int64_t>(p.row_cap, std::max<int64_t>(nt, 1)));
  kern<<<static_cast<unsigned>(rows), nth, sm, s>>>(p.act, p.sact, p.n_sub, p.cmax,
                                                    static_cast<int>(p.total), xt, mpad, m, v, nt,
                                                    p.rows);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  sum_rows_kernel<<<static_cast<unsigned>((p.total + 31) / 32), dim3(32, kSumRowGroups), 0, s>>>(
      p.rows, static_cast<int>(rows), p.total, reinterpret_cast<double*>(p.acc));
  return cudaGetLastError();
}

}  // namespace

bool subspace_build(SubPlan* p, int dim, int64_t n, const double* level_pow2, const double* index,
                    cudaStream_t stream, std::string* err) {
  subspace_free(p);
  p->stream = stream;
  if (dim < 1 || dim > 16 || n < 1) {
    *err = "subspace kernels need 1 <= dim <= 16 and a non-empty grid";
    return false;
  }
  // group grid points by level vector
  std::map<std::vector<int>, std::vector<int64_t>> groups;
  std::vector<int> lv(dim);
  for (int64_t g = 0; g < n; ++g) {
    for (int t = 0; t < dim; ++t) {
      int e = 0;
      std::frexp(level_pow2[g * dim + t], &e);
      lv[t] = e - 1;  // 2^l
      if (lv[t] < 1 || lv[t] > 20) {
        *err = "subspace kernels need levels in [1, 20]";
        return false;
      }
    }
    groups[lv].push_back(g);
  }
  std::vector<int4> desc, sinfo, act, sact;
  std::vector<uint32_t> base;
  int64_t cmax = 0;
  int na_max = 0;
  int64_t act_work = 0;
  // subspaces in order of their number of active (level > 1) dimensions, so that neighbouring
  // threads of the owner-computes kernels run the same number of evaluations
  std::vector<const std::pair<const std::vector<int>, std::vector<int64_t>>*> order;
  for (const auto& kv : groups) order.push_back(&kv);
  auto n_active = [](const std::vector<int>& l) {
    return static_cast<int>(std::count_if(l.begin(), l.end(), [](int v) { return v > 1; }));
  };
  std::stable_sort(order.begin(), order.end(), [&](const auto* a, const auto* b) {
    return n_active(a->first) < n_active(b->first);
  });
  std::vector<int> pos(static_cast<size_t>(n));
  int64_t offset = 0;
  for (const auto* kvp : order) {
    const auto& kv = *kvp;
    const std::vector<int>& l = kv.first;
    std::vector<int64_t> stride(dim);
    int64_t size = 1;
    for (int t = dim - 1; t >= 0; --t) {  // row-major over dimensions
      stride[t] = size;
      size *= int64_t(1) << (l[t] - 1);
    }
    if (offset + size > kSubMaxTotal) {
      *err = "grid has more subspace positions than the subspace kernels index";
      return false;
    }
    uint32_t b = static_cast<uint32_t>(offset);
    for (int t = 0; t < dim; ++t) {
      const float S = std::ldexp(1.0f, l[t] - 1);
      const float L = std::ldexp(1.0f, l[t]);
      int4 q;
      std::memcpy(&q.x, &S, 4);
      std::memcpy(&q.y, &L, 4);
      q.z = static_cast<int>(stride[t]);
      q.w = 0;
      desc.push_back(q);
      b -= kMagicBits * static_cast<uint32_t>(stride[t]);  // mod 2^32
    }
    base.push_back(b);
    sinfo.push_back(make_int4(static_cast<int>(offset), static_cast<int>(size),
                              static_cast<int>(b - static_cast<uint32_t>(offset)), 0));
    cmax = std::max(cmax, size);
    // active dimensions: (t, S bits, L bits, stride); the base counts only their magic offsets
    uint32_t cb = 0;
    int na = 0;
    for (int t = 0; t < dim; ++t) {
      if (l[t] <= 1) continue;
      const float S = std::ldexp(1.0f, l[t] - 1);
      const float L = std::ldexp(1.0f, l[t]);
      int4 q;
      q.x = t;
      std::memcpy(&q.y, &S, 4);
      std::memcpy(&q.z, &L, 4);
      q.w = static_cast<int>(stride[t]);
      act.push_back(q);
      cb -= kMagicBits * static_cast<uint32_t>(stride[t]);
      ++na;
    }
    for (int t = na; t < dim; ++t) act.push_back(make_int4(0, 0, 0, 0));
    na_max = std::max(na_max, na);
    act_work += na;
    sact.push_back(make_int4(static_cast<int>(static_cast<uint32_t>(offset) + cb),
                             static_cast<int>(size), static_cast<int>(cb), na));
    for (int64_t g : kv.second) {
      int64_t f = offset;
      for (int t = 0; t < dim; ++t) f += ((static_cast<int64_t>(index[g * dim + t]) - 1) / 2) * stride[t];
      pos[g] = static_cast<int>(f);
    }
    offset += size;
  }
  p->dim = dim;
  p->n_sub = static_cast<int>(groups.size());
  p->total = offset;
  p->h_pos = pos;
  p->h_sub.clear();
  for (const int4& q : sinfo) p->h_sub.push_back(make_int2(q.x, q.y));
  p->n = n;
  p->cmax = static_cast<int>(cmax);
  p->na_max = na_max;
  p->act_work = act_work;
  // partial rows of the owner-computes multTranspose: up to 16 CTAs per SM (fewer for wide CTAs),
  // at most 256 MB
  int dev = 0, sms = 1;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    *err = "subspace plan: device query failed";
    return false;
  }
  const int nth = own_threads(*p, false);
  p->row_cap = std::min<int64_t>(static_cast<int64_t>(sms) * std::min(16, std::max(2, 1024 / nth)),
                                 std::max<int64_t>(1, (int64_t(256) << 20) / (8 * offset)));
  auto alloc = [&](auto** q, size_t bytes) { return dev_malloc(q, bytes, stream) == cudaSuccess; };
  auto put = [&](void* dst, const void* src, size_t bytes) {
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream) == cudaSuccess;
  };
  bool ok = alloc(&p->desc, sizeof(int4) * desc.size()) &&
            alloc(&p->sinfo, sizeof(int4) * sinfo.size()) &&
            alloc(&p->act, sizeof(int4) * act.size()) &&
            alloc(&p->sact, sizeof(int4) * sact.size()) &&
            alloc(&p->rows, sizeof(double) * p->row_cap * offset) &&
            alloc(&p->base, sizeof(uint32_t) * base.size()) &&
            alloc(&p->pos, sizeof(int) * pos.size()) &&
            alloc(&p->asub, sizeof(float) * offset) &&
            alloc(&p->asub2, sizeof(float2) * offset) &&
            alloc(&p->acc, sizeof(unsigned long long) * offset) &&
            alloc(&p->maxbits, sizeof(unsigned int));
  // (pageable sources: each copy has taken the data when it returns)
  ok = ok && put(p->desc, desc.data(), sizeof(int4) * desc.size()) &&
       put(p->sinfo, sinfo.data(), sizeof(int4) * sinfo.size()) &&
       put(p->act, act.data(), sizeof(int4) * act.size()) &&
       put(p->sact, sact.data(), sizeof(int4) * sact.size()) &&
       put(p->base, base.data(), sizeof(uint32_t) * base.size()) &&
       put(p->pos, pos.data(), sizeof(int) * pos.size());
  if (!ok) {
    subspace_free(p);
    *err = "subspace plan allocation failed";
    return false;
  }
  if (p->total > kSubMaxPositions && !subspace_owner_fits(*p, false)) {
    subspace_free(p);
    *err = "grid has too many positions for the fixed-point scatter and a subspace too wide for "
           "the owner-computes multTranspose";
    return false;
  }
  return true;
}

void subspace_free(SubPlan* p) {
  const cudaStream_t st = p->stream;
  void* ptrs[] = {p->desc, p->sinfo, p->act,  p->sact,    p->pmat,  p->pmat_lo, p->pmat16,
                  p->cmat, p->cpair, p->rows, p->base, p->pos,  p->asub,    p->asub2,
                  p->acc,  p->maxbits};
  for (void* q : ptrs) dev_free(q, st);
  *p = SubPlan{};
}

#define SUB_DIMS(F) F(1) F(2) F(3) F(4) F(5) F(6) F(7) F(8) F(9) F(10) F(11) F(12) F(13) F(14) F(15) F(16)

cudaError_t subspace_scatter_alpha(const SubPlan& p, cudaStream_t s, const float* alpha32) {
  cudaError_t e = cudaMemsetAsync(p.asub, 0, sizeof(float) * p.total, s);
  if (e != cudaSuccess) return e;
  scatter_alpha_kernel<<<static_cast<unsigned>(std::min<int64_t>(1216, (p.n + 255) / 256)), 256, 0, s>>>(
      alpha32, p.pos, p.n, p.asub);
  return cudaGetLastError();
}

cudaError_t subspace_mat_build(const SubPlan& p, cudaStream_t s, const float* xh,
                               const float* xl, int64_t mpad, int64_t m, int num_sms) {
  switch (p.dim) {
#define F(D) \
  case D:    \
    return launch_mat_build<D>(p, s, xh, xl, mpad, m, num_sms);
    SUB_DIMS(F)
#undef F
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t subspace_scatter_alpha_df(const SubPlan& p, cudaStream_t s, const float* ah,
                                      const float* al) {
  cudaError_t e = cudaMemsetAsync(p.asub2, 0, sizeof(float2) * p.total, s);
  if (e != cudaSuccess) return e;
  scatter_alpha_df_kernel<<<static_cast<unsigned>(std::min<int64_t>(1216, (p.n + 255) / 256)), 256, 0, s>>>(
      ah, al, p.pos, p.n, p.asub2);
  return cudaGetLastError();
}

cudaError_t subspace_finish_rows(const SubPlan& p, cudaStream_t s, int64_t nrows, int64_t npad,
                                 double* out64, const double* add, double scale_add) {
  sum_rows_kernel<<<static_cast<unsigned>((p.total + 31) / 32), dim3(32, kSumRowGroups), 0, s>>>(
      p.rows, static_cast<int>(nrows), p.total, reinterpret_cast<double*>(p.acc));
  gather_sums_kernel<<<static_cast<unsigned>(std::min<int64_t>(1216, (npad + 255) / 256)), 256, 0, s>>>(
      reinterpret_cast<const double*>(p.acc), p.pos, p.n, npad, add, scale_add, out64);
  return cudaGetLastError();
}

cudaError_t subspace_mult(const SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad,
                          int64_t m, const float* alpha32, float* out32, double* out64,
                          int64_t j_begin, int64_t j_end, int num_sms) {
  cudaError_t e = subspace_scatter_alpha(p, s, alpha32);
  if (e != cudaSuccess) return e;
  const int64_t tile = kActR * kActThreads;
  const int64_t t0 = j_begin / tile;
  const int64_t nt = (j_end + tile - 1) / tile - t0;
  if (nt <= 0) return cudaGetLastError();
  switch (p.dim) {
#define F(D) \
  case D:    \
    return launch_mult<D>(p, s, xt, mpad, m, out32, out64, t0, nt, num_sms);
    SUB_DIMS(F)
#undef F
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t subspace_mult_df(const SubPlan& p, cudaStream_t s, const float* xh, const float* xl,
                             int64_t mpad, int64_t m, const float* ah, const float* al,
                             double* out64, int64_t j_begin, int64_t j_end, int num_sms) {
  cudaError_t e = cudaMemsetAsync(p.asub2, 0, sizeof(float2) * p.total, s);
  if (e != cudaSuccess) return e;
  scatter_alpha_df_kernel<<<static_cast<unsigned>(std::min<int64_t>(1216, (p.n + 255) / 256)), 256, 0, s>>>(
      ah, al, p.pos, p.n, p.asub2);
  const int64_t tile = kDfThreads * kDfR;
  const int64_t t0 = j_begin / tile;
  const int64_t nt = (j_end + tile - 1) / tile - t0;
  if (nt <= 0) return cudaGetLastError();
  switch (p.dim) {
#define F(D) \
  case D:    \
    return launch_mult_df<D>(p, s, xh, xl, mpad, m, out64, t0, nt, num_sms);
    SUB_DIMS(F)
#undef F
    default:
      return cudaErrorInvalidValue;
  }
}

namespace {

cudaError_t own_finish(const SubPlan& p, cudaStream_t s, int64_t npad, double* out64,
                       const double* add, double scale_add) {
  gather_sums_kernel<<<static_cast<unsigned>(std::min<int64_t>(1216, (npad + 255) / 256)), 256, 0, s>>>(
      reinterpret_cast<const double*>(p.acc), p.pos, p.n, npad, add, scale_add, out64);
  return cudaGetLastError();
}
}  // namespace

bool subspace_owner_fits(const SubPlan& p, bool df) {
  const size_t sm = df ? own_smem(p, p.dim, true) : act_own_smem(p, p.dim);
  return p.n_sub > 0 && p.cmax > 0 && p.rows != nullptr && sm <= kOwnSmemBudget;
}

cudaError_t subspace_multt(const SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad,
                           int64_t m, const float* v32, int64_t npad, double* out64,
                           const double* add, double scale_add, int num_sms) {
  cudaError_t e = cudaSuccess;
  if (subspace_owner_fits(p, false)) {
    switch (p.dim) {
#define F(D)                                                                                 \
  case D:                                                                                    \
    e = launch_multt_act<D>(p, s, xt, mpad, m, v32, num_sms);                                \
    break;
      SUB_DIMS(F)
#undef F
      default:
        return cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    return own_finish(p, s, npad, out64, add, scale_add);
  }
  if (p.total > kSubMaxPositions) return cudaErrorInvalidValue;  // (rejected at build)
  e = cudaMemsetAsync(p.maxbits, 0, sizeof(unsigned int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(p.acc, 0, sizeof(unsigned long long) * p.total, s);
  if (e != cudaSuccess) return e;
  maxabs_kernel<<<static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>(608, (m + 255) / 256))), 256, 0, s>>>(
      v32, m, p.maxbits);
  switch (p.dim) {
#define F(D)                                                  \
  case D:                                                     \
    e = launch_multt<D>(p, s, xt, mpad, m, v32, num_sms);     \
    break;
    SUB_DIMS(F)
#undef F
    default:
      return cudaErrorInvalidValue;
  }
  if (e != cudaSuccess) return e;
  gather_result_kernel<<<static_cast<unsigned>(std::min<int64_t>(1216, (npad + 255) / 256)), 256, 0, s>>>(
      p.acc, p.pos, p.n, npad, p.maxbits, static_cast<float>(std::max<int64_t>(m, 1)), add,
      scale_add, out64);
  return cudaGetLastError();
}

cudaError_t subspace_multt_df(const SubPlan& p, cudaStream_t s, const float* xh, const float* xl,
                              int64_t mpad, int64_t m, const float* vh, const float* vl,
                              int64_t npad, double* out64, const double* add, double scale_add,
                              int num_sms) {
  if (!subspace_owner_fits(p, true)) return cudaErrorInvalidValue;
  cudaError_t e = cudaSuccess;
  switch (p.dim) {
#define F(D)                                                                   \
  case D:                                                                      \
    e = launch_multt_own<D, true>(p, s, xh, xl, mpad, m, vh, vl, num_sms);     \
    break;
    SUB_DIMS(F)
#undef F
    default:
      return cudaErrorInvalidValue;
  }
  if (e != cudaSuccess) return e;
  return own_finish(p, s, npad, out64, add, scale_add);
}

}  // namespace sgmev

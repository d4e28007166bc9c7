// Materialised subspace products (FP32). For a fixed data set and grid the product
// p_s(x_j) = prod_t h_{l_t}(x_{j,t}) of the one possibly non-zero basis function of subspace s at
// point j does not change between calls, so it is computed once (mat_build_kernel) and kept in
// HBM as P[g][s][4] (g = j / 4, s padded to a multiple of 32, FP32: 4 bytes per point and
// subspace). mult and multTranspose then stream P once per call: they are bounded by HBM
// bandwidth instead of the hat arithmetic. The cell index of (j, s) is recomputed from x (one
// rounded-down FMA and one integer multiply-add per active dimension) rather than stored.
//
// Both kernels are owner-computes: thread k of a pass owns subspace s = pass * blockDim + k and
// walks the CTA's tiles of points; a warp reads P[g][32 consecutive s][4] as 512 contiguous bytes.
//   mult:  lane s forms alpha_s[cell] * p for 4 points; a butterfly over the warp (xor 16, 8, then
//          4, 2, 1) reduces the 4 values to 4 per-point sums, which go to per-warp partials in
//          shared memory; after all passes the partials are added in warp order.
//   multT: lane s adds v_j * p into its cells ([cell][thread] in shared memory, conflict-free) and
//          flushes them into the CTA's FP64 row every kFlushTiles tiles; rows are added in CTA
//          order.
// Every sum has a fixed order, so results are the same bit for bit from run to run.
#include <cuda_runtime.h>

#include <algorithm>

#include "subspace.h"
#include "subspace_common.cuh"

namespace sgmev {
namespace {

using namespace subk;

constexpr int kMatThreads = 512;              // subspaces per pass
constexpr int kGroups = kOwnTile / 4;         // point groups per tile
constexpr int kMatWarps = kMatThreads / 32;
// point groups in flight per thread: a ring of loads issued this many groups ahead of their use
// (kGroups is a multiple of both)
constexpr int kMultAhead = 4, kMulttAhead = 4;
static_assert(kGroups % kMultAhead == 0 && kGroups % kMulttAhead == 0, "ring must divide a tile");
// multT: FP32 sums over this many tiles (1024 points) before they go into the FP64 row
constexpr int kFlushTiles = 4;

// rows of a tile for the cell recomputation: (v or 0, x_0, ..., x_{d-1}); points outside the
// domain get x = 0.5 (their P entries are 0)
template <int DIM>
struct MatRow {
  static constexpr int W = (1 + DIM + 3) / 4 * 4;
};

template <int DIM>
__device__ __forceinline__ void mat_stage_tile(float* s_pt, int64_t tile,
                                               const float* __restrict__ xt, int64_t mpad,
                                               int64_t m, const float* __restrict__ v) {
  constexpr int W = MatRow<DIM>::W;
  const int64_t j0 = tile * kOwnTile;
  for (int k = threadIdx.x; k < kOwnTile * DIM; k += blockDim.x) {
    const int t = k / kOwnTile, jj = k - t * kOwnTile;
    s_pt[jj * W + 1 + t] = xt[static_cast<int64_t>(t) * mpad + j0 + jj];
  }
  __syncthreads();
  for (int jj = threadIdx.x; jj < kOwnTile; jj += blockDim.x) {
    float* row = s_pt + jj * W;
    const int64_t j = j0 + jj;
    bool inside = j < m;
#pragma unroll
    for (int t = 0; t < DIM; ++t) inside = inside && act_inside(row[1 + t]);
    if (!inside) {
#pragma unroll
      for (int t = 0; t < DIM; ++t) row[1 + t] = 0.5f;
    }
    row[0] = (v && inside) ? v[j] : 0.0f;
  }
  __syncthreads();
}

// cell index of a subspace with active dimensions q[0 .. na) at a row (x at offset 1 + t)
__device__ __forceinline__ uint32_t mat_cell(const float* __restrict__ row,
                                             const int4* __restrict__ q, int na, uint32_t cbase) {
  uint32_t c = cbase;
  for (int a = 0; a < na; ++a) {
    const int4 d = q[a];
    c += __float_as_uint(__fmaf_rd(row[1 + d.x], __int_as_float(d.y), kMagic)) *
         static_cast<uint32_t>(d.w);
  }
  return c;
}

// registers for up to NA active dimensions
template <int NA>
struct MatDesc {
  int off[NA > 0 ? NA : 1];
  float S[NA > 0 ? NA : 1];
  uint32_t st[NA > 0 ? NA : 1];
  __device__ __forceinline__ void load(const int4* __restrict__ q) {
#pragma unroll
    for (int a = 0; a < NA; ++a) {
      off[a] = 1 + q[a].x;
      S[a] = __int_as_float(q[a].y);
      st[a] = static_cast<uint32_t>(q[a].w);
    }
  }
  __device__ __forceinline__ uint32_t cell(const float* __restrict__ row, uint32_t cbase) const {
    uint32_t c = cbase;
#pragma unroll
    for (int a = 0; a < NA; ++a) c += __float_as_uint(__fmaf_rd(row[off[a]], S[a], kMagic)) * st[a];
    return c;
  }
};

// ---- build -----------------------------------------------------------------------------
template <int NA>
__device__ __forceinline__ void build_tile(const float* __restrict__ s_pt, int w,
                                           const int4* __restrict__ q, int na, uint32_t cbase,
                                           float4* __restrict__ dst, int64_t s_pad) {
  ActDesc<(NA > 0 ? NA : 1)> desc;
  if (NA > 0) desc.load(q);
  for (int g = 0; g < kGroups; ++g) {
    float pv[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float* row = s_pt + (4 * g + i) * w;
      uint32_t c;
      pv[i] = NA > 0 ? desc.eval(row, cbase, c)
                     : (NA == 0 ? row[0] : act_eval_dyn(row, q, na, cbase, c));
    }
    dst[static_cast<int64_t>(g) * s_pad] = make_float4(pv[0], pv[1], pv[2], pv[3]);
  }
}

template <int DIM>
__global__ void __launch_bounds__(kMatThreads, 1) mat_build_kernel(
    const int4* __restrict__ act, const int4* __restrict__ sact, int n_sub, int s_pad,
    const float* __restrict__ xt, int64_t mpad, int64_t m, int64_t n_tiles,
    float4* __restrict__ pm) {
  constexpr int W = ActRow<DIM>::W;
  extern __shared__ __align__(16) unsigned char smem[];
  float* s_pt = reinterpret_cast<float*>(smem);  // [kOwnTile][W]
  const int tid = threadIdx.x;
  for (int s0 = 0; s0 < s_pad; s0 += blockDim.x) {
    const int sid = s0 + tid;
    const bool real = sid < n_sub;
    const int4 info = real ? sact[sid] : make_int4(0, 0, 0, 0);
    const int4* q = act + static_cast<int64_t>(real ? sid : 0) * DIM;
    for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
      __syncthreads();
      act_stage_tile<DIM>(s_pt, tile, xt, mpad, m, nullptr);
      if (sid >= s_pad) continue;
      float4* dst = pm + tile * kGroups * static_cast<int64_t>(s_pad) + sid;
      if (!real) {
        for (int g = 0; g < kGroups; ++g)
          dst[static_cast<int64_t>(g) * s_pad] = make_float4(0.f, 0.f, 0.f, 0.f);
        continue;
      }
      const uint32_t cbase = static_cast<uint32_t>(info.z);
      switch (info.w) {
        case 0: build_tile<0>(s_pt, W, q, 0, cbase, dst, s_pad); break;
        case 1: build_tile<1>(s_pt, W, q, 1, cbase, dst, s_pad); break;
        case 2: build_tile<(DIM < 2 ? DIM : 2)>(s_pt, W, q, 2, cbase, dst, s_pad); break;
        case 3: build_tile<(DIM < 3 ? DIM : 3)>(s_pt, W, q, 3, cbase, dst, s_pad); break;
        case 4: build_tile<(DIM < 4 ? DIM : 4)>(s_pt, W, q, 4, cbase, dst, s_pad); break;
        default: build_tile<-1>(s_pt, W, q, info.w, cbase, dst, s_pad); break;
      }
    }
  }
}

// ---- mult --------------------------------------------------------------------------------
// lane sums of 4 values -> the 32-lane sum of value (2 * bit4 + bit3) of the lane index
__device__ __forceinline__ float reduce4(float v0, float v1, float v2, float v3, int lane) {
  const bool hi = lane & 16;
  float a0 = hi ? v2 : v0, a1 = hi ? v3 : v1;
  const float s0 = hi ? v0 : v2, s1 = hi ? v1 : v3;
  a0 += __shfl_xor_sync(0xffffffffu, s0, 16);
  a1 += __shfl_xor_sync(0xffffffffu, s1, 16);
  const bool b3 = lane & 8;
  float b = b3 ? a1 : a0;
  b += __shfl_xor_sync(0xffffffffu, b3 ? a0 : a1, 8);
  b += __shfl_xor_sync(0xffffffffu, b, 4);
  b += __shfl_xor_sync(0xffffffffu, b, 2);
  b += __shfl_xor_sync(0xffffffffu, b, 1);
  return b;
}

template <int NA>
__device__ __forceinline__ void mult_tile(const float* __restrict__ s_pt, int w,
                                          const int4* __restrict__ q, int na, uint32_t cbase,
                                          int cmax, const float* __restrict__ s_at, int s_pad_a,
                                          int sid, const float4* __restrict__ src, int64_t s_pad,
                                          float* __restrict__ s_part, bool first, int lane) {
  MatDesc<(NA > 0 ? NA : 1)> desc;
  if (NA > 0) desc.load(q);
  const float* a_col = s_at + sid;
  float4 ring[kMultAhead];
#pragma unroll
  for (int u = 0; u < kMultAhead; ++u) ring[u] = __ldcs(src + static_cast<int64_t>(u) * s_pad);
  for (int g0 = 0; g0 < kGroups; g0 += kMultAhead) {
#pragma unroll
    for (int u = 0; u < kMultAhead; ++u) {
      const int g = g0 + u;
      const float4 cur = ring[u];
      if (g + kMultAhead < kGroups) ring[u] = __ldcs(src + static_cast<int64_t>(g + kMultAhead) * s_pad);
      float cv[4];
      const float pp[4] = {cur.x, cur.y, cur.z, cur.w};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float* row = s_pt + (4 * g + i) * w;
        const uint32_t c = NA > 0 ? desc.cell(row, cbase) : (NA == 0 ? cbase : mat_cell(row, q, na, cbase));
        cv[i] = a_col[min(c, static_cast<uint32_t>(cmax - 1)) * s_pad_a] * pp[i];
      }
      const float r = reduce4(cv[0], cv[1], cv[2], cv[3], lane);
      if ((lane & 7) == 0) {
        float* dst = s_part + 4 * g + (lane >> 3);
        *dst = first ? r : *dst + r;
      }
    }
  }
}

template <int DIM>
__global__ void __launch_bounds__(kMatThreads, 2) mat_mult_kernel(
    const int4* __restrict__ act, const int4* __restrict__ sact, int n_sub, int s_pad, int cmax,
    const float* __restrict__ asub, const float* __restrict__ xt, int64_t mpad, int64_t m,
    int64_t tile_begin, int64_t n_tiles, const float4* __restrict__ pm,
    float* __restrict__ out32, double* __restrict__ out64) {
  constexpr int W = MatRow<DIM>::W;
  extern __shared__ __align__(16) unsigned char smem[];
  float* s_pt = reinterpret_cast<float*>(smem);          // [kOwnTile][W]
  float* s_part = s_pt + kOwnTile * W;                    // [warps][kOwnTile]
  float* s_at = s_part + kMatWarps * kOwnTile;            // [cmax][s_pad] alpha by (cell, subspace)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // alpha transposed: s_at[c * s_pad + s] = alpha at position offset_s + c (0 beyond the cells)
  for (int k = tid; k < cmax * s_pad; k += blockDim.x) {
    const int c = k / s_pad, sidx = k - c * s_pad;
    float a = 0.0f;
    if (sidx < n_sub) {
      const int4 info = sact[sidx];
      const int off = static_cast<int>(static_cast<uint32_t>(info.x) - static_cast<uint32_t>(info.z));
      if (c < info.y) a = asub[off + c];
    }
    s_at[k] = a;
  }
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t gt = tile_begin + tile;
    __syncthreads();  // previous tile's rows and partials are consumed
    mat_stage_tile<DIM>(s_pt, gt, xt, mpad, m, nullptr);
    for (int s0 = 0; s0 < s_pad; s0 += blockDim.x) {
      const int sid = s0 + tid;
      if (s0 + warp * 32 < s_pad) {  // whole warps: s_pad is a multiple of 32
        const bool real = sid < n_sub;
        const int4 info = real ? sact[sid] : make_int4(0, 0, 0, 0);
        const int4* q = act + static_cast<int64_t>(real ? sid : 0) * DIM;
        const uint32_t cbase = static_cast<uint32_t>(info.z);
        const float4* src = pm + gt * kGroups * static_cast<int64_t>(s_pad) + sid;
        float* part = s_part + warp * kOwnTile;
        const bool first = s0 == 0;
        // the butterfly needs the whole warp on one path: dispatch on the warp's largest count
        // (descriptor entries past a subspace's own count are zero: S = 0 and stride 0 leave the
        // cell index unchanged)
        const int na = __reduce_max_sync(0xffffffffu, info.w);
        switch (na) {
          case 0: mult_tile<0>(s_pt, W, q, 0, cbase, cmax, s_at, s_pad, sid, src, s_pad, part, first, lane); break;
          case 1: mult_tile<1>(s_pt, W, q, 1, cbase, cmax, s_at, s_pad, sid, src, s_pad, part, first, lane); break;
          case 2: mult_tile<(DIM < 2 ? DIM : 2)>(s_pt, W, q, 2, cbase, cmax, s_at, s_pad, sid, src, s_pad, part, first, lane); break;
          case 3: mult_tile<(DIM < 3 ? DIM : 3)>(s_pt, W, q, 3, cbase, cmax, s_at, s_pad, sid, src, s_pad, part, first, lane); break;
          case 4: mult_tile<(DIM < 4 ? DIM : 4)>(s_pt, W, q, 4, cbase, cmax, s_at, s_pad, sid, src, s_pad, part, first, lane); break;
          default: mult_tile<-1>(s_pt, W, q, na, cbase, cmax, s_at, s_pad, sid, src, s_pad, part, first, lane); break;
        }
      }
    }
    __syncthreads();
    // warp w wrote its partials in pass 0 iff w * 32 < s_pad (s_pad is a multiple of 32)
    const int wrote = min(kMatWarps, s_pad / 32);
    for (int jj = tid; jj < kOwnTile; jj += blockDim.x) {
      float r = 0.0f;
      for (int w = 0; w < wrote; ++w) r += s_part[w * kOwnTile + jj];
      const int64_t j = gt * kOwnTile + jj;
      const float v = j < m ? r : 0.0f;
      if (out32) out32[j] = v;
      if (out64) out64[j] = static_cast<double>(v);
    }
  }
}

// ---- multTranspose -------------------------------------------------------------------------
template <int NA>
__device__ __forceinline__ void multt_tile(const float* __restrict__ s_pt, int w,
                                           const int4* __restrict__ q, int na, uint32_t cbase,
                                           int cmax, const float4* __restrict__ src,
                                           int64_t s_pad, float* __restrict__ acc, int nth) {
  MatDesc<(NA > 0 ? NA : 1)> desc;
  if (NA > 0) desc.load(q);
  float4 ring[kMulttAhead];
#pragma unroll
  for (int u = 0; u < kMulttAhead; ++u) ring[u] = __ldcs(src + static_cast<int64_t>(u) * s_pad);
  for (int g0 = 0; g0 < kGroups; g0 += kMulttAhead) {
#pragma unroll
    for (int u = 0; u < kMulttAhead; ++u) {
      const float4 cur = ring[u];
      const int gn = g0 + u + kMulttAhead;
      if (gn < kGroups) ring[u] = __ldcs(src + static_cast<int64_t>(gn) * s_pad);
      const float pp[4] = {cur.x, cur.y, cur.z, cur.w};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float* row = s_pt + (4 * (g0 + u) + i) * w;
        const uint32_t c = NA > 0 ? desc.cell(row, cbase) : (NA == 0 ? cbase : mat_cell(row, q, na, cbase));
        acc[min(c, static_cast<uint32_t>(cmax - 1)) * nth] += row[0] * pp[i];
      }
    }
  }
}

template <int DIM>
__global__ void __launch_bounds__(kMatThreads, 2) mat_multt_kernel(
    const int4* __restrict__ act, const int4* __restrict__ sact, int n_sub, int s_pad, int cmax,
    int total, const float* __restrict__ xt, int64_t mpad, int64_t m,
    const float* __restrict__ v, int64_t n_tiles, const float4* __restrict__ pm,
    double* __restrict__ rows) {
  constexpr int W = MatRow<DIM>::W;
  extern __shared__ __align__(16) unsigned char smem[];
  float* s_pt = reinterpret_cast<float*>(smem);  // [kOwnTile][W]
  float* s_acc = s_pt + kOwnTile * W;            // [cmax][blockDim]
  double* row = rows + static_cast<int64_t>(blockIdx.x) * total;
  const int tid = threadIdx.x, nth = blockDim.x;
  for (int s0 = 0; s0 < n_sub; s0 += nth) {
    const int sid = s0 + tid;
    const bool real = sid < n_sub;
    const int4 info = real ? sact[sid] : make_int4(0, 0, 0, 0);
    const uint32_t offset = static_cast<uint32_t>(info.x) - static_cast<uint32_t>(info.z);
    const uint32_t cbase = static_cast<uint32_t>(info.z);
    const int4* q = act + static_cast<int64_t>(real ? sid : 0) * DIM;
    for (int c = 0; c < info.y; ++c) s_acc[c * nth + tid] = 0.0f;
    bool first = true;
    int since = 0;  // tiles summed in s_acc since the last flush
    for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
      __syncthreads();
      mat_stage_tile<DIM>(s_pt, tile, xt, mpad, m, v);
      if (real) {
        const float4* src = pm + tile * kGroups * static_cast<int64_t>(s_pad) + sid;
        float* acc = s_acc + tid;
        switch (info.w) {
          case 0: multt_tile<0>(s_pt, W, q, 0, cbase, cmax, src, s_pad, acc, nth); break;
          case 1: multt_tile<1>(s_pt, W, q, 1, cbase, cmax, src, s_pad, acc, nth); break;
          case 2: multt_tile<(DIM < 2 ? DIM : 2)>(s_pt, W, q, 2, cbase, cmax, src, s_pad, acc, nth); break;
          case 3: multt_tile<(DIM < 3 ? DIM : 3)>(s_pt, W, q, 3, cbase, cmax, src, s_pad, acc, nth); break;
          case 4: multt_tile<(DIM < 4 ? DIM : 4)>(s_pt, W, q, 4, cbase, cmax, src, s_pad, acc, nth); break;
          default: multt_tile<-1>(s_pt, W, q, info.w, cbase, cmax, src, s_pad, acc, nth); break;
        }
      }
      ++since;
      if (since == kFlushTiles || tile + gridDim.x >= n_tiles) {
        if (real) {
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
    if (real && first)  // no tile for this CTA: its row holds zeros
      for (int c = 0; c < info.y; ++c) row[offset + c] = 0.0;
  }
}

size_t mat_rows_smem(int dim, bool act_rows) {
  return sizeof(float) * kOwnTile * (act_rows ? ((2 + 2 * dim + 3) / 4 * 4) : ((1 + dim + 3) / 4 * 4));
}

int mat_threads(const SubPlan& p) {
  return static_cast<int>(std::min<int64_t>(kMatThreads, p.s_pad));
}

size_t mat_mult_smem(int dim, int cmax, int64_t s_pad) {
  return mat_rows_smem(dim, false) + sizeof(float) * kMatWarps * kOwnTile +
         sizeof(float) * static_cast<size_t>(cmax) * s_pad;
}

size_t mat_multt_smem(int dim, int cmax, int64_t s_pad) {
  return mat_rows_smem(dim, false) +
         sizeof(float) * static_cast<size_t>(cmax) * std::min<int64_t>(kMatThreads, s_pad);
}

template <int DIM>
cudaError_t launch_build(SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad, int64_t m,
                         int num_sms) {
  const size_t sm = mat_rows_smem(DIM, true);
  auto kern = mat_build_kernel<DIM>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
  if (e != cudaSuccess) return e;
  const int64_t nt = mpad / kOwnTile;
  const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(nt, 2LL * num_sms));
  kern<<<static_cast<unsigned>(blocks), mat_threads(p), sm, s>>>(p.act, p.sact, p.n_sub,
                                                                 static_cast<int>(p.s_pad), xt,
                                                                 mpad, m, nt, p.pmat);
  return cudaGetLastError();
}

template <int DIM>
cudaError_t launch_mat_mult(const SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad,
                            int64_t m, float* out32, double* out64, int64_t t0, int64_t nt,
                            int num_sms) {
  const size_t sm = mat_mult_smem(p.dim, p.cmax, p.s_pad);
  auto kern = mat_mult_kernel<DIM>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kMatThreads, sm);
  if (e != cudaSuccess) return e;
  const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(nt, static_cast<int64_t>(std::max(1, per_sm)) * num_sms));
  kern<<<static_cast<unsigned>(blocks), kMatThreads, sm, s>>>(
      p.act, p.sact, p.n_sub, static_cast<int>(p.s_pad), p.cmax, p.asub, xt, mpad, m, t0, nt,
      p.pmat, out32, out64);
  return cudaGetLastError();
}

template <int DIM>
cudaError_t launch_mat_multt(const SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad,
                             int64_t m, const float* v, int num_sms, int64_t* rows_used) {
  const size_t sm = mat_multt_smem(p.dim, p.cmax, p.s_pad);
  auto kern = mat_multt_kernel<DIM>;
  const int nth = mat_threads(p);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nth, sm);
  if (e != cudaSuccess) return e;
  const int64_t nt = mpad / kOwnTile;
  const int64_t rows = std::min<int64_t>(std::max(1, per_sm) * static_cast<int64_t>(num_sms), p.row_cap);
  kern<<<static_cast<unsigned>(rows), nth, sm, s>>>(p.act, p.sact, p.n_sub, static_cast<int>(p.s_pad),
                                                    p.cmax, static_cast<int>(p.total), xt, mpad, m,
                                                    v, nt, p.pmat, p.rows);
  *rows_used = rows;
  return cudaGetLastError();
}

#define MAT_DIMS(F) F(1) F(2) F(3) F(4) F(5) F(6) F(7) F(8) F(9) F(10) F(11) F(12) F(13) F(14) F(15) F(16)

constexpr size_t kMatSmemBudget = 200 * 1024;

}  // namespace

bool subspace_mat_fits(const SubPlan& p) {
  const int64_t s_pad = (p.n_sub + 31) / 32 * 32;
  return p.n_sub > 0 && p.cmax > 0 && p.rows != nullptr &&
         mat_mult_smem(p.dim, p.cmax, s_pad) <= kMatSmemBudget &&
         mat_multt_smem(p.dim, p.cmax, s_pad) <= kMatSmemBudget;
}

int64_t subspace_mat_bytes(const SubPlan& p, int64_t mpad) {
  return mpad * ((p.n_sub + 31) / 32 * 32) * static_cast<int64_t>(sizeof(float));
}

cudaError_t subspace_materialize(SubPlan* p, cudaStream_t s, const float* xt, int64_t mpad,
                                 int64_t m, int num_sms) {
  if (p->pmat) {
    cudaFree(p->pmat);
    p->pmat = nullptr;
  }
  p->s_pad = (p->n_sub + 31) / 32 * 32;
  p->mat_mpad = mpad;
  cudaError_t e = cudaMalloc(&p->pmat, static_cast<size_t>(subspace_mat_bytes(*p, mpad)));
  if (e != cudaSuccess) {
    p->pmat = nullptr;
    (void)cudaGetLastError();
    return e;
  }
  switch (p->dim) {
#define F(D)                                                 \
  case D:                                                    \
    e = launch_build<D>(*p, s, xt, mpad, m, num_sms);        \
    break;
    MAT_DIMS(F)
#undef F
    default:
      e = cudaErrorInvalidValue;
  }
  return e;
}

cudaError_t subspace_mult_mat(const SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad,
                              int64_t m, const float* alpha32, float* out32, double* out64,
                              int64_t j_begin, int64_t j_end, int num_sms) {
  if (!p.pmat || p.mat_mpad != mpad) return cudaErrorInvalidValue;
  cudaError_t e = subspace_scatter_alpha(p, s, alpha32);
  if (e != cudaSuccess) return e;
  const int64_t t0 = j_begin / kOwnTile;
  const int64_t nt = (j_end + kOwnTile - 1) / kOwnTile - t0;
  if (nt <= 0) return cudaSuccess;
  switch (p.dim) {
#define F(D) \
  case D:    \
    return launch_mat_mult<D>(p, s, xt, mpad, m, out32, out64, t0, nt, num_sms);
    MAT_DIMS(F)
#undef F
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t subspace_multt_mat(const SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad,
                               int64_t m, const float* v32, int64_t npad, double* out64,
                               const double* add, double scale_add, int num_sms) {
  if (!p.pmat || p.mat_mpad != mpad) return cudaErrorInvalidValue;
  cudaError_t e = cudaSuccess;
  int64_t rows = 0;
  switch (p.dim) {
#define F(D)                                                            \
  case D:                                                               \
    e = launch_mat_multt<D>(p, s, xt, mpad, m, v32, num_sms, &rows);    \
    break;
    MAT_DIMS(F)
#undef F
    default:
      return cudaErrorInvalidValue;
  }
  if (e != cudaSuccess) return e;
  return subspace_finish_rows(p, s, rows, npad, out64, add, scale_add);
}

}  // namespace sgmev

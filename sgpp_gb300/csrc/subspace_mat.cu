// Materialised subspace products (FP32). For a fixed data set and grid, the product
// p_s(x_j) = prod_t h_{l_t}(x_{j,t}) of the one possibly non-zero basis function of subspace s at
// point j, and that function's cell index c_s(x_j) within its subspace, do not change between
// calls. They are computed once (mat_build_kernel) and kept in HBM as
//     P[g][s] : float4, the products of points 4g .. 4g+3        (4 bytes per point and subspace)
//     C[g][s] : uint32, their cell indices, one byte each          (1 byte per point and subspace)
// with s padded to a multiple of 32 (padded entries 0). mult and multTranspose then stream P and
// C once per call and touch no coordinates: 5 bytes per (point, subspace) and a handful of
// instructions, so they are bounded by HBM bandwidth rather than the hat arithmetic. Points
// outside the domain have P = 0 (and cell 0), so they need no test.
//
// Both kernels are owner-computes: thread k of a pass owns subspace s = pass * blockDim + k and
// walks the CTA's tiles of points; a warp reads P[g][32 consecutive s] as 512 contiguous bytes
// (and C as 128), through a four-deep ring of loads in registers.
//   mult:  lane s forms alpha_s[c] * p for 4 points; a butterfly over the warp (xor 16, 8, then
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
constexpr int kMatMaxCells = 256;             // cell indices are stored in one byte
// point groups in flight per thread: a ring of loads issued this many groups ahead of their use
constexpr int kAhead = 4;
static_assert(kGroups % kAhead == 0, "the ring must divide a tile");
// multT: FP32 sums over this many tiles (1024 points) before they go into the FP64 row
constexpr int kFlushTiles = 4;

// ---- build -----------------------------------------------------------------------------
template <int NA>
__device__ __forceinline__ void build_tile(const float* __restrict__ s_pt, int w,
                                           const int4* __restrict__ q, int na, uint32_t cbase,
                                           float4* __restrict__ dst, uint32_t* __restrict__ cdst,
                                           int64_t s_pad) {
  ActDesc<(NA > 0 ? NA : 1)> desc;
  if (NA > 0) desc.load(q);
  for (int g = 0; g < kGroups; ++g) {
    float pv[4];
    uint32_t cells = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float* row = s_pt + (4 * g + i) * w;
      uint32_t c = cbase;
      pv[i] = NA > 0 ? desc.eval(row, cbase, c)
                     : (NA == 0 ? row[0] : act_eval_dyn(row, q, na, cbase, c));
      cells |= (c & 0xFFu) << (8 * i);
    }
    dst[static_cast<int64_t>(g) * s_pad] = make_float4(pv[0], pv[1], pv[2], pv[3]);
    cdst[static_cast<int64_t>(g) * s_pad] = cells;
  }
}

template <int DIM>
__global__ void __launch_bounds__(kMatThreads, 1) mat_build_kernel(
    const int4* __restrict__ act, const int4* __restrict__ sact, int n_sub, int s_pad,
    const float* __restrict__ xt, int64_t mpad, int64_t m, int64_t n_tiles,
    float4* __restrict__ pm, uint32_t* __restrict__ cm) {
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
      const int64_t at = tile * kGroups * static_cast<int64_t>(s_pad) + sid;
      if (!real) {
        for (int g = 0; g < kGroups; ++g) {
          pm[at + static_cast<int64_t>(g) * s_pad] = make_float4(0.f, 0.f, 0.f, 0.f);
          cm[at + static_cast<int64_t>(g) * s_pad] = 0u;
        }
        continue;
      }
      const uint32_t cbase = static_cast<uint32_t>(info.z);
      float4* dst = pm + at;
      uint32_t* cdst = cm + at;
      switch (info.w) {
        case 0: build_tile<0>(s_pt, W, q, 0, cbase, dst, cdst, s_pad); break;
        case 1: build_tile<1>(s_pt, W, q, 1, cbase, dst, cdst, s_pad); break;
        case 2: build_tile<(DIM < 2 ? DIM : 2)>(s_pt, W, q, 2, cbase, dst, cdst, s_pad); break;
        case 3: build_tile<(DIM < 3 ? DIM : 3)>(s_pt, W, q, 3, cbase, dst, cdst, s_pad); break;
        case 4: build_tile<(DIM < 4 ? DIM : 4)>(s_pt, W, q, 4, cbase, dst, cdst, s_pad); break;
        default: build_tile<-1>(s_pt, W, q, info.w, cbase, dst, cdst, s_pad); break;
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

__global__ void __launch_bounds__(kMatThreads, 2) mat_mult_kernel(
    const int4* __restrict__ sact, int n_sub, int s_pad, int cmax,
    const float* __restrict__ asub, int64_t m, int64_t tile_begin, int64_t n_tiles,
    const float4* __restrict__ pm, const uint32_t* __restrict__ cm,
    float* __restrict__ out32, double* __restrict__ out64) {
  extern __shared__ __align__(16) unsigned char smem[];
  float* s_part = reinterpret_cast<float*>(smem);   // [warps][kOwnTile]
  float* s_at = s_part + kMatWarps * kOwnTile;      // [cmax][s_pad] alpha by (cell, subspace)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t cm1 = static_cast<uint32_t>(cmax - 1);
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
  __syncthreads();
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t gt = tile_begin + tile;
    for (int s0 = 0; s0 < s_pad; s0 += blockDim.x) {
      if (s0 + warp * 32 >= s_pad) continue;  // whole warps: s_pad is a multiple of 32
      const int sid = s0 + tid;
      const int64_t at = gt * kGroups * static_cast<int64_t>(s_pad) + sid;
      const float4* src = pm + at;
      const uint32_t* csrc = cm + at;
      const float* a_col = s_at + sid;
      float* part = s_part + warp * kOwnTile;
      const bool first = s0 == 0;
      float4 ring[kAhead];
      uint32_t cring[kAhead];
#pragma unroll
      for (int u = 0; u < kAhead; ++u) {
        ring[u] = __ldcs(src + static_cast<int64_t>(u) * s_pad);
        cring[u] = __ldcs(csrc + static_cast<int64_t>(u) * s_pad);
      }
      for (int g0 = 0; g0 < kGroups; g0 += kAhead) {
#pragma unroll
        for (int u = 0; u < kAhead; ++u) {
          const int g = g0 + u;
          const float4 p = ring[u];
          const uint32_t cs = cring[u];
          if (g + kAhead < kGroups) {
            ring[u] = __ldcs(src + static_cast<int64_t>(g + kAhead) * s_pad);
            cring[u] = __ldcs(csrc + static_cast<int64_t>(g + kAhead) * s_pad);
          }
          // (the clamps only guard shared memory against a corrupted cell table)
          const float v0 = a_col[min(cs & 0xFFu, cm1) * s_pad] * p.x;
          const float v1 = a_col[min((cs >> 8) & 0xFFu, cm1) * s_pad] * p.y;
          const float v2 = a_col[min((cs >> 16) & 0xFFu, cm1) * s_pad] * p.z;
          const float v3 = a_col[min(cs >> 24, cm1) * s_pad] * p.w;
          const float r = reduce4(v0, v1, v2, v3, lane);
          if ((lane & 7) == 0) {
            float* dst = part + 4 * g + (lane >> 3);
            *dst = first ? r : *dst + r;
          }
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
    __syncthreads();  // the partials are read before the next tile overwrites them
  }
}

// ---- multTranspose -------------------------------------------------------------------------
__global__ void __launch_bounds__(kMatThreads, 2) mat_multt_kernel(
    const int4* __restrict__ sact, int n_sub, int s_pad, int cmax, int total,
    const float* __restrict__ v, int64_t n_tiles, const float4* __restrict__ pm,
    const uint32_t* __restrict__ cm, double* __restrict__ rows) {
  extern __shared__ __align__(16) unsigned char smem[];
  float* s_acc = reinterpret_cast<float*>(smem);  // [cmax][blockDim]
  double* row = rows + static_cast<int64_t>(blockIdx.x) * total;
  const int tid = threadIdx.x, nth = blockDim.x;
  const uint32_t cm1 = static_cast<uint32_t>(cmax - 1);
  const float4* v4 = reinterpret_cast<const float4*>(v);
  for (int s0 = 0; s0 < n_sub; s0 += nth) {
    const int sid = s0 + tid;
    if (sid >= n_sub) continue;  // no barriers below: threads run independently
    const int4 info = sact[sid];
    const uint32_t offset = static_cast<uint32_t>(info.x) - static_cast<uint32_t>(info.z);
    float* acc = s_acc + tid;
    for (int c = 0; c < info.y; ++c) acc[c * nth] = 0.0f;
    bool first = true;
    int since = 0;  // tiles summed in s_acc since the last flush
    for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
      const int64_t at = tile * kGroups * static_cast<int64_t>(s_pad) + sid;
      const float4* src = pm + at;
      const uint32_t* csrc = cm + at;
      const float4* vt = v4 + tile * kGroups;
      float4 ring[kAhead];
      uint32_t cring[kAhead];
#pragma unroll
      for (int u = 0; u < kAhead; ++u) {
        ring[u] = __ldcs(src + static_cast<int64_t>(u) * s_pad);
        cring[u] = __ldcs(csrc + static_cast<int64_t>(u) * s_pad);
      }
      for (int g0 = 0; g0 < kGroups; g0 += kAhead) {
#pragma unroll
        for (int u = 0; u < kAhead; ++u) {
          const int g = g0 + u;
          const float4 p = ring[u];
          const uint32_t cs = cring[u];
          if (g + kAhead < kGroups) {
            ring[u] = __ldcs(src + static_cast<int64_t>(g + kAhead) * s_pad);
            cring[u] = __ldcs(csrc + static_cast<int64_t>(g + kAhead) * s_pad);
          }
          const float4 vv = vt[g];  // the same four values for every lane
          acc[min(cs & 0xFFu, cm1) * nth] += vv.x * p.x;
          acc[min((cs >> 8) & 0xFFu, cm1) * nth] += vv.y * p.y;
          acc[min((cs >> 16) & 0xFFu, cm1) * nth] += vv.z * p.z;
          acc[min(cs >> 24, cm1) * nth] += vv.w * p.w;
        }
      }
      ++since;
      if (since == kFlushTiles || tile + gridDim.x >= n_tiles) {
        for (int c = 0; c < info.y; ++c) {
          double* dst = row + offset + c;
          *dst = first ? static_cast<double>(acc[c * nth]) : *dst + static_cast<double>(acc[c * nth]);
          acc[c * nth] = 0.0f;
        }
        first = false;
        since = 0;
      }
    }
    if (first)  // no tile for this CTA: its row holds zeros
      for (int c = 0; c < info.y; ++c) row[offset + c] = 0.0;
  }
}

size_t build_smem(int dim) { return sizeof(float) * kOwnTile * ((2 + 2 * dim + 3) / 4 * 4); }

int mat_threads(int64_t s_pad) { return static_cast<int>(std::min<int64_t>(kMatThreads, s_pad)); }

size_t mat_mult_smem(int cmax, int64_t s_pad) {
  return sizeof(float) * kMatWarps * kOwnTile + sizeof(float) * static_cast<size_t>(cmax) * s_pad;
}

size_t mat_multt_smem(int cmax, int64_t s_pad) {
  return sizeof(float) * static_cast<size_t>(cmax) * mat_threads(s_pad);
}

template <int DIM>
cudaError_t launch_build(SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad, int64_t m,
                         int num_sms) {
  const size_t sm = build_smem(DIM);
  auto kern = mat_build_kernel<DIM>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
  if (e != cudaSuccess) return e;
  const int64_t nt = mpad / kOwnTile;
  const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(nt, 2LL * num_sms));
  kern<<<static_cast<unsigned>(blocks), mat_threads(p.s_pad), sm, s>>>(
      p.act, p.sact, p.n_sub, static_cast<int>(p.s_pad), xt, mpad, m, nt, p.pmat, p.cmat);
  return cudaGetLastError();
}

#define MAT_DIMS(F) F(1) F(2) F(3) F(4) F(5) F(6) F(7) F(8) F(9) F(10) F(11) F(12) F(13) F(14) F(15) F(16)

constexpr size_t kMatSmemBudget = 200 * 1024;

}  // namespace

bool subspace_mat_fits(const SubPlan& p) {
  const int64_t s_pad = (p.n_sub + 31) / 32 * 32;
  return p.n_sub > 0 && p.cmax > 0 && p.cmax <= kMatMaxCells && p.rows != nullptr &&
         mat_mult_smem(p.cmax, s_pad) <= kMatSmemBudget &&
         mat_multt_smem(p.cmax, s_pad) <= kMatSmemBudget;
}

int64_t subspace_mat_bytes(const SubPlan& p, int64_t mpad) {
  return mpad * ((p.n_sub + 31) / 32 * 32) * static_cast<int64_t>(sizeof(float) + 1);
}

cudaError_t subspace_materialize(SubPlan* p, cudaStream_t s, const float* xt, int64_t mpad,
                                 int64_t m, int num_sms) {
  cudaFree(p->pmat);
  cudaFree(p->cmat);
  p->pmat = nullptr;
  p->cmat = nullptr;
  p->s_pad = (p->n_sub + 31) / 32 * 32;
  p->mat_mpad = mpad;
  const size_t entries = static_cast<size_t>(mpad / 4) * static_cast<size_t>(p->s_pad);
  cudaError_t e = cudaMalloc(&p->pmat, entries * sizeof(float4));
  if (e == cudaSuccess) e = cudaMalloc(&p->cmat, entries * sizeof(uint32_t));
  if (e != cudaSuccess) {
    cudaFree(p->pmat);
    p->pmat = nullptr;
    p->cmat = nullptr;
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

cudaError_t subspace_mult_mat(const SubPlan& p, cudaStream_t s, const float* /*xt*/, int64_t mpad,
                              int64_t m, const float* alpha32, float* out32, double* out64,
                              int64_t j_begin, int64_t j_end, int num_sms) {
  if (!p.pmat || !p.cmat || p.mat_mpad != mpad) return cudaErrorInvalidValue;
  cudaError_t e = subspace_scatter_alpha(p, s, alpha32);
  if (e != cudaSuccess) return e;
  const int64_t t0 = j_begin / kOwnTile;
  const int64_t nt = (j_end + kOwnTile - 1) / kOwnTile - t0;
  if (nt <= 0) return cudaSuccess;
  const size_t sm = mat_mult_smem(p.cmax, p.s_pad);
  e = cudaFuncSetAttribute(mat_mult_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mat_mult_kernel, kMatThreads, sm);
  if (e != cudaSuccess) return e;
  const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(nt, static_cast<int64_t>(std::max(1, per_sm)) * num_sms));
  mat_mult_kernel<<<static_cast<unsigned>(blocks), kMatThreads, sm, s>>>(
      p.sact, p.n_sub, static_cast<int>(p.s_pad), p.cmax, p.asub, m, t0, nt, p.pmat, p.cmat,
      out32, out64);
  return cudaGetLastError();
}

cudaError_t subspace_multt_mat(const SubPlan& p, cudaStream_t s, const float* /*xt*/, int64_t mpad,
                               int64_t m, const float* v32, int64_t npad, double* out64,
                               const double* add, double scale_add, int num_sms) {
  (void)m;
  if (!p.pmat || !p.cmat || p.mat_mpad != mpad) return cudaErrorInvalidValue;
  const size_t sm = mat_multt_smem(p.cmax, p.s_pad);
  const int nth = mat_threads(p.s_pad);
  cudaError_t e = cudaFuncSetAttribute(mat_multt_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mat_multt_kernel, nth, sm);
  if (e != cudaSuccess) return e;
  const int64_t nt = mpad / kOwnTile;
  const int64_t rows = std::min<int64_t>(std::max(1, per_sm) * static_cast<int64_t>(num_sms), p.row_cap);
  mat_multt_kernel<<<static_cast<unsigned>(rows), nth, sm, s>>>(
      p.sact, p.n_sub, static_cast<int>(p.s_pad), p.cmax, static_cast<int>(p.total), v32, nt,
      p.pmat, p.cmat, p.rows);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return subspace_finish_rows(p, s, rows, npad, out64, add, scale_add);
}

}  // namespace sgmev

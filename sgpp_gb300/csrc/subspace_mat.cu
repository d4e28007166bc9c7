// Materialised subspace products. For a fixed data set and grid, the product
// p_s(x_j) = prod_t h_{l_t}(x_{j,t}) of the one possibly non-zero basis function of subspace s at
// point j, and that function's cell index c_s(x_j) within its subspace, do not change between
// calls. They are computed once, in float-float arithmetic (sub_mat_build_kernel in subspace.cu),
// and kept in HBM as
//     P_hi[g][s], P_lo[g][s] : float4, the products of points 4g .. 4g+3 as float-float pairs
//     C[g][s]                : their cell indices, a byte each (uint32) or, when no subspace has
//                              more than 16 cells, a nibble each (uint16)
// with s padded to a multiple of 32 (padded entries 0), and for the inner solves of mixed fits an
// FP16 copy of P_hi with a copy of the cell words, both laid out by pairs of point groups (see
// the FP16 section). The FP32 mult and multTranspose stream P_hi and C (4.5-5 bytes per point and
// subspace), the FP64-accurate ones all three (8.5-9 bytes), the FP16 ones the copy (2.5-3); none
// touches a coordinate, so they are bounded by HBM bandwidth rather than the hat arithmetic.
// Points outside the domain have P = 0 (and cell 0), so they need no test.
//
// The kernels are owner-computes: thread k of a pass owns subspace s = pass * blockDim + k and
// walks a contiguous range of tiles of points; a warp reads P[g][32 consecutive s] as one
// contiguous run, through a ring of loads in registers that runs on from one tile into the next.
//   mult:  lane s forms alpha_s[c] * p for 4 points, for subspaces s and s + 32 at once (their
//          terms added in registers); a butterfly over the warp (xor 16, 8, then 4, 2, 1) reduces
//          the 4 values to 4 per-point sums, which go to per-warp partials in shared memory;
//          after all passes the partials are added in warp order.
//   multT: lane s adds v_j * p into its cells ([cell][thread] in shared memory, conflict-free) and
//          flushes them every kFlushTiles tiles into FP64 sums (float-float in the FP16 kernel);
//          rows are added in row order. The FP16/FP32 kernels give each pass of subspaces its own
//          CTA: the CTAs of all passes of one stream of tiles share a row and read the parts of
//          the same product rows together.
// The float-float variants do the same with float-float products, sums and butterfly.
// Every sum has a fixed order, so results are the same bit for bit from run to run.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "devmem.h"
#include "kernels.cuh"
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
// (fewer for the float-float kernels, whose arithmetic holds more registers)
constexpr int kAhead = 4, kAheadDf = 2;
static_assert(kGroups % kAhead == 0 && kGroups % kAheadDf == 0, "the ring must divide a tile");
// multT: FP32 sums over this many tiles (1024 points) before they go into the FP64 row
constexpr int kFlushTiles = 4;

// Cell words: four points' cell indices in one word, a byte each (uint32_t, grids whose
// subspaces have up to 256 cells) or a nibble each (uint16_t, up to 16 cells: 0.5 byte per entry
// instead of 1, which the streaming kernels feel directly, being bound by HBM bytes).
template <typename CW>
__device__ __forceinline__ uint32_t cell_of(uint32_t w, int i) {
  constexpr int kBits = sizeof(CW) * 2;
  return (w >> (kBits * i)) & ((1u << kBits) - 1u);
}

// Streaming loads of the products and cells: each entry is read once per launch, so they skip
// L1 allocation (ld.global.L1::no_allocate) and leave L1 to the vectors that are re-read.
__device__ __forceinline__ uint2 ld_stream(const uint2* p) {
  uint2 v;
  asm("ld.global.L1::no_allocate.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
  return v;
}
__device__ __forceinline__ float4 ld_stream(const float4* p) {
  float4 v;
  asm("ld.global.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
      : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
      : "l"(p));
  return v;
}
__device__ __forceinline__ uint4 ld_stream(const uint4* p) {
  uint4 v;
  asm("ld.global.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
      : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
      : "l"(p));
  return v;
}
__device__ __forceinline__ uint16_t ld_stream(const uint16_t* p) {
  unsigned short v;
  asm("ld.global.L1::no_allocate.u16 %0, [%1];" : "=h"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ uint32_t ld_stream(const uint32_t* p) {
  uint32_t v;
  asm("ld.global.L1::no_allocate.u32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
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

// four FP16 products (two half2 words) as floats
__device__ __forceinline__ float4 halves4(uint32_t lo, uint32_t hi) {
  const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&lo));
  const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&hi));
  return make_float4(a.x, a.y, b.x, b.y);
}

// mult: a lane takes subspaces s and s + 32 of the same four points (two 32-wide blocks per
// warp), adds their four terms in registers and then runs one butterfly, so the butterfly's
// cost is shared by two subspaces. A warp whose second block lies beyond s_pad reads its first
// block twice and multiplies the copy by a zero column of alpha (s_at is kMultBlock-padded).
constexpr int kMultBlock = 64;  // subspaces per warp and pass
constexpr int kAhead2 = 2;  // groups in flight per block: the bytes of one block at kAhead
static_assert(kGroups % 4 == 0 && kGroups % 2 == 0, "the ring must divide a tile");

__host__ __device__ constexpr int mult_at_pad(int s_pad) {
  return (s_pad + kMultBlock - 1) / kMultBlock * kMultBlock;
}

// s_stride / accumulate: windows of the subspaces, as in mat_mult_half_kernel below.
template <typename CW>
__global__ void __launch_bounds__(kMatThreads, 2) mat_mult_kernel(
    const int4* __restrict__ sact, int n_sub, int s_pad, int cmax,
    const float* __restrict__ asub, int64_t m, int64_t tile_begin, int64_t n_tiles,
    const float4* __restrict__ pm, const CW* __restrict__ cm, float* __restrict__ out32,
    double* __restrict__ out64, int s_stride, int accumulate) {
  using PT = float4;
  constexpr int A = kAhead2;
  extern __shared__ __align__(16) unsigned char smem[];
  const int sp = mult_at_pad(s_pad);                // row length of s_at
  float* s_part = reinterpret_cast<float*>(smem);   // [warps][kOwnTile]
  float* s_at = s_part + kMatWarps * kOwnTile;      // [cmax][sp] alpha by (cell, subspace)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // alpha transposed: s_at[c * sp + s] = alpha at position offset_s + c (0 beyond the cells and
  // for s >= n_sub)
  for (int k = tid; k < cmax * sp; k += blockDim.x) {
    const int c = k / sp, sidx = k - c * sp;
    float a = 0.0f;
    if (sidx < n_sub) {
      const int4 info = sact[sidx];
      const int off = static_cast<int>(static_cast<uint32_t>(info.x) - static_cast<uint32_t>(info.z));
      if (c < info.y) a = asub[off + c];
    }
    s_at[k] = a;
  }
  __syncthreads();
  // the CTA's tiles are contiguous; with one pass over the subspaces the ring runs on from one
  // tile into the next without restarting
  const int64_t t_first = blockIdx.x * n_tiles / gridDim.x;
  const int64_t t_last = (blockIdx.x + 1) * n_tiles / gridDim.x;
  const bool one_pass = s_pad <= kMultBlock * kMatWarps;
  PT ring[A], ring2[A];
  CW cring[A], cring2[A];
  const PT* nsrc = nullptr;
  const CW* ncsrc = nullptr;
  for (int64_t tile = t_first; tile < t_last; ++tile) {
    const int64_t gt = tile_begin + tile;
    for (int s0 = 0; s0 < s_pad; s0 += kMultBlock * kMatWarps) {
      const int wb = s0 + warp * kMultBlock;  // first subspace of this warp's two blocks
      if (wb >= s_pad) continue;              // whole warps: s_pad is a multiple of 32
      const int sid = wb + lane;
      const bool two = wb + 32 < s_pad;       // warp-uniform
      const int off2 = two ? 32 : 0;          // the second block (the first again when absent)
      const float* a_col = s_at + sid;
      const float* a_col2 = a_col + 32;       // zeros when the second block is absent
      float* part = s_part + warp * kOwnTile;
      const bool first = s0 == 0;
      if (!one_pass || tile == t_first) {
        const int64_t at = gt * kGroups * static_cast<int64_t>(s_stride) + sid;
#pragma unroll
        for (int u = 0; u < A; ++u) {
          ring[u] = ld_stream(pm + at + static_cast<int64_t>(u) * s_stride);
          cring[u] = ld_stream(cm + at + static_cast<int64_t>(u) * s_stride);
          ring2[u] = ld_stream(pm + at + off2 + static_cast<int64_t>(u) * s_stride);
          cring2[u] = ld_stream(cm + at + off2 + static_cast<int64_t>(u) * s_stride);
        }
        nsrc = pm + at + static_cast<int64_t>(A) * s_stride;
        ncsrc = cm + at + static_cast<int64_t>(A) * s_stride;
      }
      // refills run into the next tile when the ring continues there
      const bool more = one_pass && tile + 1 < t_last;
      for (int g0 = 0; g0 < kGroups; g0 += A) {
        const bool fetch = g0 + A < kGroups || more;
#pragma unroll
        for (int u = 0; u < A; ++u) {
          const int g = g0 + u;
          const float4 p = ring[u];
          const float4 q = ring2[u];
          const uint32_t cs = cring[u], cq = cring2[u];
          if (fetch) {
            ring[u] = ld_stream(nsrc);
            cring[u] = ld_stream(ncsrc);
            ring2[u] = ld_stream(nsrc + off2);
            cring2[u] = ld_stream(ncsrc + off2);
            nsrc += s_stride;
            ncsrc += s_stride;
          }
          // cells are below cmax by construction (the build writes c < cells of s <= cmax)
          float v0 = a_col[cell_of<CW>(cs, 0) * sp] * p.x;
          float v1 = a_col[cell_of<CW>(cs, 1) * sp] * p.y;
          float v2 = a_col[cell_of<CW>(cs, 2) * sp] * p.z;
          float v3 = a_col[cell_of<CW>(cs, 3) * sp] * p.w;
          v0 = fmaf(a_col2[cell_of<CW>(cq, 0) * sp], q.x, v0);
          v1 = fmaf(a_col2[cell_of<CW>(cq, 1) * sp], q.y, v1);
          v2 = fmaf(a_col2[cell_of<CW>(cq, 2) * sp], q.z, v2);
          v3 = fmaf(a_col2[cell_of<CW>(cq, 3) * sp], q.w, v3);
          const float r = reduce4(v0, v1, v2, v3, lane);
          if ((lane & 7) == 0) {
            float* dst = part + 4 * g + (lane >> 3);
            *dst = first ? r : *dst + r;
          }
        }
      }
    }
    __syncthreads();
    // warp w wrote its partials in pass 0 iff w * kMultBlock < s_pad
    const int wrote = min(kMatWarps, (s_pad + kMultBlock - 1) / kMultBlock);
    for (int jj = tid; jj < kOwnTile; jj += blockDim.x) {
      float r = 0.0f;
      for (int w = 0; w < wrote; ++w) r += s_part[w * kOwnTile + jj];
      const int64_t j = gt * kOwnTile + jj;
      const float v = j < m ? r : 0.0f;
      if (out32) out32[j] = accumulate ? out32[j] + v : v;
      if (out64) out64[j] = accumulate ? out64[j] + static_cast<double>(v) : static_cast<double>(v);
    }
    __syncthreads();  // the partials are read before the next tile overwrites them
  }
}

// ---- multTranspose -------------------------------------------------------------------------
// SACC: the flushes go into FP64 sums in shared memory ([cmax][blockDim] doubles beside the FP32
// cells), and the CTA's row is written once per pass: the same additions in the same order as
// flushing into the row itself, without a read-modify-write of global memory per flush (the
// flushes were a tenth of the kernel's time). Used when both arrays leave room for two CTAs per SM.
template <typename CW, bool SACC>
__global__ void __launch_bounds__(kMatThreads, 2) mat_multt_kernel(
    const int4* __restrict__ sact, int n_sub, int s_pad, int cmax, int total,
    const float* __restrict__ v, int64_t n_tiles, const float4* __restrict__ pm,
    const CW* __restrict__ cm, double* __restrict__ rows, int streams) {
  using PT = float4;
  constexpr int A = kAhead;
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, nth = blockDim.x;
  double* s_sum = reinterpret_cast<double*>(smem);  // [cmax][blockDim] (SACC)
  float* s_acc = reinterpret_cast<float*>(SACC ? smem + sizeof(double) * cmax * nth : smem);  // [cmax][blockDim]
  // CTA b takes the subspaces of pass b / streams over the tiles of stream b % streams, so the
  // CTAs of all passes of a stream read the parts of the same product rows at about the same time
  const int pass = blockIdx.x / streams, stream = blockIdx.x - pass * streams;
  const int passes = gridDim.x / streams;
  double* row = rows + static_cast<int64_t>(stream) * total;
  const float4* v4 = reinterpret_cast<const float4*>(v);
  for (int s0 = pass * nth; s0 < n_sub; s0 += nth * passes) {
    const int sid = s0 + tid;
    if (sid >= n_sub) continue;  // no barriers below: threads run independently
    const int4 info = sact[sid];
    const uint32_t offset = static_cast<uint32_t>(info.x) - static_cast<uint32_t>(info.z);
    float* acc = s_acc + tid;
    for (int c = 0; c < info.y; ++c) acc[c * nth] = 0.0f;
    bool first = true;
    // the stream's tiles are contiguous and its ring runs over all of them
    const int64_t g_begin = (stream * n_tiles / streams) * kGroups;
    const int64_t g_end = ((stream + 1) * n_tiles / streams) * kGroups;
    if (g_begin < g_end) {
      const PT* src = pm + g_begin * s_pad + sid;
      const CW* csrc = cm + g_begin * s_pad + sid;
      const float4* vt = v4 + g_begin;
      PT ring[A];
      CW cring[A];
#pragma unroll
      for (int u = 0; u < A; ++u) {
        ring[u] = ld_stream(src);
        cring[u] = ld_stream(csrc);
        src += s_pad;
        csrc += s_pad;
      }
      int since = 0;  // groups summed in s_acc since the last flush
      for (int64_t g0 = g_begin; g0 < g_end; g0 += A) {
        const bool fetch = g0 + A < g_end;
#pragma unroll
        for (int u = 0; u < A; ++u) {
          const float4 p = ring[u];
          const uint32_t cs = cring[u];
          if (fetch) {
            ring[u] = ld_stream(src);
            cring[u] = ld_stream(csrc);
            src += s_pad;
            csrc += s_pad;
          }
          const float4 vv = vt[u];  // the same four values for every lane
          // cells are below cmax by construction
          acc[cell_of<CW>(cs, 0) * nth] += vv.x * p.x;
          acc[cell_of<CW>(cs, 1) * nth] += vv.y * p.y;
          acc[cell_of<CW>(cs, 2) * nth] += vv.z * p.z;
          acc[cell_of<CW>(cs, 3) * nth] += vv.w * p.w;
        }
        vt += A;
        since += A;
        if (since == kFlushTiles * kGroups || !fetch) {
          for (int c = 0; c < info.y; ++c) {
            double* dst = SACC ? s_sum + c * nth + tid : row + offset + c;
            *dst = first ? static_cast<double>(acc[c * nth]) : *dst + static_cast<double>(acc[c * nth]);
            acc[c * nth] = 0.0f;
          }
          first = false;
          since = 0;
        }
      }
    }
    if (first) {  // no tile for this CTA: its row holds zeros
      for (int c = 0; c < info.y; ++c) row[offset + c] = 0.0;
    } else if (SACC) {
      for (int c = 0; c < info.y; ++c) row[offset + c] = s_sum[c * nth + tid];
    }
  }
}

// ---- FP16 products by pairs of point groups -------------------------------------------------
// The inner solves of mixed fits stream the FP16 copy of the products, P16[k][s] (uint4: the eight
// halves of points 8k .. 8k + 7, point groups 2k and 2k + 1), with the cell words of the same
// pair, C2[k][s] (PairCells). A lane loads 16 bytes of products and 4 (nibble cells) or 8 (byte
// cells) bytes of cells per two groups: half the memory requests of one load per group, for the
// same bytes (0.483 -> 0.444 ms for B a and 0.561 -> 0.540 ms for B^T v on the benchmark
// workload). The arithmetic and its order are those of the [g][s] kernels above.
constexpr int kPairs = kGroups / 2;  // pairs of point groups per tile

template <typename CW>
struct PairCells;
template <>
struct PairCells<uint16_t> {  // two nibble words in one uint32_t, group 2k in the low half
  using T = uint32_t;
  static __device__ __forceinline__ uint32_t word(uint32_t w, int h) { return h ? w >> 16 : w; }
};
template <>
struct PairCells<uint32_t> {  // two byte words
  using T = uint2;
  static __device__ __forceinline__ uint32_t word(uint2 w, int h) { return h ? w.y : w.x; }
};

constexpr int kPairAheadMult = 2;   // pairs in flight per block: the 4 groups of the FP16 ring
constexpr int kPairAheadMultT = 4;  // pairs in flight: 8 groups
static_assert(kPairs % kPairAheadMult == 0 && kPairs % kPairAheadMultT == 0,
              "the ring must divide a tile");

// mat_mult_kernel on the pair layout: a lane takes subspaces s and s + 32, two point groups per
// ring slot. A CTA takes a contiguous range of tiles, and with one pass over the subspaces its
// ring runs from one tile into the next instead of starting again at each tile (a ring restart
// waits a full memory latency, about 2.5 us at this load, against ~30 us of work per tile).
// Windows: the kernel can take a window of the subspaces (sact, pp and cp advanced to its first
// subspace, n_sub and s_pad its count and padded count) while s_stride stays the product rows'
// length; with accumulate the window's sums are added to the outputs (the windows run as
// successive launches, in subspace order), so grids whose coefficients do not fit shared memory
// at once take several windows.
template <typename CW>
__global__ void __launch_bounds__(kMatThreads, 2) mat_mult_half_kernel(
    const int4* __restrict__ sact, int n_sub, int s_pad, int cmax,
    const float* __restrict__ asub, int64_t m, int64_t tile_begin, int64_t n_tiles,
    const uint4* __restrict__ pp, const typename PairCells<CW>::T* __restrict__ cp,
    float* __restrict__ out32, double* __restrict__ out64, float unscale, int s_stride,
    int accumulate) {
  using PC = PairCells<CW>;
  using CT = typename PC::T;
  constexpr int A = kPairAheadMult;
  extern __shared__ __align__(16) unsigned char smem[];
  const int sp = mult_at_pad(s_pad);
  float* s_part = reinterpret_cast<float*>(smem);   // [warps][kOwnTile]
  float* s_at = s_part + kMatWarps * kOwnTile;      // [cmax][sp] alpha by (cell, subspace)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int k = tid; k < cmax * sp; k += blockDim.x) {
    const int c = k / sp, sidx = k - c * sp;
    float a = 0.0f;
    if (sidx < n_sub) {
      const int4 info = sact[sidx];
      const int off = static_cast<int>(static_cast<uint32_t>(info.x) - static_cast<uint32_t>(info.z));
      if (c < info.y) a = asub[off + c];
    }
    s_at[k] = a;
  }
  __syncthreads();
  // the CTA's tiles are contiguous; with one pass over the subspaces the ring runs on from one
  // tile into the next without restarting
  const int64_t t_first = blockIdx.x * n_tiles / gridDim.x;
  const int64_t t_last = (blockIdx.x + 1) * n_tiles / gridDim.x;
  const bool one_pass = s_pad <= kMultBlock * kMatWarps;
  const int wb0 = warp * kMultBlock;
  uint4 ring[A], ring2[A];
  CT cring[A], cring2[A];
  const uint4* nsrc = nullptr;
  const CT* ncsrc = nullptr;
  for (int64_t tile = t_first; tile < t_last; ++tile) {
    const int64_t gt = tile_begin + tile;
    for (int s0 = 0; s0 < s_pad; s0 += kMultBlock * kMatWarps) {
      const int wb = s0 + wb0;
      if (wb >= s_pad) continue;  // whole warps: s_pad is a multiple of 32
      const int sid = wb + lane;
      const bool two = wb + 32 < s_pad;  // warp-uniform
      const float* a_col = s_at + sid;
      const float* a_col2 = a_col + 32;  // zeros when the second block is absent
      float* part = s_part + warp * kOwnTile;
      const bool first = s0 == 0;
      const int off2 = two ? 32 : 0;
      if (!one_pass || tile == t_first) {
        const int64_t at = gt * kPairs * static_cast<int64_t>(s_stride) + sid;
#pragma unroll
        for (int u = 0; u < A; ++u) {
          ring[u] = ld_stream(pp + at + static_cast<int64_t>(u) * s_stride);
          cring[u] = ld_stream(cp + at + static_cast<int64_t>(u) * s_stride);
          ring2[u] = ld_stream(pp + at + off2 + static_cast<int64_t>(u) * s_stride);
          cring2[u] = ld_stream(cp + at + off2 + static_cast<int64_t>(u) * s_stride);
        }
        nsrc = pp + at + static_cast<int64_t>(A) * s_stride;
        ncsrc = cp + at + static_cast<int64_t>(A) * s_stride;
      }
      // refills run into the next tile when the ring continues there
      const bool more = one_pass && tile + 1 < t_last;
      for (int k0 = 0; k0 < kPairs; k0 += A) {
        const bool fetch = k0 + A < kPairs || more;
#pragma unroll
        for (int u = 0; u < A; ++u) {
          const int k = k0 + u;
          const uint4 pw = ring[u], qw = ring2[u];
          const CT cs = cring[u], cq = cring2[u];
          if (fetch) {
            ring[u] = ld_stream(nsrc);
            cring[u] = ld_stream(ncsrc);
            ring2[u] = ld_stream(nsrc + off2);
            cring2[u] = ld_stream(ncsrc + off2);
            nsrc += s_stride;
            ncsrc += s_stride;
          }
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const float4 p = h ? halves4(pw.z, pw.w) : halves4(pw.x, pw.y);
            const float4 q = h ? halves4(qw.z, qw.w) : halves4(qw.x, qw.y);
            const uint32_t ws = PC::word(cs, h), wq = PC::word(cq, h);
            float v0 = a_col[cell_of<CW>(ws, 0) * sp] * p.x;
            float v1 = a_col[cell_of<CW>(ws, 1) * sp] * p.y;
            float v2 = a_col[cell_of<CW>(ws, 2) * sp] * p.z;
            float v3 = a_col[cell_of<CW>(ws, 3) * sp] * p.w;
            v0 = fmaf(a_col2[cell_of<CW>(wq, 0) * sp], q.x, v0);
            v1 = fmaf(a_col2[cell_of<CW>(wq, 1) * sp], q.y, v1);
            v2 = fmaf(a_col2[cell_of<CW>(wq, 2) * sp], q.z, v2);
            v3 = fmaf(a_col2[cell_of<CW>(wq, 3) * sp], q.w, v3);
            const float r = reduce4(v0, v1, v2, v3, lane);
            if ((lane & 7) == 0) {
              float* dst = part + 4 * (2 * k + h) + (lane >> 3);
              *dst = first ? r : *dst + r;
            }
          }
        }
      }
    }
    __syncthreads();
    const int wrote = min(kMatWarps, (s_pad + kMultBlock - 1) / kMultBlock);
    for (int jj = tid; jj < kOwnTile; jj += blockDim.x) {
      float r = 0.0f;
      for (int w = 0; w < wrote; ++w) r += s_part[w * kOwnTile + jj];
      const int64_t j = gt * kOwnTile + jj;
      const float v = j < m ? r * unscale : 0.0f;  // the FP16 products are scaled by 2^p16_exp
      if (out32) out32[j] = accumulate ? out32[j] + v : v;
      if (out64) out64[j] = accumulate ? out64[j] + static_cast<double>(v) : static_cast<double>(v);
    }
    __syncthreads();  // the partials are read before the next tile overwrites them
  }
}

// mat_multt_kernel on the pair layout; a stream's tiles are contiguous and its ring runs over all
// of them (0.537 -> 0.496 ms on the benchmark workload against a ring restarted per tile). The
// FP32 cell sums are flushed into float-float sums (a two-sum, at the FP32 rate) instead of FP64
// ones, whose adds run at a small fraction of that rate on this part (0.496 -> 0.487 ms); they
// become FP64 once, when the row is written.
// BATCH points share one read-modify-write round of the owner's cells: their sums are all read
// before any is written back, so the reads' latency is paid once per batch instead of once per
// point. Points of a batch in the same cell chain through registers (a point starts from the
// latest earlier value of its cell), and the stores go in point order, so the last store of a cell
// holds every term: the same additions in the same order as BATCH = 1, bit for bit.
template <typename CW, bool SACC, int BATCH>
__global__ void __launch_bounds__(kMatThreads, 2) mat_multt_half_kernel(
    const int4* __restrict__ sact, int n_sub, int s_pad, int cmax, int total,
    const float* __restrict__ v, int64_t n_tiles, const uint4* __restrict__ pp,
    const typename PairCells<CW>::T* __restrict__ cp, double* __restrict__ rows, int streams,
    double unscale) {
  using PC = PairCells<CW>;
  using CT = typename PC::T;
  constexpr int A = kPairAheadMultT;
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, nth = blockDim.x;
  float2* s_sum = reinterpret_cast<float2*>(smem);  // [cmax][blockDim] float-float (SACC)
  float* s_acc = reinterpret_cast<float*>(SACC ? smem + sizeof(double) * cmax * nth : smem);
  const int pass = blockIdx.x / streams, stream = blockIdx.x - pass * streams;
  const int passes = gridDim.x / streams;
  double* row = rows + static_cast<int64_t>(stream) * total;
  const float4* v4 = reinterpret_cast<const float4*>(v);
  for (int s0 = pass * nth; s0 < n_sub; s0 += nth * passes) {
    const int sid = s0 + tid;
    if (sid >= n_sub) continue;  // no barriers below: threads run independently
    const int4 info = sact[sid];
    const uint32_t offset = static_cast<uint32_t>(info.x) - static_cast<uint32_t>(info.z);
    float* acc = s_acc + tid;
    for (int c = 0; c < info.y; ++c) acc[c * nth] = 0.0f;
    bool first = true;
    // the stream's tiles are contiguous, so the ring runs over all of them without restarting
    const int64_t k_begin = (stream * n_tiles / streams) * kPairs;
    const int64_t k_end = ((stream + 1) * n_tiles / streams) * kPairs;
    if (k_begin < k_end) {
      const uint4* src = pp + k_begin * s_pad + sid;
      const CT* csrc = cp + k_begin * s_pad + sid;
      const float4* vt = v4 + 2 * k_begin;
      uint4 ring[A];
      CT cring[A];
#pragma unroll
      for (int u = 0; u < A; ++u) {
        ring[u] = ld_stream(src + static_cast<int64_t>(u) * s_pad);
        cring[u] = ld_stream(csrc + static_cast<int64_t>(u) * s_pad);
      }
      src += static_cast<int64_t>(A) * s_pad;
      csrc += static_cast<int64_t>(A) * s_pad;
      int since = 0;  // pairs summed in s_acc since the last flush
      for (int64_t k0 = k_begin; k0 < k_end; k0 += A) {
        const bool fetch = k0 + A < k_end;
#pragma unroll
        for (int u = 0; u < A; ++u) {
          const uint4 pw = ring[u];
          const CT cs = cring[u];
          if (fetch) {
            ring[u] = ld_stream(src);
            cring[u] = ld_stream(csrc);
            src += s_pad;
            csrc += s_pad;
          }
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const float4 p = h ? halves4(pw.z, pw.w) : halves4(pw.x, pw.y);
            const uint32_t w = PC::word(cs, h);
            const float4 vv = vt[2 * u + h];  // the same four values for every lane
            if constexpr (BATCH == 1) {
              acc[cell_of<CW>(w, 0) * nth] += vv.x * p.x;
              acc[cell_of<CW>(w, 1) * nth] += vv.y * p.y;
              acc[cell_of<CW>(w, 2) * nth] += vv.z * p.z;
              acc[cell_of<CW>(w, 3) * nth] += vv.w * p.w;
            } else {
              const float pv[4] = {p.x, p.y, p.z, p.w};
              const float vw[4] = {vv.x, vv.y, vv.z, vv.w};
#pragma unroll
              for (int b0 = 0; b0 < 4; b0 += BATCH) {
                uint32_t c[BATCH];
                float old[BATCH], nv[BATCH];
#pragma unroll
                for (int i = 0; i < BATCH; ++i) {
                  c[i] = cell_of<CW>(w, b0 + i);
                  old[i] = acc[c[i] * nth];
                }
#pragma unroll
                for (int i = 0; i < BATCH; ++i) {
                  float base = old[i];
#pragma unroll
                  for (int j = 0; j < i; ++j) base = c[i] == c[j] ? nv[j] : base;
                  nv[i] = fmaf(vw[b0 + i], pv[b0 + i], base);
                }
#pragma unroll
                for (int i = 0; i < BATCH; ++i) acc[c[i] * nth] = nv[i];
              }
            }
          }
        }
        vt += 2 * A;
        since += A;
        if (since == kFlushTiles * kPairs || !fetch) {
          for (int c = 0; c < info.y; ++c) {
            const float a = acc[c * nth];
            if constexpr (SACC) {
              float2* d = s_sum + c * nth + tid;
              if (first) {
                *d = make_float2(a, 0.0f);
              } else {
                ff t{d->x, d->y};
                add_ff(t, ff{a, 0.0f});
                *d = make_float2(t.h, t.l);
              }
            } else {
              double* dst = row + offset + c;
              const double au = static_cast<double>(a) * unscale;
              *dst = first ? au : *dst + au;
            }
            acc[c * nth] = 0.0f;
          }
          first = false;
          since = 0;
        }
      }
    }
    if (first) {
      for (int c = 0; c < info.y; ++c) row[offset + c] = 0.0;
    } else if (SACC) {
      for (int c = 0; c < info.y; ++c) {
        const float2 t = s_sum[c * nth + tid];
        row[offset + c] = (static_cast<double>(t.x) + static_cast<double>(t.y)) * unscale;
      }
    }
  }
}

// mat_multt_half_kernel with two banks of cell sums per owner ("multt_banks" = 2): the points of a
// group alternate between the banks (points 0 and 2 of four into bank 0, 1 and 3 into bank 1),
// so each round reads both banks' cells before it writes either. The two read-modify-write
// chains are independent (the banks are disjoint), so a round waits for one shared-memory
// latency where the single bank waits for two; the single-bank kernel's warps spend most of their
// stalls on exactly that wait. The banks are added into one FP32 sum per cell every kFlushTiles
// tiles (the FP32 terms carry the FP16 products' 2^-11 rounding, far above what the FP32 sums
// add) and the row gets that sum once, in FP64. The shared memory is the single bank's with its
// float-float sums: (2 + 1) x 4 bytes per cell and owner. The order of the additions differs
// from the single-bank kernel, so the results differ in the last bits; they are fixed from run to
// run.
template <typename CW>
__global__ void __launch_bounds__(kMatThreads, 2) mat_multt_half_banked_kernel(
    const int4* __restrict__ sact, int n_sub, int s_pad, int cmax, int total,
    const float* __restrict__ v, int64_t n_tiles, const uint4* __restrict__ pp,
    const typename PairCells<CW>::T* __restrict__ cp, double* __restrict__ rows, int streams,
    double unscale) {
  using PC = PairCells<CW>;
  using CT = typename PC::T;
  constexpr int A = kPairAheadMultT;
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, nth = blockDim.x;
  float* s_sum = reinterpret_cast<float*>(smem);  // [cmax][blockDim]
  float* s_b0 = s_sum + cmax * nth;               // bank 0, [cmax][blockDim]
  float* s_b1 = s_b0 + cmax * nth;                // bank 1
  const int pass = blockIdx.x / streams, stream = blockIdx.x - pass * streams;
  const int passes = gridDim.x / streams;
  double* row = rows + static_cast<int64_t>(stream) * total;
  const float4* v4 = reinterpret_cast<const float4*>(v);
  for (int s0 = pass * nth; s0 < n_sub; s0 += nth * passes) {
    const int sid = s0 + tid;
    if (sid >= n_sub) continue;  // no barriers below: threads run independently
    const int4 info = sact[sid];
    const uint32_t offset = static_cast<uint32_t>(info.x) - static_cast<uint32_t>(info.z);
    float* b0 = s_b0 + tid;
    float* b1 = s_b1 + tid;
    float* sum = s_sum + tid;
    for (int c = 0; c < info.y; ++c) {
      b0[c * nth] = 0.0f;
      b1[c * nth] = 0.0f;
      sum[c * nth] = 0.0f;
    }
    const int64_t k_begin = (stream * n_tiles / streams) * kPairs;
    const int64_t k_end = ((stream + 1) * n_tiles / streams) * kPairs;
    if (k_begin < k_end) {
      const uint4* src = pp + k_begin * s_pad + sid;
      const CT* csrc = cp + k_begin * s_pad + sid;
      const float4* vt = v4 + 2 * k_begin;
      uint4 ring[A];
      CT cring[A];
#pragma unroll
      for (int u = 0; u < A; ++u) {
        ring[u] = ld_stream(src + static_cast<int64_t>(u) * s_pad);
        cring[u] = ld_stream(csrc + static_cast<int64_t>(u) * s_pad);
      }
      src += static_cast<int64_t>(A) * s_pad;
      csrc += static_cast<int64_t>(A) * s_pad;
      int since = 0;
      for (int64_t k0 = k_begin; k0 < k_end; k0 += A) {
        const bool fetch = k0 + A < k_end;
#pragma unroll
        for (int u = 0; u < A; ++u) {
          const uint4 pw = ring[u];
          const CT cs = cring[u];
          if (fetch) {
            ring[u] = ld_stream(src);
            cring[u] = ld_stream(csrc);
            src += s_pad;
            csrc += s_pad;
          }
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const float4 p = h ? halves4(pw.z, pw.w) : halves4(pw.x, pw.y);
            const uint32_t w = PC::word(cs, h);
            const float4 vv = vt[2 * u + h];
            {
              const uint32_t c0 = cell_of<CW>(w, 0) * nth, c1 = cell_of<CW>(w, 1) * nth;
              const float o0 = b0[c0], o1 = b1[c1];
              b0[c0] = fmaf(vv.x, p.x, o0);
              b1[c1] = fmaf(vv.y, p.y, o1);
            }
            {
              const uint32_t c2 = cell_of<CW>(w, 2) * nth, c3 = cell_of<CW>(w, 3) * nth;
              const float o2 = b0[c2], o3 = b1[c3];
              b0[c2] = fmaf(vv.z, p.z, o2);
              b1[c3] = fmaf(vv.w, p.w, o3);
            }
          }
        }
        vt += 2 * A;
        since += A;
        if (since == kFlushTiles * kPairs || !fetch) {
          for (int c = 0; c < info.y; ++c) {
            sum[c * nth] += b0[c * nth] + b1[c * nth];
            b0[c * nth] = 0.0f;
            b1[c * nth] = 0.0f;
          }
          since = 0;
        }
      }
    }
    for (int c = 0; c < info.y; ++c) row[offset + c] = static_cast<double>(sum[c * nth]) * unscale;
  }
}

// mat_multt_half_kernel with three CTAs per SM ("multt_ctas" = 3): one bank of FP32 cell sums per
// owner (16 cells x 512 owners x 4 bytes = 32 KB of shared memory per CTA), added over all of the
// stream's points and written to the row once, in FP64; two pairs of groups in flight per thread
// instead of four, so that the thread fits 42 registers. Half as many warps again as the two-CTA
// kernels hide the latency of the read-modify-write chains. The FP32 sums add up to a few thousand
// terms that carry the FP16 products' 2^-11 rounding, far above what the FP32 additions lose.
template <typename CW>
__global__ void __launch_bounds__(kMatThreads, 3) mat_multt_half_lean_kernel(
    const int4* __restrict__ sact, int n_sub, int s_pad, int cmax, int total,
    const float* __restrict__ v, int64_t n_tiles, const uint4* __restrict__ pp,
    const typename PairCells<CW>::T* __restrict__ cp, double* __restrict__ rows, int streams,
    double unscale) {
  using PC = PairCells<CW>;
  using CT = typename PC::T;
  constexpr int A = 2;
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, nth = blockDim.x;
  float* s_acc = reinterpret_cast<float*>(smem);  // [cmax][blockDim]
  const int pass = blockIdx.x / streams, stream = blockIdx.x - pass * streams;
  const int passes = gridDim.x / streams;
  double* row = rows + static_cast<int64_t>(stream) * total;
  const float4* v4 = reinterpret_cast<const float4*>(v);
  for (int s0 = pass * nth; s0 < n_sub; s0 += nth * passes) {
    const int sid = s0 + tid;
    if (sid >= n_sub) continue;  // no barriers below: threads run independently
    const int4 info = sact[sid];
    const uint32_t offset = static_cast<uint32_t>(info.x) - static_cast<uint32_t>(info.z);
    float* acc = s_acc + tid;
    for (int c = 0; c < info.y; ++c) acc[c * nth] = 0.0f;
    const int64_t k_begin = (stream * n_tiles / streams) * kPairs;
    const int64_t k_end = ((stream + 1) * n_tiles / streams) * kPairs;
    if (k_begin < k_end) {
      const uint4* src = pp + k_begin * s_pad + sid;
      const CT* csrc = cp + k_begin * s_pad + sid;
      const float4* vt = v4 + 2 * k_begin;
      uint4 ring[A];
      CT cring[A];
#pragma unroll
      for (int u = 0; u < A; ++u) {
        ring[u] = ld_stream(src + static_cast<int64_t>(u) * s_pad);
        cring[u] = ld_stream(csrc + static_cast<int64_t>(u) * s_pad);
      }
      src += static_cast<int64_t>(A) * s_pad;
      csrc += static_cast<int64_t>(A) * s_pad;
      for (int64_t k0 = k_begin; k0 < k_end; k0 += A) {
        const bool fetch = k0 + A < k_end;
#pragma unroll
        for (int u = 0; u < A; ++u) {
          const uint4 pw = ring[u];
          const CT cs = cring[u];
          if (fetch) {
            ring[u] = ld_stream(src);
            cring[u] = ld_stream(csrc);
            src += s_pad;
            csrc += s_pad;
          }
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const float4 p = h ? halves4(pw.z, pw.w) : halves4(pw.x, pw.y);
            const uint32_t w = PC::word(cs, h);
            const float4 vv = vt[2 * u + h];
            acc[cell_of<CW>(w, 0) * nth] += vv.x * p.x;
            acc[cell_of<CW>(w, 1) * nth] += vv.y * p.y;
            acc[cell_of<CW>(w, 2) * nth] += vv.z * p.z;
            acc[cell_of<CW>(w, 3) * nth] += vv.w * p.w;
          }
        }
        vt += 2 * A;
      }
    }
    for (int c = 0; c < info.y; ++c)
      row[offset + c] = static_cast<double>(acc[c * nth]) * unscale;
  }
}

// ---- float-float (FP64-accurate) variants -------------------------------------------------
__device__ __forceinline__ ff shfl_ff(ff v, int mask) {
  return ff{__shfl_xor_sync(0xffffffffu, v.h, mask), __shfl_xor_sync(0xffffffffu, v.l, mask)};
}

// reduce4 in float-float
__device__ __forceinline__ ff reduce4_ff(ff v0, ff v1, ff v2, ff v3, int lane) {
  const bool hi = lane & 16;
  ff a0 = hi ? v2 : v0, a1 = hi ? v3 : v1;
  const ff s0 = hi ? v0 : v2, s1 = hi ? v1 : v3;
  add_ff(a0, shfl_ff(s0, 16));
  add_ff(a1, shfl_ff(s1, 16));
  const bool b3 = lane & 8;
  ff b = b3 ? a1 : a0;
  add_ff(b, shfl_ff(b3 ? a0 : a1, 8));
  add_ff(b, shfl_ff(b, 4));
  add_ff(b, shfl_ff(b, 2));
  add_ff(b, shfl_ff(b, 1));
  return b;
}

// The float-float mult with the structure of mat_mult_kernel: a lane takes subspaces s and s + 32
// of the same four points, adds their float-float terms and runs one float-float butterfly.
template <typename CW>
__global__ void __launch_bounds__(kMatThreads, 1) mat_mult_df_kernel(
    const int4* __restrict__ sact, int n_sub, int s_pad, int cmax,
    const float2* __restrict__ asub2, int64_t m, int64_t tile_begin, int64_t n_tiles,
    const float4* __restrict__ phi, const float4* __restrict__ plo,
    const CW* __restrict__ cm, double* __restrict__ out64) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int sp = mult_at_pad(s_pad);                  // row length of s_at
  float2* s_part = reinterpret_cast<float2*>(smem);  // [warps][kOwnTile]
  float2* s_at = s_part + kMatWarps * kOwnTile;      // [cmax][sp]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int k = tid; k < cmax * sp; k += blockDim.x) {
    const int c = k / sp, sidx = k - c * sp;
    float2 a = make_float2(0.0f, 0.0f);
    if (sidx < n_sub) {
      const int4 info = sact[sidx];
      const int off = static_cast<int>(static_cast<uint32_t>(info.x) - static_cast<uint32_t>(info.z));
      if (c < info.y) a = asub2[off + c];
    }
    s_at[k] = a;
  }
  __syncthreads();
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t gt = tile_begin + tile;
    for (int s0 = 0; s0 < s_pad; s0 += kMultBlock * kMatWarps) {
      const int wb = s0 + warp * kMultBlock;
      if (wb >= s_pad) continue;  // whole warps: s_pad is a multiple of 32
      const int sid = wb + lane;
      const bool two = wb + 32 < s_pad;  // warp-uniform
      const int64_t at = gt * kGroups * static_cast<int64_t>(s_pad) + sid;
      const int64_t at2 = two ? at + 32 : at;  // the first block again, times a zero column
      const float2* a_col = s_at + sid;
      const float2* a_col2 = a_col + 32;
      float2* part = s_part + warp * kOwnTile;
      const bool first = s0 == 0;
      float4 rh[kAheadDf], rl[kAheadDf], qh[kAheadDf], ql[kAheadDf];
      CW rc[kAheadDf], qc[kAheadDf];
#pragma unroll
      for (int u = 0; u < kAheadDf; ++u) {
        rh[u] = __ldcs(phi + at + static_cast<int64_t>(u) * s_pad);
        rl[u] = __ldcs(plo + at + static_cast<int64_t>(u) * s_pad);
        rc[u] = __ldcs(cm + at + static_cast<int64_t>(u) * s_pad);
        qh[u] = __ldcs(phi + at2 + static_cast<int64_t>(u) * s_pad);
        ql[u] = __ldcs(plo + at2 + static_cast<int64_t>(u) * s_pad);
        qc[u] = __ldcs(cm + at2 + static_cast<int64_t>(u) * s_pad);
      }
      for (int g0 = 0; g0 < kGroups; g0 += kAheadDf) {
#pragma unroll
        for (int u = 0; u < kAheadDf; ++u) {
          const int g = g0 + u;
          const float4 ph = rh[u], pl = rl[u], gh = qh[u], gl = ql[u];
          const uint32_t cs = rc[u], cq = qc[u];
          if (g + kAheadDf < kGroups) {
            const int64_t o = static_cast<int64_t>(g + kAheadDf) * s_pad;
            rh[u] = __ldcs(phi + at + o);
            rl[u] = __ldcs(plo + at + o);
            rc[u] = __ldcs(cm + at + o);
            qh[u] = __ldcs(phi + at2 + o);
            ql[u] = __ldcs(plo + at2 + o);
            qc[u] = __ldcs(cm + at2 + o);
          }
          // cells are below cmax by construction
          const float ph_[4] = {ph.x, ph.y, ph.z, ph.w}, pl_[4] = {pl.x, pl.y, pl.z, pl.w};
          const float gh_[4] = {gh.x, gh.y, gh.z, gh.w}, gl_[4] = {gl.x, gl.y, gl.z, gl.w};
          ff v[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const float2 a = a_col[cell_of<CW>(cs, i) * sp];
            const float2 b2 = a_col2[cell_of<CW>(cq, i) * sp];
            v[i] = mul_ff(ff{ph_[i], pl_[i]}, ff{a.x, a.y});
            add_ff(v[i], mul_ff(ff{gh_[i], gl_[i]}, ff{b2.x, b2.y}));
          }
          const ff r = reduce4_ff(v[0], v[1], v[2], v[3], lane);
          if ((lane & 7) == 0) {
            float2* dst = part + 4 * g + (lane >> 3);
            ff acc = first ? ff{0.0f, 0.0f} : ff{dst->x, dst->y};
            add_ff(acc, r);
            *dst = make_float2(acc.h, acc.l);
          }
        }
      }
    }
    __syncthreads();
    // warp w wrote its partials in pass 0 iff w * kMultBlock < s_pad
    const int wrote = min(kMatWarps, (s_pad + kMultBlock - 1) / kMultBlock);
    for (int jj = tid; jj < kOwnTile; jj += blockDim.x) {
      ff r{0.0f, 0.0f};
      for (int w = 0; w < wrote; ++w) {
        const float2 q = s_part[w * kOwnTile + jj];
        add_ff(r, ff{q.x, q.y});
      }
      const int64_t j = gt * kOwnTile + jj;
      out64[j] = j < m ? static_cast<double>(r.h) + static_cast<double>(r.l) : 0.0;
    }
    __syncthreads();
  }
}

// SACC as in mat_multt_kernel: the flushes go into FP64 sums in shared memory and the row is
// written once per pass.
template <typename CW, bool SACC>
__global__ void __launch_bounds__(kMatThreads, 1) mat_multt_df_kernel(
    const int4* __restrict__ sact, int n_sub, int s_pad, int cmax, int total,
    const float* __restrict__ vh, const float* __restrict__ vl, int64_t n_tiles,
    const float4* __restrict__ phi, const float4* __restrict__ plo,
    const CW* __restrict__ cm, double* __restrict__ rows) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, nth = blockDim.x;
  double* s_sum = reinterpret_cast<double*>(smem);  // [cmax][blockDim] (SACC)
  float2* s_acc = reinterpret_cast<float2*>(SACC ? smem + sizeof(double) * cmax * nth : smem);  // [cmax][blockDim]
  double* row = rows + static_cast<int64_t>(blockIdx.x) * total;
  const uint32_t cm1 = static_cast<uint32_t>(cmax - 1);
  const float4* vh4 = reinterpret_cast<const float4*>(vh);
  const float4* vl4 = reinterpret_cast<const float4*>(vl);
  for (int s0 = 0; s0 < n_sub; s0 += nth) {
    const int sid = s0 + tid;
    if (sid >= n_sub) continue;  // no barriers below: threads run independently
    const int4 info = sact[sid];
    const uint32_t offset = static_cast<uint32_t>(info.x) - static_cast<uint32_t>(info.z);
    float2* acc = s_acc + tid;
    for (int c = 0; c < info.y; ++c) acc[c * nth] = make_float2(0.0f, 0.0f);
    bool first = true;
    // the CTA's tiles are contiguous and the ring runs over all of them, instead of starting again
    // at each tile
    const int64_t g_begin = (blockIdx.x * n_tiles / gridDim.x) * kGroups;
    const int64_t g_end = ((blockIdx.x + 1) * n_tiles / gridDim.x) * kGroups;
    if (g_begin < g_end) {
      int64_t nxt = g_begin * s_pad + sid;
      float4 rh[kAheadDf], rl[kAheadDf];
      CW rc[kAheadDf];
#pragma unroll
      for (int u = 0; u < kAheadDf; ++u) {
        rh[u] = ld_stream(phi + nxt);
        rl[u] = ld_stream(plo + nxt);
        rc[u] = ld_stream(cm + nxt);
        nxt += s_pad;
      }
      int since = 0;  // groups summed in s_acc since the last flush
      for (int64_t g0 = g_begin; g0 < g_end; g0 += kAheadDf) {
        const bool fetch = g0 + kAheadDf < g_end;
#pragma unroll
        for (int u = 0; u < kAheadDf; ++u) {
          const int64_t g = g0 + u;
          const float4 ph = rh[u], pl = rl[u];
          const uint32_t cs = rc[u];
          if (fetch) {
            rh[u] = ld_stream(phi + nxt);
            rl[u] = ld_stream(plo + nxt);
            rc[u] = ld_stream(cm + nxt);
            nxt += s_pad;
          }
          const float4 vvh = vh4[g], vvl = vl4[g];
          const float ph_[4] = {ph.x, ph.y, ph.z, ph.w}, pl_[4] = {pl.x, pl.y, pl.z, pl.w};
          const float vh_[4] = {vvh.x, vvh.y, vvh.z, vvh.w}, vl_[4] = {vvl.x, vvl.y, vvl.z, vvl.w};
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            float2* slot = acc + min(cell_of<CW>(cs, i), cm1) * nth;
            ff a{slot->x, slot->y};
            add_ff(a, mul_ff(ff{ph_[i], pl_[i]}, ff{vh_[i], vl_[i]}));
            *slot = make_float2(a.h, a.l);
          }
        }
        since += kAheadDf;
        if (since == kFlushTiles * kGroups || !fetch) {
          for (int c = 0; c < info.y; ++c) {
            const float2 a = acc[c * nth];
            const double v = static_cast<double>(a.x) + static_cast<double>(a.y);
            double* dst = SACC ? s_sum + c * nth + tid : row + offset + c;
            *dst = first ? v : *dst + v;
            acc[c * nth] = make_float2(0.0f, 0.0f);
          }
          first = false;
          since = 0;
        }
      }
    }
    if (first) {
      for (int c = 0; c < info.y; ++c) row[offset + c] = 0.0;
    } else if (SACC) {
      for (int c = 0; c < info.y; ++c) row[offset + c] = s_sum[c * nth + tid];
    }
  }
}

// ---- fused system product B^T (B a) --------------------------------------------------------
// One CTA owns every subspace (s_pad <= kSysMaxSub, in passes of blockDim) and walks tiles of
// kSysTile points: phase A streams the tile's P and C from HBM and forms (B a)_j exactly as
// mat_mult_kernel (butterfly, per-warp partials, warp-order sum); phase B streams the same tile
// again, now from L2, and adds (B a)_j * p into the owner's cells as mat_multt_kernel. So P and
// C leave HBM once per system product instead of twice. While a tile is processed, one thread asks
// L2 for the CTA's next tile (two bulk prefetches, a hint with nothing to wait for), so that HBM
// stays busy during phase B; a tile and its successor take 2 * T * s_pad * 5 bytes per CTA
// (~50 MB of L2 for all CTAs at T = 32, s_pad = 1024).
constexpr int kSysTile = 32;                 // points per tile
constexpr int kSysGroups = kSysTile / 4;
constexpr int kSysAhead = 4;                 // ring depth
constexpr int kSysThreads = 1024;            // one CTA per SM, one subspace per thread
constexpr int kSysWarps = kSysThreads / 32;
constexpr int kSysFlushTiles = 32;           // FP32 sums over 1024 points per flush
constexpr int kSysMaxSub = 1024;
static_assert(kSysGroups % kSysAhead == 0, "the ring must divide a tile");

template <typename CW>
__global__ void __launch_bounds__(kSysThreads, 1) mat_system_kernel(
    const int4* __restrict__ sact, int n_sub, int s_pad, int cmax, int total,
    const float* __restrict__ asub, int64_t n_tiles, const float4* __restrict__ pm,
    const CW* __restrict__ cm, double* __restrict__ rows) {
  extern __shared__ __align__(16) unsigned char smem[];
  float* s_at = reinterpret_cast<float*>(smem);            // [cmax][s_pad] alpha by (cell, s)
  float* s_acc = s_at + static_cast<size_t>(cmax) * s_pad;  // [cmax][s_pad] sums by (cell, s)
  float* s_part = s_acc + static_cast<size_t>(cmax) * s_pad;  // [warps][kSysTile]
  float* s_ba = s_part + kSysWarps * kSysTile;               // [kSysTile] (B a)_j
  double* row = rows + static_cast<int64_t>(blockIdx.x) * total;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t cm1 = static_cast<uint32_t>(cmax - 1);
  for (int k = tid; k < cmax * s_pad; k += blockDim.x) {
    const int c = k / s_pad, sidx = k - c * s_pad;
    float a = 0.0f;
    if (sidx < n_sub) {
      const int4 info = sact[sidx];
      const int off = static_cast<int>(static_cast<uint32_t>(info.x) - static_cast<uint32_t>(info.z));
      if (c < info.y) a = asub[off + c];
    }
    s_at[k] = a;
    s_acc[k] = 0.0f;
  }
  __syncthreads();
  int since = 0;
  bool first = true;
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t g_base = tile * kSysGroups;  // first point group of the tile
    if (tid == 0 && tile + gridDim.x < n_tiles) {
      const int64_t nb = (tile + gridDim.x) * kSysGroups * static_cast<int64_t>(s_pad);
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(pm + nb),
                   "r"(static_cast<uint32_t>(sizeof(float4) * kSysGroups * s_pad)) : "memory");
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(cm + nb),
                   "r"(static_cast<uint32_t>(sizeof(CW) * kSysGroups * s_pad)) : "memory");
    }
    // phase A: (B a)_j for the tile's points
    for (int s0 = 0; s0 < s_pad; s0 += blockDim.x) {
      if (s0 + warp * 32 >= s_pad) continue;
      const int sid = s0 + tid;
      const int64_t at = g_base * s_pad + sid;
      const float* a_col = s_at + sid;
      float* part = s_part + warp * kSysTile;
      const bool pass0 = s0 == 0;
      float4 ring[kSysAhead];
      CW cring[kSysAhead];
#pragma unroll
      for (int u = 0; u < kSysAhead; ++u) {
        ring[u] = __ldcg(pm + at + static_cast<int64_t>(u) * s_pad);
        cring[u] = __ldcg(cm + at + static_cast<int64_t>(u) * s_pad);
      }
      for (int g0 = 0; g0 < kSysGroups; g0 += kSysAhead) {
#pragma unroll
        for (int u = 0; u < kSysAhead; ++u) {
          const int g = g0 + u;
          const float4 p = ring[u];
          const uint32_t cs = cring[u];
          if (g + kSysAhead < kSysGroups) {
            ring[u] = __ldcg(pm + at + static_cast<int64_t>(g + kSysAhead) * s_pad);
            cring[u] = __ldcg(cm + at + static_cast<int64_t>(g + kSysAhead) * s_pad);
          }
          const float v0 = a_col[min(cell_of<CW>(cs, 0), cm1) * s_pad] * p.x;
          const float v1 = a_col[min(cell_of<CW>(cs, 1), cm1) * s_pad] * p.y;
          const float v2 = a_col[min(cell_of<CW>(cs, 2), cm1) * s_pad] * p.z;
          const float v3 = a_col[min(cell_of<CW>(cs, 3), cm1) * s_pad] * p.w;
          const float r = reduce4(v0, v1, v2, v3, lane);
          if ((lane & 7) == 0) {
            float* dst = part + 4 * g + (lane >> 3);
            *dst = pass0 ? r : *dst + r;
          }
        }
      }
    }
    __syncthreads();
    const int wrote = min(kSysWarps, s_pad / 32);
    for (int jj = tid; jj < kSysTile; jj += blockDim.x) {
      float r = 0.0f;
      for (int w = 0; w < wrote; ++w) r += s_part[w * kSysTile + jj];
      s_ba[jj] = r;  // points outside the data have P = 0, so their (B a)_j is 0
    }
    __syncthreads();
    // phase B: the owner of subspace s adds (B a)_j * p_s(x_j) into its cells
    for (int s0 = 0; s0 < s_pad; s0 += blockDim.x) {
      const int sid = s0 + tid;
      if (sid >= n_sub) continue;
      const int64_t at = g_base * s_pad + sid;
      float* acc = s_acc + sid;
      float4 ring[kSysAhead];
      CW cring[kSysAhead];
#pragma unroll
      for (int u = 0; u < kSysAhead; ++u) {
        ring[u] = __ldcs(pm + at + static_cast<int64_t>(u) * s_pad);
        cring[u] = __ldcs(cm + at + static_cast<int64_t>(u) * s_pad);
      }
      for (int g0 = 0; g0 < kSysGroups; g0 += kSysAhead) {
#pragma unroll
        for (int u = 0; u < kSysAhead; ++u) {
          const int g = g0 + u;
          const float4 p = ring[u];
          const uint32_t cs = cring[u];
          if (g + kSysAhead < kSysGroups) {
            ring[u] = __ldcs(pm + at + static_cast<int64_t>(g + kSysAhead) * s_pad);
            cring[u] = __ldcs(cm + at + static_cast<int64_t>(g + kSysAhead) * s_pad);
          }
          const float4 ba = *reinterpret_cast<const float4*>(s_ba + 4 * g);
          acc[min(cell_of<CW>(cs, 0), cm1) * s_pad] += ba.x * p.x;
          acc[min(cell_of<CW>(cs, 1), cm1) * s_pad] += ba.y * p.y;
          acc[min(cell_of<CW>(cs, 2), cm1) * s_pad] += ba.z * p.z;
          acc[min(cell_of<CW>(cs, 3), cm1) * s_pad] += ba.w * p.w;
        }
      }
    }
    ++since;
    const bool last = tile + gridDim.x >= n_tiles;
    if (since == kSysFlushTiles || last) {
      for (int s0 = 0; s0 < n_sub; s0 += blockDim.x) {
        const int sid = s0 + tid;
        if (sid >= n_sub) continue;
        const int4 info = sact[sid];
        const uint32_t offset = static_cast<uint32_t>(info.x) - static_cast<uint32_t>(info.z);
        for (int c = 0; c < info.y; ++c) {
          float& a = s_acc[c * s_pad + sid];
          double* dst = row + offset + c;
          *dst = first ? static_cast<double>(a) : *dst + static_cast<double>(a);
          a = 0.0f;
        }
      }
      first = false;
      since = 0;
    }
    __syncthreads();  // s_part and s_ba are rewritten by the next tile
  }
  if (first) {  // no tile for this CTA: its row holds zeros
    for (int s0 = 0; s0 < n_sub; s0 += blockDim.x) {
      const int sid = s0 + tid;
      if (sid >= n_sub) continue;
      const int4 info = sact[sid];
      const uint32_t offset = static_cast<uint32_t>(info.x) - static_cast<uint32_t>(info.z);
      for (int c = 0; c < info.y; ++c) row[offset + c] = 0.0;
    }
  }
}

size_t mat_system_smem(int cmax, int64_t s_pad) {
  return sizeof(float) * (2 * static_cast<size_t>(cmax) * s_pad + kSysWarps * kSysTile + kSysTile);
}

int mat_threads(int64_t s_pad) { return static_cast<int>(std::min<int64_t>(kMatThreads, s_pad)); }

size_t mat_mult_smem(int cmax, int64_t s_pad) {
  return sizeof(float) * kMatWarps * kOwnTile +
         sizeof(float) * static_cast<size_t>(cmax) * mult_at_pad(static_cast<int>(s_pad));
}

// FP64 flush sums in shared memory when FP32 cells and FP64 sums leave room for two CTAs per SM
bool mat_multt_sacc(int cmax, int64_t s_pad) {
  return (sizeof(float) + sizeof(double)) * static_cast<size_t>(cmax) * mat_threads(s_pad) <=
         96 * 1024;
}

size_t mat_multt_smem(int cmax, int64_t s_pad) {
  const size_t per = mat_multt_sacc(cmax, s_pad) ? sizeof(float) + sizeof(double) : sizeof(float);
  return per * static_cast<size_t>(cmax) * mat_threads(s_pad);
}

size_t mat_mult_df_smem(int cmax, int64_t s_pad) {
  return sizeof(float2) * kMatWarps * kOwnTile +
         sizeof(float2) * static_cast<size_t>(cmax) * mult_at_pad(static_cast<int>(s_pad));
}

// FP64 flush sums in shared memory while float-float cells and FP64 sums stay within 128 KB (the
// float-float kernels run one CTA per SM)
bool mat_multt_df_sacc(int cmax, int64_t s_pad) {
  return (sizeof(float2) + sizeof(double)) * static_cast<size_t>(cmax) * mat_threads(s_pad) <=
         128 * 1024;
}

size_t mat_multt_df_smem(int cmax, int64_t s_pad) {
  const size_t per = mat_multt_df_sacc(cmax, s_pad) ? sizeof(float2) + sizeof(double) : sizeof(float2);
  return per * static_cast<size_t>(cmax) * mat_threads(s_pad);
}

constexpr size_t kMatSmemBudget = 200 * 1024;

// subspaces per window of the materialised mult: all of them when their coefficients fit the
// shared memory budget, else the largest multiple of kMultBlock that does (0 if none)
int mat_mult_window(int cmax, int64_t s_pad) {
  if (mat_mult_smem(cmax, s_pad) <= kMatSmemBudget) return static_cast<int>(s_pad);
  int w = 0;
  while (w + kMultBlock < s_pad && mat_mult_smem(cmax, w + kMultBlock) <= kMatSmemBudget)
    w += kMultBlock;
  return w;
}

}  // namespace

bool subspace_mat_fits(const SubPlan& p, bool df) {
  const int64_t s_pad = (p.n_sub + 31) / 32 * 32;
  if (!(p.n_sub > 0 && p.cmax > 0 && p.cmax <= kMatMaxCells && p.rows != nullptr)) return false;
  if (df)
    return mat_mult_df_smem(p.cmax, s_pad) <= kMatSmemBudget &&
           mat_multt_df_smem(p.cmax, s_pad) <= kMatSmemBudget;
  // the mult takes its subspaces in windows where all coefficients do not fit at once
  return mat_mult_window(p.cmax, s_pad) > 0 && mat_multt_smem(p.cmax, s_pad) <= kMatSmemBudget;
}

// nibble cells when every subspace has at most 16 cells
bool mat_cell4(const SubPlan& p) { return p.cmax <= 16; }

void subspace_mat_release(SubPlan* p, cudaStream_t s) {
  dev_free(p->pmat, s);
  dev_free(p->pmat_lo, s);
  dev_free(p->pmat16, s);
  dev_free(p->cmat, s);
  dev_free(p->cpair, s);
  p->pmat = p->pmat_lo = nullptr;
  p->pmat16 = nullptr;
  p->cmat = p->cpair = nullptr;
}

int64_t subspace_mat_bytes(const SubPlan& p, int64_t mpad) {
  // P_hi, P_lo (4 + 4 bytes), the FP16 copy (2) and the cells: byte cells (1) and their pair copy
  // (1), or during the build the byte cells beside the nibbles (0.5) and their pair copy (0.5)
  const double per = 2 * sizeof(float) + 2 + 2.0;
  return static_cast<int64_t>(static_cast<double>(mpad) * ((p.n_sub + 31) / 32 * 32) * per);
}

namespace {
// byte cells [g][s] -> nibble cells [g][s] (four per uint16) and their pair copy [g / 2][s] (two
// nibble words per uint32)
__global__ void pack_cells_kernel(const uint32_t* __restrict__ in, int64_t n_pairs, int s_pad,
                                  uint16_t* __restrict__ out, uint32_t* __restrict__ pair) {
  const int64_t n = n_pairs * s_pad;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < n;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t k = e / s_pad;
    const int64_t a = e + k * s_pad;  // group 2k of the same subspace, then group 2k + 1
    uint32_t nib[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint32_t w = in[a + h * s_pad];
      nib[h] = (w & 0xFu) | ((w >> 4) & 0xF0u) | ((w >> 8) & 0xF00u) | ((w >> 12) & 0xF000u);
      out[a + h * s_pad] = static_cast<uint16_t>(nib[h]);
    }
    pair[e] = nib[0] | (nib[1] << 16);
  }
}

// byte cells [g][s] -> their pair copy [g / 2][s] (two words per uint2)
__global__ void pair_cells_kernel(const uint32_t* __restrict__ in, int64_t n_pairs, int s_pad,
                                  uint2* __restrict__ pair) {
  const int64_t n = n_pairs * s_pad;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < n;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t a = e + (e / s_pad) * s_pad;
    pair[e] = make_uint2(in[a], in[a + s_pad]);
  }
}
}  // namespace

cudaError_t subspace_materialize(SubPlan* p, cudaStream_t s, const float* xh, const float* xl,
                                 int64_t mpad, int64_t m, int num_sms) {
  auto release = [&](uint32_t* cm8) {
    dev_free(p->pmat, s);
    dev_free(p->pmat_lo, s);
    dev_free(p->pmat16, s);
    dev_free(p->cpair, s);
    if (cm8 != p->cmat) dev_free(cm8, s);
    dev_free(p->cmat, s);
    p->pmat = p->pmat_lo = nullptr;
    p->pmat16 = nullptr;
    p->cmat = p->cpair = nullptr;
  };
  release(nullptr);  // a previous build of this plan
  p->cell_bits = 8;
  p->s_pad = (p->n_sub + 31) / 32 * 32;
  p->mat_mpad = mpad;
  const size_t entries = static_cast<size_t>(mpad / 4) * static_cast<size_t>(p->s_pad);
  const int64_t n_pairs = mpad / 8;  // mpad is a multiple of the tile (256 points)
  uint32_t* cm8 = nullptr;
  cudaError_t e = dev_malloc(&p->pmat, entries * sizeof(float4), s);
  if (e == cudaSuccess) e = dev_malloc(&p->pmat_lo, entries * sizeof(float4), s);
  if (e == cudaSuccess) e = dev_malloc(&p->pmat16, entries / 2 * sizeof(uint4), s);
  if (e == cudaSuccess) e = dev_malloc(&cm8, entries * sizeof(uint32_t), s);
  if (e != cudaSuccess) {
    release(cm8);
    (void)cudaGetLastError();
    return e;
  }
  p->cmat = cm8;
  e = subspace_mat_build(*p, s, xh, xl, mpad, m, num_sms);
  const unsigned blocks = static_cast<unsigned>(std::min<int64_t>(
      16 * num_sms, std::max<int64_t>(1, (n_pairs * p->s_pad + 255) / 256)));
  if (e == cudaSuccess && mat_cell4(*p)) {
    // nibble cells, and their pair copy for the FP16 kernels (0.5 + 0.5 byte per entry)
    uint16_t* cm4 = nullptr;
    uint32_t* cp = nullptr;
    e = dev_malloc(&cm4, entries * sizeof(uint16_t), s);
    if (e == cudaSuccess) e = dev_malloc(&cp, entries / 2 * sizeof(uint32_t), s);
    if (e == cudaSuccess) {
      pack_cells_kernel<<<blocks, 256, 0, s>>>(cm8, n_pairs, static_cast<int>(p->s_pad), cm4, cp);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
      dev_free(cm8, s);
      p->cmat = cm4;
      p->cpair = cp;
      p->cell_bits = 4;
    } else {
      dev_free(cm4, s);
      dev_free(cp, s);
    }
  } else if (e == cudaSuccess) {
    uint2* cp = nullptr;
    e = dev_malloc(&cp, entries / 2 * sizeof(uint2), s);
    if (e == cudaSuccess) {
      pair_cells_kernel<<<blocks, 256, 0, s>>>(cm8, n_pairs, static_cast<int>(p->s_pad), cp);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) p->cpair = cp;
    else dev_free(cp, s);
  }
  if (e != cudaSuccess) {
    release(cm8);
    (void)cudaGetLastError();
    return e;
  }
  return cudaSuccess;
}

bool subspace_system_mat_fits(const SubPlan& p) {
  const int64_t s_pad = (p.n_sub + 31) / 32 * 32;
  return subspace_mat_fits(p, false) && s_pad <= kSysMaxSub &&
         mat_system_smem(p.cmax, s_pad) <= kMatSmemBudget;
}

namespace {
template <typename CW>
cudaError_t launch_system(const SubPlan& p, cudaStream_t s, int64_t nt, int64_t rows) {
  auto kern = mat_system_kernel<CW>;
  const size_t sm = mat_system_smem(p.cmax, p.s_pad);
  cudaError_t e = set_smem_cap(kern, sm);
  if (e != cudaSuccess) return e;
  kern<<<static_cast<unsigned>(rows), kSysThreads, sm, s>>>(
      p.sact, p.n_sub, static_cast<int>(p.s_pad), p.cmax, static_cast<int>(p.total), p.asub, nt,
      p.pmat, static_cast<const CW*>(p.cmat), p.rows);
  return cudaGetLastError();
}

template <typename CW>
cudaError_t launch_mult_df(const SubPlan& p, cudaStream_t s, int64_t m, double* out64, int64_t t0,
                           int64_t nt, int num_sms) {
  auto kern = mat_mult_df_kernel<CW>;
  const size_t sm = mat_mult_df_smem(p.cmax, p.s_pad);
  cudaError_t e = set_smem_cap(kern, sm);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kMatThreads, sm);
  if (e != cudaSuccess) return e;
  const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(nt, static_cast<int64_t>(std::max(1, per_sm)) * num_sms));
  kern<<<static_cast<unsigned>(blocks), kMatThreads, sm, s>>>(
      p.sact, p.n_sub, static_cast<int>(p.s_pad), p.cmax, p.asub2, m, t0, nt, p.pmat, p.pmat_lo,
      static_cast<const CW*>(p.cmat), out64);
  return cudaGetLastError();
}

template <typename CW>
cudaError_t launch_multt_df(const SubPlan& p, cudaStream_t s, int64_t mpad, const float* vh,
                            const float* vl, int num_sms, int64_t* rows) {
  auto kern = mat_multt_df_sacc(p.cmax, p.s_pad) ? mat_multt_df_kernel<CW, true>
                                                 : mat_multt_df_kernel<CW, false>;
  const size_t sm = mat_multt_df_smem(p.cmax, p.s_pad);
  const int nth = mat_threads(p.s_pad);
  cudaError_t e = set_smem_cap(kern, sm);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nth, sm);
  if (e != cudaSuccess) return e;
  const int64_t nt = mpad / kOwnTile;
  *rows = std::min<int64_t>(std::max(1, per_sm) * static_cast<int64_t>(num_sms), std::min<int64_t>(p.row_cap, std::max<int64_t>(nt, 1)));
  kern<<<static_cast<unsigned>(*rows), nth, sm, s>>>(
      p.sact, p.n_sub, static_cast<int>(p.s_pad), p.cmax, static_cast<int>(p.total), vh, vl, nt,
      p.pmat, p.pmat_lo, static_cast<const CW*>(p.cmat), p.rows);
  return cudaGetLastError();
}

// HALF: the FP16 kernels on the pair layout (pmat16, cpair), else the FP32 ones ([g][s]: pmat, cmat)
template <bool HALF, typename CW>
cudaError_t launch_mat_mult(const SubPlan& p, cudaStream_t s, int64_t m, float* out32,
                            double* out64, int64_t t0, int64_t nt, int num_sms) {
  // all subspaces in one launch when their coefficients fit shared memory, else windows of w
  // subspaces in subspace order, each launch adding its sums to the outputs
  const int w = mat_mult_window(p.cmax, p.s_pad);
  if (w <= 0) return cudaErrorInvalidConfiguration;
  auto run = [&](auto kern, auto pm, auto cm, auto... extra) -> cudaError_t {
    const size_t smw = mat_mult_smem(p.cmax, std::min<int64_t>(w, p.s_pad));
    cudaError_t e = set_smem_cap(kern, smw);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kMatThreads, smw);
    if (e != cudaSuccess) return e;
    const int64_t blocks = std::max<int64_t>(
        1, std::min<int64_t>(nt, static_cast<int64_t>(std::max(1, per_sm)) * num_sms));
    for (int sb = 0; sb < p.n_sub; sb += w) {
      const int cnt = std::min(w, p.n_sub - sb);
      // the window's padded count stays within the padded rows: sb is a multiple of 64
      const int cnt_pad = w >= p.s_pad ? static_cast<int>(p.s_pad) : (cnt + 31) / 32 * 32;
      kern<<<static_cast<unsigned>(blocks), kMatThreads, mat_mult_smem(p.cmax, cnt_pad), s>>>(
          p.sact + sb, cnt, cnt_pad, p.cmax, p.asub, m, t0, nt, pm + sb, cm + sb, out32, out64,
          extra..., static_cast<int>(p.s_pad), sb > 0 ? 1 : 0);
      e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  };
  if constexpr (HALF)
    return run(mat_mult_half_kernel<CW>, static_cast<const uint4*>(p.pmat16),
               static_cast<const typename PairCells<CW>::T*>(p.cpair),
               std::ldexp(1.0f, -p16_exp(p)));
  else
    return run(mat_mult_kernel<CW>, static_cast<const float4*>(p.pmat),
               static_cast<const CW*>(p.cmat));
}
template <bool HALF, typename CW>
cudaError_t launch_mat_multt(const SubPlan& p, cudaStream_t s, int64_t mpad, const float* v32,
                             int num_sms, int64_t* rows) {
  const size_t sm = mat_multt_smem(p.cmax, p.s_pad);
  const int nth = mat_threads(p.s_pad);
  const bool sacc = mat_multt_sacc(p.cmax, p.s_pad);
  auto go = [&](auto kern, auto pm, auto cm, auto... extra) -> cudaError_t {
    cudaError_t e = set_smem_cap(kern, sm);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nth, sm);
    if (e != cudaSuccess) return e;
    const int64_t nt = mpad / kOwnTile;
    // one CTA per (stream, pass): the resident CTAs split into passes, each stream a row
    const int64_t passes = (p.n_sub + nth - 1) / nth;
    const int64_t streams = std::max<int64_t>(
        1, std::min<int64_t>(std::max(1, per_sm) * static_cast<int64_t>(num_sms) / passes,
                             std::min<int64_t>(p.row_cap, std::max<int64_t>(nt, 1))));
    *rows = streams;
    kern<<<static_cast<unsigned>(streams * passes), nth, sm, s>>>(
        p.sact, p.n_sub, static_cast<int>(p.s_pad), p.cmax, static_cast<int>(p.total), v32, nt,
        pm, cm, p.rows, static_cast<int>(streams), extra...);
    return cudaGetLastError();
  };
  // the three-CTA kernel: FP32 cell sums only (4 bytes per cell and owner)
  auto go_lean = [&](auto kern, auto pm, auto cm, auto... extra) -> cudaError_t {
    const size_t sml = sizeof(float) * static_cast<size_t>(p.cmax) * nth;
    cudaError_t e = set_smem_cap(kern, sml);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nth, sml);
    if (e != cudaSuccess) return e;
    const int64_t nt = mpad / kOwnTile;
    const int64_t passes = (p.n_sub + nth - 1) / nth;
    const int64_t streams = std::max<int64_t>(
        1, std::min<int64_t>(std::max(1, per_sm) * static_cast<int64_t>(num_sms) / passes,
                             std::min<int64_t>(p.row_cap, std::max<int64_t>(nt, 1))));
    *rows = streams;
    kern<<<static_cast<unsigned>(streams * passes), nth, sml, s>>>(
        p.sact, p.n_sub, static_cast<int>(p.s_pad), p.cmax, static_cast<int>(p.total), v32, nt,
        pm, cm, p.rows, static_cast<int>(streams), extra...);
    return cudaGetLastError();
  };
  if constexpr (HALF) {
    const uint4* pm = p.pmat16;
    const auto* cm = static_cast<const typename PairCells<CW>::T*>(p.cpair);
    const double un = std::ldexp(1.0, -p16_exp(p));
    // two banks take the shared memory of the single bank with its float-float sums
    // three CTAs per SM while their FP32 cell sums leave room for three (else the kernels above)
    if (p.multt_ctas == 3 && sizeof(float) * static_cast<size_t>(p.cmax) * nth <= 72 * 1024)
      return go_lean(mat_multt_half_lean_kernel<CW>, pm, cm, un);
    if (p.multt_banks == 2 && sacc) return go(mat_multt_half_banked_kernel<CW>, pm, cm, un);
    switch (p.multt_batch) {
      case 2:
        return sacc ? go(mat_multt_half_kernel<CW, true, 2>, pm, cm, un)
                    : go(mat_multt_half_kernel<CW, false, 2>, pm, cm, un);
      case 4:
        return sacc ? go(mat_multt_half_kernel<CW, true, 4>, pm, cm, un)
                    : go(mat_multt_half_kernel<CW, false, 4>, pm, cm, un);
      default:
        return sacc ? go(mat_multt_half_kernel<CW, true, 1>, pm, cm, un)
                    : go(mat_multt_half_kernel<CW, false, 1>, pm, cm, un);
    }
  } else {
    const float4* pm = p.pmat;
    const CW* cm = static_cast<const CW*>(p.cmat);
    return sacc ? go(mat_multt_kernel<CW, true>, pm, cm) : go(mat_multt_kernel<CW, false>, pm, cm);
  }
}
}  // namespace

cudaError_t subspace_system_mat(const SubPlan& p, cudaStream_t s, int64_t mpad,
                                const float* alpha32, int64_t npad, double* out64,
                                const double* add, double scale_add, int num_sms) {
  if (!p.pmat || !p.cmat || p.mat_mpad != mpad) return cudaErrorInvalidValue;
  cudaError_t e = subspace_scatter_alpha(p, s, alpha32);
  if (e != cudaSuccess) return e;
  const int64_t nt = mpad / kSysTile;
  const int64_t rows = std::min<int64_t>(num_sms, std::min<int64_t>(p.row_cap, std::max<int64_t>(nt, 1)));
  e = p.cell_bits == 4 ? launch_system<uint16_t>(p, s, nt, rows)
                       : launch_system<uint32_t>(p, s, nt, rows);
  if (e != cudaSuccess) return e;
  return subspace_finish_rows(p, s, rows, npad, out64, add, scale_add);
}

cudaError_t subspace_mult_mat_df(const SubPlan& p, cudaStream_t s, int64_t mpad, int64_t m,
                                 const float* ah, const float* al, double* out64, int64_t j_begin,
                                 int64_t j_end, int num_sms) {
  if (!p.pmat || !p.pmat_lo || !p.cmat || p.mat_mpad != mpad) return cudaErrorInvalidValue;
  cudaError_t e = subspace_scatter_alpha_df(p, s, ah, al);
  if (e != cudaSuccess) return e;
  const int64_t t0 = j_begin / kOwnTile;
  const int64_t nt = (j_end + kOwnTile - 1) / kOwnTile - t0;
  if (nt <= 0) return cudaSuccess;
  return p.cell_bits == 4 ? launch_mult_df<uint16_t>(p, s, m, out64, t0, nt, num_sms)
                          : launch_mult_df<uint32_t>(p, s, m, out64, t0, nt, num_sms);
}

cudaError_t subspace_multt_mat_df(const SubPlan& p, cudaStream_t s, int64_t mpad,
                                  const float* vh, const float* vl, int64_t npad, double* out64,
                                  const double* add, double scale_add, int num_sms) {
  if (!p.pmat || !p.pmat_lo || !p.cmat || p.mat_mpad != mpad) return cudaErrorInvalidValue;
  int64_t rows = 0;
  cudaError_t e = p.cell_bits == 4 ? launch_multt_df<uint16_t>(p, s, mpad, vh, vl, num_sms, &rows)
                                   : launch_multt_df<uint32_t>(p, s, mpad, vh, vl, num_sms, &rows);
  if (e != cudaSuccess) return e;
  return subspace_finish_rows(p, s, rows, npad, out64, add, scale_add);
}

cudaError_t subspace_mult_mat(const SubPlan& p, cudaStream_t s, const float* /*xt*/, int64_t mpad,
                              int64_t m, const float* alpha32, float* out32, double* out64,
                              int64_t j_begin, int64_t j_end, int num_sms, bool half) {
  if (!p.pmat || !p.pmat16 || !p.cmat || !p.cpair || p.mat_mpad != mpad) return cudaErrorInvalidValue;
  cudaError_t e = subspace_scatter_alpha(p, s, alpha32);
  if (e != cudaSuccess) return e;
  const int64_t t0 = j_begin / kOwnTile;
  const int64_t nt = (j_end + kOwnTile - 1) / kOwnTile - t0;
  if (nt <= 0) return cudaSuccess;
  if (p.cell_bits == 4)
    return half ? launch_mat_mult<true, uint16_t>(p, s, m, out32, out64, t0, nt, num_sms)
                : launch_mat_mult<false, uint16_t>(p, s, m, out32, out64, t0, nt, num_sms);
  return half ? launch_mat_mult<true, uint32_t>(p, s, m, out32, out64, t0, nt, num_sms)
              : launch_mat_mult<false, uint32_t>(p, s, m, out32, out64, t0, nt, num_sms);
}

cudaError_t subspace_multt_mat(const SubPlan& p, cudaStream_t s, const float* /*xt*/, int64_t mpad,
                               int64_t /*m*/, const float* v32, int64_t npad, double* out64,
                               const double* add, double scale_add, int num_sms, bool half) {
  if (!p.pmat || !p.pmat16 || !p.cmat || !p.cpair || p.mat_mpad != mpad) return cudaErrorInvalidValue;
  int64_t rows = 0;
  cudaError_t e;
  if (p.cell_bits == 4)
    e = half ? launch_mat_multt<true, uint16_t>(p, s, mpad, v32, num_sms, &rows)
             : launch_mat_multt<false, uint16_t>(p, s, mpad, v32, num_sms, &rows);
  else
    e = half ? launch_mat_multt<true, uint32_t>(p, s, mpad, v32, num_sms, &rows)
             : launch_mat_multt<false, uint32_t>(p, s, mpad, v32, num_sms, &rows);
  if (e != cudaSuccess) return e;
  return subspace_finish_rows(p, s, rows, npad, out64, add, scale_add);
}

}  // namespace sgmev

// Batched multi-problem, multi-right-hand-side kernels (one launch per phase for all problems).
//
// A batch holds independent regression problems ("slots") of uneven dimension d, grid size N and
// data size M, each with K right-hand sides. Each launch runs a fixed number of persistent CTAs
// that pull work items from a device list (one atomic counter per launch); an item is one tile
// of one slot, so results do not depend on which CTA ran it (deterministic).
//
//   mult item  (slot, data tile of BLOCK*R points, grid range [g0, g1), chunk q):
//       part[q][j][c] = sum_{g in range} alpha[g][c] * prod_t hat(x_jt; g)
//   multT item (slot, grid tile of BLOCK*RG points, data range [j0, j1), chunk q):
//       part[q][g][c] = sum_{j in range} v[j][c] * prod_t hat(x_jt; g)
//
// Vectors with K columns are stored row-major ([point][c]); a row of K floats is loaded as
// float4s from shared memory (broadcast), so K FMAs per (grid point, data point) pair run on the
// FP32 pipes beside the 3 d hat instructions. Two arithmetic policies:
//   F32  hat products and sums in FP32 (the inner CG)
//   DF   float-float ("df64") products and sums (the FP64-accurate refinement residual)
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.cuh"

namespace sgmev {

struct BatchSlot {   // device-side per-slot table entry
  int dim;
  int active;        // 1 if the slot takes part in the current launch
  int64_t n, npad, m, mpad;
  int64_t grid_off;  // element offset into the grid pools (li32 / gq), npad * dim entries
  int64_t data_off;  // element offset into the data pools (xh / xl), dim * mpad entries
  int64_t nvec_off;  // element offset into N-side pools, npad * K entries
  int64_t mvec_off;  // element offset into M-side pools, mpad * K entries
  int64_t part_off;  // element offset into the partial pool
  int nchunk[4];     // chunks per tile of the four item lists (mult/multT x FP32/df64)
};

struct BatchItem {
  int slot;
  int chunk;
  int64_t tile;
  int64_t begin, end;
};

constexpr int kBB = 128;   // threads per CTA
constexpr int kBGT = 32;   // grid points per shared tile (mult)
constexpr int kBDT = 64;   // data points per shared tile (multT)

// register blocking per (arithmetic, K): data points per thread (mult), grid points per thread
// (multT); chosen so that the K accumulators and the coordinates fit without spills at d = 16
__host__ __device__ constexpr int batch_r(bool df, int K) { return K == 1 ? 4 : (df ? 1 : 2); }
__host__ __device__ constexpr int batch_rg(bool df, int K) { return K == 1 ? 2 : (df ? 1 : 2); }

// ---------------- arithmetic policies ----------------
struct PolicyF32 {
  struct Acc {
    float v;
  };
  __device__ static Acc zero() { return Acc{0.0f}; }
  struct P {
    float v;
  };
  __device__ static P first(float xh, float xl, float2 li, float4 gq) {
    return P{hat_first(xh, li)};
  }
  __device__ static P next(P p, float xh, float xl, float2 li, float4 gq) {
    return P{hat_next(p.v, xh, li)};
  }
  // acc += p * (ch + cl)
  __device__ static void fma_acc(Acc& a, P p, float ch, float cl) { a.v = fmaf(p.v, ch, a.v); }
  __device__ static void renorm(Acc&) {}
  __device__ static float2 out(Acc a) { return make_float2(a.v, 0.0f); }
};

struct PolicyDF {
  struct Acc {
    ff v;
  };
  __device__ static Acc zero() { return Acc{ff{0.0f, 0.0f}}; }
  struct P {
    ff v;
  };
  __device__ static P first(float xh, float xl, float2 li, float4 gq) {
    return P{hat_ff(xh, xl, gq)};
  }
  __device__ static P next(P p, float xh, float xl, float2 li, float4 gq) {
    return P{mul_ff(p.v, hat_ff(xh, xl, gq))};
  }
  __device__ static void fma_acc(Acc& a, P p, float ch, float cl) {
    add_ff(a.v, mul_ff(p.v, ff{ch, cl}));
  }
  __device__ static void renorm(Acc& a) { renorm_ff(a.v); }
  __device__ static float2 out(Acc a) { return make_float2(a.v.h, a.v.l); }
};

template <class Pol>
struct IsDF {
  static constexpr bool value = false;
};
template <>
struct IsDF<PolicyDF> {
  static constexpr bool value = true;
};

// ---------------- batched mult ----------------
// alpha pools: ah/al [npad * K] row-major (al unused for F32); part: float2 (hi, lo) per entry
template <class Pol, int DIM, int K, int R = batch_r(IsDF<Pol>::value, K)>
__device__ void batch_mult_item(const BatchSlot& s, const BatchItem& it, const float* __restrict__ xh_pool,
                                const float* __restrict__ xl_pool, const float2* __restrict__ li_pool,
                                const float4* __restrict__ gq_pool, const float* __restrict__ ah_pool,
                                const float* __restrict__ al_pool, float2* __restrict__ part_pool,
                                float2* s_li, float4* s_gq, float* s_ah, float* s_al) {
  constexpr bool DF = IsDF<Pol>::value;
  const float* xh = xh_pool + s.data_off;
  const float* xl = xl_pool + s.data_off;
  const int64_t j0 = it.tile * (kBB * R) + threadIdx.x;
  float x[R][DIM];
  float xlo[DF ? R : 1][DF ? DIM : 1];
#pragma unroll
  for (int r = 0; r < R; ++r) {
#pragma unroll
    for (int t = 0; t < DIM; ++t) {
      x[r][t] = xh[static_cast<int64_t>(t) * s.mpad + j0 + r * kBB];
      if constexpr (DF) xlo[r][t] = xl[static_cast<int64_t>(t) * s.mpad + j0 + r * kBB];
    }
  }
  typename Pol::Acc acc[R][K];
#pragma unroll
  for (int r = 0; r < R; ++r) {
#pragma unroll
    for (int c = 0; c < K; ++c) acc[r][c] = Pol::zero();
  }
  const float2* li = li_pool + s.grid_off;
  const float4* gq = gq_pool + s.grid_off;
  const float* ah = ah_pool + s.nvec_off;
  const float* al = al_pool + s.nvec_off;
  for (int64_t g0 = it.begin; g0 < it.end; g0 += kBGT) {
    __syncthreads();
    for (int k = threadIdx.x; k < kBGT * DIM; k += kBB) {
      if constexpr (DF) s_gq[k] = gq[g0 * DIM + k];
      else s_li[k] = li[g0 * DIM + k];
    }
    for (int k = threadIdx.x; k < kBGT * K; k += kBB) {
      s_ah[k] = ah[g0 * K + k];
      if constexpr (DF) s_al[k] = al[g0 * K + k];
    }
    __syncthreads();
    for (int g = 0; g < kBGT; ++g) {
      typename Pol::P p[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if constexpr (DF) p[r] = Pol::first(x[r][0], xlo[r][0], float2{}, s_gq[g * DIM]);
        else p[r] = Pol::first(x[r][0], 0.0f, s_li[g * DIM], float4{});
      }
#pragma unroll
      for (int t = 1; t < DIM; ++t) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          if constexpr (DF) p[r] = Pol::next(p[r], x[r][t], xlo[r][t], float2{}, s_gq[g * DIM + t]);
          else p[r] = Pol::next(p[r], x[r][t], 0.0f, s_li[g * DIM + t], float4{});
        }
      }
#pragma unroll
      for (int c = 0; c < K; ++c) {
        const float ch = s_ah[g * K + c];
        const float cl = DF ? s_al[g * K + c] : 0.0f;
#pragma unroll
        for (int r = 0; r < R; ++r) Pol::fma_acc(acc[r][c], p[r], ch, cl);
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
#pragma unroll
      for (int c = 0; c < K; ++c) Pol::renorm(acc[r][c]);
    }
  }
  float2* out = part_pool + s.part_off + static_cast<int64_t>(it.chunk) * s.mpad * K;
  static_assert(R >= 1, "blocking");
#pragma unroll
  for (int r = 0; r < R; ++r) {
#pragma unroll
    for (int c = 0; c < K; ++c) out[(j0 + r * kBB) * K + c] = Pol::out(acc[r][c]);
  }
}

// ---------------- batched multT ----------------
// v pools: vh/vl [mpad * K] row-major; part: float2 per (grid point, column)
template <class Pol, int DIM, int K, int RG = batch_rg(IsDF<Pol>::value, K)>
__device__ void batch_multt_item(const BatchSlot& s, const BatchItem& it, const float* __restrict__ xh_pool,
                                 const float* __restrict__ xl_pool, const float2* __restrict__ li_pool,
                                 const float4* __restrict__ gq_pool, const float* __restrict__ vh_pool,
                                 const float* __restrict__ vl_pool, float2* __restrict__ part_pool,
                                 float* s_xh, float* s_xl, float* s_vh, float* s_vl) {
  constexpr bool DF = IsDF<Pol>::value;
  const int64_t g0 = it.tile * (kBB * RG) + threadIdx.x;
  const float2* li = li_pool + s.grid_off;
  const float4* gq = gq_pool + s.grid_off;
  float2 l[DF ? 1 : RG][DF ? 1 : DIM];
  float4 q[DF ? RG : 1][DF ? DIM : 1];
#pragma unroll
  for (int k = 0; k < RG; ++k) {
#pragma unroll
    for (int t = 0; t < DIM; ++t) {
      if constexpr (DF) q[k][t] = gq[(g0 + k * kBB) * DIM + t];
      else l[k][t] = li[(g0 + k * kBB) * DIM + t];
    }
  }
  typename Pol::Acc acc[RG][K];
#pragma unroll
  for (int k = 0; k < RG; ++k) {
#pragma unroll
    for (int c = 0; c < K; ++c) acc[k][c] = Pol::zero();
  }
  const float* xh = xh_pool + s.data_off;
  const float* xl = xl_pool + s.data_off;
  const float* vh = vh_pool + s.mvec_off;
  const float* vl = vl_pool + s.mvec_off;
  for (int64_t jt = it.begin; jt < it.end; jt += kBDT) {
    __syncthreads();
#pragma unroll
    for (int t = 0; t < DIM; ++t) {
      for (int k = threadIdx.x; k < kBDT; k += kBB) {
        s_xh[t * kBDT + k] = xh[static_cast<int64_t>(t) * s.mpad + jt + k];
        if constexpr (DF) s_xl[t * kBDT + k] = xl[static_cast<int64_t>(t) * s.mpad + jt + k];
      }
    }
    for (int k = threadIdx.x; k < kBDT * K; k += kBB) {
      s_vh[k] = vh[jt * K + k];
      if constexpr (DF) s_vl[k] = vl[jt * K + k];
    }
    __syncthreads();
    for (int j = 0; j < kBDT; ++j) {
      typename Pol::P p[RG];
#pragma unroll
      for (int k = 0; k < RG; ++k) {
        if constexpr (DF) p[k] = Pol::first(s_xh[j], s_xl[j], float2{}, q[k][0]);
        else p[k] = Pol::first(s_xh[j], 0.0f, l[k][0], float4{});
      }
#pragma unroll
      for (int t = 1; t < DIM; ++t) {
        const float xv = s_xh[t * kBDT + j];
        const float xw = DF ? s_xl[t * kBDT + j] : 0.0f;
#pragma unroll
        for (int k = 0; k < RG; ++k) {
          if constexpr (DF) p[k] = Pol::next(p[k], xv, xw, float2{}, q[k][t]);
          else p[k] = Pol::next(p[k], xv, 0.0f, l[k][t], float4{});
        }
      }
#pragma unroll
      for (int c = 0; c < K; ++c) {
        const float ch = s_vh[j * K + c];
        const float cl = DF ? s_vl[j * K + c] : 0.0f;
#pragma unroll
        for (int k = 0; k < RG; ++k) Pol::fma_acc(acc[k][c], p[k], ch, cl);
      }
    }
#pragma unroll
    for (int k = 0; k < RG; ++k) {
#pragma unroll
      for (int c = 0; c < K; ++c) Pol::renorm(acc[k][c]);
    }
  }
  float2* out = part_pool + s.part_off + static_cast<int64_t>(it.chunk) * s.npad * K;
#pragma unroll
  for (int k = 0; k < RG; ++k) {
#pragma unroll
    for (int c = 0; c < K; ++c) out[(g0 + k * kBB) * K + c] = Pol::out(acc[k][c]);
  }
}

}  // namespace sgmev

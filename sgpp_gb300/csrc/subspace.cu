// Subspace-skipping evaluation of the hat basis in FP32 (the reference's DEFAULT operator does
// the same on the CPU by hierarchical descent, base/src/sgpp/base/algorithm/AlgorithmEvaluation.hpp
// :129-179; SUBSPACELINEAR by flat subspace arrays, DatadrivenOpFactory.cpp:453-470).
//
// For a data point x and a subspace with level vector l, exactly one basis function can be
// non-zero: in dimension t its index is i_t = 2 k_t + 1 with k_t = floor(x_t 2^{l_t - 1}). So a
// product costs one evaluation per subspace instead of one per grid point. The kernels are
// branch-free per dimension: with S = 2^{l-1}, L = 2^l and xc = x clamped into [0, 1),
//     y5 = fma(xc, S, -0.5)               exact when xc S >= 0.5 (xc S is exact: S = 2^k)
//     r  = y5 + 1.5*2^23                  rounds to the integer k; r = 1.5*2^23 + k exactly
//     t  = fma(x, L, -(2 (r - 1.5*2^23) + 1)),  h = sat(1 - |t|),  p *= h
//     flat += bits(r) * stride            (the offset term is folded into the subspace base)
// Rounding xc S - 0.5 to the nearest integer gives floor(xc S) except at exact cell boundaries,
// where both neighbouring hats are 0, so the choice there does not matter; xc S < S - 0.5 keeps k
// at most S - 1, and x outside [0, 1) selects an edge cell whose hat is 0. (The constant
// 1.5*2^23 - 0.5 is not an FP32 number, so the 0.5 is subtracted in its own exact step.)
//
//   mult        gather: result_j = sum_s asub[pos_s(x_j)] * prod_t h_t; asub in shared memory
//   multT       scatter: contributions v_j * prod_t h_t are rounded to 43-bit fixed point (one
//               power-of-two scale from max|v| and M), split into a high word and a 22-bit low
//               word, added into two shared-memory int32 accumulators, and flushed into a global
//               int64 vector after every 512-point tile (so no word sum can overflow); integer
//               addition is exact and associative, so the result is the same bit for bit
//               whatever the order of the atomic updates
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "subspace.h"

namespace sgmev {

namespace {

constexpr int kSDT = 64;                  // subspaces per shared-memory descriptor tile
constexpr unsigned kMagicBits = 0x4B400000u;  // bits of 1.5 * 2^23
constexpr float kMagic = 12582912.0f;         // 1.5 * 2^23
constexpr float kBelowOne = 0.99999994f;      // largest float < 1

constexpr int kMultThreads = 128, kMultR = 4;
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
      const float rr = fmaf(pt.xc[r][t], S, -0.5f) + kMagic;
      const float nI = fmaf(rr - kMagic, -2.0f, -1.0f);
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

template <int DIM>
__global__ void __launch_bounds__(kMultThreads) sub_mult_kernel(
    const int4* __restrict__ desc, const uint32_t* __restrict__ base, int n_sub,
    const float* __restrict__ asub, int total, const float* __restrict__ xt, int64_t mpad,
    int64_t m, int64_t tile_begin, int64_t n_tiles, float* __restrict__ out32,
    double* __restrict__ out64) {
  extern __shared__ __align__(16) unsigned char smem[];
  int4* s_desc = reinterpret_cast<int4*>(smem);
  uint32_t* s_base = reinterpret_cast<uint32_t*>(s_desc + kSDT * DIM);
  float* s_a = reinterpret_cast<float*>(s_base + kSDT);
  for (int k = threadIdx.x; k < total; k += kMultThreads) s_a[k] = asub[k];
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t j0 = (tile_begin + tile) * (kMultThreads * kMultR) + threadIdx.x;
    Pt<DIM, kMultR> pt;
    load_points(pt, xt, mpad, j0, kMultThreads);
    float acc[kMultR];
#pragma unroll
    for (int r = 0; r < kMultR; ++r) acc[r] = 0.0f;
    for (int s0 = 0; s0 < n_sub; s0 += kSDT) {
      const int cnt = min(kSDT, n_sub - s0);
      __syncthreads();
      for (int k = threadIdx.x; k < cnt * DIM; k += kMultThreads) s_desc[k] = desc[s0 * DIM + k];
      for (int k = threadIdx.x; k < cnt; k += kMultThreads) s_base[k] = base[s0 + k];
      __syncthreads();
      for (int s = 0; s < cnt; ++s) {
        uint32_t flat[kMultR];
        float p[kMultR];
        eval_subspace<DIM, kMultR>(pt, s_desc + s * DIM, s_base[s], static_cast<uint32_t>(total - 1),
                                   flat, p);
#pragma unroll
        for (int r = 0; r < kMultR; ++r) acc[r] = fmaf(s_a[flat[r]], p[r], acc[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < kMultR; ++r) {
      const int64_t j = j0 + r * kMultThreads;
      const float v = j < m ? acc[r] : 0.0f;
      if (out32) out32[j] = v;
      if (out64) out64[j] = static_cast<double>(v);
    }
  }
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

size_t mult_smem(int dim, int64_t total) {
  return sizeof(int4) * kSDT * dim + sizeof(uint32_t) * kSDT + sizeof(float) * total;
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
  const size_t sm = mult_smem(DIM, p.total);
  cudaError_t e = cudaFuncSetAttribute(sub_mult_kernel<DIM>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
  if (e != cudaSuccess) return e;
  const int64_t blocks = std::min<int64_t>(nt, static_cast<int64_t>(num_sms) * 8);
  sub_mult_kernel<DIM><<<static_cast<unsigned>(std::max<int64_t>(blocks, 1)), kMultThreads, sm, s>>>(
      p.desc, p.base, p.n_sub, p.asub, static_cast<int>(p.total), xt, mpad, m, t0, nt, out32, out64);
  return cudaGetLastError();
}

template <int DIM>
cudaError_t launch_multt(const SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad,
                         int64_t m, const float* v, int num_sms) {
  const size_t sm = multt_smem(DIM, p.total);
  cudaError_t e = cudaFuncSetAttribute(sub_multt_kernel<DIM>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
  if (e != cudaSuccess) return e;
  const int64_t nt = mpad / (kMulttThreads * kMulttR);
  const int64_t blocks = multt_blocks(mpad, num_sms);
  sub_multt_kernel<DIM><<<static_cast<unsigned>(blocks), kMulttThreads, sm, s>>>(
      p.desc, p.base, p.n_sub, static_cast<int>(p.total), xt, mpad, m, nt, v, p.maxbits,
      static_cast<float>(std::max<int64_t>(m, 1)), p.acc);
  return cudaGetLastError();
}

}  // namespace

bool subspace_build(SubPlan* p, int dim, int64_t n, const double* level_pow2, const double* index,
                    std::string* err) {
  subspace_free(p);
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
  std::vector<int4> desc;
  std::vector<uint32_t> base;
  std::vector<int> pos(static_cast<size_t>(n));
  int64_t offset = 0;
  for (const auto& kv : groups) {
    const std::vector<int>& l = kv.first;
    std::vector<int64_t> stride(dim);
    int64_t size = 1;
    for (int t = dim - 1; t >= 0; --t) {  // row-major over dimensions
      stride[t] = size;
      size *= int64_t(1) << (l[t] - 1);
    }
    if (offset + size > kSubMaxPositions) {
      *err = "grid has more subspace positions than the shared-memory kernels hold";
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
  p->n = n;
  bool ok = cudaMalloc(&p->desc, sizeof(int4) * desc.size()) == cudaSuccess &&
            cudaMalloc(&p->base, sizeof(uint32_t) * base.size()) == cudaSuccess &&
            cudaMalloc(&p->pos, sizeof(int) * pos.size()) == cudaSuccess &&
            cudaMalloc(&p->asub, sizeof(float) * offset) == cudaSuccess &&
            cudaMalloc(&p->acc, sizeof(unsigned long long) * offset) == cudaSuccess &&
            cudaMalloc(&p->maxbits, sizeof(unsigned int)) == cudaSuccess;
  ok = ok && cudaMemcpy(p->desc, desc.data(), sizeof(int4) * desc.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(p->base, base.data(), sizeof(uint32_t) * base.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(p->pos, pos.data(), sizeof(int) * pos.size(), cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    subspace_free(p);
    *err = "subspace plan allocation failed";
    return false;
  }
  return true;
}

void subspace_free(SubPlan* p) {
  cudaFree(p->desc);
  cudaFree(p->base);
  cudaFree(p->pos);
  cudaFree(p->asub);
  cudaFree(p->acc);
  cudaFree(p->maxbits);
  *p = SubPlan{};
}

#define SUB_DIMS(F) F(1) F(2) F(3) F(4) F(5) F(6) F(7) F(8) F(9) F(10) F(11) F(12) F(13) F(14) F(15) F(16)

cudaError_t subspace_mult(const SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad,
                          int64_t m, const float* alpha32, float* out32, double* out64,
                          int64_t j_begin, int64_t j_end, int num_sms) {
  cudaError_t e = cudaMemsetAsync(p.asub, 0, sizeof(float) * p.total, s);
  if (e != cudaSuccess) return e;
  scatter_alpha_kernel<<<static_cast<unsigned>(std::min<int64_t>(1216, (p.n + 255) / 256)), 256, 0, s>>>(
      alpha32, p.pos, p.n, p.asub);
  const int64_t tile = kMultThreads * kMultR;
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

cudaError_t subspace_multt(const SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad,
                           int64_t m, const float* v32, int64_t npad, double* out64,
                           const double* add, double scale_add, int num_sms) {
  cudaError_t e = cudaMemsetAsync(p.maxbits, 0, sizeof(unsigned int), s);
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

}  // namespace sgmev

// libsgpp_gb300: GB300 multi-evaluation operator behind the C ABI declared in include/sgmev.h.
//
// Host-side structure (one op = one grid + one data set, as the reference operator):
//   staging   data rows -> dim-major FP64 and FP32 copies, grid (2^l, i) -> interleaved pairs
//   plans     per precision: CTA tile shapes and the 2-D split (tiles x chunks) sized so that
//             every launch has at least `target_ctas` CTAs on the 152 SMs
//   products  mult / multT = one tile kernel writing partials + one fixed-order reduce kernel
//   system    B^T(B a) + lambda*M*a: mult, reduce into the M-vector, multT, reduce (+ lambda term)
//   fit       conjugate gradients with every vector on the device; scalars come back to the
//             host once per dot product to drive the loop exactly like
//             solver/src/sgpp/solver/sle/ConjugateGradients.cpp:22-151
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sgmev.h"
#include "dense.h"
#include "kernels.cuh"
#include "devmem.h"
#include "subspace.h"
#include "block_tc.h"

namespace sgmev {

thread_local std::string g_last_error;

static int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define SGMEV_CUDA(call)                                                                 \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      return fail(e_ == cudaErrorMemoryAllocation ? SGMEV_ERR_OOM : SGMEV_ERR_CUDA,      \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                   \
    }                                                                                    \
  } while (0)

#define SGMEV_TRY(expr)   \
  do {                    \
    int rc_ = (expr);     \
    if (rc_ != SGMEV_OK) return rc_; \
  } while (0)

constexpr int64_t kMPadTo = 1024;
constexpr int64_t kNPadTo = 512;
constexpr int kReduceBlocks = 1216;  // 8 x 152 SMs
constexpr int kDotBlocks = 304;
constexpr int kDotThreads = 256;
constexpr int kCgSlots = 10;

static inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
static inline int64_t round_up(int64_t a, int64_t b) { return ceil_div(a, b) * b; }

struct Plan {
  int64_t tiles = 0;   // CTAs along the tiled axis
  int64_t nsplit = 1;  // CTAs along the split axis
  int64_t chunk = 0;   // elements of the split axis per CTA
  bool generic = false;
};

}  // namespace sgmev

using namespace sgmev;

struct sgmev_op {
  int dim = 0;
  int64_t n = 0, m = 0, npad = 0, mpad = 0;
  int precision = SGMEV_FP64;
  int device = 0;
  int num_sms = 152;
  int64_t target_ctas = 4 * 152;

  double* xt64 = nullptr;
  float* xt32 = nullptr;    // float(x)
  float* xt32lo = nullptr;  // float(x - float(x)): the df64 low part
  double2* li64 = nullptr;
  float2* li32 = nullptr;
  float4* gq = nullptr;     // df64 grid constants (2^l, 1 - i, 1 + i, 0)
  double* gs64 = nullptr;   // ModLinear: per-grid-point factor 2^b (0 on padding)
  float* gs32 = nullptr;
  int64_t npad_cap = 0;
  bool mod = false;         // modified linear basis (ModLinear grid; params "basis")
  bool in_cube = true;      // every data coordinate lies in [0, 1]

  // work vectors
  double* a64 = nullptr;   // [npad] converted input (mult) / padded grid vector
  float* a32 = nullptr;    // [npad]
  float* a32lo = nullptr;  // [npad] df64 low part
  double* v64 = nullptr;   // [mpad] data-side vector (mult output / multT input)
  float* v32 = nullptr;    // [mpad]
  float* v32lo = nullptr;  // [mpad] df64 low part
  double* out64 = nullptr; // [max(npad, mpad)]
  void* part = nullptr;
  size_t part_bytes = 0;
  int64_t part_elems = 0;  // capacity of `part` in doubles

  // CG vectors (FP64, npad each)
  double* cg = nullptr;  // kCgSlots vectors: b, x, r, d, q, t, outer residual, dx, z, 1/diag
  bool pc_valid = false;  // 1/diag(B^T B + lm I) in slot 9 is current
  double pc_lm = 0.0;
  double* dot_part = nullptr;
  double* dot_out = nullptr;
  double* scal = nullptr;      // CG scalars on the device (+ the last-block ticket at scal + 8)
  double* host_scalar = nullptr;  // pinned

  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
  cudaEvent_t ev_switch = nullptr;  // orders a new stream after the work of the previous one
  double last_seconds = -1.0;
  int64_t launches = 0;
  bool precond = false;  // Jacobi-preconditioned inner CG in the mixed fits (params "precond")
  double inner_tol = 1e-4;  // relative tolerance of the inner solves of mixed fits ("inner_tol")
  int mat_mode = 1;         // materialised FP32 products: 0 off, 1 auto, 2 on ("materialize")
  bool mat_multt = true;    // multTranspose streams them too ("materialize_multt")
  // FP32 system products B^T (B a) in one fused pass over the materialised products instead of
  // the mult and multTranspose kernels ("system_product": "fused"; the separate kernels, each
  // at the HBM copy bandwidth, are faster: 1.44 against 1.50 ms on the benchmark workload)
  bool fused_system = false;
  bool mat_failed = false;  // a build was refused or failed for the current grid
  // the products were built only to pack the block products (the materialised kernels do not take
  // this grid) and are gone: the other products run on the on-the-fly kernels
  bool mat_block_only = false;
  bool inner_half = true;   // inner solves of mixed fits use the FP16 products ("inner_products")
  bool use_half = false;    // set while such an inner solve runs
  int algo = 2;          // FP32 products: 0 dense, 1 subspace, 2 auto (params "algo")
  SubPlan sub;           // subspace tables of the current grid
  bool sub_ok = false;   // sub is built and chosen for the FP32 products
  // BF16 tensor-core products with 16 right-hand sides (built on the first block call)
  sgmev::BlockPlan blk;
  bool blk_ok = false;
  bool blk_failed = false;
  std::string blk_err;
  sgmev::BlockShape blk_shape;  // launch shape ("block_*" knobs or the autotuner)
  // inner tolerance of block fits ("block_inner_tol"); 0: the operand type's default (1e-4 for
  // FP16 products, 1e-3 for BF16 ones, whose 2^-8 rounding limits what a tighter solve gains)
  double block_inner_tol = 0.0;
  bool block_f16 = true;          // FP16 block products ("block_products": "f16", default) or BF16
  int multt_batch = 1;  // points per read-modify-write round of the FP16 multTranspose ("multt_batch")
  int multt_banks = 1;  // banks of cell sums per owner in the FP16 multTranspose ("multt_banks")
  int multt_ctas = 2;   // CTAs per SM of the FP16 multTranspose ("multt_ctas")

  std::vector<double> bb_left, bb_width;

  // optional per-kernel timing (sgmev_profile): one event pair per tile-kernel launch,
  // resolved when read
  bool profile = false;
  std::vector<cudaEvent_t> prof_events;  // pool, 2 per launch
  std::vector<int> prof_kind;            // kind of launch i
  size_t prof_used = 0;                  // launches recorded since the last reset
  int64_t prof_count[19] = {0};
  double prof_seconds[19] = {0.0};
};

namespace sgmev {

// kinds of timed tile kernels (sgmev_tools.h SGMEV_KERNEL_*)
enum {
  KIND_MULT_FP32 = 0,
  KIND_MULTT_FP32 = 1,
  KIND_MULT_FP64 = 2,
  KIND_MULTT_FP64 = 3,
  KIND_MULT_DF64 = 4,
  KIND_MULTT_DF64 = 5,
  KIND_MULT_SUB32 = 6,
  KIND_MULTT_SUB32 = 7,
  KIND_MULT_SUBDF = 8,
  KIND_MULTT_SUBDF = 9,
  KIND_MULT_MAT32 = 10,
  KIND_MULTT_MAT32 = 11,
  KIND_MULT_MATDF = 12,
  KIND_MULTT_MATDF = 13,
  KIND_SYSTEM_MAT32 = 14,
  KIND_MULT_MAT16 = 15,
  KIND_MULTT_MAT16 = 16,
  KIND_BLOCK_MULT = 17,
  KIND_BLOCK_MULTT = 18
};
constexpr int kKinds = 19;

template <typename T>
static const T* gscale(const sgmev_op* op);
template <>
const float* gscale<float>(const sgmev_op* op) { return op->gs32; }
template <>
const double* gscale<double>(const sgmev_op* op) { return op->gs64; }

template <typename T>
static int kind_mult() { return sizeof(T) == 4 ? KIND_MULT_FP32 : KIND_MULT_FP64; }
template <typename T>
static int kind_multt() { return sizeof(T) == 4 ? KIND_MULTT_FP32 : KIND_MULTT_FP64; }

static long prof_begin(sgmev_op* op, int kind) {
  if (!op->profile) return -1;
  if (op->prof_events.size() < 2 * (op->prof_used + 1)) {
    const size_t grow = std::max<size_t>(64, op->prof_events.size());
    for (size_t k = 0; k < grow; ++k) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return -1;
      op->prof_events.push_back(e);
    }
  }
  if (op->prof_kind.size() < op->prof_used + 1) op->prof_kind.resize(op->prof_used + 1);
  const long i = static_cast<long>(op->prof_used++);
  op->prof_kind[i] = kind;
  cudaEventRecord(op->prof_events[2 * i], op->stream);
  return i;
}

static void prof_end(sgmev_op* op, long i) {
  if (i >= 0) cudaEventRecord(op->prof_events[2 * i + 1], op->stream);
}

// ---------------------------------------------------------------------------------------
// staging kernels
// ---------------------------------------------------------------------------------------
__global__ void stage_data_kernel(const double* __restrict__ rows, int64_t m, int dim,
                                  int64_t mpad, const double* __restrict__ bb_left,
                                  const double* __restrict__ bb_width, double* __restrict__ xt64,
                                  float* __restrict__ xt32, float* __restrict__ xt32lo) {
  const int64_t total = mpad * dim;
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < total;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int t = static_cast<int>(k / mpad);
    const int64_t j = k - static_cast<int64_t>(t) * mpad;
    double x = 0.0;
    if (j < m) {
      x = rows[j * dim + t];
      if (bb_left) x = (x - bb_left[t]) / bb_width[t];
    }
    xt64[k] = x;
    const float h = static_cast<float>(x);
    xt32[k] = h;
    xt32lo[k] = static_cast<float>(x - static_cast<double>(h));
  }
}

__global__ void stage_grid_kernel(const double* __restrict__ level_pow2,
                                  const double* __restrict__ index, int64_t n, int dim,
                                  int64_t npad, double2* __restrict__ li64,
                                  float2* __restrict__ li32, float4* __restrict__ gq) {
  const int64_t total = npad * dim;
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < total;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double L = 0.0, I = 2.0;  // padded row: t = -2, hat = 0
    if (k < n * dim) {
      L = level_pow2[k];
      I = index[k];
    }
    li64[k] = make_double2(L, I);
    li32[k] = make_float2(static_cast<float>(L), static_cast<float>(I));
    // padded rows (L = 0): a = 1 - 2 = -1, b = 1 + 2 = 3, so min(a, b) < 0 and the hat is 0
    gq[k] = make_float4(static_cast<float>(L), static_cast<float>(1.0 - I),
                        static_cast<float>(1.0 + I), 0.0f);
  }
}

// ModLinear: (2^l, i) rows -> the scaled pairs and float-float constants of kernels.cuh and the
// per-grid-point factors 2^b; one thread per grid point (padded rows: hat 0, factor 0)
__global__ void stage_grid_mod_kernel(const double* __restrict__ level_pow2,
                                      const double* __restrict__ index, int64_t n, int dim,
                                      int64_t npad, double2* __restrict__ li64,
                                      float2* __restrict__ li32, float4* __restrict__ gq,
                                      double* __restrict__ gs64, float* __restrict__ gs32) {
  for (int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; g < npad;
       g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double scale = g < n ? 1.0 : 0.0;
    for (int t = 0; t < dim; ++t) {
      const int64_t k = g * dim + t;
      double a = 0.0, c = 2.0;                  // padded row: t = -2, hat 0
      float4 q = make_float4(0.0f, -1.0f, 3.0f, 0.0f);
      if (g < n) {
        const double L = level_pow2[k], I = index[k];
        if (L == 2.0) {                         // level 1: constant 1
          a = 0.0;
          c = 0.0;
          q = make_float4(0.0f, 1.0f, 1.0f, 0.0f);
        } else if (I == 1.0) {                  // 2 (1 - (L / 2) x)
          a = 0.5 * L;
          c = -0.0;
          q = make_float4(static_cast<float>(0.5 * L), kModOpen, 1.0f, 0.0f);
          scale *= 2.0;
        } else if (I == L - 1.0) {              // 2 (1 - (L / 2) (1 - x))
          a = -0.5 * L;
          c = -0.5 * L;
          q = make_float4(static_cast<float>(0.5 * L), static_cast<float>(1.0 - 0.5 * L),
                          kModOpen, 0.0f);
          scale *= 2.0;
        } else {
          a = L;
          c = I;
          q = make_float4(static_cast<float>(L), static_cast<float>(1.0 - I),
                          static_cast<float>(1.0 + I), 0.0f);
        }
      }
      li64[k] = make_double2(a, c);
      li32[k] = make_float2(static_cast<float>(a), static_cast<float>(c));
      gq[k] = q;
    }
    gs64[g] = scale;
    gs32[g] = static_cast<float>(scale);
  }
}

// flag |= 1 when a staged coordinate lies outside [0, 1] (or is NaN)
__global__ void cube_check_kernel(const double* __restrict__ xt, int64_t total,
                                  unsigned int* __restrict__ flag) {
  bool out = false;
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < total;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const double x = xt[k];
    out = out || !(x >= 0.0 && x <= 1.0);
  }
  if (__syncthreads_or(out) && threadIdx.x == 0) atomicOr(flag, 1u);
}

__global__ void convert_pad_kernel(const double* __restrict__ in, int64_t n, int64_t npad,
                                   double* __restrict__ out64, float* __restrict__ out32,
                                   float* __restrict__ out32lo) {
  for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < npad;
       k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const double v = k < n ? in[k] : 0.0;
    if (out64) out64[k] = v;
    const float h = static_cast<float>(v);
    if (out32) out32[k] = h;
    if (out32lo) out32lo[k] = static_cast<float>(v - static_cast<double>(h));
  }
}

// deterministic dot product: fixed grid, fixed tree
__global__ void dot_partial_kernel(const double* __restrict__ a, const double* __restrict__ b,
                                   int64_t n, double* __restrict__ part) {
  __shared__ double s[kDotThreads];
  double acc = 0.0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    acc = fma(a[i], b[i], acc);
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kDotThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

__global__ void dot_final_kernel(const double* __restrict__ part, int np, double* __restrict__ out) {
  __shared__ double s[kDotThreads];
  double acc = 0.0;
  for (int i = threadIdx.x; i < np; i += kDotThreads) acc += part[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kDotThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}

// y = a*x + y
__global__ void axpy_kernel(int64_t n, double a, const double* __restrict__ x,
                            double* __restrict__ y) {
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    y[i] = fma(a, x[i], y[i]);
}

// d = beta*d + r
__global__ void xpby_kernel(int64_t n, const double* __restrict__ r, double beta,
                            double* __restrict__ d) {
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    d[i] = fma(beta, d[i], r[i]);
}

// ---- CG with its scalars on the device ---------------------------------------------------
// scal[0] delta_new, [1] delta_old, [2] d.q, [3] alpha, [4] beta; a ticket counter (scal + 8)
// lets the last block of a launch add the partials. Every sum has the thread mapping and the
// tree of dot_partial_kernel + dot_final_kernel, so the scalars are bit-identical to the
// host-driven loop's.
__device__ __forceinline__ double block_tree_sum(double acc, double* s) {
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kDotThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  return s[0];
}

// the last block to finish sums part[0..gridDim.x) as dot_final_kernel does; true in its threads
__device__ __forceinline__ bool last_block_total(double block_sum, double* part,
                                                 unsigned int* ticket, double* s,
                                                 double* total) {
  __shared__ bool is_last;
  if (threadIdx.x == 0) {
    part[blockIdx.x] = block_sum;
    __threadfence();
    is_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!is_last) return false;
  __threadfence();
  double acc = 0.0;
  for (int i = threadIdx.x; i < static_cast<int>(gridDim.x); i += kDotThreads)
    acc += reinterpret_cast<volatile double*>(part)[i];
  *total = block_tree_sum(acc, s);
  if (threadIdx.x == 0) *ticket = 0u;
  return true;
}

// dq = d.q, alpha = delta_new / dq (0 when dq is 0: the loop then stops without a step)
__global__ void __launch_bounds__(kDotThreads) cg_alpha_kernel(const double* __restrict__ d,
                                                              const double* __restrict__ q,
                                                              int64_t n, double* __restrict__ part,
                                                              double* __restrict__ scal) {
  __shared__ double s[kDotThreads];
  double acc = 0.0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    acc = fma(d[i], q[i], acc);
  const double b = block_tree_sum(acc, s);
  double dq = 0.0;
  if (last_block_total(b, part, reinterpret_cast<unsigned int*>(scal + 8), s, &dq) &&
      threadIdx.x == 0) {
    scal[2] = dq;
    scal[3] = dq != 0.0 ? scal[0] / dq : 0.0;
  }
}

// x += alpha d; r -= alpha q (unless r_fixed: r was recomputed); then delta_old = delta_new,
// delta_new = r.r, beta = delta_new / delta_old. with_x = false skips the x update.
__global__ void __launch_bounds__(kDotThreads) cg_update_kernel(int64_t n, const double* __restrict__ d,
                                                               const double* __restrict__ q,
                                                               double* __restrict__ x,
                                                               double* __restrict__ r, int with_x,
                                                               int r_fixed,
                                                               double* __restrict__ part,
                                                               double* __restrict__ scal) {
  __shared__ double s[kDotThreads];
  const double a = scal[3];
  double acc = 0.0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (with_x) x[i] = fma(a, d[i], x[i]);
    double ri = r[i];
    if (!r_fixed) {
      ri = fma(-a, q[i], ri);
      r[i] = ri;
    }
    acc = fma(ri, ri, acc);
  }
  const double b = block_tree_sum(acc, s);
  double rr = 0.0;
  if (last_block_total(b, part, reinterpret_cast<unsigned int*>(scal + 8), s, &rr) &&
      threadIdx.x == 0) {
    scal[1] = scal[0];
    scal[0] = rr;
    scal[4] = rr / scal[1];
  }
}

// x += alpha d (alpha on the device)
__global__ void axpy_dev_kernel(int64_t n, const double* __restrict__ scal,
                                const double* __restrict__ d, double* __restrict__ x) {
  const double a = scal[3];
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    x[i] = fma(a, d[i], x[i]);
}

// d = beta d + r (beta on the device)
__global__ void xpby_dev_kernel(int64_t n, const double* __restrict__ r,
                                const double* __restrict__ scal, double* __restrict__ d) {
  const double beta = scal[4];
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    d[i] = fma(beta, d[i], r[i]);
}

// z = a * b (elementwise)
__global__ void mul_kernel(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                           double* __restrict__ z) {
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    z[i] = a[i] * b[i];
}

// inv[i] = 1 / (diag[i] + lm) for i < n, 0 in the padding
__global__ void inv_diag_kernel(int64_t n, int64_t npad, const double* __restrict__ diag,
                                double lm, double* __restrict__ inv) {
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < npad;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const double dv = diag[i] + lm;
    inv[i] = (i < n && dv > 0.0) ? 1.0 / dv : 0.0;
  }
}

// v[j] = 1 for j < m, 0 in the padding (FP32)
__global__ void ones_kernel(int64_t m, int64_t mpad, float* __restrict__ v) {
  for (int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; j < mpad;
       j += static_cast<int64_t>(gridDim.x) * blockDim.x)
    v[j] = j < m ? 1.0f : 0.0f;
}

// z = x - y
__global__ void sub_kernel(int64_t n, const double* __restrict__ x, const double* __restrict__ y,
                           double* __restrict__ z) {
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    z[i] = x[i] - y[i];
}

// ---------------------------------------------------------------------------------------
// launch planning and dispatch
// ---------------------------------------------------------------------------------------
template <typename T>
static Plan plan_mult(const sgmev_op* op, int64_t tiles_total) {
  Plan p;
  p.generic = op->dim > kMaxTemplDim;
  p.tiles = tiles_total;
  // splits along the grid axis: at most one per grid tile and at most what the partial buffer
  // holds at a stride of mpad
  const int64_t max_split = std::max<int64_t>(
      1, std::min<int64_t>(op->npad / kGT, op->part_elems / op->mpad));
  int64_t want = ceil_div(op->target_ctas, std::max<int64_t>(p.tiles, 1));
  want = std::max<int64_t>(1, std::min(want, max_split));
  p.chunk = round_up(ceil_div(op->npad, want), kGT);
  p.nsplit = ceil_div(op->npad, p.chunk);
  return p;
}

template <typename T>
static Plan plan_multt(const sgmev_op* op, int64_t tiles_total) {
  Plan p;
  p.generic = op->dim > kMaxTemplDim;
  p.tiles = tiles_total;
  const int64_t max_split = std::max<int64_t>(
      1, std::min<int64_t>(op->mpad / kDT, op->part_elems / op->npad));
  int64_t want = ceil_div(op->target_ctas, std::max<int64_t>(p.tiles, 1));
  want = std::max<int64_t>(1, std::min(want, max_split));
  p.chunk = round_up(ceil_div(op->mpad, want), kDT);
  p.nsplit = ceil_div(op->mpad, p.chunk);
  return p;
}

template <typename T, int DIM>
static void launch_mult_dim(sgmev_op* op, const T* xt, const typename Pair<T>::type* li,
                            const T* alpha, const Plan& p, int64_t tile_offset, T* part) {
  constexpr int R = Blocking<T>::mult_r(DIM);
  dim3 grid(static_cast<unsigned>(p.tiles), static_cast<unsigned>(p.nsplit));
  mult_kernel<T, DIM, R, kBlock, kGT><<<grid, kBlock, 0, op->stream>>>(
      xt, op->mpad, li, alpha, op->npad, p.chunk, tile_offset, part);
}

template <typename T, int DIM>
static void launch_multt_dim(sgmev_op* op, const T* xt, const T* v,
                             const typename Pair<T>::type* li, const Plan& p, int64_t tile_offset,
                             T* part) {
  constexpr int RG = Blocking<T>::multt_r(DIM);
  dim3 grid(static_cast<unsigned>(p.tiles), static_cast<unsigned>(p.nsplit));
  mult_transpose_kernel<T, DIM, RG, kBlock, kDT><<<grid, kBlock, 0, op->stream>>>(
      xt, v, op->mpad, li, op->npad, p.chunk, tile_offset, part);
}

// mult over data range [j_begin, j_end): partial sums into op->part, returns the plan used.
template <typename T>
static int run_mult(sgmev_op* op, const T* xt, const typename Pair<T>::type* li, const T* alpha,
                    int64_t j_begin, int64_t j_end, Plan* used) {
  T* part = static_cast<T*>(op->part);
  if (op->dim <= kMaxTemplDim) {
    const int64_t tile_pts = kBlock * Blocking<T>::mult_r(op->dim);
    const int64_t t0 = j_begin / tile_pts;
    const int64_t t1 = ceil_div(j_end, tile_pts);
    Plan p = plan_mult<T>(op, t1 - t0);
    const long ev = prof_begin(op, kind_mult<T>());
    if (op->mod) {
      mod_mult_launch<T>(op->dim, dim3(static_cast<unsigned>(p.tiles), static_cast<unsigned>(p.nsplit)),
                         op->stream, xt, op->mpad, li, alpha, gscale<T>(op), op->npad, p.chunk,
                         t0, 0, part);
    } else {
      switch (op->dim) {
#define F(D)                                                         \
  case D:                                                            \
    launch_mult_dim<T, D>(op, xt, li, alpha, p, t0, part);           \
    break;
        SGMEV_DIM_CASES(F)
#undef F
        default:
          break;
      }
    }
    prof_end(op, ev);
    *used = p;
  } else {
    const int64_t count = j_end - j_begin;
    Plan p = plan_mult<T>(op, ceil_div(count, kBlock));
    dim3 grid(static_cast<unsigned>(p.tiles), static_cast<unsigned>(p.nsplit));
    const long ev = prof_begin(op, kind_mult<T>());
    if (op->mod) {
      mod_mult_launch<T>(op->dim, grid, op->stream, xt, op->mpad, li, alpha, gscale<T>(op),
                         op->npad, p.chunk, j_begin, count, part);
    } else {
      mult_generic_kernel<T><<<grid, kBlock, 0, op->stream>>>(xt, op->mpad, op->dim, li, alpha,
                                                              op->npad, p.chunk, j_begin, count,
                                                              part);
    }
    prof_end(op, ev);
    *used = p;
  }
  op->launches += 1;
  SGMEV_CUDA(cudaGetLastError());
  return SGMEV_OK;
}

template <typename T>
static int run_multt(sgmev_op* op, const T* xt, const T* v, const typename Pair<T>::type* li,
                     int64_t g_begin, int64_t g_end, Plan* used) {
  T* part = static_cast<T*>(op->part);
  if (op->dim <= kMaxTemplDim) {
    const int64_t tile_pts = kBlock * Blocking<T>::multt_r(op->dim);
    const int64_t t0 = g_begin / tile_pts;
    const int64_t t1 = ceil_div(g_end, tile_pts);
    Plan p = plan_multt<T>(op, t1 - t0);
    const long ev = prof_begin(op, kind_multt<T>());
    if (op->mod) {
      mod_multt_launch<T, false>(op->dim, dim3(static_cast<unsigned>(p.tiles), static_cast<unsigned>(p.nsplit)),
                                 op->stream, xt, v, op->mpad, li, gscale<T>(op), op->npad, p.chunk,
                                 t0, 0, part);
    } else {
      switch (op->dim) {
#define F(D)                                                      \
  case D:                                                         \
    launch_multt_dim<T, D>(op, xt, v, li, p, t0, part);           \
    break;
        SGMEV_DIM_CASES(F)
#undef F
        default:
          break;
      }
    }
    prof_end(op, ev);
    *used = p;
  } else {
    const int64_t count = g_end - g_begin;
    Plan p = plan_multt<T>(op, ceil_div(count, kBlock));
    dim3 grid(static_cast<unsigned>(p.tiles), static_cast<unsigned>(p.nsplit));
    const long ev = prof_begin(op, kind_multt<T>());
    if (op->mod) {
      mod_multt_launch<T, false>(op->dim, grid, op->stream, xt, v, op->mpad, li, gscale<T>(op),
                                 op->npad, p.chunk, g_begin, count, part);
    } else {
      mult_transpose_generic_kernel<T><<<grid, kBlock, 0, op->stream>>>(
          xt, v, op->mpad, op->dim, li, op->npad, p.chunk, g_begin, count, part);
    }
    prof_end(op, ev);
    *used = p;
  }
  op->launches += 1;
  SGMEV_CUDA(cudaGetLastError());
  return SGMEV_OK;
}

template <typename TP, typename TO>
static int run_reduce(sgmev_op* op, int nsplit, int64_t stride, int64_t begin, int64_t n_valid,
                      int64_t n_total, TO* out, const double* add, double scale) {
  const int64_t work = std::max<int64_t>(n_total - begin, 1);
  const unsigned blocks =
      static_cast<unsigned>(std::min<int64_t>(kReduceBlocks, ceil_div(work, 256)));
  reduce_splits_kernel<TP, TO><<<blocks, 256, 0, op->stream>>>(
      static_cast<const TP*>(op->part), nsplit, stride, begin, n_valid, n_total, out, add, scale);
  op->launches += 1;
  SGMEV_CUDA(cudaGetLastError());
  return SGMEV_OK;
}

static unsigned vec_blocks(int64_t n) {
  return static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>(kReduceBlocks, ceil_div(n, 256))));
}

template <int DIM>
static void launch_mult_df_dim(sgmev_op* op, const float* ah, const float* al, const Plan& p,
                               int64_t tile_offset, float2* part) {
  dim3 grid(static_cast<unsigned>(p.tiles), static_cast<unsigned>(p.nsplit));
  mult_df_kernel<DIM, kDfMultR, kBlock, kGT><<<grid, kBlock, 0, op->stream>>>(
      op->xt32, op->xt32lo, op->mpad, op->gq, ah, al, op->npad, p.chunk, tile_offset, part);
}

template <int DIM>
static void launch_multt_df_dim(sgmev_op* op, const float* vh, const float* vl, const Plan& p,
                                int64_t tile_offset, float2* part) {
  dim3 grid(static_cast<unsigned>(p.tiles), static_cast<unsigned>(p.nsplit));
  mult_transpose_df_kernel<DIM, kDfMulttRG, kBlock, kDT><<<grid, kBlock, 0, op->stream>>>(
      op->xt32, op->xt32lo, vh, vl, op->mpad, op->gq, op->npad, p.chunk, tile_offset, part);
}

static int run_mult_df(sgmev_op* op, const float* ah, const float* al, int64_t j_begin,
                       int64_t j_end, Plan* used) {
  float2* part = static_cast<float2*>(op->part);
  if (op->dim <= kMaxTemplDim) {
    const int64_t tile_pts = kBlock * kDfMultR;
    const int64_t t0 = j_begin / tile_pts;
    const int64_t t1 = ceil_div(j_end, tile_pts);
    Plan p = plan_mult<float>(op, t1 - t0);
    const long ev = prof_begin(op, KIND_MULT_DF64);
    if (op->mod) {
      mod_mult_df_launch(op->dim, dim3(static_cast<unsigned>(p.tiles), static_cast<unsigned>(p.nsplit)),
                         op->stream, op->xt32, op->xt32lo, op->mpad, op->gq, ah, al, op->gs32,
                         op->npad, p.chunk, t0, 0, part);
    } else {
      switch (op->dim) {
#define F(D)                                               \
  case D:                                                  \
    launch_mult_df_dim<D>(op, ah, al, p, t0, part);        \
    break;
        SGMEV_DIM_CASES(F)
#undef F
        default:
          break;
      }
    }
    prof_end(op, ev);
    *used = p;
  } else {
    const int64_t count = j_end - j_begin;
    Plan p = plan_mult<float>(op, ceil_div(count, kBlock));
    dim3 grid(static_cast<unsigned>(p.tiles), static_cast<unsigned>(p.nsplit));
    const long ev = prof_begin(op, KIND_MULT_DF64);
    if (op->mod) {
      mod_mult_df_launch(op->dim, grid, op->stream, op->xt32, op->xt32lo, op->mpad, op->gq, ah,
                         al, op->gs32, op->npad, p.chunk, j_begin, count, part);
    } else {
      mult_df_generic_kernel<false><<<grid, kBlock, 0, op->stream>>>(
          op->xt32, op->xt32lo, op->mpad, op->dim, op->gq, ah, al, op->npad, p.chunk, j_begin,
          count, part);
    }
    prof_end(op, ev);
    *used = p;
  }
  op->launches += 1;
  SGMEV_CUDA(cudaGetLastError());
  return SGMEV_OK;
}

static int run_multt_df(sgmev_op* op, const float* vh, const float* vl, int64_t g_begin,
                        int64_t g_end, Plan* used) {
  float2* part = static_cast<float2*>(op->part);
  if (op->dim <= kMaxTemplDim) {
    const int64_t tile_pts = kBlock * kDfMulttRG;
    const int64_t t0 = g_begin / tile_pts;
    const int64_t t1 = ceil_div(g_end, tile_pts);
    Plan p = plan_multt<float>(op, t1 - t0);
    const long ev = prof_begin(op, KIND_MULTT_DF64);
    if (op->mod) {
      mod_multt_df_launch(op->dim, dim3(static_cast<unsigned>(p.tiles), static_cast<unsigned>(p.nsplit)),
                          op->stream, op->xt32, op->xt32lo, vh, vl, op->mpad, op->gq, op->gs32,
                          op->npad, p.chunk, t0, 0, part);
    } else {
      switch (op->dim) {
#define F(D)                                                \
  case D:                                                   \
    launch_multt_df_dim<D>(op, vh, vl, p, t0, part);        \
    break;
        SGMEV_DIM_CASES(F)
#undef F
        default:
          break;
      }
    }
    prof_end(op, ev);
    *used = p;
  } else {
    const int64_t count = g_end - g_begin;
    Plan p = plan_multt<float>(op, ceil_div(count, kBlock));
    dim3 grid(static_cast<unsigned>(p.tiles), static_cast<unsigned>(p.nsplit));
    const long ev = prof_begin(op, KIND_MULTT_DF64);
    if (op->mod) {
      mod_multt_df_launch(op->dim, grid, op->stream, op->xt32, op->xt32lo, vh, vl, op->mpad,
                          op->gq, op->gs32, op->npad, p.chunk, g_begin, count, part);
    } else {
      mult_transpose_df_generic_kernel<false><<<grid, kBlock, 0, op->stream>>>(
          op->xt32, op->xt32lo, vh, vl, op->mpad, op->dim, op->gq, op->npad, p.chunk, g_begin,
          count, part);
    }
    prof_end(op, ev);
    *used = p;
  }
  op->launches += 1;
  SGMEV_CUDA(cudaGetLastError());
  return SGMEV_OK;
}

// data points per mult tile / grid points per multT tile for a precision (tile-aligned ranges)
static int64_t mult_tile_pts(const sgmev_op* op, int prec) {
  if (op->dim > kMaxTemplDim) return 1;
  if (prec == SGMEV_FP64) return kBlock * Blocking<double>::mult_r(op->dim);
  if (prec == SGMEV_DF64) return kBlock * kDfMultR;
  return kBlock * Blocking<float>::mult_r(op->dim);
}

static int64_t multt_tile_pts(const sgmev_op* op, int prec) {
  if (op->dim > kMaxTemplDim) return 1;
  if (prec == SGMEV_FP64) return kBlock * Blocking<double>::multt_r(op->dim);
  if (prec == SGMEV_DF64) return kBlock * kDfMulttRG;
  return kBlock * Blocking<float>::multt_r(op->dim);
}

// ---------------------------------------------------------------------------------------
// device-side products on padded device vectors
// ---------------------------------------------------------------------------------------
// Materialised FP32 subspace products: built on the first FP32 product after the grid was
// staged, when the "materialize" knob allows it and they fit (auto: at most half of the free
// device memory and 64 GiB); a failed build falls back to the on-the-fly kernels for this grid.
static bool mat_ready(sgmev_op* op) {
  using namespace sgmev;
  if (op->mat_block_only) return false;
  if (op->sub.pmat) return true;
  if (op->mat_mode == 0 || op->mat_failed || !subspace_mat_fits(op->sub, false)) return false;
  // ModLinear products are built for data in the cube (the cell of a boundary-adjacent function
  // is clamped there); data outside it stays on the dense kernels, which extrapolate
  if (op->mod && !op->in_cube) return false;
  const int64_t bytes = subspace_mat_bytes(op->sub, op->mpad);
  if (op->mat_mode == 1) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      (void)cudaGetLastError();
      op->mat_failed = true;
      return false;
    }
    if (static_cast<double>(bytes) > std::min(0.5 * static_cast<double>(free_b), 64.0 * (1ull << 30))) {
      op->mat_failed = true;
      return false;
    }
  }
  if (subspace_materialize(&op->sub, op->stream, op->xt32, op->xt32lo, op->mpad, op->m,
                           op->num_sms) != cudaSuccess) {
    (void)cudaGetLastError();
    subspace_mat_release(&op->sub, op->stream);
    op->mat_failed = true;
    return false;
  }
  op->launches += 1;
  return true;
}

// Inputs per precision: FP64 a64; FP32 a32; DF64 (a32, a32lo) — all padded to npad.
// out64 / out32 [mpad] (zero beyond m) = B a over data range [j_begin, j_end).
static int dev_mult(sgmev_op* op, int prec, const double* a64, const float* a32,
                    const float* a32lo, double* out64, float* out32, int64_t j_begin,
                    int64_t j_end) {
  if (j_end <= j_begin) return SGMEV_OK;
  Plan p;
  const int64_t total = j_end;
  const int64_t valid = std::min(op->m, total);
  if (prec == SGMEV_FP64) {
    SGMEV_TRY(run_mult<double>(op, op->xt64, op->li64, a64, j_begin, j_end, &p));
    if (out64) SGMEV_TRY((run_reduce<double, double>(op, (int)p.nsplit, op->mpad, j_begin, valid, total, out64, nullptr, 0.0)));
    if (out32) SGMEV_TRY((run_reduce<double, float>(op, (int)p.nsplit, op->mpad, j_begin, valid, total, out32, nullptr, 0.0)));
  } else if (prec == SGMEV_DF64 && op->sub_ok && out64 && !out32 && mat_ready(op) &&
             subspace_mat_fits(op->sub, true)) {
    const long ev = prof_begin(op, KIND_MULT_MATDF);
    SGMEV_CUDA(subspace_mult_mat_df(op->sub, op->stream, op->mpad, op->m, a32, a32lo, out64,
                                    j_begin, j_end, op->num_sms));
    prof_end(op, ev);
    op->launches += 2;
  } else if (prec == SGMEV_DF64 && op->sub_ok && !op->mod && out64 && !out32) {
    const long ev = prof_begin(op, KIND_MULT_SUBDF);
    SGMEV_CUDA(subspace_mult_df(op->sub, op->stream, op->xt32, op->xt32lo, op->mpad, op->m, a32,
                                a32lo, out64, j_begin, j_end, op->num_sms));
    prof_end(op, ev);
    op->launches += 2;
  } else if (prec == SGMEV_DF64) {
    SGMEV_TRY(run_mult_df(op, a32, a32lo, j_begin, j_end, &p));
    if (out64) SGMEV_TRY((run_reduce<float2, double>(op, (int)p.nsplit, op->mpad, j_begin, valid, total, out64, nullptr, 0.0)));
    if (out32) SGMEV_TRY((run_reduce<float2, float>(op, (int)p.nsplit, op->mpad, j_begin, valid, total, out32, nullptr, 0.0)));
  } else if (op->sub_ok && mat_ready(op)) {
    const long ev = prof_begin(op, op->use_half ? KIND_MULT_MAT16 : KIND_MULT_MAT32);
    SGMEV_CUDA(subspace_mult_mat(op->sub, op->stream, op->xt32, op->mpad, op->m, a32, out32, out64,
                                 j_begin, j_end, op->num_sms, op->use_half));
    prof_end(op, ev);
    op->launches += 2;
  } else if (op->sub_ok && !op->mod) {
    const long ev = prof_begin(op, KIND_MULT_SUB32);
    SGMEV_CUDA(subspace_mult(op->sub, op->stream, op->xt32, op->mpad, op->m, a32, out32, out64,
                             j_begin, j_end, op->num_sms));
    prof_end(op, ev);
    op->launches += 2;
  } else {
    SGMEV_TRY(run_mult<float>(op, op->xt32, op->li32, a32, j_begin, j_end, &p));
    if (out64) SGMEV_TRY((run_reduce<float, double>(op, (int)p.nsplit, op->mpad, j_begin, valid, total, out64, nullptr, 0.0)));
    if (out32) SGMEV_TRY((run_reduce<float, float>(op, (int)p.nsplit, op->mpad, j_begin, valid, total, out32, nullptr, 0.0)));
  }
  return SGMEV_OK;
}

// out64[g_begin..g_end) = B^T v (+ scale * add); inputs FP64 v64, FP32 v32, DF64 (v32, v32lo)
static int dev_multt(sgmev_op* op, int prec, const double* v64, const float* v32,
                     const float* v32lo, double* out64, int64_t g_begin, int64_t g_end,
                     const double* add, double scale) {
  if (g_end <= g_begin) return SGMEV_OK;
  Plan p;
  const int64_t valid = std::min(op->n, g_end);
  if (prec == SGMEV_FP64) {
    SGMEV_TRY(run_multt<double>(op, op->xt64, v64, op->li64, g_begin, g_end, &p));
    SGMEV_TRY((run_reduce<double, double>(op, (int)p.nsplit, op->npad, g_begin, valid, g_end, out64, add, scale)));
  } else if (prec == SGMEV_DF64 && op->sub_ok && op->mat_multt && mat_ready(op) &&
             subspace_mat_fits(op->sub, true)) {
    // the subspace sums produce every grid entry at once (the range is a subset of them)
    const long ev = prof_begin(op, KIND_MULTT_MATDF);
    SGMEV_CUDA(subspace_multt_mat_df(op->sub, op->stream, op->mpad, v32, v32lo, op->npad, out64,
                                     add, scale, op->num_sms));
    prof_end(op, ev);
    op->launches += 3;
  } else if (prec == SGMEV_DF64 && op->sub_ok && !op->mod && subspace_owner_fits(op->sub, true)) {
    // the subspace sums produce every grid entry at once (the range is a subset of them)
    const long ev = prof_begin(op, KIND_MULTT_SUBDF);
    SGMEV_CUDA(subspace_multt_df(op->sub, op->stream, op->xt32, op->xt32lo, op->mpad, op->m, v32,
                                 v32lo, op->npad, out64, add, scale, op->num_sms));
    prof_end(op, ev);
    op->launches += 3;
  } else if (prec == SGMEV_DF64) {
    SGMEV_TRY(run_multt_df(op, v32, v32lo, g_begin, g_end, &p));
    SGMEV_TRY((run_reduce<float2, double>(op, (int)p.nsplit, op->npad, g_begin, valid, g_end, out64, add, scale)));
  } else if (op->sub_ok && op->mat_multt && mat_ready(op)) {
    // the subspace sums produce every grid entry at once (the range is a subset of them)
    const long ev = prof_begin(op, op->use_half ? KIND_MULTT_MAT16 : KIND_MULTT_MAT32);
    SGMEV_CUDA(subspace_multt_mat(op->sub, op->stream, op->xt32, op->mpad, op->m, v32, op->npad,
                                  out64, add, scale, op->num_sms, op->use_half));
    prof_end(op, ev);
    op->launches += 3;
  } else if (op->sub_ok && !op->mod) {
    // the subspace scatter produces every grid entry at once (the range is a subset of it)
    const long ev = prof_begin(op, KIND_MULTT_SUB32);
    SGMEV_CUDA(subspace_multt(op->sub, op->stream, op->xt32, op->mpad, op->m, v32, op->npad,
                              out64, add, scale, op->num_sms));
    prof_end(op, ev);
    op->launches += 3;
  } else {
    SGMEV_TRY(run_multt<float>(op, op->xt32, v32, op->li32, g_begin, g_end, &p));
    SGMEV_TRY((run_reduce<float, double>(op, (int)p.nsplit, op->npad, g_begin, valid, g_end, out64, add, scale)));
  }
  return SGMEV_OK;
}

static int dev_convert(sgmev_op* op, const double* in, int64_t n, int64_t npad, double* o64,
                       float* o32, float* o32lo) {
  convert_pad_kernel<<<vec_blocks(npad), 256, 0, op->stream>>>(in, n, npad, o64, o32, o32lo);
  op->launches += 1;
  SGMEV_CUDA(cudaGetLastError());
  return SGMEV_OK;
}

// out64[npad] = B^T (B a) + lm * a, a given as padded FP64 device vector [npad]
static int dev_system(sgmev_op* op, int prec, const double* a64, double* out64, double lm) {
  if (prec == SGMEV_FP32) {
    SGMEV_TRY(dev_convert(op, a64, op->npad, op->npad, nullptr, op->a32, nullptr));
    if (op->fused_system && !op->use_half && op->sub_ok && op->mat_multt && mat_ready(op) &&
        subspace_system_mat_fits(op->sub)) {
      // one pass over the materialised products for B^T (B a)
      const long ev = prof_begin(op, KIND_SYSTEM_MAT32);
      SGMEV_CUDA(subspace_system_mat(op->sub, op->stream, op->mpad, op->a32, op->npad, out64, a64,
                                     lm, op->num_sms));
      prof_end(op, ev);
      op->launches += 4;
      return SGMEV_OK;
    }
    SGMEV_TRY(dev_mult(op, prec, nullptr, op->a32, nullptr, nullptr, op->v32, 0, op->mpad));
    SGMEV_TRY(dev_multt(op, prec, nullptr, op->v32, nullptr, out64, 0, op->npad, a64, lm));
  } else if (prec == SGMEV_DF64) {
    SGMEV_TRY(dev_convert(op, a64, op->npad, op->npad, nullptr, op->a32, op->a32lo));
    SGMEV_TRY(dev_mult(op, prec, nullptr, op->a32, op->a32lo, op->v64, nullptr, 0, op->mpad));
    SGMEV_TRY(dev_convert(op, op->v64, op->mpad, op->mpad, nullptr, op->v32, op->v32lo));
    SGMEV_TRY(dev_multt(op, prec, nullptr, op->v32, op->v32lo, out64, 0, op->npad, a64, lm));
  } else {
    SGMEV_TRY(dev_mult(op, prec, a64, nullptr, nullptr, op->v64, nullptr, 0, op->mpad));
    SGMEV_TRY(dev_multt(op, prec, op->v64, nullptr, nullptr, out64, 0, op->npad, a64, lm));
  }
  return SGMEV_OK;
}

static int dev_dot(sgmev_op* op, const double* a, const double* b, int64_t n, double* host_out) {
  dot_partial_kernel<<<kDotBlocks, kDotThreads, 0, op->stream>>>(a, b, n, op->dot_part);
  dot_final_kernel<<<1, kDotThreads, 0, op->stream>>>(op->dot_part, kDotBlocks, op->dot_out);
  op->launches += 2;
  SGMEV_CUDA(cudaGetLastError());
  SGMEV_CUDA(cudaMemcpyAsync(op->host_scalar, op->dot_out, sizeof(double),
                             cudaMemcpyDeviceToHost, op->stream));
  SGMEV_CUDA(cudaStreamSynchronize(op->stream));
  *host_out = *op->host_scalar;
  return SGMEV_OK;
}

static int dev_axpy(sgmev_op* op, int64_t n, double a, const double* x, double* y) {
  axpy_kernel<<<vec_blocks(n), 256, 0, op->stream>>>(n, a, x, y);
  op->launches += 1;
  SGMEV_CUDA(cudaGetLastError());
  return SGMEV_OK;
}

// ---------------------------------------------------------------------------------------
// allocation helpers
// ---------------------------------------------------------------------------------------
template <typename T>
static int dalloc(cudaStream_t s, T** p, size_t count) {
  if (*p) {
    dev_free(*p, s);
    *p = nullptr;
  }
  if (count == 0) count = 1;
  SGMEV_CUDA(dev_malloc(p, count * sizeof(T), s));
  return SGMEV_OK;
}

// Partial-sum capacity: enough for the full-range plans of both products (the split count
// a full-range launch wants is ceil(target_ctas / tiles)), and at least 8 strides of each axis.
// Ranged launches clamp their split count to this capacity.
static int64_t part_need_elems(const sgmev_op* op) {
  int64_t need = 8 * std::max(op->mpad, op->npad);
  const int rm[2] = {Blocking<float>::mult_r(op->dim), Blocking<double>::mult_r(op->dim)};
  const int rt[2] = {Blocking<float>::multt_r(op->dim), Blocking<double>::multt_r(op->dim)};
  for (int k = 0; k < 2; ++k) {
    const int64_t mt = op->dim > kMaxTemplDim ? ceil_div(op->mpad, kBlock) : op->mpad / (kBlock * rm[k]);
    const int64_t nt = op->dim > kMaxTemplDim ? ceil_div(op->npad, kBlock) : op->npad / (kBlock * rt[k]);
    const int64_t sm = std::min<int64_t>(op->npad / kGT, ceil_div(op->target_ctas, std::max<int64_t>(mt, 1)));
    const int64_t st = std::min<int64_t>(op->mpad / kDT, ceil_div(op->target_ctas, std::max<int64_t>(nt, 1)));
    need = std::max(need, std::max(sm * op->mpad, st * op->npad));
  }
  return need;
}

static int check_grid(int dim, int64_t n, const double* level_pow2, const double* index) {
  for (int64_t k = 0; k < n * dim; ++k) {
    const double L = level_pow2[k], I = index[k];
    if (!(L >= 2.0) || L > 1099511627776.0 || std::floor(L) != L) {
      return fail(SGMEV_ERR_UNSUPPORTED,
                  "level entry " + std::to_string(k) + " is not 2^l with l >= 1 (hat basis "
                  "without boundary only)");
    }
    const double lg = std::log2(L);
    if (std::floor(lg) != lg) {
      return fail(SGMEV_ERR_UNSUPPORTED, "level entry " + std::to_string(k) + " is not a power of two");
    }
    if (!(I >= 1.0) || !(I < L) || std::floor(I) != I || std::fmod(I, 2.0) != 1.0) {
      return fail(SGMEV_ERR_UNSUPPORTED,
                  "index entry " + std::to_string(k) + " is not an odd integer in (0, 2^l)");
    }
  }
  return SGMEV_OK;
}

static int stage_grid(sgmev_op* op, int64_t n, const double* level_pow2, const double* index) {
  const int64_t npad = std::max<int64_t>(round_up(std::max<int64_t>(n, 1), kNPadTo), kNPadTo);
  if (npad > op->npad_cap) {
    SGMEV_TRY(dalloc(op->stream, &op->li64, static_cast<size_t>(npad * op->dim)));
    SGMEV_TRY(dalloc(op->stream, &op->li32, static_cast<size_t>(npad * op->dim)));
    SGMEV_TRY(dalloc(op->stream, &op->gq, static_cast<size_t>(npad * op->dim)));
    if (op->mod) {
      SGMEV_TRY(dalloc(op->stream, &op->gs64, static_cast<size_t>(npad)));
      SGMEV_TRY(dalloc(op->stream, &op->gs32, static_cast<size_t>(npad)));
    }
    SGMEV_TRY(dalloc(op->stream, &op->a64, static_cast<size_t>(npad)));
    SGMEV_TRY(dalloc(op->stream, &op->a32, static_cast<size_t>(npad)));
    SGMEV_TRY(dalloc(op->stream, &op->a32lo, static_cast<size_t>(npad)));
    SGMEV_TRY(dalloc(op->stream, &op->cg, static_cast<size_t>(npad) * kCgSlots));
    op->npad_cap = npad;
  }
  op->n = n;
  op->npad = npad;
  op->pc_valid = false;
  double* d_l = nullptr;
  double* d_i = nullptr;
  const size_t bytes = sizeof(double) * static_cast<size_t>(std::max<int64_t>(n * op->dim, 1));
  SGMEV_CUDA(dev_malloc(&d_l, bytes, op->stream));
  cudaError_t e = dev_malloc(&d_i, bytes, op->stream);
  if (e != cudaSuccess) {
    dev_free(d_l, op->stream);
    return fail(SGMEV_ERR_OOM, std::string("device allocation: ") + cudaGetErrorString(e));
  }
  if (n > 0) {
    cudaMemcpyAsync(d_l, level_pow2, bytes, cudaMemcpyHostToDevice, op->stream);
    cudaMemcpyAsync(d_i, index, bytes, cudaMemcpyHostToDevice, op->stream);
  }
  if (op->mod) {
    stage_grid_mod_kernel<<<vec_blocks(npad), 256, 0, op->stream>>>(
        d_l, d_i, n, op->dim, npad, op->li64, op->li32, op->gq, op->gs64, op->gs32);
  } else {
    stage_grid_kernel<<<vec_blocks(npad * op->dim), 256, 0, op->stream>>>(
        d_l, d_i, n, op->dim, npad, op->li64, op->li32, op->gq);
  }
  op->launches += 1;
  e = cudaStreamSynchronize(op->stream);
  dev_free(d_l, op->stream);
  dev_free(d_i, op->stream);
  if (e != cudaSuccess) return fail(SGMEV_ERR_CUDA, std::string("stage grid: ") + cudaGetErrorString(e));
  // subspace tables for the FP32 products: used when chosen ("algo") and cheaper by the
  // instruction count per data point (one basis function per subspace, ~8 per active dimension
  // and ~10 per subspace, against 3 per dimension for every grid point)
  op->sub_ok = false;
  op->mat_failed = false;
  op->mat_block_only = false;
  block_free(&op->blk);
  op->blk_ok = false;
  op->blk_failed = false;
  subspace_free(&op->sub);
  if (op->algo != 0 && n > 0) {
    std::string why;
    if (subspace_build(&op->sub, op->dim, n, level_pow2, index, op->stream, &why)) {
      op->sub.mod = op->mod;
      op->sub.multt_batch = op->multt_batch;
      op->sub.multt_banks = op->multt_banks;
      op->sub.multt_ctas = op->multt_ctas;
      const double dense_cost = 3.0 * op->dim * static_cast<double>(n);
      const double sub_cost = 8.0 * static_cast<double>(op->sub.act_work) + 10.0 * op->sub.n_sub;
      op->sub_ok = op->algo == 1 || sub_cost * 1.5 < dense_cost;
      if (!op->sub_ok) subspace_free(&op->sub);
    } else if (op->algo == 1) {
      return fail(SGMEV_ERR_UNSUPPORTED, "algo \"subspace\": " + why);
    }
  }
  // output vector and split partials depend on npad
  SGMEV_TRY(dalloc(op->stream, &op->out64, static_cast<size_t>(std::max(op->npad, op->mpad))));
  const int64_t elems = part_need_elems(op);
  const size_t need = static_cast<size_t>(elems) * sizeof(double);
  if (need > op->part_bytes) {
    dev_free(op->part, op->stream);
    op->part = nullptr;
    op->part_bytes = 0;
    op->part_elems = 0;
    SGMEV_CUDA(dev_malloc(&op->part, need, op->stream));
    op->part_bytes = need;
  }
  op->part_elems = static_cast<int64_t>(op->part_bytes / sizeof(double));
  return SGMEV_OK;
}

static void release(sgmev_op* op) {
  // the operator's own work is done before its memory is handed back (a wait on its streams
  // only; frees are stream-ordered and never synchronise the device). The current stream was
  // ordered after every stream the op used before (sgmev_set_stream), so waiting on it and on
  // the op's own stream covers all of the op's work.
  if (op->stream) cudaStreamSynchronize(op->stream);
  if (op->own_stream && op->own_stream != op->stream) cudaStreamSynchronize(op->own_stream);
  block_free(&op->blk);
  subspace_free(&op->sub);
  void* ptrs[] = {op->xt64, op->xt32, op->xt32lo, op->li64, op->li32, op->gq, op->gs64, op->gs32, op->a64,
                  op->a32,  op->a32lo, op->v64,   op->v32,  op->v32lo, op->out64, op->part,
                  op->cg,   op->dot_part, op->dot_out, op->scal};
  for (void* p : ptrs) dev_free(p, op->stream);
  pinned_release(op->host_scalar);
  op->host_scalar = nullptr;
  for (cudaEvent_t e : op->prof_events) cudaEventDestroy(e);
  if (op->ev_start) cudaEventDestroy(op->ev_start);
  if (op->ev_stop) cudaEventDestroy(op->ev_stop);
  if (op->ev_switch) cudaEventDestroy(op->ev_switch);
  if (op->own_stream) cudaStreamDestroy(op->own_stream);
  (void)cudaGetLastError();
}

static int begin_timed(sgmev_op* op) {
  SGMEV_CUDA(cudaEventRecord(op->ev_start, op->stream));
  return SGMEV_OK;
}

static int end_timed(sgmev_op* op, bool sync) {
  SGMEV_CUDA(cudaEventRecord(op->ev_stop, op->stream));
  if (sync) {
    SGMEV_CUDA(cudaEventSynchronize(op->ev_stop));
    float ms = 0.f;
    SGMEV_CUDA(cudaEventElapsedTime(&ms, op->ev_start, op->ev_stop));
    op->last_seconds = ms * 1e-3;
  }
  return SGMEV_OK;
}

// Value of a string entry "key": "value" in a flat JSON object (the operator's parameters);
// empty if absent. Only what the parameters here need: no nesting, no escapes.
static std::string json_string(const char* json, const char* key) {
  if (!json) return "";
  const std::string s(json);
  const std::string k = std::string("\"") + key + "\"";
  size_t p = s.find(k);
  if (p == std::string::npos) return "";
  p = s.find(':', p + k.size());
  if (p == std::string::npos) return "";
  p = s.find('"', p + 1);
  if (p == std::string::npos) return "";
  const size_t e = s.find('"', p + 1);
  if (e == std::string::npos) return "";
  return s.substr(p + 1, e - p - 1);
}

// Launch-shape knobs (the autotuner's choices): "multt_batch", "multt_banks", "multt_ctas" and the
// "block_*" shape of the tensor-core block products. They change no result (multt_batch), only the
// order of the FP16 multTranspose's additions (multt_banks, multt_ctas), or only how the block
// products are cut into launches, so they may also change on a live operator (sgmev_set_params).
static int apply_shape_params(sgmev_op* op, const char* params_json) {
  using namespace sgmev;
  const std::string mb = json_string(params_json, "multt_batch");
  int batch = op->multt_batch;
  if (!mb.empty()) {
    if (mb != "1" && mb != "2" && mb != "4")
      return fail(SGMEV_ERR_INVALID, "params: multt_batch must be 1, 2 or 4");
    batch = mb[0] - '0';
  }
  const std::string mc = json_string(params_json, "multt_ctas");
  int ctas = op->multt_ctas;
  if (!mc.empty()) {
    if (mc != "2" && mc != "3") return fail(SGMEV_ERR_INVALID, "params: multt_ctas must be 2 or 3");
    ctas = mc[0] - '0';
  }
  const std::string mk = json_string(params_json, "multt_banks");
  int banks = op->multt_banks;
  if (!mk.empty()) {
    if (mk != "1" && mk != "2") return fail(SGMEV_ERR_INVALID, "params: multt_banks must be 1 or 2");
    banks = mk[0] - '0';
  }
  BlockShape sh = op->blk_shape;
  const char* knobs[] = {"block_mult_tiles", "block_mult_groups", "block_multt_groups",
                         "block_stages", "block_loads", "block_window", "block_teams"};
  int* fields[] = {&sh.mult_tiles, &sh.mult_groups, &sh.multt_groups, &sh.stages, &sh.loads,
                   &sh.window, &sh.teams};
  for (int k = 0; k < 7; ++k) {
    const std::string v = json_string(params_json, knobs[k]);
    if (v.empty()) continue;
    char* end = nullptr;
    const long x = std::strtol(v.c_str(), &end, 10);
    if (!end || *end != '\0' || x < 1 || x > 64)
      return fail(SGMEV_ERR_INVALID, std::string("params: ") + knobs[k] + " must be an integer in [1, 64]");
    *fields[k] = static_cast<int>(x);
  }
  const std::string ma = json_string(params_json, "block_mult_a");
  if (!ma.empty()) {
    if (ma != "tmem" && ma != "smem")
      return fail(SGMEV_ERR_INVALID, "params: block_mult_a must be \"tmem\" or \"smem\"");
    sh.mult_tmem = ma == "tmem" ? 1 : 0;
  }
  op->multt_batch = batch;
  op->sub.multt_batch = batch;
  op->multt_banks = banks;
  op->sub.multt_banks = banks;
  op->multt_ctas = ctas;
  op->sub.multt_ctas = ctas;
  op->blk_shape = sh;
  op->blk.shape = sh;
  return SGMEV_OK;
}

static int check_op(const sgmev_op* op) {
  if (!op) return fail(SGMEV_ERR_INVALID, "op is NULL");
  return SGMEV_OK;
}

// resolve recorded launch timings into the per-kind totals (needs the stream idle)
static int prof_resolve(sgmev_op* op) {
  for (size_t i = 0; i < op->prof_used; ++i) {
    float ms = 0.f;
    SGMEV_CUDA(cudaEventElapsedTime(&ms, op->prof_events[2 * i], op->prof_events[2 * i + 1]));
    op->prof_count[op->prof_kind[i]] += 1;
    op->prof_seconds[op->prof_kind[i]] += ms * 1e-3;
  }
  op->prof_used = 0;
  return SGMEV_OK;
}

}  // namespace sgmev

// =========================================================================================
// C ABI
// =========================================================================================
extern "C" {

SGMEV_API const char* sgmev_last_error(void) { return sgmev::g_last_error.c_str(); }

SGMEV_API int sgmev_version(void) { return 10000; }

SGMEV_API int sgmev_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

SGMEV_API int sgmev_create(sgmev_op** out, int dim, int64_t n_grid, const double* level_pow2,
                           const double* index, int64_t n_data, const double* data,
                           const double* bb_left, const double* bb_right, int precision,
                           const char* params_json) {
  using namespace sgmev;
  g_last_error.clear();
  if (!out) return fail(SGMEV_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (dim < 1) return fail(SGMEV_ERR_INVALID, "dim must be >= 1");
  if (n_grid < 0 || n_data < 0) return fail(SGMEV_ERR_INVALID, "negative size");
  if (n_grid > 0 && (!level_pow2 || !index)) return fail(SGMEV_ERR_INVALID, "level/index is NULL");
  if (n_data > 0 && !data) return fail(SGMEV_ERR_INVALID, "data is NULL");
  if ((bb_left == nullptr) != (bb_right == nullptr))
    return fail(SGMEV_ERR_INVALID, "bounding box needs both left and right");
  if (precision != SGMEV_FP64 && precision != SGMEV_FP32 && precision != SGMEV_DF64)
    return fail(SGMEV_ERR_INVALID, "precision must be SGMEV_FP64, SGMEV_FP32 or SGMEV_DF64");
  if (n_data > (int64_t(1) << 40) || n_grid > (int64_t(1) << 34))
    return fail(SGMEV_ERR_INVALID, "problem too large");
  SGMEV_TRY(check_grid(dim, n_grid, level_pow2, index));
  if (bb_left) {
    for (int t = 0; t < dim; ++t)
      if (!(bb_right[t] > bb_left[t]))
        return fail(SGMEV_ERR_INVALID, "bounding box interval " + std::to_string(t) + " is empty");
  }
  const std::string precond = json_string(params_json, "precond");
  const std::string algo = json_string(params_json, "algo");
  if (!algo.empty() && algo != "dense" && algo != "subspace" && algo != "auto")
    return fail(SGMEV_ERR_INVALID, "params: algo must be \"dense\", \"subspace\" or \"auto\"");
  if (!precond.empty() && precond != "jacobi" && precond != "none")
    return fail(SGMEV_ERR_INVALID, "params: precond must be \"jacobi\" or \"none\"");
  const std::string mat = json_string(params_json, "materialize");
  if (!mat.empty() && mat != "auto" && mat != "on" && mat != "off")
    return fail(SGMEV_ERR_INVALID, "params: materialize must be \"auto\", \"on\" or \"off\"");
  const std::string inner_p = json_string(params_json, "inner_products");
  if (!inner_p.empty() && inner_p != "half" && inner_p != "float")
    return fail(SGMEV_ERR_INVALID, "params: inner_products must be \"half\" or \"float\"");
  const std::string basis = json_string(params_json, "basis");
  if (!basis.empty() && basis != "linear" && basis != "modlinear")
    return fail(SGMEV_ERR_INVALID, "params: basis must be \"linear\" or \"modlinear\"");
  const std::string sys_p = json_string(params_json, "system_product");
  if (!sys_p.empty() && sys_p != "separate" && sys_p != "fused")
    return fail(SGMEV_ERR_INVALID, "params: system_product must be \"separate\" or \"fused\"");
  const std::string mat_t = json_string(params_json, "materialize_multt");
  if (!mat_t.empty() && mat_t != "on" && mat_t != "off")
    return fail(SGMEV_ERR_INVALID, "params: materialize_multt must be \"on\" or \"off\"");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(SGMEV_ERR_NO_DEVICE, "no CUDA device is visible");
  }

  sgmev_op* op = new sgmev_op;
  op->dim = dim;
  op->precision = precision;
  op->m = n_data;
  op->mpad = std::max<int64_t>(round_up(std::max<int64_t>(n_data, 1), kMPadTo), kMPadTo);
  op->precond = precond == "jacobi";
  op->mat_mode = mat == "off" ? 0 : (mat == "on" ? 2 : 1);
  op->mat_multt = mat_t != "off";
  op->fused_system = sys_p == "fused";
  op->inner_half = inner_p != "float";
  op->mod = basis == "modlinear";
  {
    const std::string it = json_string(params_json, "inner_tol");
    if (!it.empty()) {
      char* end = nullptr;
      const double v = std::strtod(it.c_str(), &end);
      if (!end || *end != '\0' || !(v > 0.0) || !(v < 1.0)) {
        release(op);
        delete op;
        return fail(SGMEV_ERR_INVALID, "params: inner_tol must be a number in (0, 1)");
      }
      op->inner_tol = v;
    }
    const std::string bt = json_string(params_json, "block_inner_tol");
    if (!bt.empty()) {
      char* end = nullptr;
      const double v = std::strtod(bt.c_str(), &end);
      if (!end || *end != '\0' || !(v > 0.0) || !(v < 1.0)) {
        release(op);
        delete op;
        return fail(SGMEV_ERR_INVALID, "params: block_inner_tol must be a number in (0, 1)");
      }
      op->block_inner_tol = v;
    }
    const std::string bp = json_string(params_json, "block_products");
    if (!bp.empty()) {
      if (bp != "bf16" && bp != "f16") {
        release(op);
        delete op;
        return fail(SGMEV_ERR_INVALID, "params: block_products must be \"bf16\" or \"f16\"");
      }
      op->block_f16 = bp == "f16";
    }
    const int rc_shape = apply_shape_params(op, params_json);
    if (rc_shape != SGMEV_OK) {
      release(op);
      delete op;
      return rc_shape;
    }
  }
  op->algo = algo == "dense" ? 0 : (algo == "subspace" ? 1 : 2);
  auto bail = [&](int rc) {
    release(op);
    delete op;
    return rc;
  };
#define CREATE_CUDA(call)                                                               \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return bail(fail(e_ == cudaErrorMemoryAllocation ? SGMEV_ERR_OOM : SGMEV_ERR_CUDA, \
                       std::string(#call) + ": " + cudaGetErrorString(e_)));            \
  } while (0)
#define CREATE_TRY(expr)               \
  do {                                 \
    int rc_ = (expr);                  \
    if (rc_ != SGMEV_OK) return bail(rc_); \
  } while (0)

  CREATE_CUDA(cudaGetDevice(&op->device));
  CREATE_CUDA(cudaDeviceGetAttribute(&op->num_sms, cudaDevAttrMultiProcessorCount, op->device));
  op->target_ctas = static_cast<int64_t>(op->num_sms) * 4;
  CREATE_CUDA(cudaStreamCreateWithFlags(&op->own_stream, cudaStreamNonBlocking));
  op->stream = op->own_stream;
  CREATE_CUDA(cudaEventCreate(&op->ev_start));
  CREATE_CUDA(cudaEventCreate(&op->ev_stop));
  CREATE_CUDA(cudaEventCreateWithFlags(&op->ev_switch, cudaEventDisableTiming));
  op->host_scalar = static_cast<double*>(pinned_block());
  if (!op->host_scalar) return bail(fail(SGMEV_ERR_OOM, "pinned host block"));
  CREATE_TRY(dalloc(op->stream, &op->dot_part, kDotBlocks));
  CREATE_TRY(dalloc(op->stream, &op->dot_out, 8));
  CREATE_TRY(dalloc(op->stream, &op->scal, 16));
  CREATE_CUDA(cudaMemsetAsync(op->scal, 0, sizeof(double) * 16, op->stream));

  // data
  CREATE_TRY(dalloc(op->stream, &op->xt64, static_cast<size_t>(op->mpad * dim)));
  CREATE_TRY(dalloc(op->stream, &op->xt32, static_cast<size_t>(op->mpad * dim)));
  CREATE_TRY(dalloc(op->stream, &op->xt32lo, static_cast<size_t>(op->mpad * dim)));
  CREATE_TRY(dalloc(op->stream, &op->v64, static_cast<size_t>(op->mpad)));
  CREATE_TRY(dalloc(op->stream, &op->v32, static_cast<size_t>(op->mpad)));
  CREATE_TRY(dalloc(op->stream, &op->v32lo, static_cast<size_t>(op->mpad)));
  {
    double* d_rows = nullptr;
    double* d_bb = nullptr;
    const size_t rbytes = sizeof(double) * static_cast<size_t>(std::max<int64_t>(n_data * dim, 1));
    CREATE_CUDA(dev_malloc(&d_rows, rbytes, op->stream));
    if (n_data > 0) cudaMemcpyAsync(d_rows, data, rbytes, cudaMemcpyHostToDevice, op->stream);
    if (bb_left) {
      op->bb_left.assign(bb_left, bb_left + dim);
      op->bb_width.resize(dim);
      std::vector<double> hb(2 * dim);
      for (int t = 0; t < dim; ++t) {
        op->bb_width[t] = bb_right[t] - bb_left[t];
        hb[t] = bb_left[t];
        hb[dim + t] = op->bb_width[t];
      }
      cudaError_t e = dev_malloc(&d_bb, sizeof(double) * 2 * dim, op->stream);
      if (e != cudaSuccess) {
        dev_free(d_rows, op->stream);
        return bail(fail(SGMEV_ERR_OOM, "device allocation for the bounding box"));
      }
      cudaMemcpyAsync(d_bb, hb.data(), sizeof(double) * 2 * dim, cudaMemcpyHostToDevice, op->stream);
    }
    stage_data_kernel<<<vec_blocks(op->mpad * dim), 256, 0, op->stream>>>(
        d_rows, n_data, dim, op->mpad, d_bb, d_bb ? d_bb + dim : nullptr, op->xt64, op->xt32,
        op->xt32lo);
    op->launches += 1;
    unsigned int* flag = reinterpret_cast<unsigned int*>(op->dot_out);
    if (op->mod) {
      // the ModLinear subspace products want the data in the cube (see mat_ready)
      cudaMemsetAsync(flag, 0, sizeof(unsigned int), op->stream);
      cube_check_kernel<<<vec_blocks(op->mpad * dim), 256, 0, op->stream>>>(
          op->xt64, op->mpad * dim, flag);
      op->launches += 1;
      cudaMemcpyAsync(op->host_scalar, flag, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                      op->stream);
    }
    cudaError_t e = cudaStreamSynchronize(op->stream);
    dev_free(d_rows, op->stream);
    dev_free(d_bb, op->stream);
    if (e != cudaSuccess) return bail(fail(SGMEV_ERR_CUDA, std::string("stage data: ") + cudaGetErrorString(e)));
    if (op->mod) op->in_cube = *reinterpret_cast<const unsigned int*>(op->host_scalar) == 0;
  }
  CREATE_TRY(stage_grid(op, n_grid, level_pow2, index));
#undef CREATE_CUDA
#undef CREATE_TRY
  *out = op;
  return SGMEV_OK;
}

SGMEV_API int sgmev_destroy(sgmev_op* op) {
  if (!op) return SGMEV_OK;
  if (op->stream) cudaStreamSynchronize(op->stream);
  sgmev::release(op);
  delete op;
  return SGMEV_OK;
}

SGMEV_API int sgmev_prepare(sgmev_op* op, int64_t n_grid, const double* level_pow2,
                            const double* index) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  if (n_grid < 0) return fail(SGMEV_ERR_INVALID, "negative size");
  if (n_grid > 0 && (!level_pow2 || !index)) return fail(SGMEV_ERR_INVALID, "level/index is NULL");
  SGMEV_TRY(check_grid(op->dim, n_grid, level_pow2, index));
  SGMEV_CUDA(cudaStreamSynchronize(op->stream));
  return stage_grid(op, n_grid, level_pow2, index);
}

SGMEV_API int sgmev_get_sizes(const sgmev_op* op, int* dim, int64_t* n_grid, int64_t* n_data) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  if (dim) *dim = op->dim;
  if (n_grid) *n_grid = op->n;
  if (n_data) *n_data = op->m;
  return SGMEV_OK;
}

SGMEV_API int sgmev_set_stream(sgmev_op* op, void* stream) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  cudaStream_t next = stream ? static_cast<cudaStream_t>(stream) : op->own_stream;
  if (next != op->stream) {
    // work enqueued from now on (including stream-ordered frees of the op's buffers) runs after
    // everything the op enqueued on the previous stream
    SGMEV_CUDA(cudaEventRecord(op->ev_switch, op->stream));
    SGMEV_CUDA(cudaStreamWaitEvent(next, op->ev_switch, 0));
    op->stream = next;
  }
  return SGMEV_OK;
}

SGMEV_API int sgmev_set_params(sgmev_op* op, const char* params_json) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  if (!params_json) return SGMEV_OK;
  static const char* allowed[] = {"multt_batch", "multt_banks", "multt_ctas", "block_mult_tiles", "block_mult_groups",
                                  "block_multt_groups", "block_stages", "block_loads",
                                  "block_mult_a", "block_window", "block_teams"};
  // every key must be a launch-shape knob
  for (const char* c = params_json; (c = std::strchr(c, '"')) != nullptr;) {
    const char* e = std::strchr(c + 1, '"');
    if (!e) break;
    const std::string key(c + 1, e);
    const char* after = e + 1;
    while (*after == ' ') ++after;
    if (*after == ':') {
      bool ok = false;
      for (const char* a : allowed) ok = ok || key == a;
      if (!ok) return fail(SGMEV_ERR_INVALID, "sgmev_set_params: \"" + key + "\" is not a launch-shape knob");
    }
    c = e + 1;
  }
  SGMEV_CUDA(cudaStreamSynchronize(op->stream));
  int cap = 0;
  SGMEV_CUDA(cudaDeviceGetAttribute(&cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, op->device));
  const BlockShape before = op->blk_shape;
  SGMEV_TRY(apply_shape_params(op, params_json));
  if (!block_shape_ok(op->blk_shape, cap)) {
    op->blk_shape = before;
    op->blk.shape = before;
    return fail(SGMEV_ERR_INVALID, "invalid block launch shape (teams must be at most the stages and divide the loads; window at most 3; the stages and coefficient rows must fit shared and tensor memory)");
  }
  return SGMEV_OK;
}

SGMEV_API int sgmev_synchronize(sgmev_op* op) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  SGMEV_CUDA(cudaStreamSynchronize(op->stream));
  return SGMEV_OK;
}

SGMEV_API int64_t sgmev_kernel_launches(const sgmev_op* op) { return op ? op->launches : 0; }

SGMEV_API double sgmev_get_duration(sgmev_op* op) { return op ? op->last_seconds : -1.0; }

static int mult_common(sgmev_op* op, const double* alpha_dev_or_null, const double* alpha_host,
                       double* result_dev, double* result_host, int64_t start, int64_t end) {
  using namespace sgmev;
  const int prec = op->precision;
  SGMEV_TRY(begin_timed(op));
  const double* src = alpha_dev_or_null;
  if (alpha_host) {
    if (op->n > 0)
      SGMEV_CUDA(cudaMemcpyAsync(op->out64, alpha_host, sizeof(double) * op->n,
                                 cudaMemcpyHostToDevice, op->stream));
    src = op->out64;
  }
  SGMEV_TRY(dev_convert(op, src, op->n, op->npad, prec == SGMEV_FP64 ? op->a64 : nullptr,
                        prec == SGMEV_FP64 ? nullptr : op->a32,
                        prec == SGMEV_DF64 ? op->a32lo : nullptr));
  // tile-aligned data range covering [start, end)
  const int64_t tile_pts = mult_tile_pts(op, prec);
  const int64_t jb = (start / tile_pts) * tile_pts;
  const int64_t je = std::min(op->mpad, round_up(end, tile_pts));
  SGMEV_TRY(dev_mult(op, prec, op->a64, op->a32, op->a32lo, op->v64, nullptr, jb, je));
  if (result_host) {
    if (end > start)
      SGMEV_CUDA(cudaMemcpyAsync(result_host + start, op->v64 + start,
                                 sizeof(double) * (end - start), cudaMemcpyDeviceToHost,
                                 op->stream));
  } else if (result_dev && end > start) {
    SGMEV_CUDA(cudaMemcpyAsync(result_dev + start, op->v64 + start, sizeof(double) * (end - start),
                               cudaMemcpyDeviceToDevice, op->stream));
  }
  SGMEV_TRY(end_timed(op, result_host != nullptr));
  return SGMEV_OK;
}

static int multt_common(sgmev_op* op, const double* src_dev, const double* src_host,
                        double* result_dev, double* result_host, int64_t start, int64_t end) {
  using namespace sgmev;
  const int prec = op->precision;
  SGMEV_TRY(begin_timed(op));
  const double* src = src_dev;
  if (src_host) {
    if (op->m > 0)
      SGMEV_CUDA(cudaMemcpyAsync(op->out64, src_host, sizeof(double) * op->m,
                                 cudaMemcpyHostToDevice, op->stream));
    src = op->out64;
  }
  SGMEV_TRY(dev_convert(op, src, op->m, op->mpad, prec == SGMEV_FP64 ? op->v64 : nullptr,
                        prec == SGMEV_FP64 ? nullptr : op->v32,
                        prec == SGMEV_DF64 ? op->v32lo : nullptr));
  const int64_t tile_pts = multt_tile_pts(op, prec);
  const int64_t gb = (start / tile_pts) * tile_pts;
  const int64_t ge = std::min(op->npad, round_up(end, tile_pts));
  double* tmp = op->cg + 7 * op->npad;  // spare CG slot as result staging
  SGMEV_TRY(dev_multt(op, prec, op->v64, op->v32, op->v32lo, tmp, gb, ge, nullptr, 0.0));
  if (result_host) {
    if (end > start)
      SGMEV_CUDA(cudaMemcpyAsync(result_host + start, tmp + start, sizeof(double) * (end - start),
                                 cudaMemcpyDeviceToHost, op->stream));
  } else if (result_dev && end > start) {
    SGMEV_CUDA(cudaMemcpyAsync(result_dev + start, tmp + start, sizeof(double) * (end - start),
                               cudaMemcpyDeviceToDevice, op->stream));
  }
  SGMEV_TRY(end_timed(op, result_host != nullptr));
  return SGMEV_OK;
}

SGMEV_API int sgmev_mult(sgmev_op* op, const double* alpha, double* result) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  if ((op->n > 0 && !alpha) || (op->m > 0 && !result)) return fail(SGMEV_ERR_INVALID, "NULL vector");
  return mult_common(op, nullptr, alpha, nullptr, result, 0, op->m);
}

SGMEV_API int sgmev_mult_transpose(sgmev_op* op, const double* source, double* result) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  if ((op->m > 0 && !source) || (op->n > 0 && !result)) return fail(SGMEV_ERR_INVALID, "NULL vector");
  return multt_common(op, nullptr, source, nullptr, result, 0, op->n);
}

SGMEV_API int sgmev_mult_range(sgmev_op* op, const double* alpha, double* result,
                               int64_t start_data, int64_t end_data) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  if (start_data < 0 || end_data > op->m || start_data > end_data)
    return fail(SGMEV_ERR_INVALID, "data range out of bounds");
  if ((op->n > 0 && !alpha) || (end_data > start_data && !result)) return fail(SGMEV_ERR_INVALID, "NULL vector");
  return mult_common(op, nullptr, alpha, nullptr, result, start_data, end_data);
}

SGMEV_API int sgmev_mult_transpose_range(sgmev_op* op, const double* source, double* result,
                                         int64_t start_grid, int64_t end_grid) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  if (start_grid < 0 || end_grid > op->n || start_grid > end_grid)
    return fail(SGMEV_ERR_INVALID, "grid range out of bounds");
  if ((op->m > 0 && !source) || (end_grid > start_grid && !result)) return fail(SGMEV_ERR_INVALID, "NULL vector");
  return multt_common(op, nullptr, source, nullptr, result, start_grid, end_grid);
}

SGMEV_API int sgmev_mult_device(sgmev_op* op, const double* d_alpha, double* d_result) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  if ((op->n > 0 && !d_alpha) || (op->m > 0 && !d_result)) return fail(SGMEV_ERR_INVALID, "NULL vector");
  return mult_common(op, d_alpha, nullptr, d_result, nullptr, 0, op->m);
}

SGMEV_API int sgmev_mult_transpose_device(sgmev_op* op, const double* d_source,
                                          double* d_result) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  if ((op->m > 0 && !d_source) || (op->n > 0 && !d_result)) return fail(SGMEV_ERR_INVALID, "NULL vector");
  return multt_common(op, d_source, nullptr, d_result, nullptr, 0, op->n);
}

static int system_common(sgmev_op* op, const double* a_dev, const double* a_host, double* r_dev,
                         double* r_host, double lm) {
  using namespace sgmev;
  SGMEV_TRY(begin_timed(op));
  double* a = op->cg + 6 * op->npad;  // padded copy of the input
  double* r = op->cg + 7 * op->npad;
  const double* src = a_dev;
  if (a_host) {
    if (op->n > 0)
      SGMEV_CUDA(cudaMemcpyAsync(op->out64, a_host, sizeof(double) * op->n,
                                 cudaMemcpyHostToDevice, op->stream));
    src = op->out64;
  }
  SGMEV_TRY(dev_convert(op, src, op->n, op->npad, a, nullptr, nullptr));
  SGMEV_TRY(dev_system(op, op->precision, a, r, lm));
  if (r_host) {
    if (op->n > 0)
      SGMEV_CUDA(cudaMemcpyAsync(r_host, r, sizeof(double) * op->n, cudaMemcpyDeviceToHost, op->stream));
  } else if (op->n > 0) {
    SGMEV_CUDA(cudaMemcpyAsync(r_dev, r, sizeof(double) * op->n, cudaMemcpyDeviceToDevice, op->stream));
  }
  SGMEV_TRY(end_timed(op, r_host != nullptr));
  return SGMEV_OK;
}

SGMEV_API int sgmev_system_apply(sgmev_op* op, const double* alpha, double* result,
                                 double lambda_times_m) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  if (op->n > 0 && (!alpha || !result)) return fail(SGMEV_ERR_INVALID, "NULL vector");
  return system_common(op, nullptr, alpha, nullptr, result, lambda_times_m);
}

SGMEV_API int sgmev_system_apply_device(sgmev_op* op, const double* d_alpha, double* d_result,
                                        double lambda_times_m) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  if (op->n > 0 && (!d_alpha || !d_result)) return fail(SGMEV_ERR_INVALID, "NULL vector");
  return system_common(op, d_alpha, nullptr, d_result, nullptr, lambda_times_m);
}

// CG on (B^T B + lm I) x = rhs with operator precision `prec`; all vectors padded device FP64.
// Mirrors ConjugateGradients::solve (ConjugateGradients.cpp:22-151). x is the start vector
// when reuse, otherwise zeroed. delta0_scale multiplies the starting delta (epsilon^2).
static int cg_core(sgmev_op* op, int prec, const double* rhs, double* x, double lm,
                   int64_t imax, double eps, bool reuse, int64_t* iters, double* delta_final) {
  using namespace sgmev;
  const int64_t np = op->npad;
  double* r = op->cg + 2 * np;
  double* d = op->cg + 3 * np;
  double* q = op->cg + 4 * np;
  double* t = op->cg + 5 * np;
  const double eps2 = eps * eps;
  double delta_0 = 0.0;
  SGMEV_CUDA(cudaMemcpyAsync(r, rhs, sizeof(double) * np, cudaMemcpyDeviceToDevice, op->stream));
  if (reuse) {
    // A * 0 = 0, so r = rhs (ConjugateGradients.cpp:58-62)
    SGMEV_TRY(dev_dot(op, r, r, np, &delta_0));
    delta_0 *= eps2;
  } else {
    SGMEV_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * np, op->stream));
  }
  if (reuse) {
    // r = rhs - A x (ConjugateGradients.cpp:68-70); for x = 0 this product is exactly zero
    // (0 * hat = 0, sums of zeros, lambda * 0), so the cold start skips it.
    SGMEV_TRY(dev_system(op, prec, x, t, lm));
    sub_kernel<<<vec_blocks(np), 256, 0, op->stream>>>(np, r, t, r);
    op->launches += 1;
  }
  SGMEV_CUDA(cudaMemcpyAsync(d, r, sizeof(double) * np, cudaMemcpyDeviceToDevice, op->stream));
  // the scalars live on the device (alpha and beta never visit the host); the host reads
  // delta_new and d.q once per iteration for the stopping test
  double* sc = op->scal;
  double* host = op->host_scalar;  // pinned: [0] delta_new, [1] delta_old, [2] d.q
  auto read_scalars = [&]() -> int {
    SGMEV_CUDA(cudaMemcpyAsync(host, sc, sizeof(double) * 3, cudaMemcpyDeviceToHost, op->stream));
    SGMEV_CUDA(cudaStreamSynchronize(op->stream));
    return SGMEV_OK;
  };
  // delta_new = r.r (the update kernel without steps)
  cg_update_kernel<<<kDotBlocks, kDotThreads, 0, op->stream>>>(np, d, q, x, r, 0, 1,
                                                                 op->dot_part, sc);
  op->launches += 1;
  SGMEV_CUDA(cudaGetLastError());
  SGMEV_TRY(read_scalars());
  double delta_new = host[0];
  if (!reuse) delta_0 = delta_new * eps2;
  int64_t it = 0;
  while (it < imax && delta_new > delta_0 && delta_new > 0.0) {
    SGMEV_TRY(dev_system(op, prec, d, q, lm));
    cg_alpha_kernel<<<kDotBlocks, kDotThreads, 0, op->stream>>>(d, q, np, op->dot_part, sc);
    op->launches += 1;
    if (it % 50 == 0 && it > 0) {
      // the true residual every 50 iterations (ConjugateGradients.cpp:99-104)
      axpy_dev_kernel<<<vec_blocks(np), 256, 0, op->stream>>>(np, sc, d, x);
      SGMEV_TRY(dev_system(op, prec, x, t, lm));
      sub_kernel<<<vec_blocks(np), 256, 0, op->stream>>>(np, rhs, t, r);
      cg_update_kernel<<<kDotBlocks, kDotThreads, 0, op->stream>>>(np, d, q, x, r, 0, 1,
                                                                     op->dot_part, sc);
      op->launches += 3;
    } else {
      cg_update_kernel<<<kDotBlocks, kDotThreads, 0, op->stream>>>(np, d, q, x, r, 1, 0,
                                                                     op->dot_part, sc);
      op->launches += 1;
    }
    xpby_dev_kernel<<<vec_blocks(np), 256, 0, op->stream>>>(np, r, sc, d);
    op->launches += 1;
    SGMEV_CUDA(cudaGetLastError());
    SGMEV_TRY(read_scalars());
    // d.q == 0: alpha was 0, so x and r did not move; stop as the reference does before a step
    if (host[2] == 0.0) break;
    delta_new = host[0];
    ++it;
  }
  SGMEV_CUDA(cudaGetLastError());
  *iters = it;
  *delta_final = delta_new;
  return SGMEV_OK;
}

// 1/diag(B^T B + lm I) into CG slot 9 (Jacobi preconditioner), from one FP32 squared-hat
// multTranspose with v = 1: diag_i = sum_j prod_t hat_t(x_j)^2. Cached until the grid or lm changes.
static int dev_precond(sgmev_op* op, double lm) {
  using namespace sgmev;
  const int64_t np = op->npad;
  double* inv = op->cg + 9 * np;
  if (op->pc_valid && op->pc_lm == lm) return SGMEV_OK;
  ones_kernel<<<vec_blocks(op->mpad), 256, 0, op->stream>>>(op->m, op->mpad, op->v32);
  op->launches += 1;
  Plan p;
  float* part = static_cast<float*>(op->part);
  if (op->mod) {
    const bool tiled = op->dim <= kMaxTemplDim;
    p = plan_multt<float>(op, tiled ? np / (kBlock * Blocking<float>::multt_r(op->dim))
                                    : ceil_div(np, kBlock));
    dim3 grid(static_cast<unsigned>(p.tiles), static_cast<unsigned>(p.nsplit));
    mod_multt_launch<float, true>(op->dim, grid, op->stream, op->xt32, op->v32, op->mpad,
                                  op->li32, op->gs32, np, p.chunk, 0, np, part);
  } else if (op->dim <= kMaxTemplDim) {
    const int64_t tiles = np / (kBlock * Blocking<float>::multt_r(op->dim));
    p = plan_multt<float>(op, tiles);
    dim3 grid(static_cast<unsigned>(p.tiles), static_cast<unsigned>(p.nsplit));
    switch (op->dim) {
#define F(D)                                                                                     \
  case D:                                                                                        \
    mult_transpose_kernel<float, D, Blocking<float>::multt_r(D), kBlock, kDT, true>              \
        <<<grid, kBlock, 0, op->stream>>>(op->xt32, op->v32, op->mpad, op->li32, np, p.chunk, 0, \
                                          part);                                                 \
    break;
      SGMEV_DIM_CASES(F)
#undef F
      default:
        break;
    }
  } else {
    p = plan_multt<float>(op, ceil_div(np, kBlock));
    dim3 grid(static_cast<unsigned>(p.tiles), static_cast<unsigned>(p.nsplit));
    mult_transpose_generic_kernel<float, true><<<grid, kBlock, 0, op->stream>>>(
        op->xt32, op->v32, op->mpad, op->dim, op->li32, np, p.chunk, 0, np, part);
  }
  op->launches += 1;
  SGMEV_CUDA(cudaGetLastError());
  double* diag = op->cg + 8 * np;
  SGMEV_TRY((run_reduce<float, double>(op, (int)p.nsplit, np, 0, op->n, np, diag, nullptr, 0.0)));
  inv_diag_kernel<<<vec_blocks(np), 256, 0, op->stream>>>(op->n, np, diag, lm, inv);
  op->launches += 1;
  SGMEV_CUDA(cudaGetLastError());
  op->pc_valid = true;
  op->pc_lm = lm;
  return SGMEV_OK;
}

// Jacobi-preconditioned CG from x = 0 on (B^T B + lm I) x = rhs with operator precision `prec`
// (the inner correction solve of the mixed fit). Stops when the preconditioned residual norm
// r.z falls below eps^2 times its start value, or after imax iterations.
static int pcg_core(sgmev_op* op, int prec, const double* rhs, double* x, double lm,
                    int64_t imax, double eps, int64_t* iters) {
  using namespace sgmev;
  const int64_t np = op->npad;
  double* r = op->cg + 2 * np;
  double* d = op->cg + 3 * np;
  double* q = op->cg + 4 * np;
  double* z = op->cg + 8 * np;
  const double* inv = op->cg + 9 * np;
  SGMEV_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * np, op->stream));
  SGMEV_CUDA(cudaMemcpyAsync(r, rhs, sizeof(double) * np, cudaMemcpyDeviceToDevice, op->stream));
  mul_kernel<<<vec_blocks(np), 256, 0, op->stream>>>(np, inv, r, z);
  op->launches += 1;
  SGMEV_CUDA(cudaMemcpyAsync(d, z, sizeof(double) * np, cudaMemcpyDeviceToDevice, op->stream));
  double delta_new = 0.0;
  SGMEV_TRY(dev_dot(op, r, z, np, &delta_new));
  const double delta_0 = delta_new * eps * eps;
  int64_t it = 0;
  while (it < imax && delta_new > delta_0 && delta_new > 0.0) {
    SGMEV_TRY(dev_system(op, prec, d, q, lm));
    double dq = 0.0;
    SGMEV_TRY(dev_dot(op, d, q, np, &dq));
    if (dq == 0.0) break;
    const double a = delta_new / dq;
    SGMEV_TRY(dev_axpy(op, np, a, d, x));
    SGMEV_TRY(dev_axpy(op, np, -a, q, r));
    mul_kernel<<<vec_blocks(np), 256, 0, op->stream>>>(np, inv, r, z);
    op->launches += 1;
    const double delta_old = delta_new;
    SGMEV_TRY(dev_dot(op, r, z, np, &delta_new));
    xpby_kernel<<<vec_blocks(np), 256, 0, op->stream>>>(np, z, delta_new / delta_old, d);
    op->launches += 1;
    ++it;
  }
  SGMEV_CUDA(cudaGetLastError());
  *iters = it;
  return SGMEV_OK;
}

static int fit_common(sgmev_op* op, int mode, const double* y, bool y_on_device, double lambda,
                      int64_t max_iterations, double epsilon, int reuse, double* alpha,
                      bool alpha_on_device, int64_t* iterations, double* residual);

SGMEV_API int sgmev_fit(sgmev_op* op, int mode, const double* y, double lambda,
                        int64_t max_iterations, double epsilon, int reuse, double* alpha,
                        int64_t* iterations, double* residual) {
  return fit_common(op, mode, y, false, lambda, max_iterations, epsilon, reuse, alpha, false,
                    iterations, residual);
}

SGMEV_API int sgmev_fit_device(sgmev_op* op, int mode, const double* d_y, double lambda,
                               int64_t max_iterations, double epsilon, int reuse, double* d_alpha,
                               int64_t* iterations, double* residual) {
  return fit_common(op, mode, d_y, true, lambda, max_iterations, epsilon, reuse, d_alpha, true,
                    iterations, residual);
}

static int fit_common(sgmev_op* op, int mode, const double* y, bool y_on_device, double lambda,
                      int64_t max_iterations, double epsilon, int reuse, double* alpha,
                      bool alpha_on_device, int64_t* iterations, double* residual) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  if ((op->m > 0 && !y) || (op->n > 0 && !alpha)) return fail(SGMEV_ERR_INVALID, "NULL vector");
  if (mode != SGMEV_SOLVE_PLAIN && mode != SGMEV_SOLVE_MIXED && mode != SGMEV_SOLVE_MIXED_NATIVE64)
    return fail(SGMEV_ERR_INVALID, "mode must be SGMEV_SOLVE_PLAIN, _MIXED or _MIXED_NATIVE64");
  // precision of b = B^T y and of the outer residual
  const int res_prec = mode == SGMEV_SOLVE_MIXED            ? SGMEV_DF64
                       : mode == SGMEV_SOLVE_MIXED_NATIVE64 ? SGMEV_FP64
                                                            : op->precision;
  if (!(epsilon > 0.0) || max_iterations < 0) return fail(SGMEV_ERR_INVALID, "bad epsilon/max_iterations");
  const int64_t np = op->npad;
  double* b = op->cg;
  double* x = op->cg + np;
  const double lm = static_cast<double>(op->m) * lambda;
  SGMEV_TRY(begin_timed(op));
  // b = B^T y in FP64 (generateb)
  if (op->m > 0)
    SGMEV_CUDA(cudaMemcpyAsync(op->out64, y, sizeof(double) * op->m,
                               y_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                               op->stream));
  SGMEV_TRY(dev_convert(op, op->out64, op->m, op->mpad, op->v64, op->v32, op->v32lo));
  SGMEV_TRY(dev_multt(op, res_prec, op->v64, op->v32, op->v32lo, b, 0, np, nullptr, 0.0));
  if (reuse) {
    double* tmp = op->cg + 7 * np;
    if (op->n > 0)
      SGMEV_CUDA(cudaMemcpyAsync(tmp, alpha, sizeof(double) * op->n,
                                 alpha_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                 op->stream));
    SGMEV_TRY(dev_convert(op, tmp, op->n, np, x, nullptr, nullptr));
  }
  int64_t total_it = 0;
  double res = 0.0;
  if (mode == SGMEV_SOLVE_PLAIN) {
    SGMEV_TRY(cg_core(op, op->precision, b, x, lm, max_iterations, epsilon, reuse != 0, &total_it, &res));
  } else {
    // iterative refinement: r = b - A x with the FP64-accurate operator (df64 or native FP64),
    // solve A32 dx = r by CG with FP32 kernels and FP64 vectors, x += dx
    double* rr = op->cg + 6 * np;  // outer residual (cg_core uses slots 2..5)
    double* dx = op->cg + 7 * np;
    if (!reuse) SGMEV_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * np, op->stream));
    double rnorm2 = 0.0, r0 = 0.0;
    const double eps_inner = op->inner_tol;
    if (op->precond) SGMEV_TRY(dev_precond(op, lm));
    for (int outer = 0; outer < 64; ++outer) {
      if (outer == 0 && !reuse) {
        // cold start: A * 0 is exactly zero, so the first residual is b itself
        SGMEV_CUDA(cudaMemcpyAsync(rr, b, sizeof(double) * np, cudaMemcpyDeviceToDevice, op->stream));
      } else {
        SGMEV_TRY(dev_system(op, res_prec, x, rr, lm));
        sub_kernel<<<vec_blocks(np), 256, 0, op->stream>>>(np, b, rr, rr);
        op->launches += 1;
      }
      SGMEV_TRY(dev_dot(op, rr, rr, np, &rnorm2));
      if (outer == 0) r0 = rnorm2;
      res = rnorm2;
      if (rnorm2 <= epsilon * epsilon * r0 || rnorm2 == 0.0 || total_it >= max_iterations) break;
      int64_t it = 0;
      double dres = 0.0;
      const double want = std::max(eps_inner, epsilon * std::sqrt(r0 / rnorm2) * 0.5);
      // the inner solve may use the FP16 copy of the materialised products: the outer residual
      // is FP64-accurate, so the refinement still converges to the FP64 solution
      struct HalfScope {
        sgmev_op* o;
        // ModLinear products reach 2^(active dimensions): FP16 holds them up to 15
        explicit HalfScope(sgmev_op* op_) : o(op_) {
          o->use_half = o->inner_half && (!o->mod || o->sub.na_max <= 15);
        }
        ~HalfScope() { o->use_half = false; }
      } half_scope(op);
      if (op->precond) {
        SGMEV_TRY(pcg_core(op, SGMEV_FP32, rr, dx, lm, max_iterations - total_it,
                           std::min(want, 0.5), &it));
      } else {
        SGMEV_TRY(cg_core(op, SGMEV_FP32, rr, dx, lm, max_iterations - total_it,
                          std::min(want, 0.5), false, &it, &dres));
      }
      total_it += it;
      SGMEV_TRY(dev_axpy(op, np, 1.0, dx, x));
    }
  }
  if (op->n > 0)
    SGMEV_CUDA(cudaMemcpyAsync(alpha, x, sizeof(double) * op->n,
                               alpha_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                               op->stream));
  SGMEV_TRY(end_timed(op, true));
  if (iterations) *iterations = total_it;
  if (residual) *residual = res;
  return SGMEV_OK;
}

SGMEV_API int sgmev_profile(sgmev_op* op, int enable) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  SGMEV_CUDA(cudaStreamSynchronize(op->stream));
  op->profile = enable != 0;
  op->prof_used = 0;
  for (int k = 0; k < kKinds; ++k) {
    op->prof_count[k] = 0;
    op->prof_seconds[k] = 0.0;
  }
  return SGMEV_OK;
}

SGMEV_API int sgmev_profile_read(sgmev_op* op, int kind, int64_t* launches, double* seconds) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  if (kind < 0 || kind >= kKinds) return fail(SGMEV_ERR_INVALID, "unknown kernel kind");
  SGMEV_CUDA(cudaStreamSynchronize(op->stream));
  SGMEV_TRY(prof_resolve(op));
  if (launches) *launches = op->prof_count[kind];
  if (seconds) *seconds = op->prof_seconds[kind];
  return SGMEV_OK;
}

// ---- 16 right-hand sides: BF16 tensor-core block products and block fits ------------------
// The materialised products of a grid the materialised kernels do not take, built only to pack
// the block products from (same memory rule as mat_ready); false when they cannot be built.
static bool block_materialize(sgmev_op* op) {
  using namespace sgmev;
  if (op->mat_mode == 0 || op->mat_block_only || (op->mod && !op->in_cube)) return false;
  if (op->sub.n_sub <= 0 || op->sub.cmax <= 0 || op->sub.cmax > kBlockMaxCells) return false;
  const int64_t bytes = subspace_mat_bytes(op->sub, op->mpad);
  if (op->mat_mode == 1) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      (void)cudaGetLastError();
      return false;
    }
    if (static_cast<double>(bytes) > std::min(0.5 * static_cast<double>(free_b), 64.0 * (1ull << 30)))
      return false;
  }
  if (subspace_materialize(&op->sub, op->stream, op->xt32, op->xt32lo, op->mpad, op->m,
                           op->num_sms) != cudaSuccess) {
    (void)cudaGetLastError();
    subspace_mat_release(&op->sub, op->stream);
    return false;
  }
  op->launches += 1;
  return true;
}

// The block products need the subspace plan and its materialised products (grids whose subspaces
// have at most 128 cells); they are built on the first block call and kept until prepare().
static int block_ready(sgmev_op* op) {
  using namespace sgmev;
  if (op->blk_ok) return SGMEV_OK;
  if (op->blk_failed) return fail(SGMEV_ERR_UNSUPPORTED, "block products: " + op->blk_err);
  int cap = 0;
  SGMEV_CUDA(cudaDeviceGetAttribute(&cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, op->device));
  if (!block_shape_ok(op->blk_shape, cap))
    return fail(SGMEV_ERR_INVALID, "invalid block launch shape (teams must be at most the stages and divide the loads; window at most 3; the stages and coefficient rows must fit shared and tensor memory)");
  // The block products are packed from the materialised products. Where the materialised
  // kernels do not take the grid (their coefficients live in shared memory: grids with many
  // subspaces of many cells), the products are built only for the packing and freed after it.
  const bool block_only = op->sub_ok && !mat_ready(op) && block_materialize(op);
  if (!op->sub_ok || (!block_only && !mat_ready(op))) {
    op->blk_failed = true;
    op->blk_err = "they stream the materialised subspace products (params \"algo\": \"subspace\", "
                  "\"materialize\": not \"off\"), which this operator does not have";
    return fail(SGMEV_ERR_UNSUPPORTED, "block products: " + op->blk_err);
  }
  std::string err;
  const bool built = block_build(&op->blk, op->sub, op->m, op->mpad, op->block_f16, op->stream,
                                 op->num_sms, &err);
  if (block_only) {
    subspace_mat_release(&op->sub, op->stream);
    op->mat_block_only = true;
  }
  if (!built) {
    op->blk_failed = true;
    op->blk_err = err;
    return fail(SGMEV_ERR_UNSUPPORTED, "block products: " + err);
  }
  op->blk.shape = op->blk_shape;
  op->launches += 1;
  op->blk_ok = true;
  return SGMEV_OK;
}

static int block_check(sgmev_op* op) {
  using namespace sgmev;
  int st = 0;
  SGMEV_CUDA(block_status(op->blk, op->stream, &st));
  if (st != 0)
    return fail(SGMEV_ERR_CUDA, "block products: a wait of the tensor-core kernels ran out (status " +
                                    std::to_string(st) + ")");
  return SGMEV_OK;
}

// q = B^T (B d) + lm d for 16 columns, on the tensor cores
static int block_system(sgmev_op* op, const double* d, double* q, double lm) {
  using namespace sgmev;
  const long e0 = prof_begin(op, KIND_BLOCK_MULT);
  SGMEV_CUDA(block_mult(op->blk, op->stream, d, op->npad, nullptr, op->num_sms));
  prof_end(op, e0);
  const long e1 = prof_begin(op, KIND_BLOCK_MULTT);
  SGMEV_CUDA(block_multt(op->blk, op->stream, nullptr, op->npad, q, d, lm, op->num_sms));
  prof_end(op, e1);
  op->launches += 4;
  return SGMEV_OK;
}

struct DevBuf {  // stream-ordered scratch of one call
  cudaStream_t s;
  void* p = nullptr;
  explicit DevBuf(cudaStream_t st) : s(st) {}
  ~DevBuf() { sgmev::dev_free(p, s); }
};

static int block_products_common(sgmev_op* op, bool transpose, const double* in, double* out) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  if ((!in || !out) && (op->n > 0 && op->m > 0)) return fail(SGMEV_ERR_INVALID, "NULL vector");
  SGMEV_TRY(block_ready(op));
  const int64_t np = op->npad, mp = op->mpad, K = kBlockRhs;
  const int64_t n_in = transpose ? op->m : op->n, pad_in = transpose ? mp : np;
  const int64_t n_out = transpose ? op->n : op->m, pad_out = transpose ? np : mp;
  DevBuf buf(op->stream);
  SGMEV_CUDA(dev_malloc(&buf.p, sizeof(double) * K * (pad_in + pad_out), op->stream));
  double* d_in = static_cast<double*>(buf.p);
  double* d_out = d_in + K * pad_in;
  SGMEV_TRY(begin_timed(op));
  SGMEV_CUDA(cudaMemsetAsync(d_in, 0, sizeof(double) * K * pad_in, op->stream));
  if (n_in > 0)
    SGMEV_CUDA(cudaMemcpy2DAsync(d_in, sizeof(double) * pad_in, in, sizeof(double) * n_in,
                                 sizeof(double) * n_in, K, cudaMemcpyHostToDevice, op->stream));
  if (transpose) {
    const long ev = prof_begin(op, KIND_BLOCK_MULTT);
    SGMEV_CUDA(block_multt(op->blk, op->stream, d_in, np, d_out, nullptr, 0.0, op->num_sms));
    prof_end(op, ev);
  } else {
    const long ev = prof_begin(op, KIND_BLOCK_MULT);
    SGMEV_CUDA(block_mult(op->blk, op->stream, d_in, np, d_out, op->num_sms));
    prof_end(op, ev);
  }
  op->launches += 3;
  if (n_out > 0)
    SGMEV_CUDA(cudaMemcpy2DAsync(out, sizeof(double) * n_out, d_out, sizeof(double) * pad_out,
                                 sizeof(double) * n_out, K, cudaMemcpyDeviceToHost, op->stream));
  SGMEV_TRY(end_timed(op, true));
  return block_check(op);
}

SGMEV_API int sgmev_mult_block(sgmev_op* op, const double* alpha, double* result) {
  return block_products_common(op, false, alpha, result);
}

SGMEV_API int sgmev_mult_transpose_block(sgmev_op* op, const double* source, double* result) {
  return block_products_common(op, true, source, result);
}

static int fit_block_common(sgmev_op* op, const double* y, bool y_dev, double lambda,
                            int64_t max_iterations, double epsilon, double* alpha, bool a_dev,
                            int64_t* iterations, double* residuals) {
  using namespace sgmev;
  SGMEV_TRY(check_op(op));
  if ((op->m > 0 && !y) || (op->n > 0 && !alpha)) return fail(SGMEV_ERR_INVALID, "NULL vector");
  if (!(epsilon > 0.0) || max_iterations < 0) return fail(SGMEV_ERR_INVALID, "bad epsilon/max_iterations");
  SGMEV_TRY(block_ready(op));
  const int K = kBlockRhs;
  const int64_t np = op->npad;
  const double lm = static_cast<double>(op->m) * lambda;
  // b, x, outer residual rr, inner solution e, inner residual r, direction d, product q, temp t
  DevBuf buf(op->stream);
  const size_t vec = static_cast<size_t>(K) * np;
  const size_t parts = static_cast<size_t>(K) * kBlockDotBlocks;
  SGMEV_CUDA(dev_malloc(&buf.p, sizeof(double) * (8 * vec + 2 * parts + kBlockScalars), op->stream));
  double* b = static_cast<double*>(buf.p);
  double* x = b + vec;
  double* rr = x + vec;
  double* e = rr + vec;
  double* r = e + vec;
  double* d = r + vec;
  double* q = d + vec;
  double* t = q + vec;
  double* part_a = t + vec;
  double* part_b = part_a + parts;
  double* sc = part_b + parts;
  SGMEV_CUDA(cudaMemsetAsync(sc, 0, sizeof(double) * kBlockScalars, op->stream));
  SGMEV_TRY(begin_timed(op));
  // b_k = B^T y_k with the FP64-accurate df64 products (generateb per column)
  for (int k = 0; k < K; ++k) {
    if (op->m > 0)
      SGMEV_CUDA(cudaMemcpyAsync(op->out64, y + static_cast<int64_t>(k) * op->m,
                                 sizeof(double) * op->m,
                                 y_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                 op->stream));
    SGMEV_TRY(dev_convert(op, op->out64, op->m, op->mpad, op->v64, op->v32, op->v32lo));
    SGMEV_TRY(dev_multt(op, SGMEV_DF64, op->v64, op->v32, op->v32lo, b + k * np, 0, np, nullptr,
                        0.0));
  }
  SGMEV_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * vec, op->stream));
  std::vector<double> host(3 * K + parts), rho(K, 0.0), rho0(K, 0.0), tol2(K, 0.0);
  std::vector<int64_t> col_it(K, 0);
  std::vector<char> done(K, 0);
  auto block_norms = [&](const double* v, std::vector<double>& out) -> int {
    SGMEV_CUDA(block_dot(op->stream, v, v, np, part_a));
    SGMEV_CUDA(cudaMemcpyAsync(host.data(), part_a, sizeof(double) * parts, cudaMemcpyDeviceToHost,
                               op->stream));
    SGMEV_CUDA(cudaStreamSynchronize(op->stream));
    for (int k = 0; k < K; ++k) {
      double acc = 0.0;
      for (int bl = 0; bl < kBlockDotBlocks; ++bl) acc += host[k * kBlockDotBlocks + bl];
      out[k] = acc;
    }
    op->launches += 1;
    return SGMEV_OK;
  };
  int64_t total_it = 0;
  for (int outer = 0; outer < 64; ++outer) {
    if (outer == 0) {
      SGMEV_CUDA(cudaMemcpyAsync(rr, b, sizeof(double) * vec, cudaMemcpyDeviceToDevice, op->stream));
    } else {
      for (int k = 0; k < K; ++k) {
        if (done[k]) continue;  // x_k did not move: its residual stands
        SGMEV_TRY(dev_system(op, SGMEV_DF64, x + k * np, t, lm));
        sub_kernel<<<vec_blocks(np), 256, 0, op->stream>>>(np, b + k * np, t, rr + k * np);
        op->launches += 1;
      }
    }
    SGMEV_TRY(block_norms(rr, rho));
    if (outer == 0) rho0 = rho;
    bool all_done = true;
    for (int k = 0; k < K; ++k) {
      done[k] = done[k] || rho[k] <= epsilon * epsilon * rho0[k] || rho[k] == 0.0;
      all_done = all_done && done[k];
      const double inner_tol =
          op->block_inner_tol > 0.0 ? op->block_inner_tol : (op->block_f16 ? 1e-4 : 1e-3);
      const double want = std::min(0.5, std::max(inner_tol,
                                                 epsilon * std::sqrt(rho0[k] / std::max(rho[k], 1e-300)) * 0.5));
      tol2[k] = done[k] ? HUGE_VAL : want * want;
    }
    if (all_done || total_it >= max_iterations) break;
    // inner block CG on A e = rr with the BF16 tensor-core products, e = 0 at the start
    SGMEV_CUDA(cudaMemcpyAsync(sc + kScTol2, tol2.data(), sizeof(double) * K, cudaMemcpyHostToDevice,
                               op->stream));
    SGMEV_CUDA(cudaMemcpyAsync(r, rr, sizeof(double) * vec, cudaMemcpyDeviceToDevice, op->stream));
    SGMEV_CUDA(block_cg_init(op->stream, r, d, e, np, part_a, sc));
    op->launches += 2;
    int cur = 0;
    int64_t steps = 0;
    while (total_it < max_iterations) {
      SGMEV_CUDA(cudaMemcpyAsync(host.data(), sc + kScDelta + cur * K, sizeof(double) * K,
                                 cudaMemcpyDeviceToHost, op->stream));
      SGMEV_CUDA(cudaMemcpyAsync(host.data() + K, sc + kScDelta0, sizeof(double) * K,
                                 cudaMemcpyDeviceToHost, op->stream));
      SGMEV_CUDA(cudaMemcpyAsync(host.data() + 2 * K, sc + kScStalled, sizeof(double) * K,
                                 cudaMemcpyDeviceToHost, op->stream));
      SGMEV_CUDA(cudaStreamSynchronize(op->stream));
      int active = 0;
      bool stalled = false;
      for (int k = 0; k < K; ++k) {
        if (host[2 * K + k] != 0.0 && tol2[k] != HUGE_VAL) {
          tol2[k] = HUGE_VAL;  // d.q = 0: the column cannot move (the reference stops there too)
          stalled = true;
        }
        if (host[k] > tol2[k] * host[K + k]) {
          ++active;
          ++col_it[k];
        }
      }
      if (stalled)
        SGMEV_CUDA(cudaMemcpyAsync(sc + kScTol2, tol2.data(), sizeof(double) * K,
                                   cudaMemcpyHostToDevice, op->stream));
      if (active == 0) break;
      SGMEV_TRY(block_system(op, d, q, lm));
      SGMEV_CUDA(block_cg_step(op->stream, e, r, d, q, np, part_a, part_b, sc, cur));
      op->launches += 3;
      cur ^= 1;
      ++total_it;
      ++steps;
    }
    axpy_kernel<<<vec_blocks(static_cast<int64_t>(vec)), 256, 0, op->stream>>>(
        static_cast<int64_t>(vec), 1.0, e, x);
    op->launches += 1;
    SGMEV_TRY(block_check(op));
    if (steps == 0) break;  // no column could take a step: further refinement cannot move
  }
  for (int k = 0; k < K; ++k)
    if (op->n > 0)
      SGMEV_CUDA(cudaMemcpyAsync(alpha + static_cast<int64_t>(k) * op->n, x + k * np,
                                 sizeof(double) * op->n,
                                 a_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                 op->stream));
  SGMEV_TRY(end_timed(op, true));
  SGMEV_TRY(block_check(op));
  for (int k = 0; k < K; ++k) {
    if (iterations) iterations[k] = col_it[k];
    if (residuals) residuals[k] = rho[k];
  }
  return SGMEV_OK;
}

SGMEV_API int sgmev_fit_block(sgmev_op* op, const double* y, double lambda,
                              int64_t max_iterations, double epsilon, double* alpha,
                              int64_t* iterations, double* residuals) {
  return fit_block_common(op, y, false, lambda, max_iterations, epsilon, alpha, false, iterations,
                          residuals);
}

SGMEV_API int sgmev_fit_block_device(sgmev_op* op, const double* d_y, double lambda,
                                     int64_t max_iterations, double epsilon, double* d_alpha,
                                     int64_t* iterations, double* residuals) {
  return fit_block_common(op, d_y, true, lambda, max_iterations, epsilon, d_alpha, true,
                          iterations, residuals);
}

}  // extern "C"

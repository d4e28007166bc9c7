// Subspace-skipping evaluation of the hat basis (FP32): one basis function per subspace and
// data point instead of every grid point (internal interface of libsgpp_gb300).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace sgmev {

// Allow `kern` the device's largest dynamic shared memory, after checking that `need` fits. Every
// caller sets the same value, so operators running in several host threads cannot undo one
// another's setting between the call and their launch (the attribute belongs to the kernel, not
// to the launch).
template <typename Kernel>
inline cudaError_t set_smem_cap(Kernel kern, size_t need) {
  int dev = 0, cap = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  if (need > static_cast<size_t>(cap)) return cudaErrorInvalidValue;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
}

// A grid regrouped by subspace (level vector). Positions: each subspace owns the contiguous range
// [offset, offset + prod_t 2^{l_t - 1}) in subspace order; a grid point's position is
// offset + sum_t ((i_t - 1) / 2) * stride_t. Positions without a grid point (adaptive grids)
// carry alpha = 0 and are ignored on output.
struct SubPlan {
  int dim = 0;
  int n_sub = 0;
  int64_t total = 0;      // positions
  int64_t n = 0;          // grid points
  int4* desc = nullptr;   // [n_sub * dim] (bits(2^{l-1}), bits(2^l), stride, 0)
  uint32_t* base = nullptr;  // [n_sub] offset - sum_t bits(1.5*2^23) * stride_t (mod 2^32)
  int* pos = nullptr;     // [n] grid point -> position
  float* asub = nullptr;  // [total] alpha in subspace order
  float2* asub2 = nullptr;  // [total] alpha as float-float pairs (df64 mult)
  unsigned long long* acc = nullptr;  // [total] fixed-point accumulators / FP64 sums (multT)
  unsigned int* maxbits = nullptr;    // max |v| as float bits
  int4* sinfo = nullptr;  // [n_sub] (offset, cells, offset-free base, 0)
  int4* act = nullptr;    // [n_sub * dim] active dimensions (t, bits(S), bits(L), stride), padded
  int4* sact = nullptr;   // [n_sub] (base over active dimensions, cells, its offset-free part, count)
  int na_max = 0;         // most active dimensions of a subspace

  int64_t act_work = 0;   // active dimensions summed over subspaces
  int cmax = 0;           // largest cell count of a subspace
  double* rows = nullptr;  // [row_cap * total] per-CTA partial sums (owner-computes multT)
  int64_t row_cap = 0;
  // materialised products as float-float pairs P_hi[j / 4][s][j % 4], P_lo[...] (s padded to
  // s_pad, a multiple of 32) and the cell index of each within its subspace, C[j / 4][s] (four
  // bytes, point j % 4 in byte j % 4), for the data of mat_mpad padded points; nullptr when not
  // built
  float4* pmat = nullptr;
  float4* pmat_lo = nullptr;
  // the same products rounded to FP16 by pairs of point groups: P16[j / 8][s] holds the eight
  // halves of points 8 (j / 8) .. 8 (j / 8) + 7, so the FP16 kernels load two groups at once
  uint4* pmat16 = nullptr;
  void* cmat = nullptr;  // cell words: uint32_t (a byte per point) or uint16_t (a nibble)
  // the cell words by pairs of point groups, C2[j / 8][s] (two uint16_t words in a uint32_t, or
  // two uint32_t in a uint2), for the FP16 kernels
  void* cpair = nullptr;
  int cell_bits = 8;     // 8 or 4 bits per cell in cmat
  int64_t s_pad = 0;
  int64_t mat_mpad = 0;
  cudaStream_t stream = nullptr;  // device memory of the plan is allocated and freed on it
  // host copies: (offset, cells) per subspace and the position of every grid point
  std::vector<int2> h_sub;
  std::vector<int> h_pos;
  bool mod = false;  // modified linear basis (ModLinear): only the materialised products support it
  // points per read-modify-write round of the FP16 multTranspose's cell sums (1, 2 or 4; the
  // same bits for each)
  int multt_batch = 1;
  // banks of cell sums per owner in the FP16 multTranspose (1, or 2: two independent
  // read-modify-write chains; other bits than one bank)
  int multt_banks = 1;
  // CTAs per SM of the FP16 multTranspose: 2, or 3 (one bank of FP32 cell sums, no flush sums,
  // fewer loads in flight per thread; other last bits)
  int multt_ctas = 2;
};

// The FP16 copy of the materialised products holds 2^p16_exp(p) x the products, so that they
// stay out of FP16's subnormal range (a product of many hats is small: in 10 dimensions typically
// about 2^-14, where FP16 keeps only a few bits); the FP16 kernels multiply their sums by
// 2^-p16_exp. Products are at most 1 (hats), or 2^(active dimensions) for the modified basis
// inside the cube; scaled, the largest stays at or below 2^13.
inline int p16_exp(const SubPlan& p) { return 13 - (p.mod ? (p.na_max < 15 ? p.na_max : 15) : 0); }

// position count up to which alpha is staged in shared memory (and the fixed-point scatter, two
// 4-byte accumulators per position, can run); larger grids read alpha from global memory
constexpr int64_t kSubMaxPositions = 24 * 1024;
// largest position count of a plan (32-bit indices, per-CTA rows of FP64 sums)
constexpr int64_t kSubMaxTotal = int64_t(1) << 27;

// Build the plan from the eval arrays (host, [n x dim] 2^l and i). Returns false (and leaves
// the plan empty) when the grid has more than kSubMaxTotal positions, a subspace that the
// owner-computes multTranspose cannot hold (beyond kSubMaxPositions), or dim is not templated.
bool subspace_build(SubPlan* p, int dim, int64_t n, const double* level_pow2,
                    const double* index, cudaStream_t stream, std::string* err);
void subspace_free(SubPlan* p);

// out[j] (FP32 and/or FP64, zero beyond m) = sum_g alpha_g phi_g(x_j) for j in [j_begin, j_end)
// (tile-aligned to 512); alpha32 [n] FP32.
cudaError_t subspace_mult(const SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad,
                          int64_t m, const float* alpha32, float* out32, double* out64,
                          int64_t j_begin, int64_t j_end, int num_sms);

// FP64-accurate (float-float) mult: out64[j] for j in [j_begin, j_end) (tile-aligned to 512),
// x as (xh, xl) dim-major pairs, alpha as (ah, al) [n]
cudaError_t subspace_mult_df(const SubPlan& p, cudaStream_t s, const float* xh, const float* xl,
                             int64_t mpad, int64_t m, const float* ah, const float* al,
                             double* out64, int64_t j_begin, int64_t j_end, int num_sms);

// true when the owner-computes multTranspose holds its per-cell sums in shared memory (FP32 or
// float-float); otherwise subspace_multt falls back to the fixed-point scatter and
// subspace_multt_df must not be called
bool subspace_owner_fits(const SubPlan& p, bool df);

// out64[g] (g < n; zero in [n, npad)) = sum_j v_j phi_g(x_j) (+ scale_add * add[g]); v32 [mpad]
cudaError_t subspace_multt(const SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad,
                           int64_t m, const float* v32, int64_t npad, double* out64,
                           const double* add, double scale_add, int num_sms);

// internal steps shared by the subspace sources: alpha (FP32, [n]) into asub in position order,
// and out64 = gather of the sum of `nrows` partial rows (+ scale_add * add)
cudaError_t subspace_scatter_alpha(const SubPlan& p, cudaStream_t s, const float* alpha32);
cudaError_t subspace_finish_rows(const SubPlan& p, cudaStream_t s, int64_t nrows, int64_t npad,
                                 double* out64, const double* add, double scale_add);
cudaError_t subspace_scatter_alpha_df(const SubPlan& p, cudaStream_t s, const float* ah,
                                      const float* al);
// fills pmat, pmat_lo, pmat16 and cmat (allocated, s_pad set) from the float-float data (xh, xl);
// cpair is derived from cmat afterwards
cudaError_t subspace_mat_build(const SubPlan& p, cudaStream_t s, const float* xh,
                               const float* xl, int64_t mpad, int64_t m, int num_sms);

// Materialised products: bytes they take for mpad points, whether the FP32 (df = false) or
// float-float (df = true) kernels' shared memory fits the plan, building them from the
// float-float data (allocates; the data must not change afterwards), and the products that
// stream them (same contracts as subspace_mult / subspace_multt / subspace_mult_df /
// subspace_multt_df).
int64_t subspace_mat_bytes(const SubPlan& p, int64_t mpad);
// free the materialised products of the plan (stream-ordered on s)
void subspace_mat_release(SubPlan* p, cudaStream_t s);
// whether the materialised kernels take the grid (FP32 / FP16 ones, or with df the float-float
// ones); the FP32 / FP16 mult takes its subspaces in windows where all coefficients do not fit
// shared memory at once
bool subspace_mat_fits(const SubPlan& p, bool df);
cudaError_t subspace_materialize(SubPlan* p, cudaStream_t s, const float* xh, const float* xl,
                                 int64_t mpad, int64_t m, int num_sms);
// fused FP32 system product out64 = B^T (B alpha) (+ scale_add * add), one pass over the
// materialised products (grids of at most 1024 subspaces)
bool subspace_system_mat_fits(const SubPlan& p);
cudaError_t subspace_system_mat(const SubPlan& p, cudaStream_t s, int64_t mpad,
                                const float* alpha32, int64_t npad, double* out64,
                                const double* add, double scale_add, int num_sms);
cudaError_t subspace_mult_mat_df(const SubPlan& p, cudaStream_t s, int64_t mpad, int64_t m,
                                 const float* ah, const float* al, double* out64, int64_t j_begin,
                                 int64_t j_end, int num_sms);
cudaError_t subspace_multt_mat_df(const SubPlan& p, cudaStream_t s, int64_t mpad,
                                  const float* vh, const float* vl, int64_t npad, double* out64,
                                  const double* add, double scale_add, int num_sms);
// half: stream the FP16 copy of the products (3 bytes per entry instead of 5; products good to
// 2^-11, for the inner solves of mixed fits)
cudaError_t subspace_mult_mat(const SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad,
                              int64_t m, const float* alpha32, float* out32, double* out64,
                              int64_t j_begin, int64_t j_end, int num_sms, bool half = false);
cudaError_t subspace_multt_mat(const SubPlan& p, cudaStream_t s, const float* xt, int64_t mpad,
                               int64_t m, const float* v32, int64_t npad, double* out64,
                               const double* add, double scale_add, int num_sms,
                               bool half = false);

// FP64-accurate (float-float) multTranspose: x as (xh, xl), v as (vh, vl) [mpad]
cudaError_t subspace_multt_df(const SubPlan& p, cudaStream_t s, const float* xh, const float* xl,
                              int64_t mpad, int64_t m, const float* vh, const float* vl,
                              int64_t npad, double* out64, const double* add, double scale_add,
                              int num_sms);

}  // namespace sgmev

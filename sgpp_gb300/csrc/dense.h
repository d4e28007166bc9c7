// Dense (every grid point per data point) launch shapes shared by sgmev.cu and dense_mod.cu
// (internal to libsgpp_gb300).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.cuh"

namespace sgmev {

constexpr int kBlock = 128;
constexpr int kGT = 32;  // grid points per shared-memory tile (mult)
constexpr int kDT = 64;  // data points per shared-memory tile (multT)
constexpr int kMaxTemplDim = 16;

// Register blocking per precision and dimension (data points per thread for mult, grid points
// per thread for multT).
template <typename T>
struct Blocking;
template <>
struct Blocking<float> {
  static constexpr int mult_r(int dim) { return dim <= 12 ? 8 : 4; }
  static constexpr int multt_r(int) { return 4; }
};
template <>
struct Blocking<double> {
  static constexpr int mult_r(int) { return 4; }
  static constexpr int multt_r(int) { return 2; }
};

// df64 tile kernels (float-float), R = 4 data points / RG = 2 grid points per thread
constexpr int kDfMultR = 4;
constexpr int kDfMulttRG = 2;

#define SGMEV_DIM_CASES(F) \
  F(1) F(2) F(3) F(4) F(5) F(6) F(7) F(8) F(9) F(10) F(11) F(12) F(13) F(14) F(15) F(16)

// Launches of the ModLinear (modified linear basis) dense kernels, instantiated in dense_mod.cu
// so that they compile beside the Linear ones. dim <= kMaxTemplDim: the tiled kernels, `offset`
// = first tile; larger dim: the generic kernels, `offset` = first index and `count` indices.
// gscale holds the per-grid-point factors 2^b (kernels.cuh).
template <typename T>
void mod_mult_launch(int dim, dim3 grid, cudaStream_t s, const T* xt, int64_t mpad,
                     const typename Pair<T>::type* li, const T* alpha, const T* gscale,
                     int64_t npad, int64_t chunk, int64_t offset, int64_t count, T* part);
template <typename T, bool SQ>
void mod_multt_launch(int dim, dim3 grid, cudaStream_t s, const T* xt, const T* v, int64_t mpad,
                      const typename Pair<T>::type* li, const T* gscale, int64_t npad,
                      int64_t chunk, int64_t offset, int64_t count, T* part);
void mod_mult_df_launch(int dim, dim3 grid, cudaStream_t s, const float* xh, const float* xl,
                        int64_t mpad, const float4* gq, const float* ah, const float* al,
                        const float* gscale, int64_t npad, int64_t chunk, int64_t offset,
                        int64_t count, float2* part);
void mod_multt_df_launch(int dim, dim3 grid, cudaStream_t s, const float* xh, const float* xl,
                         const float* vh, const float* vl, int64_t mpad, const float4* gq,
                         const float* gscale, int64_t npad, int64_t chunk, int64_t offset,
                         int64_t count, float2* part);

}  // namespace sgmev

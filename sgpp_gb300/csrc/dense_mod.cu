// ModLinear instantiations of the dense kernels (kernels.cuh with MOD = true), in a translation
// unit of their own so that they compile in parallel with the Linear ones in sgmev.cu.
#include "dense.h"

namespace sgmev {

template <typename T>
void mod_mult_launch(int dim, dim3 grid, cudaStream_t s, const T* xt, int64_t mpad,
                     const typename Pair<T>::type* li, const T* alpha, const T* gscale,
                     int64_t npad, int64_t chunk, int64_t offset, int64_t count, T* part) {
  switch (dim) {
#define F(D)                                                                                   \
  case D:                                                                                      \
    mult_kernel<T, D, Blocking<T>::mult_r(D), kBlock, kGT, true>                               \
        <<<grid, kBlock, 0, s>>>(xt, mpad, li, alpha, npad, chunk, offset, part, gscale);      \
    break;
    SGMEV_DIM_CASES(F)
#undef F
    default:
      mult_generic_kernel<T, true><<<grid, kBlock, 0, s>>>(xt, mpad, dim, li, alpha, npad, chunk,
                                                           offset, count, part, gscale);
      break;
  }
}

template <typename T, bool SQ>
void mod_multt_launch(int dim, dim3 grid, cudaStream_t s, const T* xt, const T* v, int64_t mpad,
                      const typename Pair<T>::type* li, const T* gscale, int64_t npad,
                      int64_t chunk, int64_t offset, int64_t count, T* part) {
  switch (dim) {
#define F(D)                                                                                  \
  case D:                                                                                     \
    mult_transpose_kernel<T, D, Blocking<T>::multt_r(D), kBlock, kDT, SQ, true>               \
        <<<grid, kBlock, 0, s>>>(xt, v, mpad, li, npad, chunk, offset, part, gscale);         \
    break;
    SGMEV_DIM_CASES(F)
#undef F
    default:
      mult_transpose_generic_kernel<T, SQ, true><<<grid, kBlock, 0, s>>>(
          xt, v, mpad, dim, li, npad, chunk, offset, count, part, gscale);
      break;
  }
}

void mod_mult_df_launch(int dim, dim3 grid, cudaStream_t s, const float* xh, const float* xl,
                        int64_t mpad, const float4* gq, const float* ah, const float* al,
                        const float* gscale, int64_t npad, int64_t chunk, int64_t offset,
                        int64_t count, float2* part) {
  switch (dim) {
#define F(D)                                                                                 \
  case D:                                                                                    \
    mult_df_kernel<D, kDfMultR, kBlock, kGT, true><<<grid, kBlock, 0, s>>>(                  \
        xh, xl, mpad, gq, ah, al, npad, chunk, offset, part, gscale);                        \
    break;
    SGMEV_DIM_CASES(F)
#undef F
    default:
      mult_df_generic_kernel<true><<<grid, kBlock, 0, s>>>(xh, xl, mpad, dim, gq, ah, al, npad,
                                                           chunk, offset, count, part, gscale);
      break;
  }
}

void mod_multt_df_launch(int dim, dim3 grid, cudaStream_t s, const float* xh, const float* xl,
                         const float* vh, const float* vl, int64_t mpad, const float4* gq,
                         const float* gscale, int64_t npad, int64_t chunk, int64_t offset,
                         int64_t count, float2* part) {
  switch (dim) {
#define F(D)                                                                                 \
  case D:                                                                                    \
    mult_transpose_df_kernel<D, kDfMulttRG, kBlock, kDT, true><<<grid, kBlock, 0, s>>>(      \
        xh, xl, vh, vl, mpad, gq, npad, chunk, offset, part, gscale);                        \
    break;
    SGMEV_DIM_CASES(F)
#undef F
    default:
      mult_transpose_df_generic_kernel<true><<<grid, kBlock, 0, s>>>(
          xh, xl, vh, vl, mpad, dim, gq, npad, chunk, offset, count, part, gscale);
      break;
  }
}

template void mod_mult_launch<float>(int, dim3, cudaStream_t, const float*, int64_t,
                                     const float2*, const float*, const float*, int64_t, int64_t,
                                     int64_t, int64_t, float*);
template void mod_mult_launch<double>(int, dim3, cudaStream_t, const double*, int64_t,
                                      const double2*, const double*, const double*, int64_t,
                                      int64_t, int64_t, int64_t, double*);
template void mod_multt_launch<float, false>(int, dim3, cudaStream_t, const float*, const float*,
                                             int64_t, const float2*, const float*, int64_t,
                                             int64_t, int64_t, int64_t, float*);
template void mod_multt_launch<float, true>(int, dim3, cudaStream_t, const float*, const float*,
                                            int64_t, const float2*, const float*, int64_t,
                                            int64_t, int64_t, int64_t, float*);
template void mod_multt_launch<double, false>(int, dim3, cudaStream_t, const double*,
                                              const double*, int64_t, const double2*,
                                              const double*, int64_t, int64_t, int64_t, int64_t,
                                              double*);

}  // namespace sgmev

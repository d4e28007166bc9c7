/*
 * sgmev_tools.h — measurement helpers of libsgpp_gb300.so (no counterpart in the reference;
 * used by the benchmark to obtain the roofline denominators on the GPU it runs on).
 */
#ifndef SGMEV_TOOLS_H_
#define SGMEV_TOOLS_H_

#include <stdint.h>

#include "sgmev.h"

#ifdef __cplusplus
extern "C" {
#endif

/*
 * Measured vector FMA throughput of the current device: a kernel of independent fused
 * multiply-add chains on every SM, timed with CUDA events. precision: SGMEV_FP64 or SGMEV_FP32.
 * *flops_per_second counts one FMA as two floating-point operations; *sm_clock_khz is the
 * clock the device reported (cudaDevAttrClockRate).
 */
SGMEV_API int sgmev_fma_peak(int precision, double* flops_per_second, int* sm_clock_khz);

#ifdef __cplusplus
}
#endif

#endif /* SGMEV_TOOLS_H_ */

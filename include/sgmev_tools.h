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

/*
 * Per-kernel timing of an op's tile kernels. sgmev_profile(op, 1) resets the counters and
 * records a CUDA event pair around every following mult / multTranspose tile-kernel launch on
 * the op's stream; sgmev_profile_read() synchronises the stream and returns, for one kernel
 * kind, the number of launches and their summed device time since the reset.
 */
#define SGMEV_KERNEL_MULT_FP32 0
#define SGMEV_KERNEL_MULTT_FP32 1
#define SGMEV_KERNEL_MULT_FP64 2
#define SGMEV_KERNEL_MULTT_FP64 3
#define SGMEV_KERNEL_MULT_DF64 4
#define SGMEV_KERNEL_MULTT_DF64 5
#define SGMEV_KERNEL_MULT_SUB32 6  /* FP32 subspace-skipping mult */
#define SGMEV_KERNEL_MULTT_SUB32 7 /* FP32 subspace-skipping multTranspose */
#define SGMEV_KERNEL_MULT_SUBDF 8  /* df64 subspace-skipping mult */
#define SGMEV_KERNEL_MULTT_SUBDF 9 /* df64 subspace-skipping multTranspose */
#define SGMEV_KERNEL_MULT_MAT32 10 /* FP32 mult streaming the materialised subspace products */
#define SGMEV_KERNEL_MULTT_MAT32 11 /* FP32 multTranspose streaming them */
#define SGMEV_KERNEL_MULT_MATDF 12 /* df64 mult streaming them */
#define SGMEV_KERNEL_MULTT_MATDF 13 /* df64 multTranspose streaming them */
#define SGMEV_KERNEL_SYSTEM_MAT32 14 /* FP32 B^T (B a) in one pass over them */
#define SGMEV_KERNEL_MULT_MAT16 15 /* mult streaming their FP16 copy (inner solves of mixed fits) */
#define SGMEV_KERNEL_MULTT_MAT16 16 /* multTranspose streaming it */
#define SGMEV_KERNEL_BLOCK_MULT 17  /* B [a_1 .. a_16], BF16 tensor-core tiles */
#define SGMEV_KERNEL_BLOCK_MULTT 18 /* B^T [v_1 .. v_16], BF16 tensor-core tiles */
SGMEV_API int sgmev_profile(sgmev_op* op, int enable);
SGMEV_API int sgmev_profile_read(sgmev_op* op, int kind, int64_t* launches, double* seconds);

#ifdef __cplusplus
}
#endif

#endif /* SGMEV_TOOLS_H_ */

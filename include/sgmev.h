/*
 * sgmev.h — C ABI of the GB300 (sm_103a) multi-evaluation library libsgpp_gb300.so.
 *
 * The library computes SG++'s OperationMultipleEval products for the piecewise-linear hat
 * basis on Linear (no-boundary) sparse grids, on the GPU:
 *
 *   mult           result_j = sum_i alpha_i  prod_t max(1 - |2^{l_it} x_jt - i_it|, 0)
 *   multTranspose  result_i = sum_j source_j prod_t max(1 - |2^{l_it} x_jt - i_it|, 0)
 *
 * and the same products for the modified linear basis of ModLinear grids (params "basis"):
 * a level-1 factor is 1, i = 1 gives max(2 - 2^l x, 0), i = 2^l - 1 gives max(2^l x - i + 1, 0)
 * (base/.../basis/LinearModifiedBasis.hpp:40-58, streamed as
 * datadriven/.../OperationMultiEvalModMaskStreaming).
 *
 * All entry points take plain host pointers (or, for the *_device variants, device pointers)
 * and sizes; none uses C++ or torch types. Every function returns SGMEV_OK (0) or a negative
 * status; sgmev_last_error() then returns a message for the calling thread. No entry point
 * calls exit() or aborts.
 *
 * Threading: one op handle per host thread at a time (like the reference operators, which are
 * driven by single-threaded callers). Each handle owns a CUDA stream unless one is set with
 * sgmev_set_stream().
 *
 * Layouts are the reference's own, so a maintainer passes SG++ buffers unchanged:
 *   level_pow2, index : [n_grid x dim] row-major doubles, 2^l and i
 *                       (HashGridStorage::getLevelIndexArraysForEval,
 *                        base/src/sgpp/base/grid/storage/hashmap/HashGridStorage.cpp:433-450)
 *   data              : [n_data x dim] row-major doubles (base::DataMatrix, DataMatrix.hpp:28)
 *   vectors           : contiguous doubles (base::DataVector)
 */
#ifndef SGMEV_H_
#define SGMEV_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define SGMEV_API __attribute__((visibility("default")))
#else
#define SGMEV_API
#endif

/* ---- status codes -------------------------------------------------------------------- */
#define SGMEV_OK 0
#define SGMEV_ERR_INVALID (-1)     /* bad argument (null pointer, size, layout) */
#define SGMEV_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define SGMEV_ERR_NO_DEVICE (-3)   /* no CUDA device visible */
#define SGMEV_ERR_UNSUPPORTED (-4) /* combination not supported (e.g. non-hat grid type) */
#define SGMEV_ERR_NOT_CONVERGED (-5)
#define SGMEV_ERR_OOM (-6)         /* device allocation failed */

/* ---- precision of the evaluation kernels ---------------------------------------------- */
#define SGMEV_FP64 0 /* native double: the plain FP64 path (parity 1e-12 vs the reference) */
#define SGMEV_FP32 1 /* single-precision hat products and tile sums; FP64 cross-tile sums */
#define SGMEV_DF64 2 /* FP64-accurate float-float ("df64") arithmetic on the FP32 pipes: every
                        1-D hat exact, products and sums with ~2^-47 relative rounding; parity
                        1e-12 like SGMEV_FP64, at a fraction of native FP64's cost on GB300 */

typedef struct sgmev_op sgmev_op;

/* Message of the last failing call on this thread ("" if none). Never NULL. */
SGMEV_API const char* sgmev_last_error(void);

/* Library/ABI version, e.g. 10000 for 1.0.0. */
SGMEV_API int sgmev_version(void);

/* Number of visible CUDA devices (0 if none); never fails. */
SGMEV_API int sgmev_device_count(void);

/*
 * Create an operator for one grid and one data set; replaces
 *   sgpp::op_factory::createOperationMultipleEval(Grid&, DataMatrix&, OperationMultipleEvalConfiguration&)
 *   datadriven/src/sgpp/datadriven/DatadrivenOpFactory.cpp:409-552 (new branches: Linear and
 *   ModLinear grids, STREAMING type, CUDA subtype) and the operator constructors
 *   datadriven/.../OperationMultiEvalStreaming/OperationMultiEvalStreaming.cpp:13-25 and
 *   datadriven/.../OperationMultiEvalModMaskStreaming/OperationMultiEvalModMaskStreaming.cpp:19-29.
 * The data are copied to the device once (dim-major, padded), as the reference operator copies
 * and transposes its dataset; the caller's buffers may be freed afterwards.
 * bb_left/bb_right: optional bounding box ([dim] each, both NULL for the unit cube); data are
 * mapped by (x - left) / (right - left) as BoundingBox::transformPointToUnitCube
 * (base/src/sgpp/base/grid/common/BoundingBox.hpp:223-227).
 * precision: SGMEV_FP64, SGMEV_FP32 or SGMEV_DF64. params_json: optional flat JSON object of
 * string knobs (may be NULL): "precond": "none" (default) or "jacobi" — the preconditioner of the
 * inner correction solves of SGMEV_SOLVE_MIXED* fits (SGMEV_SOLVE_PLAIN is never preconditioned).
 * Jacobi (diag(B^T B) + lambda*M) doubled the iteration count on clustered (Gaussian-mixture) data,
 * where fine-level hats see few points, so it is off unless asked for.
 * "inner_tol": relative tolerance of the inner correction solves of mixed fits (default "1e-4").
 * "algo": "auto" (default), "dense" or "subspace" — how the FP32 products are evaluated: dense
 * (every grid point for every data point, the STREAMING algorithm) or subspace-skipping (one basis
 * function per subspace and data point, as the reference's DEFAULT operator; grids of dim <= 16
 * with at most 24,576 subspace positions); "auto" takes subspace when it needs fewer instructions.
 * "materialize": "auto" (default), "on" or "off" — whether the subspace FP32 products keep
 * p_s(x_j) for every data point and subspace in device memory (built on the first
 * FP32 product) and streams it, instead of evaluating the hats on every call; "auto" does so when
 * it takes at most half of the free device memory and 64 GiB. The products are kept as
 * float-float pairs with their cell index (8 bytes and a byte, or a nibble when no subspace has
 * more than 16 cells; grids whose subspaces have at most 256 cells), so the df64 (FP64-accurate)
 * products stream them too, beside an FP16 copy with its own copy of the cell indices for the
 * inner solves of mixed fits (11 to 12 bytes per point and subspace in all). "materialize_multt": "on"
 * (default) or "off" — whether multTranspose streams them as well as mult. "system_product":
 * "separate" (default) or "fused" — FP32 system products B^T (B a) on the materialised products
 * as the mult and multTranspose kernels or in one fused pass. "inner_products":
 * "half" (default) or "float" — the inner FP32 solves of mixed fits stream an FP16 copy of the
 * products (2.5-3 bytes per entry instead of 4.5-5; the FP64-accurate outer residual keeps the result
 * exact to the fit's tolerance).
 * "multt_batch": "1" (default), "2" or "4" — points per read-modify-write round of the owner's
 * cell sums in the FP16 multTranspose (the same bits for each; a launch-shape choice of the
 * autotuner, sgpp_gb300.autotune). "multt_banks": "1" (default) or "2" — banks of cell sums per
 * owner in the FP16 multTranspose (two independent read-modify-write chains; other last bits
 * than one bank; an autotuner choice). "multt_ctas": "2" (default) or "3" — CTAs per SM of the
 * FP16 multTranspose (three: FP32 cell sums only, fewer loads in flight per thread; other last
 * bits; an autotuner choice).
 * "basis": "linear" (default) or "modlinear" — the basis of the grid. level_pow2/index stay the
 * (2^l, i) arrays of getLevelIndexArraysForEval for both (a ModLinear grid has the same points).
 * ModLinear functions next to a face extrapolate linearly beyond it, as the reference's mask
 * evaluation does; the materialised products are used for ModLinear only when every data
 * coordinate lies in [0, 1] (otherwise the dense kernels run), and the FP16 inner products only
 * for subspaces of at most 15 active dimensions (products reach 2^15).
 */
SGMEV_API int sgmev_create(sgmev_op** out, int dim, int64_t n_grid, const double* level_pow2,
                           const double* index, int64_t n_data, const double* data,
                           const double* bb_left, const double* bb_right, int precision,
                           const char* params_json);

/* Destroy the operator and free its device memory. NULL is accepted. */
SGMEV_API int sgmev_destroy(sgmev_op* op);

/*
 * Re-stage the grid after it changed (refinement appends points); replaces
 *   OperationMultipleEval::prepare()  base/src/sgpp/base/operation/hash/OperationMultipleEval.hpp:118
 *   (STREAMING: recalculateLevelAndIndex, OperationMultiEvalStreaming.cpp:145-156,181).
 */
SGMEV_API int sgmev_prepare(sgmev_op* op, int64_t n_grid, const double* level_pow2,
                            const double* index);

/* Sizes of the staged problem. */
SGMEV_API int sgmev_get_sizes(const sgmev_op* op, int* dim, int64_t* n_grid, int64_t* n_data);

/*
 * result[n_data] = B alpha[n_grid]; replaces OperationMultipleEval::mult(alpha, result)
 *   OperationMultipleEval.hpp:55. Host buffers; blocks until the result is in `result`.
 */
SGMEV_API int sgmev_mult(sgmev_op* op, const double* alpha, double* result);

/*
 * result[n_grid] = B^T source[n_data]; replaces OperationMultipleEval::multTranspose
 *   OperationMultipleEval.hpp:81. Host buffers; blocks until done.
 */
SGMEV_API int sgmev_mult_transpose(sgmev_op* op, const double* source, double* result);

/*
 * Ranged variants; replace OperationMultipleEval.hpp:70-73 (data range of mult) and :97-100
 * (grid range of multTranspose). result is the full-length vector; only
 * result[start..end) is written.
 */
SGMEV_API int sgmev_mult_range(sgmev_op* op, const double* alpha, double* result,
                               int64_t start_data, int64_t end_data);
SGMEV_API int sgmev_mult_transpose_range(sgmev_op* op, const double* source, double* result,
                                         int64_t start_grid, int64_t end_grid);

/*
 * Device-resident variants: the same products on device pointers (doubles), enqueued on the
 * op's stream; they return without synchronising. For callers that keep vectors on the GPU.
 */
SGMEV_API int sgmev_mult_device(sgmev_op* op, const double* d_alpha, double* d_result);
SGMEV_API int sgmev_mult_transpose_device(sgmev_op* op, const double* d_source,
                                          double* d_result);

/*
 * result[n_grid] = B^T source[n_data] (FP64) for callers that cannot allocate GPU memory.
 * No counterpart in the reference. Everything is a device pointer the caller owns, in the
 * reference's layouts (level_pow2/index [n_grid x dim], data [n_data x dim] row-major, already in
 * the unit cube); work is enqueued on `stream` (NULL = the legacy default stream) and the call
 * returns without synchronising. It allocates nothing: the split partial sums live in a fixed
 * 16 MiB array inside the library (2^21 doubles), so n_grid is limited to 2,097,152
 * (SGMEV_ERR_INVALID beyond that) and dim to 64. The first call on each device looks up that
 * array's device address; make that first call before any stream capture. Calls share the array:
 * calls whose work overlaps on the GPU race and must be serialised by the caller.
 */
SGMEV_API int sgmev_mult_transpose_noalloc(int dim, int64_t n_grid, const double* d_level_pow2,
                                           const double* d_index, int64_t n_data,
                                           const double* d_data, const double* d_source,
                                           double* d_result, void* stream);

/*
 * System matrix of the least-squares regression, applied on the device:
 *   result = B^T (B alpha) + lambda_times_m * alpha
 * replaces SystemMatrixLeastSquaresIdentity::mult
 *   datadriven/src/sgpp/datadriven/algorithm/SystemMatrixLeastSquaresIdentity.cpp:32-47
 * (the reference passes lambda * number_of_instances). Host buffers; blocks.
 */
SGMEV_API int sgmev_system_apply(sgmev_op* op, const double* alpha, double* result,
                                 double lambda_times_m);
SGMEV_API int sgmev_system_apply_device(sgmev_op* op, const double* d_alpha, double* d_result,
                                        double lambda_times_m);

/*
 * Regression fit on the device: b = B^T y, then conjugate gradients on
 * (B^T B + lambda*M*I) alpha = b, all vectors resident on the GPU; replaces
 *   SystemMatrixLeastSquaresIdentity::generateb (SystemMatrixLeastSquaresIdentity.cpp:49-56) +
 *   solver::ConjugateGradients::solve (solver/src/sgpp/solver/sle/ConjugateGradients.cpp:22-151):
 *   same relative stopping test delta_new <= epsilon^2 * delta_0, same true-residual refresh
 *   every 50 iterations, same warm start (reuse != 0 keeps alpha as the start vector).
 * mode:
 *   SGMEV_SOLVE_PLAIN  — CG with the op's own precision kernels (FP64 op: the plain FP64 path).
 *   SGMEV_SOLVE_MIXED  — iterative refinement: the outer residual b - A alpha (and b) with the
 *                        FP64-accurate df64 kernels, the inner correction solves by CG with
 *                        FP32 kernels and FP64 vectors (Jacobi-preconditioned with
 *                        diag(B^T B) + lambda*M if params say "precond": "jacobi"); stops when
 *                        ||b - A alpha||^2 <= epsilon^2 * ||b - A alpha_0||^2 (true residual).
 *   SGMEV_SOLVE_MIXED_NATIVE64 — the same with native FP64 kernels for the residual.
 * Every op stages the FP64, FP32 and df64 copies of its data, so any mode works on any op.
 * y: [n_data] host; alpha: [n_grid] host in/out. iterations: total inner CG iterations;
 * residual: final delta_new (plain) or ||b - A alpha||^2 in FP64 (mixed).
 */
#define SGMEV_SOLVE_PLAIN 0
#define SGMEV_SOLVE_MIXED 1
#define SGMEV_SOLVE_MIXED_NATIVE64 2
SGMEV_API int sgmev_fit(sgmev_op* op, int mode, const double* y, double lambda,
                        int64_t max_iterations, double epsilon, int reuse, double* alpha,
                        int64_t* iterations, double* residual);

/* sgmev_fit with y [n_data] and alpha [n_grid] as device pointers (doubles). Blocks. */
SGMEV_API int sgmev_fit_device(sgmev_op* op, int mode, const double* d_y, double lambda,
                               int64_t max_iterations, double epsilon, int reuse, double* d_alpha,
                               int64_t* iterations, double* residual);

/*
 * Duration in seconds of the device work of the last mult / multTranspose / system apply /
 * fit call (CUDA events on the op's stream); replaces OperationMultipleEval::getDuration
 *   OperationMultipleEval.hpp:120. -1 before the first call.
 */
SGMEV_API double sgmev_get_duration(sgmev_op* op);

/* Use `stream` (a cudaStream_t) for all following work of this op; NULL restores the op's own.
 * The new stream is made to wait (an event) for the work the op enqueued on the previous one, so
 * sgmev_synchronize and sgmev_destroy (which frees on the current stream) cover the op's work on
 * every stream it used. */
SGMEV_API int sgmev_set_stream(sgmev_op* op, void* stream);

/* Change launch-shape knobs of a live operator: params_json may hold only "multt_batch",
 * "multt_banks", "multt_ctas" and the "block_mult_tiles", "block_mult_groups", "block_multt_groups",
 * "block_stages", "block_loads", "block_window", "block_teams", "block_mult_a" knobs (see
 * sgmev_create); they change no result bits except the order of the FP16 multTranspose's
 * additions (multt_banks, multt_ctas) and how the block products are cut into launches.
 * No counterpart in the reference (whose OpenCL kernels take such parameters from a
 * configuration file written by StaticParameterTuner,
 * datadriven/src/sgpp/datadriven/application/StaticParameterTuner.cpp:297-417); used by the
 * autotuner (sgpp_gb300.autotune). Waits for the op's stream first. */
SGMEV_API int sgmev_set_params(sgmev_op* op, const char* params_json);

/* Block until all work enqueued by this op has finished. */
SGMEV_API int sgmev_synchronize(sgmev_op* op);

/* Number of kernels this op launched so far (instrumentation for benchmarks). */
SGMEV_API int64_t sgmev_kernel_launches(const sgmev_op* op);

/* ---- 16 right-hand sides: BF16 tensor-core products and fits ---------------------------- */
/*
 * The same operator applied to 16 vectors at once, on the 5th-generation tensor cores: per tile of
 * 128 data points and group of 128 grid positions, the products of the materialised subspace
 * products (rounded to FP16, 2^-11 relative) with the 16 vectors (split into FP16 high and low
 * parts, about 2^-22; every operand scaled by a power of two into FP16's range) are tcgen05 MMAs
 * accumulating in FP32; with params "block_products": "bf16" the products are rounded to BF16
 * (2^-8) and the vectors split into BF16 parts (about 2^-16). No counterpart in the reference,
 * which applies OperationMultipleEval::mult / multTranspose (OperationMultipleEval.hpp:55, :81)
 * to one vector at a time; column k here equals those products of vector k to FP16 (or BF16)
 * accuracy.
 * Needs the subspace algorithm with materialised products (params "algo": "subspace", the default
 * where it pays) and subspaces of at most 128 cells; otherwise SGMEV_ERR_UNSUPPORTED.
 * Vectors are column-major: vector k of length n at offset k * n. Host buffers; blocks.
 * params "block_products": "f16" (default) or "bf16"; "block_inner_tol" (default "1e-4" with
 * FP16 products, "1e-3" with BF16 ones): inner tolerance of sgmev_fit_block; "block_mult_tiles",
 * "block_mult_groups", "block_multt_groups", "block_stages" (default 4), "block_loads" (default
 * 6): launch shape; "block_window" (1-3, default 2): stages whose MMAs one issue round interleaves;
 * "block_teams" (1-4, default 3, at most block_stages and dividing block_loads): producer teams
 * of 4 warps that write alternate stages; and
 * "block_mult_a": "tmem" (default) or "smem", where the mult keeps its A operand (the autotuner's
 * choices, sgpp_gb300.autotune).
 */
#define SGMEV_BLOCK_RHS 16
SGMEV_API int sgmev_mult_block(sgmev_op* op, const double* alpha, double* result);
SGMEV_API int sgmev_mult_transpose_block(sgmev_op* op, const double* source, double* result);

/*
 * 16 regression fits sharing one operator (one grid, one data set, 16 target vectors y_k):
 * per column the system of SystemMatrixLeastSquaresIdentity::mult / generateb
 * (datadriven/src/sgpp/datadriven/algorithm/SystemMatrixLeastSquaresIdentity.cpp:32-56) solved
 * as ConjugateGradients::solve would (solver/src/sgpp/solver/sle/ConjugateGradients.cpp:22-151),
 * by mixed-precision iterative refinement: b_k = B^T y_k and the outer residuals b_k - A alpha_k
 * with the FP64-accurate df64 products, the inner correction solves as one block CG over the 16
 * columns on the BF16 tensor-core products (each column its own CG scalars); a column stops when
 * ||b_k - A alpha_k||^2 <= epsilon^2 ||b_k||^2. y: [16 x n_data] column-major; alpha: [16 x n_grid]
 * out (cold start); iterations[16]: inner CG steps of each column; residuals[16]: the final
 * ||b_k - A alpha_k||^2 (either may be NULL).
 */
SGMEV_API int sgmev_fit_block(sgmev_op* op, const double* y, double lambda,
                              int64_t max_iterations, double epsilon, double* alpha,
                              int64_t* iterations, double* residuals);
/* sgmev_fit_block with y and alpha as device pointers (column-major doubles). Blocks. */
SGMEV_API int sgmev_fit_block_device(sgmev_op* op, const double* d_y, double lambda,
                                     int64_t max_iterations, double epsilon, double* d_alpha,
                                     int64_t* iterations, double* residuals);

/* ---- batched fits: many independent problems, continuous batching ----------------------- */
/*
 * A batch engine fits many independent regression problems of uneven dimension, grid size and
 * data size at once: every problem runs the mixed-precision fit of sgmev_fit (SGMEV_SOLVE_MIXED:
 * FP32 CG inside, df64 residual outside) as a state machine on the device, and one step advances
 * every unfinished problem by one inner CG iteration or one outer residual, with one launch per
 * phase for all problems (persistent CTAs pulling per-problem tiles from a device work list) and
 * the step's launches captured into one CUDA graph. Problems can be added while others run
 * (continuous batching); each result is the same alone and in any mix. Each problem carries
 * `rhs` right-hand sides (1 or 16) that share its operator B.
 * Replaces, per problem, SystemMatrixLeastSquaresIdentity::generateb + ConjugateGradients::solve
 * (datadriven/.../SystemMatrixLeastSquaresIdentity.cpp:49-56, solver/.../ConjugateGradients.cpp:22-151)
 * run for many problems; the reference has no batched counterpart.
 *   grid_capacity: total grid rows x dim over all resident problems (padded to 512 rows each);
 *   data_capacity: total data points x dim (padded to 1024 points each).
 */
typedef struct sgmev_batch sgmev_batch;
SGMEV_API int sgmev_batch_create(sgmev_batch** out, int max_slots, int rhs, int64_t grid_capacity,
                                 int64_t data_capacity, const char* params_json);
SGMEV_API int sgmev_batch_destroy(sgmev_batch* b);
/* Pool elements one problem occupies (admission by device-memory footprint). */
SGMEV_API int sgmev_batch_footprint(int dim, int64_t n_grid, int64_t n_data, int rhs,
                                    int64_t* grid_elems, int64_t* data_elems);
/* Stage one problem (host buffers: eval arrays [n_grid x dim], data [n_data x dim],
 * y [n_data x rhs] row-major) and compute b = B^T y; returns its slot. SGMEV_ERR_OOM when no slot
 * or pool space is free (the caller retries after sgmev_batch_remove). */
SGMEV_API int sgmev_batch_add(sgmev_batch* b, int dim, int64_t n_grid, const double* level_pow2,
                              const double* index, int64_t n_data, const double* data,
                              const double* y, double lambda, double epsilon,
                              int64_t max_iterations, int* slot_out);
SGMEV_API int sgmev_batch_remove(sgmev_batch* b, int slot);
/* Advance all unfinished problems by `steps` steps; phases[max_slots] receives each slot's phase
 * (0 empty, 1 outer residual pending, 2 inner CG, 3 done). */
SGMEV_API int sgmev_batch_step(sgmev_batch* b, int steps, int* phases);
/* Step until no problem is running (or max_steps); *steps_taken = steps run. */
SGMEV_API int sgmev_batch_solve(sgmev_batch* b, int64_t max_steps, int64_t* steps_taken);
/* alpha [n_grid x rhs] row-major; iterations = inner CG iterations; residual = worst column's
 * ||b - A alpha||^2 / ||b||^2 at the last outer step; phase as above. */
SGMEV_API int sgmev_batch_result(sgmev_batch* b, int slot, double* alpha, int64_t* iterations,
                                 double* residual, int* phase);
SGMEV_API int sgmev_batch_info(sgmev_batch* b, int64_t* steps, int64_t* launches,
                               int* free_slots);

/* ---- sparse-grid construction on the host (native C++) --------------------------------- */
/* ---- least-squares fitting with spatial adaptivity -----------------------------------------
 * The reference's ModelFittingLeastSquares
 *   datadriven/src/sgpp/datadriven/datamining/modules/fitting/ModelFittingLeastSquares.cpp:51-140
 * (fit / adapt / update / evaluate) over one device-resident operator: the data stay on the GPU
 * from fit() on, adapt() refines the grid on the host (SurplusRefinementFunctor), re-stages it
 * and solves again from the zero-extended alpha, which never leaves the device except for the
 * refinement functor. Solves are CG with reuse, as assembleSystemAndSolve does.
 */
typedef struct sgfit sgfit;
typedef struct {
  int level;                      /* regular grid level (RegularGridConfiguration::level_) */
  int basis;                      /* 0 Linear, 1 ModLinear (RegularGridConfiguration::type_) */
  double lambda;                  /* RegularizationConfiguration::lambda_ */
  double final_eps;               /* solverFinalConfig eps_ / maxIterations_ */
  int64_t final_max_iterations;
  double refine_eps;              /* solverRefineConfig eps_ / maxIterations_ */
  int64_t refine_max_iterations;
  int64_t num_refinements;        /* AdaptivityConfiguration::numRefinements_ */
  int64_t num_refinement_points;  /* numRefinementPoints_ */
  double refinement_threshold;    /* refinementThreshold_ */
  int mode;                       /* SGMEV_SOLVE_PLAIN (the reference's CG) or a mixed mode */
  int precision;                  /* operator precision: SGMEV_FP64, SGMEV_FP32, SGMEV_DF64 */
} sgfit_config;

/* The reference's defaults (FitterConfiguration::setupDefaults): level 3, Linear, lambda 0.01,
 * eps 1e-12 and 100 iterations for both solver configurations, one refinement of one point. */
SGMEV_API void sgfit_config_defaults(sgfit_config* config);
/* params_json: optional operator knobs as for sgmev_create ("basis" is set from the config). */
SGMEV_API int sgfit_create(sgfit** out, const sgfit_config* config, const char* params_json);
SGMEV_API int sgfit_destroy(sgfit* fitter);
/* ModelFittingLeastSquares::fit: regular grid on `dim` dimensions, alpha = 0, solve.
 * x: [m x dim] row-major, y: [m]. */
SGMEV_API int sgfit_fit(sgfit* fitter, int64_t m, int dim, const double* x, const double* y);
/* ModelFittingLeastSquares::adapt: *refined = 1 when the grid grew and was solved again. */
SGMEV_API int sgfit_adapt(sgfit* fitter, int* refined);
/* ModelFittingLeastSquares::update: the current grid and alpha on new data (fit() if none). */
SGMEV_API int sgfit_update(sgfit* fitter, int64_t m, int dim, const double* x, const double* y);
/* ModelFittingLeastSquares::evaluate(samples, results): out[m] = B(x) alpha. */
SGMEV_API int sgfit_evaluate(sgfit* fitter, int64_t m, const double* x, double* out);
/* The grid (level/index [n x dim] raw int32, NULL to get the sizes) and alpha [n]. */
SGMEV_API int sgfit_grid(const sgfit* fitter, int* dim, int64_t* n_grid, int32_t* level,
                         int32_t* index);
SGMEV_API int sgfit_alpha(const sgfit* fitter, double* alpha);
/* CG iterations and residual of the last solve, refinement rounds done. */
SGMEV_API int sgfit_stats(const sgfit* fitter, int64_t* iterations, double* residual,
                          int64_t* refinements);

/* ---- dataset ingest (host) ----------------------------------------------------------------
 * ARFF and CSV text read exactly as the reference's readers read it
 *   datadriven/src/sgpp/datadriven/tools/ARFFTools.cpp  readARFFSize / readARFF (:60-170)
 *   datadriven/src/sgpp/datadriven/tools/CSVTools.cpp   readCSVSize / readCSV
 * (the rules are listed in sgpp_gb300/csrc/datasets.cpp). The text is passed as bytes; the
 * library opens no files. The rows go to sgmev_create as they are (with the grid's bounding box,
 * if any, applied there on the device).
 */
#define SGDATA_ARFF 0
#define SGDATA_CSV 1

/* Number of admissible instances and the dimension (columns, less the target column when
 * has_targets); replaces ARFFTools::readARFFSize / CSVTools::readCSVSize. skip_first_line: CSV
 * only (a header line). targets/n_targets: optional target filter (0.001 tolerance). */
SGMEV_API int sgdata_size(int format, const char* text, int64_t len, int has_targets,
                          int skip_first_line, const double* targets, int n_targets,
                          int64_t* n_instances, int64_t* dim);

/* Read the rows: data [n_read x dim_out] row-major, y [n_read] (when has_targets); replaces
 * ARFFTools::readARFF / CSVTools::readCSV. cutoff < 0: no instance cutoff. cols/n_cols: optional
 * column selection (order kept). n_cap: rows the caller's buffers hold (sgdata_size's count). */
SGMEV_API int sgdata_read(int format, const char* text, int64_t len, int has_targets,
                          int skip_first_line, int64_t cutoff, const int64_t* cols, int n_cols,
                          const double* targets, int n_targets, double* data, double* y,
                          int64_t n_cap, int64_t* n_read, int64_t* dim_out);

/*
 * Regular Linear sparse grid without boundary in the reference's storage order; replaces
 *   Grid::createLinearGrid(d)->getGenerator().regular(level)
 *   base/src/sgpp/base/grid/Grid.cpp:73, HashGenerator.hpp:282-347.
 * Call with level/index NULL to get the size in *n_grid; then with arrays of [n_grid x dim]
 * int32 raw levels and indices.
 */
SGMEV_API int sggrid_regular(int dim, int level, int64_t* n_grid, int32_t* level_out,
                             int32_t* index_out);

/*
 * One round of surplus refinement (largest |alpha| first); replaces
 *   GridGenerator::refine(SurplusRefinementFunctor(alpha, n_points, threshold))
 *   base/.../StandardGridGenerator.cpp:64-68, HashRefinement.cpp:124-147,
 *   SurplusRefinementFunctor.cpp:23-28.
 * level/index: [cap x dim] int32, first n_grid rows filled on entry; on return *n_out rows.
 * New points are appended (existing rows keep their positions, as in the reference).
 * Points are refined by descending |alpha|, ties by position; the set of created points
 * equals the reference's (whose order follows its hash-map iteration).
 */
SGMEV_API int sggrid_refine_surplus(int dim, int64_t n_grid, int64_t cap, int32_t* level,
                                    int32_t* index, const double* alpha, int64_t n_points,
                                    double threshold, int64_t* n_out);

/* (2^l, i) as doubles in the reference's eval layout (HashGridStorage.cpp:433-450). */
SGMEV_API int sggrid_level_index_for_eval(int dim, int64_t n_grid, const int32_t* level,
                                          const int32_t* index, double* level_pow2,
                                          double* index_out);

#ifdef __cplusplus
}
#endif

#endif /* SGMEV_H_ */

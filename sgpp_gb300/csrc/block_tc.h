// Products with many right-hand sides on the tensor cores (internal interface of libsgpp_gb300).
//
// For K = 16 coefficient vectors (or data-side vectors) at once, B P and B^T Q become
// contractions: per tile of 128 points and per group of 128 "rows" (cells of subspaces), the
// weighted one-hot matrix E[point][row] = p_s(x) where row = the cell of subspace s that x lies in,
// 0 elsewhere, is formed in shared memory from the materialised products (FP16, or BF16) and
// contracted on the tensor cores (tcgen05.mma kind::f16, FP16 or BF16 operands, FP32 accumulators
// in tensor memory):
//   mult:  Q[tile][32] += E[tile][group] * C[group][32]    (C: the coefficient rows)
//   multT: R[group][32] += E[tile][group]^T * Q[tile][32]
// The 32 columns are the 16 right-hand sides split into high and low parts (x = hi + lo, about 22
// significant bits in FP16, 16 in BF16), so that only the products are rounded (2^-11 in FP16,
// 2^-8 in BF16); the two halves are added in FP32 when the accumulators are read.
//
// Rows: every subspace with C cells takes max(1, C / 8) chunks of 8 rows; subspaces are packed,
// largest first, into groups of 16 chunks (a subspace never spans two groups, so C <= 128); a
// row that is not a cell of a grid point carries coefficient 0 and is dropped on output.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "subspace.h"

namespace sgmev {

constexpr int kBlockRhs = 16;      // right-hand sides per block product
constexpr int kBlockCols = 32;     // MMA columns: high and low parts
constexpr int kBlockTile = 128;    // points per tile (MMA M for mult, K extent for multT)
constexpr int kBlockGroupRows = 128;  // rows per group (MMA M for multT)
constexpr int kBlockMaxCells = 128;   // largest subspace the block products take

// Per group and chunk q (16 chunks of 8 rows): the byte offset of the chunk's slot row in a
// stage's load buffer (slot index within the group x 512), and 128 x which of the slot's chunks q
// is (or a large base for a chunk no slot uses). 128 bytes, copied with the stage's products.
struct BlockHeader {
  int32_t row[16];
  int32_t base[16];
};

// Tunable launch shapes (picked per operator by the autotuner, sgmev_tune_block)
struct BlockShape {
  int mult_tiles = 8;      // tiles per mult CTA (their accumulators stay in tensor memory)
  int mult_groups = 32;    // groups whose coefficient rows a mult CTA holds (fewer when shared
                           // memory runs out)
  int multt_groups = 16;   // groups (accumulators) per multT CTA
  int stages = 4;          // stages of E in flight (shared or tensor memory)
  int loads = 6;           // stages of packed products in flight (bulk copies ahead of use)
  int mult_tmem = 1;       // mult keeps its A operand (the stages of E) in tensor memory
  int window = 2;          // stages whose MMAs one issue round interleaves (at most `stages`)
  int teams = 3;           // producer teams of 4 warps, each writing every teams-th stage
                           // (at most `stages` and `loads`)
};

struct BlockPlan {
  int n_groups = 0;
  int n_slots = 0;            // subspaces, in group order
  int64_t rows = 0;           // n_groups * 128
  int64_t n = 0;              // grid points
  int64_t mpad = 0;           // padded points (a multiple of 128)
  int64_t m = 0;
  int* row_gp = nullptr;      // [rows] grid point of a row, -1 when none
  int* gp_row = nullptr;      // [n] row of a grid point
  BlockHeader* gheader = nullptr;  // [n_groups] chunk headers
  int2* gslots = nullptr;     // [n_groups] first slot and slot count of each group
  uint32_t* pc = nullptr;     // [mpad / 128][n_slots][128] FP16 / BF16 product | 16 cell << 16,
                              // tile by tile
  uint16_t* coef = nullptr;   // [n_groups][4096] coefficient rows, FP16 / BF16, operand layout
  uint16_t* qtiles = nullptr; // [mpad / 128][4096] Q tiles, FP16 / BF16, operand layout
  double* part = nullptr;     // [streams][16][rows] partial rows of multT
  int part_streams = 0;
  int* status = nullptr;      // device error word (a wait that ran out)
  // FP16 operands instead of BF16 (the products keep 11 significant bits instead of 8). FP16's
  // range is narrow, so every operand is scaled by a power of two (exact, undone on output): the
  // products by 2^pexp (the largest into [2^13, 2^14), so that products down to 2^-27 of it stay
  // out of FP16's subnormals), the coefficient rows and the Q tiles per column (scales[c] and
  // scales[16 + c]): the largest coefficient of a column maps into [2^13, 2^14), and a Q tile
  // written by block_mult takes the coefficient scale times 2^-qshift, which bounds the
  // accumulators (n_slots x the largest scaled product x 2^14) by 2^14.
  bool f16 = false;
  int pexp = 0;
  int qshift = 0;
  float* scales = nullptr;    // [32]
  unsigned* colmax = nullptr; // [16] largest |value| per column (float bits), reset after use
  BlockShape shape;
  cudaStream_t stream = nullptr;
};

// Build the plan and the packed products from a materialised subspace plan (its pmat and cmat);
// false with a message when the grid has a subspace above kBlockMaxCells cells or allocation fails.
// f16: FP16 products and operands (else BF16).
bool block_build(BlockPlan* b, const SubPlan& sub, int64_t m, int64_t mpad, bool f16,
                 cudaStream_t s, int num_sms, std::string* err);
void block_free(BlockPlan* b);

// Q = B P for 16 columns: P column-major FP64 [16][npad] (grid order). Writes the Q tiles
// (input of block_multt) and, when out64 is given, Q column-major FP64 [16][mpad].
cudaError_t block_mult(BlockPlan& b, cudaStream_t s, const double* p, int64_t npad,
                       double* out64, int num_sms);
// R = B^T Q (+ scale_add * add) for the Q tiles of the last block_mult, or of `v` when given
// (column-major FP64 [16][mpad], staged into tiles first): out64 column-major [16][npad].
cudaError_t block_multt(BlockPlan& b, cudaStream_t s, const double* v, int64_t npad,
                        double* out64, const double* add, double scale_add, int num_sms);
// 0 when every wait of the block kernels completed; otherwise the kernels gave up (an error)
cudaError_t block_status(BlockPlan& b, cudaStream_t s, int* host_status);
// whether a launch shape fits the device's shared memory (smem_cap bytes per block)
bool block_shape_ok(const BlockShape& sh, int smem_cap);

// CG on 16 columns (column-major [16][np] vectors; independent systems sharing the operator).
// Scalars on the device, at these offsets of `sc` (kBlockScalars doubles): delta in two slots
// (the iteration's and the next one's), delta_0 of the solve, the squared relative tolerance of
// each column, and a flag per column whose last step had d.q = 0. Dot products go through
// `part` arrays of kBlockRhs * kBlockDotBlocks doubles.
constexpr int kBlockDotBlocks = 64;
constexpr int kScDelta = 0, kScDelta0 = 32, kScTol2 = 48, kScStalled = 64, kBlockScalars = 80;
// part[k * kBlockDotBlocks + b]: per-block sums of a_k . b_k
cudaError_t block_dot(cudaStream_t s, const double* a, const double* b, int64_t np, double* part);
// d = r, e = 0, delta = delta_0 = r.r (slot 0)
cudaError_t block_cg_init(cudaStream_t s, const double* r, double* d, double* e, int64_t np,
                          double* part, double* sc);
// one CG step on every active column (delta > tol2 * delta_0), q = A d given; reads delta from
// slot `cur` and writes the new one to slot cur ^ 1
cudaError_t block_cg_step(cudaStream_t s, double* e, double* r, double* d, const double* q,
                          int64_t np, double* part_dq, double* part_rr, double* sc, int cur);

}  // namespace sgmev

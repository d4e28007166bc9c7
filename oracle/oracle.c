/*
 * ORACLE — test infrastructure only.
 *
 * A plain-C, FP64 restatement of SG++'s multi-evaluation path for the piecewise-linear hat
 * basis on Linear (no-boundary) sparse grids, and for the modified linear basis on ModLinear
 * grids (the same grid points; boundary-adjacent functions extrapolate to the cube faces). Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py may load this library, and only as the reference results of the
 * tests (or the timed CPU baseline). The shipped CUDA path never calls into it.
 *
 * Parity pin: tests/test_oracle_golden.py checks every function here against fixtures that
 * tests/golden/make_golden.py produced from the reference's own compiled code (oracle/ref.mk
 * + oracle/ref_harness.cpp), and against the reference's known-answer test
 * base/tests/test_OperationMultipleEval.cpp:24-79.
 *
 * Conventions (the reference's eval layout, HashGridStorage.cpp:433-450):
 *   level_pow2[n*d + t] = 2^l_{n,t},  index[n*d + t] = i_{n,t}   (row-major [N x d] doubles)
 *   data[m*d + t]                                                  (row-major [M x d] doubles)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_API __attribute__((visibility("default")))

/* ------------------------------------------------------------------------------------------
 * 1-D hat, LinearBasis::eval  (base/src/sgpp/base/operation/hash/common/basis/LinearBasis.hpp:37-41)
 *   phi_{l,i}(x) = max(1 - |2^l x - i|, 0)
 * ------------------------------------------------------------------------------------------ */
static inline double hat(double level_pow2, double index, double x) {
  double v = 1.0 - fabs(level_pow2 * x - index);
  return v > 0.0 ? v : 0.0;
}

/* ------------------------------------------------------------------------------------------
 * Regular sparse grid without boundary, in the reference's storage order.
 * HashGenerator::regular_iter (base/src/sgpp/base/grid/generation/hashmap/HashGenerator.hpp:282-347),
 * T = 0: first the 1-D grid in dimension 0 (levels 1..n, odd indices ascending); then for each
 * further dimension t, every existing point g (in sequence order) keeps (1,1) in dimension t in
 * place and appends copies with (l,i) for all admissible l >= 1 (l + sum of the other levels,
 * counting not-yet-expanded dimensions as level 1, <= n + d - 1), odd i ascending.
 * Returns N, or -1 if cap is too small. lev/idx: [N x d] int32 (raw level, index).
 * ------------------------------------------------------------------------------------------ */
ORC_API int64_t orc_regular_grid(int dim, int level, int64_t cap, int32_t* lev, int32_t* idx) {
  if (dim <= 0 || level <= 0) return 0;
  int64_t n = 0;
  for (int l = 1; l <= level; ++l) {
    for (int i = 1; i < (1 << l); i += 2) {
      if (n >= cap) return -1;
      for (int t = 0; t < dim; ++t) {
        lev[n * dim + t] = 1;
        idx[n * dim + t] = 1;
      }
      lev[n * dim + 0] = l;
      idx[n * dim + 0] = i;
      ++n;
    }
  }
  for (int t = 1; t < dim; ++t) {
    const int64_t size = n;
    for (int64_t g = 0; g < size; ++g) {
      /* level sum of g with dimensions >= t still at level 1, minus one (regular_iter:306) */
      int level_sum = -1;
      int level_max = 0;
      for (int s = 0; s < dim; ++s) {
        level_sum += lev[g * dim + s];
        if (lev[g * dim + s] > level_max) level_max = lev[g * dim + s];
      }
      int first = 1;
      for (int l = 1; l + level_sum <= level + dim - 1 && (l > level_max ? l : level_max) <= level;
           ++l) {
        for (int i = 1; i < (1 << l); i += 2) {
          if (first) {
            lev[g * dim + t] = l; /* (1,1): updates g in place */
            idx[g * dim + t] = i;
            first = 0;
          } else {
            if (n >= cap) return -1;
            memcpy(&lev[n * dim], &lev[g * dim], sizeof(int32_t) * dim);
            memcpy(&idx[n * dim], &idx[g * dim], sizeof(int32_t) * dim);
            lev[n * dim + t] = l;
            idx[n * dim + t] = i;
            ++n;
          }
        }
      }
      /* restore (1,1) in dimension t for g: the in-place update above wrote l=1,i=1 anyway */
      lev[g * dim + t] = 1;
      idx[g * dim + t] = 1;
    }
  }
  return n;
}

/* Number of points of a regular grid: sum over level vectors |l|_1 <= n + d - 1 of 2^{|l|_1 - d}. */
ORC_API int64_t orc_regular_grid_size(int dim, int level) {
  /* dynamic programme over dimensions: cnt[s] = number of points with level sum s */
  if (dim <= 0 || level <= 0) return 0;
  const int smax = level + dim - 1;
  double* cnt = (double*)calloc((size_t)smax + 1, sizeof(double));
  double* nxt = (double*)calloc((size_t)smax + 1, sizeof(double));
  cnt[0] = 1.0;
  for (int t = 0; t < dim; ++t) {
    memset(nxt, 0, sizeof(double) * ((size_t)smax + 1));
    for (int s = 0; s <= smax; ++s) {
      if (cnt[s] == 0.0) continue;
      for (int l = 1; s + l <= smax && l <= level; ++l) nxt[s + l] += cnt[s] * (double)(1 << (l - 1));
    }
    double* tmp = cnt;
    cnt = nxt;
    nxt = tmp;
  }
  double total = 0.0;
  for (int s = 0; s <= smax; ++s) total += cnt[s];
  free(cnt);
  free(nxt);
  return (int64_t)total;
}

/* ------------------------------------------------------------------------------------------
 * Surplus refinement, one round.
 * HashRefinement::free_refine (base/.../HashRefinement.cpp:124-147) with
 * SurplusRefinementFunctor (value |alpha_seq|, SurplusRefinementFunctor.cpp:23-28):
 *   - refinable = points missing at least one child (l+1, 2i-1) / (l+1, 2i+1) in some
 *     dimension (collectRefinablePoints, :42-91);
 *   - keep the `n_points` largest values (addElementToCollection, :19-38);
 *   - for each kept point with value >= threshold: for every dimension, create the missing left
 *     then right child (refineGridpoint1D, :191-212); a created point first gets its missing
 *     hierarchical parents in every dimension, recursively (AbstractRefinement.cpp:36-52,
 *     createGridpointSubroutine in AbstractRefinement.hpp:229-244), then is appended.
 * The reference walks the kept points in heap order over hash-map iteration order; here they
 * are walked by descending value, ties by sequence number. The resulting point SET is
 * identical; only the sequence numbers of newly appended points can differ.
 * Returns the new N (>= n), or -1 if cap is too small. lev/idx are [cap x d], first n filled.
 * ------------------------------------------------------------------------------------------ */
typedef struct {
  int dim;
  int64_t n, cap;
  int32_t* lev;
  int32_t* idx;
  int64_t* table; /* open addressing, -1 = empty; stores sequence numbers */
  int64_t tsize;
} orc_store;

static uint64_t point_hash(const int32_t* l, const int32_t* i, int dim) {
  uint64_t h = 1469598103934665603ULL;
  for (int t = 0; t < dim; ++t) {
    h ^= (uint64_t)(uint32_t)l[t] * 0x9E3779B97F4A7C15ULL;
    h *= 1099511628211ULL;
    h ^= (uint64_t)(uint32_t)i[t] + 0x632BE59BD9B4E019ULL;
    h *= 1099511628211ULL;
  }
  return h;
}

static int64_t store_find(const orc_store* s, const int32_t* l, const int32_t* i) {
  uint64_t h = point_hash(l, i, s->dim) & (uint64_t)(s->tsize - 1);
  for (;;) {
    int64_t q = s->table[h];
    if (q < 0) return -1;
    if (memcmp(&s->lev[q * s->dim], l, sizeof(int32_t) * s->dim) == 0 &&
        memcmp(&s->idx[q * s->dim], i, sizeof(int32_t) * s->dim) == 0)
      return q;
    h = (h + 1) & (uint64_t)(s->tsize - 1);
  }
}

static int store_insert(orc_store* s, const int32_t* l, const int32_t* i) {
  if (s->n >= s->cap) return -1;
  int64_t q = s->n++;
  memcpy(&s->lev[q * s->dim], l, sizeof(int32_t) * s->dim);
  memcpy(&s->idx[q * s->dim], i, sizeof(int32_t) * s->dim);
  uint64_t h = point_hash(l, i, s->dim) & (uint64_t)(s->tsize - 1);
  while (s->table[h] >= 0) h = (h + 1) & (uint64_t)(s->tsize - 1);
  s->table[h] = q;
  return 0;
}

/* createGridpoint: parents in every dimension first (recursively), then the point itself. */
static int store_create(orc_store* s, int32_t* l, int32_t* i) {
  for (int t = 0; t < s->dim; ++t) {
    if (l[t] > 1) {
      const int32_t sl = l[t], si = i[t];
      l[t] = sl - 1;
      i[t] = (((si + 1) / 2) % 2 == 1) ? (si + 1) / 2 : (si - 1) / 2;
      if (store_find(s, l, i) < 0) {
        if (store_create(s, l, i) != 0) return -1;
      }
      l[t] = sl;
      i[t] = si;
    }
  }
  return store_insert(s, l, i);
}

typedef struct {
  double value;
  int64_t seq;
} orc_cand;

static int cand_cmp(const void* a, const void* b) {
  const orc_cand* x = (const orc_cand*)a;
  const orc_cand* y = (const orc_cand*)b;
  if (x->value > y->value) return -1;
  if (x->value < y->value) return 1;
  return x->seq < y->seq ? -1 : (x->seq > y->seq ? 1 : 0);
}

ORC_API int64_t orc_refine_surplus(int dim, int64_t n, int64_t cap, int32_t* lev, int32_t* idx,
                                   const double* alpha, int64_t n_points, double threshold) {
  if (n <= 0) return -1;
  orc_store s;
  s.dim = dim;
  s.n = 0;
  s.cap = cap;
  s.lev = lev;
  s.idx = idx;
  s.tsize = 1;
  while (s.tsize < 2 * cap + 16) s.tsize <<= 1;
  s.table = (int64_t*)malloc(sizeof(int64_t) * (size_t)s.tsize);
  for (int64_t k = 0; k < s.tsize; ++k) s.table[k] = -1;
  /* index the existing points (they already sit in lev/idx; re-insert in place) */
  for (int64_t q = 0; q < n; ++q) {
    uint64_t h = point_hash(&lev[q * dim], &idx[q * dim], dim) & (uint64_t)(s.tsize - 1);
    while (s.table[h] >= 0) h = (h + 1) & (uint64_t)(s.tsize - 1);
    s.table[h] = q;
  }
  s.n = n;

  orc_cand* cands = (orc_cand*)malloc(sizeof(orc_cand) * (size_t)n);
  int64_t nc = 0;
  int32_t* cl = (int32_t*)malloc(sizeof(int32_t) * (size_t)dim);
  int32_t* ci = (int32_t*)malloc(sizeof(int32_t) * (size_t)dim);
  for (int64_t q = 0; q < n; ++q) {
    memcpy(cl, &lev[q * dim], sizeof(int32_t) * dim);
    memcpy(ci, &idx[q * dim], sizeof(int32_t) * dim);
    int refinable = 0;
    for (int t = 0; t < dim && !refinable; ++t) {
      const int32_t sl = cl[t], si = ci[t];
      cl[t] = sl + 1;
      ci[t] = 2 * si - 1;
      if (store_find(&s, cl, ci) < 0) refinable = 1;
      ci[t] = 2 * si + 1;
      if (!refinable && store_find(&s, cl, ci) < 0) refinable = 1;
      cl[t] = sl;
      ci[t] = si;
    }
    if (refinable) {
      cands[nc].value = fabs(alpha[q]);
      cands[nc].seq = q;
      ++nc;
    }
  }
  qsort(cands, (size_t)nc, sizeof(orc_cand), cand_cmp);
  if (nc > n_points) nc = n_points;

  int rc = 0;
  for (int64_t k = 0; k < nc && rc == 0; ++k) {
    if (!(cands[k].value >= threshold)) continue;
    const int64_t q = cands[k].seq;
    int32_t* pl = (int32_t*)malloc(sizeof(int32_t) * (size_t)dim);
    int32_t* pi = (int32_t*)malloc(sizeof(int32_t) * (size_t)dim);
    memcpy(pl, &lev[q * dim], sizeof(int32_t) * dim);
    memcpy(pi, &idx[q * dim], sizeof(int32_t) * dim);
    for (int t = 0; t < dim && rc == 0; ++t) {
      const int32_t sl = pl[t], si = pi[t];
      pl[t] = sl + 1;
      pi[t] = 2 * si - 1;
      if (store_find(&s, pl, pi) < 0) rc = store_create(&s, pl, pi);
      pl[t] = sl + 1;
      pi[t] = 2 * si + 1;
      if (rc == 0 && store_find(&s, pl, pi) < 0) rc = store_create(&s, pl, pi);
      pl[t] = sl;
      pi[t] = si;
    }
    free(pl);
    free(pi);
  }
  free(cl);
  free(ci);
  free(cands);
  free(s.table);
  return rc == 0 ? s.n : -1;
}

/* level/index as the reference's eval arrays (HashGridStorage.cpp:433-450). */
ORC_API void orc_level_index_for_eval(int dim, int64_t n, const int32_t* lev, const int32_t* idx,
                                      double* level_pow2, double* index) {
  for (int64_t k = 0; k < n * dim; ++k) {
    level_pow2[k] = (double)(1u << lev[k]);
    index[k] = (double)idx[k];
  }
}

/* Bounding-box transform to the unit cube, BoundingBox.hpp:223-252: (x - left) / (right - left).
 * Points outside the box evaluate to zero on a no-boundary Linear grid either way, because every
 * hat's support lies inside (0, 1). */
ORC_API void orc_bb_to_unit(int dim, int64_t m, const double* left, const double* right,
                            const double* data, double* out) {
  for (int64_t j = 0; j < m; ++j)
    for (int t = 0; t < dim; ++t)
      out[j * dim + t] = (data[j * dim + t] - left[t]) / (right[t] - left[t]);
}

/* ------------------------------------------------------------------------------------------
 * NAIVE mult / multTranspose: OperationMultipleEvalLinearNaive.cpp:12-41 / :43-73.
 * result_j = sum_i alpha_i prod_t phi(x_jt); result_i = sum_j v_j prod_t phi(x_jt).
 * Summation order is the reference's (grid points ascending for mult, data ascending for multT).
 * ------------------------------------------------------------------------------------------ */
ORC_API void orc_mult_naive(int dim, int64_t n, const double* level_pow2, const double* index,
                            int64_t m, const double* data, const double* alpha, double* result) {
  for (int64_t j = 0; j < m; ++j) {
    double acc = 0.0;
    for (int64_t i = 0; i < n; ++i) {
      double v = 1.0;
      for (int t = 0; t < dim; ++t) {
        const double h = hat(level_pow2[i * dim + t], index[i * dim + t], data[j * dim + t]);
        if (h == 0.0) {
          v = 0.0;
          break;
        }
        v *= h;
      }
      acc += alpha[i] * v;
    }
    result[j] = acc;
  }
}

ORC_API void orc_mult_transpose_naive(int dim, int64_t n, const double* level_pow2,
                                      const double* index, int64_t m, const double* data,
                                      const double* source, double* result) {
  for (int64_t i = 0; i < n; ++i) {
    double acc = 0.0;
    for (int64_t j = 0; j < m; ++j) {
      double v = 1.0;
      for (int t = 0; t < dim; ++t) {
        const double h = hat(level_pow2[i * dim + t], index[i * dim + t], data[j * dim + t]);
        if (h == 0.0) {
          v = 0.0;
          break;
        }
        v *= h;
      }
      acc += source[j] * v;
    }
    result[i] = acc;
  }
}

/* ------------------------------------------------------------------------------------------
 * Modified linear basis, LinearModifiedBasis::eval
 * (base/src/sgpp/base/operation/hash/common/basis/LinearModifiedBasis.hpp:40-58), raw (l, i):
 *   l == 1        -> 1
 *   i == 1        -> 2 - 2^l x   for x <= 2 / 2^l, else 0
 *   i == 2^l - 1  -> 2^l x - i + 1   for x >= 1 - 2 / 2^l, else 0
 *   otherwise     -> max(1 - |2^l x - i|, 0)
 * NAIVE-shaped products over it (every grid point per data point, the summation order of
 * orc_mult_naive); the reference's DEFAULT ModLinear operator (OperationMultipleEvalModLinear.cpp,
 * AlgorithmDGEMV over this basis) gives the same values up to summation order.
 * ------------------------------------------------------------------------------------------ */
ORC_API double orc_modlinear_eval(int l, int i, double x) {
  const double hinv = (double)(1 << l);
  if (l == 1) return 1.0;
  if (i == 1) return x <= 2.0 / hinv ? 2.0 - hinv * x : 0.0;
  if (i == (1 << l) - 1) return x >= 1.0 - 2.0 / hinv ? hinv * x - (double)i + 1.0 : 0.0;
  const double v = 1.0 - fabs(hinv * x - (double)i);
  return v > 0.0 ? v : 0.0;
}

static double mod_product(int dim, const int32_t* lev, const int32_t* idx, const double* x) {
  double v = 1.0;
  for (int t = 0; t < dim; ++t) {
    const double h = orc_modlinear_eval(lev[t], idx[t], x[t]);
    if (h == 0.0) return 0.0;
    v *= h;
  }
  return v;
}

ORC_API void orc_mult_naive_mod(int dim, int64_t n, const int32_t* lev, const int32_t* idx,
                                int64_t m, const double* data, const double* alpha,
                                double* result) {
  for (int64_t j = 0; j < m; ++j) {
    double acc = 0.0;
    for (int64_t i = 0; i < n; ++i)
      acc += alpha[i] * mod_product(dim, lev + i * dim, idx + i * dim, data + j * dim);
    result[j] = acc;
  }
}

ORC_API void orc_mult_transpose_naive_mod(int dim, int64_t n, const int32_t* lev,
                                          const int32_t* idx, int64_t m, const double* data,
                                          const double* source, double* result) {
  for (int64_t i = 0; i < n; ++i) {
    double acc = 0.0;
    for (int64_t j = 0; j < m; ++j)
      acc += source[j] * mod_product(dim, lev + i * dim, idx + i * dim, data + j * dim);
    result[i] = acc;
  }
}

/* ------------------------------------------------------------------------------------------
 * STREAMING-shaped dense kernels (the CPU baseline restatement).
 * OperationMultiEvalStreaming.cpp:92-143 with the portable kernels
 * OperationMultiEvalStreaming_multImpl.cpp:577-623 and _multTransposeImpl.cpp:485-510:
 * data transposed to dim-major, data points in chunks, OpenMP over data chunks for mult and
 * over grid-point ranges for multTranspose; every (grid point, data point) product starts at
 * alpha_j (mult) or source_i (multT) and multiplies one hat per dimension.
 * Chunks here are 64 data points so that the inner loop vectorises on any host ISA.
 * ------------------------------------------------------------------------------------------ */
#define ORC_CHUNK 64

typedef struct {
  int dim;
  int64_t m, mpad;
  double* xt; /* [dim x mpad] dim-major; padded by repeating the last row (padDataset, :158-177) */
} orc_stream_data;

ORC_API void* orc_stream_prepare(int dim, int64_t m, const double* data) {
  orc_stream_data* s = (orc_stream_data*)malloc(sizeof(orc_stream_data));
  s->dim = dim;
  s->m = m;
  s->mpad = ((m + ORC_CHUNK - 1) / ORC_CHUNK) * ORC_CHUNK;
  s->xt = (double*)aligned_alloc(64, sizeof(double) * (size_t)(s->mpad * dim + 8));
  for (int t = 0; t < dim; ++t)
    for (int64_t j = 0; j < s->mpad; ++j) {
      const int64_t src = j < m ? j : m - 1;
      s->xt[t * s->mpad + j] = data[src * dim + t];
    }
  return s;
}

ORC_API void orc_stream_release(void* h) {
  orc_stream_data* s = (orc_stream_data*)h;
  if (!s) return;
  free(s->xt);
  free(s);
}

ORC_API void orc_stream_mult(void* h, int64_t n, const double* level_pow2, const double* index,
                             const double* alpha, double* result) {
  const orc_stream_data* s = (const orc_stream_data*)h;
  const int dim = s->dim;
  const int64_t nchunks = s->mpad / ORC_CHUNK;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nchunks; ++c) {
    double acc[ORC_CHUNK];
    double cur[ORC_CHUNK];
    const int64_t base = c * ORC_CHUNK;
    for (int k = 0; k < ORC_CHUNK; ++k) acc[k] = 0.0;
    for (int64_t i = 0; i < n; ++i) {
      const double a = alpha[i];
      for (int k = 0; k < ORC_CHUNK; ++k) cur[k] = a;
      for (int t = 0; t < dim; ++t) {
        const double L = level_pow2[i * dim + t];
        const double I = index[i * dim + t];
        const double* x = &s->xt[t * s->mpad + base];
        for (int k = 0; k < ORC_CHUNK; ++k) {
          const double v = 1.0 - fabs(L * x[k] - I);
          cur[k] *= v > 0.0 ? v : 0.0;
        }
      }
      for (int k = 0; k < ORC_CHUNK; ++k) acc[k] += cur[k];
    }
    for (int k = 0; k < ORC_CHUNK; ++k) {
      if (base + k < s->m) result[base + k] = acc[k];
    }
  }
}

ORC_API void orc_stream_mult_transpose(void* h, int64_t n, const double* level_pow2,
                                       const double* index, const double* source,
                                       double* result) {
  const orc_stream_data* s = (const orc_stream_data*)h;
  const int dim = s->dim;
  const int64_t nchunks = s->mpad / ORC_CHUNK;
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < n; ++i) {
    double part[ORC_CHUNK];
    double cur[ORC_CHUNK];
    for (int k = 0; k < ORC_CHUNK; ++k) part[k] = 0.0;
    for (int64_t c = 0; c < nchunks; ++c) {
      const int64_t base = c * ORC_CHUNK;
      for (int k = 0; k < ORC_CHUNK; ++k)
        cur[k] = (base + k < s->m) ? source[base + k] : 0.0; /* padding source = 0 (:124-128) */
      for (int t = 0; t < dim; ++t) {
        const double L = level_pow2[i * dim + t];
        const double I = index[i * dim + t];
        const double* x = &s->xt[t * s->mpad + base];
        for (int k = 0; k < ORC_CHUNK; ++k) {
          const double v = 1.0 - fabs(L * x[k] - I);
          cur[k] *= v > 0.0 ? v : 0.0;
        }
      }
      for (int k = 0; k < ORC_CHUNK; ++k) part[k] += cur[k];
    }
    double total = 0.0;
    for (int k = 0; k < ORC_CHUNK; ++k) total += part[k];
    result[i] = total;
  }
}

/* ------------------------------------------------------------------------------------------
 * ModLinear STREAMING (OperationMultiEvalModMaskStreaming).
 * Layout, HashGridStorage::getLevelIndexMaskArraysForModEval (HashGridStorage.cpp:519-559) and
 * OperationMultiEvalModMaskStreaming::recalculateLevelIndexMask (.cpp:182-250), per (point, dim)
 * with raw (l, i):
 *   l == 1        : level 0,     index 0, mask 0,        offset 1
 *   i == 1        : level -2^l,  index 0, mask 0,        offset 2
 *   i == 2^l - 1  : level 2^l,   index i, mask 0,        offset 1
 *   otherwise     : level 2^l,   index i, mask sign bit, offset 1
 * Evaluation, _multImpl.cpp:83-122 / _multTransposeImpl.cpp (same steps):
 *   phi = max(offset + (mask | (level * x - index)), 0)
 * where `|` is the bitwise or of the 64-bit patterns (the sign bit turns t into -|t|).
 * The mask array holds the raw bit patterns in double storage, as in the reference.
 * ------------------------------------------------------------------------------------------ */
ORC_API void orc_mod_mask_arrays(int dim, int64_t n, const int32_t* lev, const int32_t* idx,
                                 double* level, double* index, double* mask, double* offset) {
  for (int64_t g = 0; g < n; ++g)
    for (int t = 0; t < dim; ++t) {
      const int64_t k = g * dim + t;
      const int l = lev[k], i = idx[k];
      uint64_t bits = 0;
      if (l == 1) {
        level[k] = 0.0;
        index[k] = 0.0;
        offset[k] = 1.0;
      } else if (i == 1) {
        level[k] = -(double)(1 << l);
        index[k] = 0.0;
        offset[k] = 2.0;
      } else if (i == (1 << l) - 1) {
        level[k] = (double)(1 << l);
        index[k] = (double)i;
        offset[k] = 1.0;
      } else {
        level[k] = (double)(1 << l);
        index[k] = (double)i;
        bits = 0x8000000000000000ull;
        offset[k] = 1.0;
      }
      memcpy(&mask[k], &bits, sizeof bits);
    }
}

static inline double mod_mask_eval(double level, double index, double mask, double offset,
                                   double x) {
  double t = level * x - index;
  uint64_t tb, mb;
  memcpy(&tb, &t, sizeof tb);
  memcpy(&mb, &mask, sizeof mb);
  tb |= mb;
  memcpy(&t, &tb, sizeof t);
  const double v = offset + t;
  return v > 0.0 ? v : 0.0;
}

ORC_API void orc_stream_mult_mod(void* h, int64_t n, const double* level, const double* index,
                                 const double* mask, const double* offset, const double* alpha,
                                 double* result) {
  const orc_stream_data* s = (const orc_stream_data*)h;
  const int dim = s->dim;
  const int64_t nchunks = s->mpad / ORC_CHUNK;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nchunks; ++c) {
    double acc[ORC_CHUNK];
    double cur[ORC_CHUNK];
    const int64_t base = c * ORC_CHUNK;
    for (int k = 0; k < ORC_CHUNK; ++k) acc[k] = 0.0;
    for (int64_t i = 0; i < n; ++i) {
      const double a = alpha[i];
      for (int k = 0; k < ORC_CHUNK; ++k) cur[k] = a;
      for (int t = 0; t < dim; ++t) {
        const int64_t q = i * dim + t;
        const double* x = &s->xt[t * s->mpad + base];
        for (int k = 0; k < ORC_CHUNK; ++k)
          cur[k] *= mod_mask_eval(level[q], index[q], mask[q], offset[q], x[k]);
      }
      for (int k = 0; k < ORC_CHUNK; ++k) acc[k] += cur[k];
    }
    for (int k = 0; k < ORC_CHUNK; ++k) {
      if (base + k < s->m) result[base + k] = acc[k];
    }
  }
}

ORC_API void orc_stream_mult_transpose_mod(void* h, int64_t n, const double* level,
                                           const double* index, const double* mask,
                                           const double* offset, const double* source,
                                           double* result) {
  const orc_stream_data* s = (const orc_stream_data*)h;
  const int dim = s->dim;
  const int64_t nchunks = s->mpad / ORC_CHUNK;
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < n; ++i) {
    double part[ORC_CHUNK];
    double cur[ORC_CHUNK];
    for (int k = 0; k < ORC_CHUNK; ++k) part[k] = 0.0;
    for (int64_t c = 0; c < nchunks; ++c) {
      const int64_t base = c * ORC_CHUNK;
      for (int k = 0; k < ORC_CHUNK; ++k)
        cur[k] = (base + k < s->m) ? source[base + k] : 0.0; /* padding source = 0 */
      for (int t = 0; t < dim; ++t) {
        const int64_t q = i * dim + t;
        const double* x = &s->xt[t * s->mpad + base];
        for (int k = 0; k < ORC_CHUNK; ++k)
          cur[k] *= mod_mask_eval(level[q], index[q], mask[q], offset[q], x[k]);
      }
      for (int k = 0; k < ORC_CHUNK; ++k) part[k] += cur[k];
    }
    double total = 0.0;
    for (int k = 0; k < ORC_CHUNK; ++k) total += part[k];
    result[i] = total;
  }
}

ORC_API int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

ORC_API void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ------------------------------------------------------------------------------------------
 * Regression fit: SystemMatrixLeastSquaresIdentity (datadriven/.../SystemMatrixLeastSquaresIdentity.cpp:32-56)
 *   A alpha = B^T (B alpha) + (M * lambda) alpha,   b = B^T y
 * solved by ConjugateGradients::solve (solver/src/sgpp/solver/sle/ConjugateGradients.cpp:22-151):
 * relative stopping test delta_new <= eps^2 delta_0, true residual recomputed every 50
 * iterations, optional warm start (reuse).
 * ------------------------------------------------------------------------------------------ */
/* level/index arrays of either basis: mask == NULL selects the Linear (level_pow2, index) pair,
 * otherwise the ModLinear (level, index, mask, offset) streaming layout */
typedef struct {
  const double *level, *index, *mask, *offset;
} orc_arrays;

static void arr_mult(void* h, int64_t n, const orc_arrays* A, const double* a, double* out) {
  if (A->mask)
    orc_stream_mult_mod(h, n, A->level, A->index, A->mask, A->offset, a, out);
  else
    orc_stream_mult(h, n, A->level, A->index, a, out);
}

static void arr_mult_transpose(void* h, int64_t n, const orc_arrays* A, const double* v,
                               double* out) {
  if (A->mask)
    orc_stream_mult_transpose_mod(h, n, A->level, A->index, A->mask, A->offset, v, out);
  else
    orc_stream_mult_transpose(h, n, A->level, A->index, v, out);
}

static void sys_apply(void* h, int64_t n, const orc_arrays* A, double lambda_m, const double* a,
                      double* out, double* tmp) {
  arr_mult(h, n, A, a, tmp);
  arr_mult_transpose(h, n, A, tmp, out);
  for (int64_t i = 0; i < n; ++i) out[i] += lambda_m * a[i];
}

static double dot(int64_t n, const double* a, const double* b) {
  double s = 0.0;
  for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

static int cg_fit(void* h, int64_t n, const orc_arrays* A, const double* y, double lambda,
                  int64_t imax, double eps, int reuse, double* alpha, int64_t* iterations,
                  double* residual) {
  const orc_stream_data* s = (const orc_stream_data*)h;
  const double lambda_m = (double)s->m * lambda;
  double* tmp = (double*)malloc(sizeof(double) * (size_t)s->mpad);
  double* b = (double*)malloc(sizeof(double) * (size_t)n);
  double* r = (double*)malloc(sizeof(double) * (size_t)n);
  double* d = (double*)malloc(sizeof(double) * (size_t)n);
  double* q = (double*)malloc(sizeof(double) * (size_t)n);
  double* t = (double*)malloc(sizeof(double) * (size_t)n);
  arr_mult_transpose((void*)s, n, A, y, b); /* generateb, :49-56 */

  const double eps2 = eps * eps;
  double delta_0 = 0.0;
  memcpy(r, b, sizeof(double) * (size_t)n);
  if (reuse) {
    /* the reference's A*0 is zero; r = b, delta_0 = eps^2 * b.b */
    delta_0 = dot(n, r, r) * eps2;
  } else {
    for (int64_t i = 0; i < n; ++i) alpha[i] = 0.0;
  }
  sys_apply((void*)s, n, A, lambda_m, alpha, t, tmp);
  for (int64_t i = 0; i < n; ++i) r[i] -= t[i];
  memcpy(d, r, sizeof(double) * (size_t)n);
  double delta_new = dot(n, r, r);
  if (!reuse) delta_0 = delta_new * eps2;
  int64_t it = 0;
  while (it < imax && delta_new > delta_0 && delta_new > 0.0) {
    sys_apply((void*)s, n, A, lambda_m, d, q, tmp);
    const double dq = dot(n, d, q);
    if (dq == 0.0) break;
    const double a = delta_new / dq;
    for (int64_t i = 0; i < n; ++i) alpha[i] += a * d[i];
    if (it % 50 == 0 && it > 0) {
      sys_apply((void*)s, n, A, lambda_m, alpha, t, tmp);
      for (int64_t i = 0; i < n; ++i) r[i] = b[i] - t[i];
    } else {
      for (int64_t i = 0; i < n; ++i) r[i] -= a * q[i];
    }
    const double delta_old = delta_new;
    delta_new = dot(n, r, r);
    const double beta = delta_new / delta_old;
    for (int64_t i = 0; i < n; ++i) d[i] = beta * d[i] + r[i];
    ++it;
  }
  *iterations = it;
  *residual = delta_new;
  free(tmp);
  free(b);
  free(r);
  free(d);
  free(q);
  free(t);
  return 0;
}

ORC_API int orc_cg_fit(void* h, int64_t n, const double* level_pow2, const double* index,
                       const double* y, double lambda, int64_t imax, double eps, int reuse,
                       double* alpha, int64_t* iterations, double* residual) {
  const orc_arrays A = {level_pow2, index, NULL, NULL};
  return cg_fit(h, n, &A, y, lambda, imax, eps, reuse, alpha, iterations, residual);
}

/* the same fit on a ModLinear grid (the reference factory gives SystemMatrixLeastSquaresIdentity
 * OperationMultiEvalModMaskStreaming for STREAMING there, DatadrivenOpFactory.cpp:479-483) */
ORC_API int orc_cg_fit_mod(void* h, int64_t n, const double* level, const double* index,
                           const double* mask, const double* offset, const double* y,
                           double lambda, int64_t imax, double eps, int reuse, double* alpha,
                           int64_t* iterations, double* residual) {
  const orc_arrays A = {level, index, mask, offset};
  return cg_fit(h, n, &A, y, lambda, imax, eps, reuse, alpha, iterations, residual);
}

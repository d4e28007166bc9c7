// Device-resident least-squares fitting with spatial adaptivity: the reference's
// ModelFittingLeastSquares (datadriven/src/sgpp/datadriven/datamining/modules/fitting/
// ModelFittingLeastSquares.cpp) over one GPU operator. C ABI in include/sgmev.h (sgfit_*).
//
//   fit(data)    regular grid of the configured level and basis, alpha = 0, then
//                assembleSystemAndSolve with the final solver configuration (:51-64, :129-140):
//                b = B^T y, CG on (B^T B + lambda M I) alpha = b, started from alpha (reuse).
//   adapt()      while fewer than numRefinements_ rounds were done: SurplusRefinementFunctor(alpha,
//                numRefinementPoints_, refinementThreshold_) refines the grid (new points are
//                appended); if it grew, alpha is extended with zeros (resizeZero) and solved
//                again from there with the refine solver configuration (:66-101).
//   update(data) the same grid and alpha on new data, solved with the final configuration
//                (:103-113; the reference's update() calls reset(), which releases the grid it
//                then solves on; here the grid is kept, as the method intends).
//   evaluate(x)  B(x) alpha on other points (:39-49).
//
// Where the reference builds a new system matrix, and with it a new operator that copies the
// data, for every solve, here one operator holds the data on the device from fit() or update()
// on; adapt() re-stages only the grid (sgmev_prepare). y and alpha stay on the device between
// solves; a refinement round brings alpha back to the host for the refinement functor (N
// doubles) and sends the grown grid down.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sgmev.h"

namespace sgmev {
extern thread_local std::string g_last_error;
}

struct sgfit {
  sgfit_config cfg;
  std::string params;         // operator knobs (JSON), the basis added
  int dim = 0;
  int64_t n = 0;              // grid points
  std::vector<int32_t> level, index;  // [n x dim] raw levels and indices, storage order
  sgmev_op* op = nullptr;     // the operator on the current data set
  int64_t m = 0;
  double* d_y = nullptr;      // [m]
  double* d_alpha = nullptr;  // [n]
  int64_t refinements = 0;
  int64_t last_iterations = 0;
  double last_residual = 0.0;
};

namespace {

int fit_fail(int code, const std::string& msg) {
  sgmev::g_last_error = msg;
  return code;
}

#define FIT_TRY(expr)                   \
  do {                                  \
    const int rc_ = (expr);             \
    if (rc_ != SGMEV_OK) return rc_;    \
  } while (0)

#define FIT_CUDA(call)                                                                    \
  do {                                                                                    \
    const cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess)                                                                \
      return fit_fail(e_ == cudaErrorMemoryAllocation ? SGMEV_ERR_OOM : SGMEV_ERR_CUDA,   \
                      std::string(#call) + ": " + cudaGetErrorString(e_));                \
  } while (0)

std::string op_params(const sgfit* f) {
  std::string p = f->params;
  if (f->cfg.basis == 1) {
    const std::string kv = "\"basis\":\"modlinear\"";
    p = p.empty() ? "{" + kv + "}" : p.substr(0, p.size() - 1) + (p.size() > 2 ? "," : "") + kv + "}";
  }
  return p;
}

int eval_arrays(const sgfit* f, std::vector<double>& lp, std::vector<double>& ix) {
  lp.resize(static_cast<size_t>(std::max<int64_t>(f->n * f->dim, 1)));
  ix.resize(lp.size());
  return sggrid_level_index_for_eval(f->dim, f->n, f->level.data(), f->index.data(), lp.data(),
                                     ix.data());
}

// a new operator on (x, y) for the current grid; y goes to the device
int stage_data(sgfit* f, int64_t m, const double* x, const double* y) {
  std::vector<double> lp, ix;
  FIT_TRY(eval_arrays(f, lp, ix));
  if (f->op) sgmev_destroy(f->op);
  f->op = nullptr;
  const std::string p = op_params(f);
  FIT_TRY(sgmev_create(&f->op, f->dim, f->n, lp.data(), ix.data(), m, x, nullptr, nullptr,
                       f->cfg.precision, p.empty() ? nullptr : p.c_str()));
  if (f->d_y) cudaFree(f->d_y);
  f->d_y = nullptr;
  FIT_CUDA(cudaMalloc(&f->d_y, sizeof(double) * static_cast<size_t>(std::max<int64_t>(m, 1))));
  if (m > 0) FIT_CUDA(cudaMemcpy(f->d_y, y, sizeof(double) * m, cudaMemcpyHostToDevice));
  f->m = m;
  return SGMEV_OK;
}

// alpha on the device resized to `n` points: the first `keep` entries kept, the rest zero
int resize_alpha(sgfit* f, int64_t n, int64_t keep) {
  double* a = nullptr;
  FIT_CUDA(cudaMalloc(&a, sizeof(double) * static_cast<size_t>(std::max<int64_t>(n, 1))));
  FIT_CUDA(cudaMemset(a, 0, sizeof(double) * static_cast<size_t>(std::max<int64_t>(n, 1))));
  if (keep > 0 && f->d_alpha)
    FIT_CUDA(cudaMemcpy(a, f->d_alpha, sizeof(double) * keep, cudaMemcpyDeviceToDevice));
  if (f->d_alpha) cudaFree(f->d_alpha);
  f->d_alpha = a;
  return SGMEV_OK;
}

// assembleSystemAndSolve: b = B^T y, CG from the current alpha (reuse = true)
int solve(sgfit* f, double eps, int64_t max_iterations) {
  return sgmev_fit_device(f->op, f->cfg.mode, f->d_y, f->cfg.lambda, max_iterations, eps, 1,
                          f->d_alpha, &f->last_iterations, &f->last_residual);
}

int check(const sgfit* f) {
  if (!f) return fit_fail(SGMEV_ERR_INVALID, "fitter is NULL");
  return SGMEV_OK;
}

}  // namespace

extern "C" {

SGMEV_API void sgfit_config_defaults(sgfit_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  // FitterConfiguration::setupDefaults (datadriven/.../fitting/FitterConfiguration.cpp:143-218)
  c->level = 3;
  c->basis = 0;
  c->lambda = 0.01;
  c->final_eps = 1e-12;
  c->final_max_iterations = 100;
  c->refine_eps = 1e-12;
  c->refine_max_iterations = 100;
  c->num_refinements = 1;
  c->num_refinement_points = 1;
  c->refinement_threshold = 0.0;
  c->mode = SGMEV_SOLVE_PLAIN;
  c->precision = SGMEV_FP64;
}

SGMEV_API int sgfit_create(sgfit** out, const sgfit_config* cfg, const char* params_json) {
  sgmev::g_last_error.clear();
  if (!out || !cfg) return fit_fail(SGMEV_ERR_INVALID, "sgfit_create: NULL argument");
  *out = nullptr;
  if (cfg->level < 1) return fit_fail(SGMEV_ERR_INVALID, "grid level must be >= 1");
  if (cfg->basis != 0 && cfg->basis != 1)
    return fit_fail(SGMEV_ERR_INVALID, "basis must be 0 (Linear) or 1 (ModLinear)");
  if (cfg->mode != SGMEV_SOLVE_PLAIN && cfg->mode != SGMEV_SOLVE_MIXED &&
      cfg->mode != SGMEV_SOLVE_MIXED_NATIVE64)
    return fit_fail(SGMEV_ERR_INVALID, "mode must be SGMEV_SOLVE_PLAIN, _MIXED or _MIXED_NATIVE64");
  if (cfg->num_refinement_points < 0 || cfg->num_refinements < 0)
    return fit_fail(SGMEV_ERR_INVALID, "negative refinement counts");
  sgfit* f = new sgfit;
  f->cfg = *cfg;
  f->params = params_json ? params_json : "";
  while (!f->params.empty() && (f->params.back() == ' ' || f->params.back() == '\n'))
    f->params.pop_back();
  if (!f->params.empty() && (f->params.front() != '{' || f->params.back() != '}')) {
    delete f;
    return fit_fail(SGMEV_ERR_INVALID, "params_json must be a flat JSON object");
  }
  *out = f;
  return SGMEV_OK;
}

SGMEV_API int sgfit_destroy(sgfit* f) {
  if (!f) return SGMEV_OK;
  if (f->op) sgmev_destroy(f->op);
  if (f->d_y) cudaFree(f->d_y);
  if (f->d_alpha) cudaFree(f->d_alpha);
  delete f;
  return SGMEV_OK;
}

SGMEV_API int sgfit_fit(sgfit* f, int64_t m, int dim, const double* x, const double* y) {
  FIT_TRY(check(f));
  sgmev::g_last_error.clear();
  if (dim < 1 || m < 0 || (m > 0 && (!x || !y)))
    return fit_fail(SGMEV_ERR_INVALID, "sgfit_fit: bad data arguments");
  // reset(): a new regular grid of the configured level
  f->dim = dim;
  f->refinements = 0;
  int64_t n = 0;
  FIT_TRY(sggrid_regular(dim, f->cfg.level, &n, nullptr, nullptr));
  f->level.assign(static_cast<size_t>(n * dim), 0);
  f->index.assign(static_cast<size_t>(n * dim), 0);
  FIT_TRY(sggrid_regular(dim, f->cfg.level, &n, f->level.data(), f->index.data()));
  f->n = n;
  FIT_TRY(stage_data(f, m, x, y));
  FIT_TRY(resize_alpha(f, n, 0));
  return solve(f, f->cfg.final_eps, f->cfg.final_max_iterations);
}

SGMEV_API int sgfit_adapt(sgfit* f, int* refined) {
  FIT_TRY(check(f));
  sgmev::g_last_error.clear();
  if (refined) *refined = 0;
  if (!f->op)
    return fit_fail(SGMEV_ERR_INVALID,
                    "ModelFittingLeastSquares: Can't refine before initial grid is created");
  if (f->refinements >= f->cfg.num_refinements) return SGMEV_OK;
  std::vector<double> alpha(static_cast<size_t>(std::max<int64_t>(f->n, 1)));
  if (f->n > 0)
    FIT_CUDA(cudaMemcpy(alpha.data(), f->d_alpha, sizeof(double) * f->n, cudaMemcpyDeviceToHost));
  // room for the new points: children and their missing parents (grown until it fits)
  int64_t cap = f->n + f->cfg.num_refinement_points * 2 * f->dim * 8 + 1024;
  int64_t n_new = 0;
  for (int attempt = 0;; ++attempt) {
    std::vector<int32_t> lv(static_cast<size_t>(cap * f->dim)), ix(lv.size());
    std::copy(f->level.begin(), f->level.end(), lv.begin());
    std::copy(f->index.begin(), f->index.end(), ix.begin());
    const int rc = sggrid_refine_surplus(f->dim, f->n, cap, lv.data(), ix.data(), alpha.data(),
                                         f->cfg.num_refinement_points, f->cfg.refinement_threshold,
                                         &n_new);
    if (rc == SGMEV_OK) {
      lv.resize(static_cast<size_t>(n_new * f->dim));
      ix.resize(lv.size());
      f->level.swap(lv);
      f->index.swap(ix);
      break;
    }
    const bool full = sgmev::g_last_error.find("capacity") != std::string::npos;
    if (!full || attempt >= 8) return rc;
    cap *= 4;
  }
  if (n_new <= f->n) return SGMEV_OK;
  const int64_t n_old = f->n;
  f->n = n_new;
  std::vector<double> lp, ix;
  FIT_TRY(eval_arrays(f, lp, ix));
  FIT_TRY(sgmev_prepare(f->op, f->n, lp.data(), ix.data()));
  FIT_TRY(resize_alpha(f, f->n, n_old));  // alpha.resizeZero(grid size)
  FIT_TRY(solve(f, f->cfg.refine_eps, f->cfg.refine_max_iterations));
  ++f->refinements;
  if (refined) *refined = 1;
  return SGMEV_OK;
}

SGMEV_API int sgfit_update(sgfit* f, int64_t m, int dim, const double* x, const double* y) {
  FIT_TRY(check(f));
  sgmev::g_last_error.clear();
  if (!f->op) return sgfit_fit(f, m, dim, x, y);
  if (dim != f->dim || m < 0 || (m > 0 && (!x || !y)))
    return fit_fail(SGMEV_ERR_INVALID, "sgfit_update: bad data arguments");
  f->refinements = 0;  // reset() in the reference clears the refinement count
  FIT_TRY(stage_data(f, m, x, y));
  return solve(f, f->cfg.final_eps, f->cfg.final_max_iterations);
}

SGMEV_API int sgfit_evaluate(sgfit* f, int64_t m, const double* x, double* out) {
  FIT_TRY(check(f));
  sgmev::g_last_error.clear();
  if (!f->op) return fit_fail(SGMEV_ERR_INVALID, "sgfit_evaluate: no model (fit first)");
  if (m < 0 || (m > 0 && (!x || !out))) return fit_fail(SGMEV_ERR_INVALID, "sgfit_evaluate: bad arguments");
  if (m == 0) return SGMEV_OK;
  std::vector<double> alpha(static_cast<size_t>(std::max<int64_t>(f->n, 1)));
  if (f->n > 0)
    FIT_CUDA(cudaMemcpy(alpha.data(), f->d_alpha, sizeof(double) * f->n, cudaMemcpyDeviceToHost));
  std::vector<double> lp, ix;
  FIT_TRY(eval_arrays(f, lp, ix));
  sgmev_op* e = nullptr;
  const std::string p = op_params(f);
  FIT_TRY(sgmev_create(&e, f->dim, f->n, lp.data(), ix.data(), m, x, nullptr, nullptr,
                       f->cfg.precision, p.empty() ? nullptr : p.c_str()));
  const int rc = sgmev_mult(e, alpha.data(), out);
  sgmev_destroy(e);
  return rc;
}

SGMEV_API int sgfit_grid(const sgfit* f, int* dim, int64_t* n_grid, int32_t* level, int32_t* index) {
  FIT_TRY(check(f));
  if (dim) *dim = f->dim;
  if (n_grid) *n_grid = f->n;
  if (level) std::copy(f->level.begin(), f->level.end(), level);
  if (index) std::copy(f->index.begin(), f->index.end(), index);
  return SGMEV_OK;
}

SGMEV_API int sgfit_alpha(const sgfit* f, double* alpha) {
  FIT_TRY(check(f));
  if (!alpha) return fit_fail(SGMEV_ERR_INVALID, "sgfit_alpha: NULL");
  if (f->n > 0 && f->d_alpha)
    FIT_CUDA(cudaMemcpy(alpha, f->d_alpha, sizeof(double) * f->n, cudaMemcpyDeviceToHost));
  return SGMEV_OK;
}

SGMEV_API int sgfit_stats(const sgfit* f, int64_t* iterations, double* residual,
                          int64_t* refinements) {
  FIT_TRY(check(f));
  if (iterations) *iterations = f->last_iterations;
  if (residual) *residual = f->last_residual;
  if (refinements) *refinements = f->refinements;
  return SGMEV_OK;
}

}  // extern "C"

// Test infrastructure only: a thin extern "C" harness around the SG++ reference library
// (compiled from the reference's own sources by oracle/ref.mk into oracle/_ref/).
// Nothing in the shipped product links or loads this file; tests and the golden-fixture
// generator use it to pin the oracle restatement (oracle/oracle.c) and the CUDA path.
//
// What it drives, all unmodified reference code:
//   grid      sgpp::base::Grid::createLinearGrid        base/src/sgpp/base/grid/Grid.cpp:73
//             GridGenerator::regular                    base/.../StandardGridGenerator.cpp:27-30
//             GridGenerator::refine(SurplusRefinementFunctor)
//                                                       base/.../StandardGridGenerator.cpp:64-68
//             HashGridStorage::getLevelIndexArraysForEval
//                                                       base/.../HashGridStorage.cpp:433-450
//   DEFAULT   op_factory::createOperationMultipleEval(grid, data)
//             -> OperationMultipleEvalLinear            base/.../BaseOpFactory.cpp:595-598
//   NAIVE     OperationMultipleEvalLinearNaive          base/.../OperationMultipleEvalLinearNaive.cpp
//   STREAMING OperationMultiEvalStreaming               datadriven/.../OperationMultiEvalStreaming.cpp
//   ModLinear Grid::createModLinearGrid                 base/src/sgpp/base/grid/Grid.cpp
//             DEFAULT -> OperationMultipleEvalModLinear base/.../BaseOpFactory.cpp (ModLinear branch)
//             STREAMING -> OperationMultiEvalModMaskStreaming
//                                                       datadriven/.../OperationMultiEvalModMaskStreaming.cpp
//             HashGridStorage::getLevelIndexMaskArraysForModEval
//                                                       base/.../HashGridStorage.cpp:519-559
//   datasets  ARFFTools::readARFF, CSVTools::readCSV (on a string stream)
//                                                       datadriven/.../tools/ARFFTools.cpp, CSVTools.cpp
//   CG fit    SystemMatrixLeastSquaresIdentity + solver::ConjugateGradients
//                                                       datadriven/.../SystemMatrixLeastSquaresIdentity.cpp
//                                                       solver/src/sgpp/solver/sle/ConjugateGradients.cpp
//
// SystemMatrixLeastSquaresIdentity obtains its operator through the datadriven factory
// (datadriven/src/sgpp/datadriven/DatadrivenOpFactory.cpp:409). That factory's translation
// unit pulls in every datadriven operator, so this harness defines the one factory overload
// itself and routes (DEFAULT) and (STREAMING, DEFAULT) exactly as the reference factory does
// for Linear grids (DatadrivenOpFactory.cpp:439-452) and ModLinear grids (:479-483).

#include <sgpp/base/datatypes/DataMatrix.hpp>
#include <sgpp/base/datatypes/DataVector.hpp>
#include <sgpp/base/exception/factory_exception.hpp>
#include <sgpp/base/grid/Grid.hpp>
#include <sgpp/base/grid/generation/functors/SurplusRefinementFunctor.hpp>
#include <sgpp/base/grid/storage/hashmap/HashGridStorage.hpp>
#include <sgpp/base/operation/BaseOpFactory.hpp>
#include <sgpp/base/operation/hash/OperationMultipleEval.hpp>
#include <sgpp/base/operation/hash/OperationMultipleEvalLinearNaive.hpp>
#include <sgpp/base/tools/GaussLegendreQuadRule1D.hpp>
#include <sgpp/datadriven/algorithm/SystemMatrixLeastSquaresIdentity.hpp>
#include <sgpp/datadriven/operation/hash/DatadrivenOperationCommon.hpp>
#include <sgpp/datadriven/tools/ARFFTools.hpp>
#include <sgpp/datadriven/tools/CSVTools.hpp>
#include <sgpp/datadriven/operation/hash/OperationMultiEvalModMaskStreaming/OperationMultiEvalModMaskStreaming.hpp>
#include <sgpp/datadriven/operation/hash/OperationMultiEvalStreaming/OperationMultiEvalStreaming.hpp>
#include <sgpp/solver/sle/ConjugateGradients.hpp>

#ifdef _OPENMP
#include <omp.h>
#endif

#include <cstdint>
#include <cstring>
#include <exception>
#include <memory>
#include <sstream>
#include <string>

// The reference snapshot ships GaussLegendreQuadRule1D.hpp without its .cpp. Linear-grid code
// never calls it, but other base/ translation units reference the symbols, so they are defined
// here as inert stand-ins (they are never reached on the multi-evaluation path).
namespace sgpp {
namespace base {
GaussLegendreQuadRule1D::GaussLegendreQuadRule1D() {}
GaussLegendreQuadRule1D::~GaussLegendreQuadRule1D() {}
void GaussLegendreQuadRule1D::getLevelPointsAndWeightsNormalized(size_t, DataVector&,
                                                                 DataVector&) {
  throw factory_exception("GaussLegendreQuadRule1D is not part of the multi-evaluation oracle");
}
GaussLegendreQuadRule1D& GaussLegendreQuadRule1D::getInstance() {
  static GaussLegendreQuadRule1D instance;
  return instance;
}
}  // namespace base

namespace op_factory {
// Routing as in DatadrivenOpFactory.cpp:439-452 and :479-483 (DEFAULT -> base factory;
// STREAMING/DEFAULT -> OperationMultiEvalStreaming for Linear grids and
// OperationMultiEvalModMaskStreaming for ModLinear grids); every other combination throws, like
// the reference's final `throw factory_exception` (DatadrivenOpFactory.cpp:551).
base::OperationMultipleEval* createOperationMultipleEval(
    base::Grid& grid, base::DataMatrix& dataset,
    datadriven::OperationMultipleEvalConfiguration& configuration) {
  using datadriven::OperationMultipleEvalSubType;
  using datadriven::OperationMultipleEvalType;
  if (configuration.getType() == OperationMultipleEvalType::DEFAULT) {
    return createOperationMultipleEval(grid, dataset);
  }
  if (grid.getType() == base::GridType::Linear &&
      configuration.getType() == OperationMultipleEvalType::STREAMING &&
      configuration.getSubType() == OperationMultipleEvalSubType::DEFAULT) {
    return new datadriven::OperationMultiEvalStreaming(grid, dataset);
  }
  if (grid.getType() == base::GridType::ModLinear &&
      configuration.getType() == OperationMultipleEvalType::STREAMING &&
      configuration.getSubType() == OperationMultipleEvalSubType::DEFAULT) {
    return new datadriven::OperationMultiEvalModMaskStreaming(grid, dataset);
  }
  throw base::factory_exception("oracle harness: unsupported multi-eval configuration");
}
}  // namespace op_factory
}  // namespace sgpp

namespace {

thread_local std::string g_err;

struct RefGrid {
  std::unique_ptr<sgpp::base::Grid> grid;
};

enum RefKind { REF_DEFAULT = 0, REF_STREAMING = 1, REF_NAIVE = 2 };

sgpp::base::DataMatrix make_matrix(const double* rows, int64_t m, int dim) {
  sgpp::base::DataMatrix mat(static_cast<size_t>(m), static_cast<size_t>(dim));
  std::memcpy(mat.getPointer(), rows, sizeof(double) * static_cast<size_t>(m) * dim);
  return mat;
}

std::unique_ptr<sgpp::base::OperationMultipleEval> make_op(RefGrid* g,
                                                           sgpp::base::DataMatrix& data,
                                                           int kind) {
  switch (kind) {
    case REF_DEFAULT:
      return std::unique_ptr<sgpp::base::OperationMultipleEval>(
          sgpp::op_factory::createOperationMultipleEval(*g->grid, data));
    case REF_STREAMING:
      if (g->grid->getType() == sgpp::base::GridType::ModLinear)
        return std::make_unique<sgpp::datadriven::OperationMultiEvalModMaskStreaming>(*g->grid,
                                                                                      data);
      return std::make_unique<sgpp::datadriven::OperationMultiEvalStreaming>(*g->grid, data);
    case REF_NAIVE:
      if (g->grid->getType() != sgpp::base::GridType::Linear)
        throw sgpp::base::factory_exception("the NAIVE kind is Linear only");
      return std::make_unique<sgpp::base::OperationMultipleEvalLinearNaive>(*g->grid, data);
    default:
      throw sgpp::base::factory_exception("unknown reference kind");
  }
}

template <class F>
int guarded(F&& f) {
  try {
    f();
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return 1;
  } catch (...) {
    g_err = "unknown exception";
    return 1;
  }
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

void ref_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int ref_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void* ref_grid_create_linear(int dim) {
  RefGrid* g = new RefGrid;
  g->grid.reset(sgpp::base::Grid::createLinearGrid(static_cast<size_t>(dim)));
  return g;
}

void* ref_grid_create_modlinear(int dim) {
  RefGrid* g = new RefGrid;
  g->grid.reset(sgpp::base::Grid::createModLinearGrid(static_cast<size_t>(dim)));
  return g;
}

void ref_grid_destroy(void* h) { delete static_cast<RefGrid*>(h); }

int ref_grid_regular(void* h, int level) {
  return guarded([&] { static_cast<RefGrid*>(h)->grid->getGenerator().regular(level); });
}

int64_t ref_grid_size(void* h) {
  return static_cast<int64_t>(static_cast<RefGrid*>(h)->grid->getSize());
}

int ref_grid_dim(void* h) {
  return static_cast<int>(static_cast<RefGrid*>(h)->grid->getDimension());
}

// level/index in the reference's eval layout: two [N x d] row-major arrays, 2^l and i as doubles.
int ref_grid_level_index(void* h, double* level_pow2, double* index) {
  return guarded([&] {
    RefGrid* g = static_cast<RefGrid*>(h);
    auto& st = g->grid->getStorage();
    sgpp::base::DataMatrix lv(st.getSize(), st.getDimension());
    sgpp::base::DataMatrix ix(st.getSize(), st.getDimension());
    st.getLevelIndexArraysForEval(lv, ix);
    std::memcpy(level_pow2, lv.getPointer(), sizeof(double) * lv.getSize());
    std::memcpy(index, ix.getPointer(), sizeof(double) * ix.getSize());
  });
}

// The ModLinear streaming layout (HashGridStorage::getLevelIndexMaskArraysForModEval): four
// [N x d] row-major arrays; mask holds raw 64-bit sign masks in double storage.
int ref_grid_mask_arrays(void* h, double* level, double* index, double* mask, double* offset) {
  return guarded([&] {
    auto& st = static_cast<RefGrid*>(h)->grid->getStorage();
    sgpp::base::DataMatrix lv(st.getSize(), st.getDimension());
    sgpp::base::DataMatrix ix(st.getSize(), st.getDimension());
    sgpp::base::DataMatrix mk(st.getSize(), st.getDimension());
    sgpp::base::DataMatrix of(st.getSize(), st.getDimension());
    st.getLevelIndexMaskArraysForModEval(lv, ix, mk, of);
    std::memcpy(level, lv.getPointer(), sizeof(double) * lv.getSize());
    std::memcpy(index, ix.getPointer(), sizeof(double) * ix.getSize());
    std::memcpy(mask, mk.getPointer(), sizeof(double) * mk.getSize());
    std::memcpy(offset, of.getPointer(), sizeof(double) * of.getSize());
  });
}

// Raw (level, index, leaf) per grid point in storage sequence order.
int ref_grid_points(void* h, int32_t* level, int32_t* index, int32_t* leaf) {
  return guarded([&] {
    auto& st = static_cast<RefGrid*>(h)->grid->getStorage();
    const size_t d = st.getDimension();
    for (size_t s = 0; s < st.getSize(); ++s) {
      auto& p = st.getPoint(s);
      for (size_t t = 0; t < d; ++t) {
        level[s * d + t] = static_cast<int32_t>(p.getLevel(t));
        index[s * d + t] = static_cast<int32_t>(p.getIndex(t));
      }
      if (leaf) leaf[s] = p.isLeaf() ? 1 : 0;
    }
  });
}

int ref_grid_set_bounding_box(void* h, const double* left, const double* right) {
  return guarded([&] {
    auto& bb = static_cast<RefGrid*>(h)->grid->getBoundingBox();
    for (size_t t = 0; t < bb.getDimension(); ++t) {
      bb.setBoundary(t, sgpp::base::BoundingBox1D(left[t], right[t]));
    }
  });
}

// One round of surplus refinement on |alpha| (SurplusRefinementFunctor.cpp:23-28).
int ref_grid_refine_surplus(void* h, const double* alpha, int64_t n_alpha, int64_t n_points,
                            double threshold) {
  return guarded([&] {
    RefGrid* g = static_cast<RefGrid*>(h);
    sgpp::base::DataVector a(static_cast<size_t>(n_alpha));
    std::memcpy(a.getPointer(), alpha, sizeof(double) * static_cast<size_t>(n_alpha));
    sgpp::base::SurplusRefinementFunctor f(a, static_cast<size_t>(n_points), threshold);
    g->grid->getGenerator().refine(f);
  });
}

// Serialized grid text (Grid::serialize), for fixtures that want the reference's own format.
int ref_grid_serialize(void* h, char* buf, int64_t cap, int64_t* needed) {
  return guarded([&] {
    std::string s;
    static_cast<RefGrid*>(h)->grid->serialize(s);
    *needed = static_cast<int64_t>(s.size()) + 1;
    if (buf && cap >= *needed) std::memcpy(buf, s.c_str(), s.size() + 1);
  });
}

// result[m] = sum_i alpha_i phi_i(x_m)  through the chosen reference implementation.
int ref_mult(void* h, int kind, const double* data, int64_t m, const double* alpha,
             double* result, double* seconds) {
  return guarded([&] {
    RefGrid* g = static_cast<RefGrid*>(h);
    const int dim = static_cast<int>(g->grid->getDimension());
    sgpp::base::DataMatrix x = make_matrix(data, m, dim);
    auto op = make_op(g, x, kind);
    sgpp::base::DataVector a(g->grid->getSize());
    std::memcpy(a.getPointer(), alpha, sizeof(double) * a.getSize());
    sgpp::base::DataVector r(static_cast<size_t>(m));
    op->mult(a, r);
    std::memcpy(result, r.getPointer(), sizeof(double) * r.getSize());
    if (seconds) *seconds = kind == REF_STREAMING ? op->getDuration() : -1.0;
  });
}

// result[i] = sum_m source_m phi_i(x_m)
int ref_mult_transpose(void* h, int kind, const double* data, int64_t m, const double* source,
                       double* result, double* seconds) {
  return guarded([&] {
    RefGrid* g = static_cast<RefGrid*>(h);
    const int dim = static_cast<int>(g->grid->getDimension());
    sgpp::base::DataMatrix x = make_matrix(data, m, dim);
    auto op = make_op(g, x, kind);
    sgpp::base::DataVector s(static_cast<size_t>(m));
    std::memcpy(s.getPointer(), source, sizeof(double) * s.getSize());
    sgpp::base::DataVector r(g->grid->getSize());
    op->multTranspose(s, r);
    std::memcpy(result, r.getPointer(), sizeof(double) * r.getSize());
    if (seconds) *seconds = kind == REF_STREAMING ? op->getDuration() : -1.0;
  });
}

// Repeated STREAMING mult/multTranspose on one prepared operator (CPU baseline timing): the
// operator is built once, then `reps` calls run back to back; per-call durations are returned.
int ref_streaming_time(void* h, const double* data, int64_t m, const double* alpha,
                       const double* source, int reps, double* mult_seconds,
                       double* multt_seconds) {
  return guarded([&] {
    RefGrid* g = static_cast<RefGrid*>(h);
    const int dim = static_cast<int>(g->grid->getDimension());
    sgpp::base::DataMatrix x = make_matrix(data, m, dim);
    auto op = make_op(g, x, REF_STREAMING);
    sgpp::base::DataVector a(g->grid->getSize());
    std::memcpy(a.getPointer(), alpha, sizeof(double) * a.getSize());
    sgpp::base::DataVector s(static_cast<size_t>(m));
    std::memcpy(s.getPointer(), source, sizeof(double) * s.getSize());
    sgpp::base::DataVector r1(static_cast<size_t>(m));
    sgpp::base::DataVector r2(g->grid->getSize());
    for (int k = 0; k < reps; ++k) {
      op->mult(a, r1);
      mult_seconds[k] = op->getDuration();
      op->multTranspose(s, r2);
      multt_seconds[k] = op->getDuration();
    }
  });
}

// ModelFittingLeastSquares::fit followed by up to `rounds` adapt() calls
// (datadriven/.../fitting/ModelFittingLeastSquares.cpp:51-101, assembleSystemAndSolve :129-140)
// with the reference's own classes: a regular grid, SystemMatrixLeastSquaresIdentity with the
// default multiple-eval configuration, b = generateb(y), ConjugateGradients(maxIterations, eps)
// solving with reuse = true; adapt() refines with SurplusRefinementFunctor and zero-extends
// alpha. Returns the final grid (raw level/index rows, storage order), alpha, and the CG
// iterations of every solve (iters_out[rounds + 1], -1 where no solve happened).
int ref_fit_adapt(int basis, int dim, int level, const double* x, int64_t m, const double* y,
                  double lambda, double final_eps, int64_t final_maxit, double refine_eps,
                  int64_t refine_maxit, int64_t rounds, int64_t points, double threshold,
                  int64_t cap, int32_t* level_out, int32_t* index_out, double* alpha_out,
                  int64_t* n_out, int64_t* iters_out) {
  return guarded([&] {
    std::unique_ptr<sgpp::base::Grid> grid(
        basis == 1 ? sgpp::base::Grid::createModLinearGrid(static_cast<size_t>(dim))
                   : sgpp::base::Grid::createLinearGrid(static_cast<size_t>(dim)));
    grid->getGenerator().regular(level);
    sgpp::base::DataMatrix X = make_matrix(x, m, dim);
    sgpp::base::DataVector Y(static_cast<size_t>(m));
    std::memcpy(Y.getPointer(), y, sizeof(double) * static_cast<size_t>(m));
    sgpp::base::DataVector alpha(grid->getSize());
    alpha.setAll(0.0);
    auto solve = [&](double eps, int64_t maxit) -> int64_t {
      sgpp::datadriven::SystemMatrixLeastSquaresIdentity A(*grid, X, lambda);
      sgpp::datadriven::OperationMultipleEvalConfiguration cfg;
      A.setImplementation(cfg);
      sgpp::base::DataVector b(grid->getSize());
      A.generateb(Y, b);
      sgpp::solver::ConjugateGradients cg(static_cast<size_t>(maxit), eps);
      cg.solve(A, alpha, b, true, false, -1.0);
      return static_cast<int64_t>(cg.getNumberIterations());
    };
    for (int64_t r = 0; r <= rounds; ++r) iters_out[r] = -1;
    iters_out[0] = solve(final_eps, final_maxit);
    for (int64_t r = 0; r < rounds; ++r) {
      sgpp::base::SurplusRefinementFunctor f(alpha, static_cast<size_t>(points), threshold);
      const size_t n0 = grid->getSize();
      grid->getGenerator().refine(f);
      if (grid->getSize() <= n0) break;
      alpha.resizeZero(grid->getSize());
      iters_out[r + 1] = solve(refine_eps, refine_maxit);
    }
    auto& st = grid->getStorage();
    *n_out = static_cast<int64_t>(st.getSize());
    if (*n_out > cap) throw sgpp::base::factory_exception("ref_fit_adapt: cap too small");
    for (size_t s = 0; s < st.getSize(); ++s) {
      for (int t = 0; t < dim; ++t) {
        level_out[s * dim + t] = static_cast<int32_t>(st.getPoint(s).getLevel(t));
        index_out[s * dim + t] = static_cast<int32_t>(st.getPoint(s).getIndex(t));
      }
      alpha_out[s] = alpha[s];
    }
  });
}

// A data set through the reference's readers: format 0 = ARFF, 1 = CSV. Writes at most
// n_cap rows of data (row-major, dim_cap columns) and targets; *n / *d get the Dataset's sizes.
int ref_read_dataset(int format, const char* text, int64_t len, int has_targets, int skip_first,
                     int64_t cutoff, const int64_t* cols, int n_cols, const double* targets,
                     int n_targets, double* data, double* y, int64_t n_cap, int64_t dim_cap,
                     int64_t* n, int64_t* d) {
  return guarded([&] {
    const std::string content(text, static_cast<size_t>(len));
    std::vector<size_t> sel;
    for (int k = 0; k < n_cols; ++k) sel.push_back(static_cast<size_t>(cols[k]));
    std::vector<double> tg(targets, targets + n_targets);
    const size_t cut = cutoff < 0 ? static_cast<size_t>(-1) : static_cast<size_t>(cutoff);
    std::istringstream stream(content);
    sgpp::datadriven::Dataset ds =
        format == 0 ? sgpp::datadriven::ARFFTools::readARFF(stream, has_targets != 0, cut, sel, tg)
                    : sgpp::datadriven::CSVTools::readCSV(stream, skip_first != 0,
                                                          has_targets != 0, cut, sel, tg);
    *n = static_cast<int64_t>(ds.getNumberInstances());
    *d = static_cast<int64_t>(ds.getDimension());
    for (int64_t i = 0; i < *n && i < n_cap; ++i) {
      for (int64_t t = 0; t < *d && t < dim_cap; ++t)
        data[i * dim_cap + t] = ds.getData().get(static_cast<size_t>(i), static_cast<size_t>(t));
      if (has_targets) y[i] = ds.getTargets()[static_cast<size_t>(i)];
    }
  });
}

// Regression fit exactly as the reference learner does it: b = B^T y, then CG on
// (B^T B + lambda*M*I) alpha = b with SystemMatrixLeastSquaresIdentity.
int ref_cg_fit(void* h, int kind, const double* data, int64_t m, const double* y, double lambda,
               int64_t imax, double epsilon, int reuse, double* alpha_io, int64_t* iterations,
               double* residual) {
  return guarded([&] {
    RefGrid* g = static_cast<RefGrid*>(h);
    const int dim = static_cast<int>(g->grid->getDimension());
    sgpp::base::DataMatrix x = make_matrix(data, m, dim);
    sgpp::datadriven::SystemMatrixLeastSquaresIdentity A(*g->grid, x, lambda);
    sgpp::datadriven::OperationMultipleEvalConfiguration cfg(
        kind == REF_STREAMING ? sgpp::datadriven::OperationMultipleEvalType::STREAMING
                              : sgpp::datadriven::OperationMultipleEvalType::DEFAULT,
        sgpp::datadriven::OperationMultipleEvalSubType::DEFAULT);
    A.setImplementation(cfg);
    sgpp::base::DataVector yv(static_cast<size_t>(m));
    std::memcpy(yv.getPointer(), y, sizeof(double) * yv.getSize());
    sgpp::base::DataVector b(g->grid->getSize());
    A.generateb(yv, b);
    sgpp::base::DataVector alpha(g->grid->getSize());
    std::memcpy(alpha.getPointer(), alpha_io, sizeof(double) * alpha.getSize());
    sgpp::solver::ConjugateGradients cg(static_cast<size_t>(imax), epsilon);
    cg.solve(A, alpha, b, reuse != 0, false, 0.0);
    std::memcpy(alpha_io, alpha.getPointer(), sizeof(double) * alpha.getSize());
    *iterations = static_cast<int64_t>(cg.getNumberIterations());
    *residual = cg.getResiduum();
  });
}

}  // extern "C"

// Reference-side binding: an sgpp::base::OperationMultipleEval subclass that forwards to the
// GB300 library through its C ABI (sgmev.h). Header-only; a maintainer adds it to SG++'s
// datadriven module and one branch to the factory (see the branch below).
//
// Contract followed (base/src/sgpp/base/operation/hash/OperationMultipleEval.hpp:27-130):
//   * grid and dataset are held by reference, not owned; the dataset is copied to the device
//     once at construction (as OperationMultiEvalStreaming copies and transposes it,
//     OperationMultiEvalStreaming.cpp:13-25) and is fixed for the operator's life;
//   * result vectors arrive sized by the caller and are overwritten, never resized;
//   * prepare() re-stages the grid after refinement (SystemMatrixLeastSquaresIdentity.cpp:58,
//     LearnerBase.cpp:225);
//   * getDuration() returns the device seconds of the last call;
//   * failures throw sgpp::base::operation_exception (never exit()).
//
// Factory branches (DatadrivenOpFactory.cpp, inside `if (grid.getType() == base::GridType::Linear)`
// next to the STREAMING/OCLMP branches at :439-452, and the same inside
// `else if (grid.getType() == base::GridType::ModLinear)` next to :480-483):
//
//   if (configuration.getType() == datadriven::OperationMultipleEvalType::STREAMING &&
//       configuration.getSubType() == datadriven::OperationMultipleEvalSubType::CUDA) {
//     return new sgpp_gb300::OperationMultiEvalCudaLinear(grid, dataset, configuration);
//   }
//
// The operator takes its basis from the grid: the hat basis for Linear grids, the modified
// linear basis (LinearModifiedBasis.hpp:40-58, streamed by OperationMultiEvalModMaskStreaming)
// for ModLinear grids; any other grid type throws.
#pragma once

#include <sgpp/base/datatypes/DataMatrix.hpp>
#include <sgpp/base/datatypes/DataVector.hpp>
#include <sgpp/base/exception/operation_exception.hpp>
#include <sgpp/base/grid/Grid.hpp>
#include <sgpp/base/operation/hash/OperationMultipleEval.hpp>
#include <sgpp/datadriven/operation/hash/DatadrivenOperationCommon.hpp>

#include <string>
#include <vector>

#include "../sgmev.h"

namespace sgpp_gb300 {

class OperationMultiEvalCudaLinear : public sgpp::base::OperationMultipleEval {
 public:
  // precision: SGMEV_FP64 (default, parity with the reference), SGMEV_FP32 or SGMEV_DF64; read
  // from the configuration's parameters ("precision": "double" | "float" | "df64") when one is
  // given, together with the library's other knobs ("algo", "materialize", "materialize_multt",
  // "inner_tol", "precond", "inner_products", "system_product"; see include/sgmev.h), passed
  // through unchanged.
  OperationMultiEvalCudaLinear(sgpp::base::Grid& grid, sgpp::base::DataMatrix& dataset,
                               int precision = SGMEV_FP64)
      : OperationMultipleEval(grid, dataset), precision_(precision) {
    create();
  }

  OperationMultiEvalCudaLinear(sgpp::base::Grid& grid, sgpp::base::DataMatrix& dataset,
                               sgpp::datadriven::OperationMultipleEvalConfiguration& config)
      : OperationMultipleEval(grid, dataset), precision_(SGMEV_FP64) {
    auto params = config.getParameters();
    if (params && params->contains("precision")) {
      const std::string p = (*params)["precision"].get();
      if (p == "float") precision_ = SGMEV_FP32;
      if (p == "df64") precision_ = SGMEV_DF64;
    }
    if (params) {
      for (const char* key : {"algo", "materialize", "materialize_multt", "inner_tol", "precond",
                              "inner_products", "system_product"}) {
        if (!params->contains(key)) continue;
        knobs_ += knobs_.empty() ? "{" : ",";
        knobs_ += std::string("\"") + key + "\":\"" + (*params)[key].get() + "\"";
      }
      if (!knobs_.empty()) knobs_ += "}";
    }
    create();
  }

  ~OperationMultiEvalCudaLinear() override { sgmev_destroy(op_); }

  OperationMultiEvalCudaLinear(const OperationMultiEvalCudaLinear&) = delete;
  OperationMultiEvalCudaLinear& operator=(const OperationMultiEvalCudaLinear&) = delete;

  void mult(sgpp::base::DataVector& alpha, sgpp::base::DataVector& result) override {
    check_size(alpha.getSize(), n_grid_, "alpha");
    check_size(result.getSize(), n_data_, "result");
    check(sgmev_mult(op_, alpha.getPointer(), result.getPointer()));
  }

  void mult(sgpp::base::DataVector& alpha, sgpp::base::DataVector& result, size_t startIndexData,
            size_t endIndexData) override {
    check_size(alpha.getSize(), n_grid_, "alpha");
    check_size(result.getSize(), n_data_, "result");
    check(sgmev_mult_range(op_, alpha.getPointer(), result.getPointer(),
                           static_cast<int64_t>(startIndexData),
                           static_cast<int64_t>(endIndexData)));
  }

  void multTranspose(sgpp::base::DataVector& source, sgpp::base::DataVector& result) override {
    check_size(source.getSize(), n_data_, "source");
    check_size(result.getSize(), n_grid_, "result");
    check(sgmev_mult_transpose(op_, source.getPointer(), result.getPointer()));
  }

  void multTranspose(sgpp::base::DataVector& source, sgpp::base::DataVector& result,
                     size_t startIndexGrid, size_t endIndexGrid) override {
    check_size(source.getSize(), n_data_, "source");
    check_size(result.getSize(), n_grid_, "result");
    check(sgmev_mult_transpose_range(op_, source.getPointer(), result.getPointer(),
                                     static_cast<int64_t>(startIndexGrid),
                                     static_cast<int64_t>(endIndexGrid)));
  }

  void prepare() override {
    std::vector<double> level, index;
    export_grid(level, index);
    check(sgmev_prepare(op_, n_grid_, level.data(), index.data()));
  }

  double getDuration() override { return sgmev_get_duration(op_); }

  std::string getImplementationName() override {
    const std::string base = modlinear() ? "CUDA_MODLINEAR_" : "CUDA_LINEAR_";
    return base + (precision_ == SGMEV_FP32 ? "FP32" : (precision_ == SGMEV_DF64 ? "DF64" : "FP64"));
  }

 private:
  bool modlinear() const { return grid.getType() == sgpp::base::GridType::ModLinear; }

  void create() {
    if (grid.getType() != sgpp::base::GridType::Linear && !modlinear()) {
      throw sgpp::base::operation_exception("OperationMultiEvalCudaLinear: Linear and ModLinear "
                                            "grids only");
    }
    if (modlinear()) {
      knobs_ = knobs_.empty() ? std::string("{\"basis\":\"modlinear\"}")
                              : knobs_.substr(0, knobs_.size() - 1) + ",\"basis\":\"modlinear\"}";
    }
    std::vector<double> level, index;
    export_grid(level, index);
    n_data_ = static_cast<int64_t>(dataset.getNrows());
    const int dim = static_cast<int>(grid.getDimension());
    if (n_data_ > 0 && static_cast<int>(dataset.getNcols()) != dim) {
      throw sgpp::base::operation_exception("OperationMultiEvalCudaLinear: dataset dimension "
                                            "does not match the grid");
    }
    std::vector<double> left, right;
    auto& bb = grid.getBoundingBox();
    bool unit = true;
    for (int t = 0; t < dim; ++t) {
      const auto b = bb.getBoundary(static_cast<size_t>(t));
      left.push_back(b.leftBoundary);
      right.push_back(b.rightBoundary);
      unit = unit && b.leftBoundary == 0.0 && b.rightBoundary == 1.0;
    }
    check(sgmev_create(&op_, dim, n_grid_, level.data(), index.data(), n_data_,
                       dataset.getPointer(), unit ? nullptr : left.data(),
                       unit ? nullptr : right.data(), precision_,
                       knobs_.empty() ? nullptr : knobs_.c_str()));
  }

  void export_grid(std::vector<double>& level, std::vector<double>& index) {
    auto& storage = grid.getStorage();
    const size_t n = storage.getSize(), d = storage.getDimension();
    sgpp::base::DataMatrix lv(n, d), ix(n, d);
    storage.getLevelIndexArraysForEval(lv, ix);  // HashGridStorage.cpp:433-450
    level.assign(lv.getPointer(), lv.getPointer() + n * d);
    index.assign(ix.getPointer(), ix.getPointer() + n * d);
    n_grid_ = static_cast<int64_t>(n);
  }

  static void check_size(size_t got, int64_t want, const char* what) {
    if (static_cast<int64_t>(got) != want) {
      throw sgpp::base::operation_exception(std::string("OperationMultiEvalCudaLinear: ") + what +
                                            " has the wrong size");
    }
  }

  static void check(int rc) {
    if (rc != SGMEV_OK) {
      throw sgpp::base::operation_exception(std::string("OperationMultiEvalCudaLinear: ") +
                                            sgmev_last_error());
    }
  }

  sgmev_op* op_ = nullptr;
  int precision_;
  std::string knobs_;  // flat JSON object of string knobs, or empty
  int64_t n_grid_ = 0;
  int64_t n_data_ = 0;
};

}  // namespace sgpp_gb300

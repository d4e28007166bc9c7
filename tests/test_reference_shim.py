"""The reference-side binding (include/sgpp_gb300/OperationMultiEvalCudaLinear.hpp) compiles
against SG++'s own headers, links with SG++'s library and this project's C-ABI library, and is
driven by the reference's SystemMatrixLeastSquaresIdentity + ConjugateGradients unchanged.

Needs the reference sources (headers) and oracle/_ref/libsgpp_ref.so; skipped where they are
absent. Without a GPU the operator's constructor must throw sgpp::base::operation_exception
(no exit(), no CPU fallback); with a GPU the driver checks the CUDA results against SG++'s own
DEFAULT operator and runs a CG fit through the reference's classes.
"""
import os
import subprocess

import pytest

from conftest import ROOT
from oracle import reference_source

REF = reference_source() or ""
REF_LIB = os.path.join(ROOT, "oracle", "_ref")

DRIVER = r"""
#include <cmath>
#include <cstdio>
#include <memory>
#include <random>

#include <sgpp/base/exception/factory_exception.hpp>
#include <sgpp/base/grid/Grid.hpp>
#include <sgpp/base/operation/BaseOpFactory.hpp>
#include <sgpp/datadriven/algorithm/SystemMatrixLeastSquaresIdentity.hpp>
#include <sgpp/datadriven/operation/hash/OperationMultiEvalModMaskStreaming/OperationMultiEvalModMaskStreaming.hpp>
#include <sgpp/datadriven/operation/hash/OperationMultiEvalStreaming/OperationMultiEvalStreaming.hpp>
#include <sgpp/solver/sle/ConjugateGradients.hpp>

#include "sgpp_gb300/OperationMultiEvalCudaLinear.hpp"

using sgpp::base::DataMatrix;
using sgpp::base::DataVector;
namespace dd = sgpp::datadriven;

// The datadriven factory with the two added branches ((Linear | ModLinear), STREAMING, CUDA);
// the other routes are the reference's for these grids (DatadrivenOpFactory.cpp:436-452 and
// :479-483). Defined in the executable, it takes precedence over the library's definition, as the
// patched factory would.
namespace sgpp {
namespace op_factory {
base::OperationMultipleEval* createOperationMultipleEval(
    base::Grid& grid, base::DataMatrix& dataset, dd::OperationMultipleEvalConfiguration& cfg) {
  if (cfg.getType() == dd::OperationMultipleEvalType::DEFAULT)
    return createOperationMultipleEval(grid, dataset);
  if (grid.getType() == base::GridType::Linear &&
      cfg.getType() == dd::OperationMultipleEvalType::STREAMING) {
    if (cfg.getSubType() == dd::OperationMultipleEvalSubType::DEFAULT)
      return new dd::OperationMultiEvalStreaming(grid, dataset);
    if (cfg.getSubType() == dd::OperationMultipleEvalSubType::CUDA)
      return new sgpp_gb300::OperationMultiEvalCudaLinear(grid, dataset, cfg);
  }
  if (grid.getType() == base::GridType::ModLinear &&
      cfg.getType() == dd::OperationMultipleEvalType::STREAMING) {
    if (cfg.getSubType() == dd::OperationMultipleEvalSubType::DEFAULT)
      return new dd::OperationMultiEvalModMaskStreaming(grid, dataset);
    if (cfg.getSubType() == dd::OperationMultipleEvalSubType::CUDA)
      return new sgpp_gb300::OperationMultiEvalCudaLinear(grid, dataset, cfg);
  }
  throw base::factory_exception("OperationMultiEval is not implemented for this grid type.");
}
}  // namespace op_factory
}  // namespace sgpp

int main() {
  {
    // a grid of another basis is refused before any device work
    std::unique_ptr<sgpp::base::Grid> poly(sgpp::base::Grid::createPolyGrid(2, 3));
    poly->getGenerator().regular(2);
    DataMatrix px(4, 2);
    try {
      sgpp_gb300::OperationMultiEvalCudaLinear op(*poly, px);
      std::printf("POLY_ACCEPTED\n");
      return 4;
    } catch (sgpp::base::operation_exception& e) {
      std::printf("POLY_REJECTED %s\n", e.what());
    }
  }
  std::unique_ptr<sgpp::base::Grid> grid(sgpp::base::Grid::createLinearGrid(4));
  grid->getGenerator().regular(4);
  const size_t n = grid->getSize(), m = 2000;
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  DataMatrix x(m, 4);
  DataVector y(m);
  for (size_t j = 0; j < m; ++j) {
    for (size_t t = 0; t < 4; ++t) x.set(j, t, u(rng));
    y[j] = std::sin(3.0 * x.get(j, 0)) + x.get(j, 1) * x.get(j, 2);
  }
  DataVector alpha(n), ref(m), got(m);
  for (size_t i = 0; i < n; ++i) alpha[i] = u(rng) - 0.5;

  // reference-driven regression fit: DEFAULT operator, then the CUDA operator
  dd::SystemMatrixLeastSquaresIdentity A(*grid, x, 1e-3);
  DataVector b_ref(n), a_ref(n);
  A.generateb(y, b_ref);
  sgpp::solver::ConjugateGradients cg_ref(500, 1e-10);
  cg_ref.solve(A, a_ref, b_ref, false, false, 0.0);

  dd::OperationMultipleEvalConfiguration cuda_cfg(dd::OperationMultipleEvalType::STREAMING,
                                                  dd::OperationMultipleEvalSubType::CUDA);
  try {
    A.setImplementation(cuda_cfg);
  } catch (sgpp::base::operation_exception& e) {
    std::printf("OPERATION_EXCEPTION %s\n", e.what());
    return 3;
  }
  DataVector b(n), a(n);
  A.generateb(y, b);
  sgpp::solver::ConjugateGradients cg(500, 1e-10);
  cg.solve(A, a, b, false, false, 0.0);
  double ea = 0.0, ma = 0.0;
  for (size_t i = 0; i < n; ++i) {
    ea = std::fmax(ea, std::fabs(a[i] - a_ref[i]));
    ma = std::fmax(ma, std::fabs(a_ref[i]));
  }
  std::printf("FIT_REL_ERR %.3e iterations %zu / %zu\n", ea / ma, cg.getNumberIterations(),
              cg_ref.getNumberIterations());

  // direct operator parity against the DEFAULT operator
  sgpp_gb300::OperationMultiEvalCudaLinear cuda(*grid, x);
  std::unique_ptr<sgpp::base::OperationMultipleEval> def(
      sgpp::op_factory::createOperationMultipleEval(*grid, x));
  def->mult(alpha, ref);
  cuda.mult(alpha, got);
  double err = 0.0, mx = 0.0;
  for (size_t j = 0; j < m; ++j) {
    err = std::fmax(err, std::fabs(got[j] - ref[j]));
    mx = std::fmax(mx, std::fabs(ref[j]));
  }
  std::printf("MULT_REL_ERR %.3e\n", err / mx);

  // ModLinear: the reference's streaming route (OperationMultiEvalModMaskStreaming) against the
  // CUDA one, through the same system matrix and CG
  std::unique_ptr<sgpp::base::Grid> mgrid(sgpp::base::Grid::createModLinearGrid(4));
  mgrid->getGenerator().regular(4);
  const size_t nm = mgrid->getSize();
  dd::SystemMatrixLeastSquaresIdentity AM(*mgrid, x, 1e-3);
  AM.setImplementation(dd::OperationMultipleEvalConfiguration(
      dd::OperationMultipleEvalType::STREAMING, dd::OperationMultipleEvalSubType::DEFAULT));
  DataVector bm_ref(nm), am_ref(nm), bm(nm), am(nm);
  AM.generateb(y, bm_ref);
  sgpp::solver::ConjugateGradients cgm_ref(2000, 1e-10);
  cgm_ref.solve(AM, am_ref, bm_ref, false, false, 0.0);
  AM.setImplementation(cuda_cfg);
  AM.generateb(y, bm);
  sgpp::solver::ConjugateGradients cgm(2000, 1e-10);
  cgm.solve(AM, am, bm, false, false, 0.0);
  double em = 0.0, mm = 0.0;
  for (size_t i = 0; i < nm; ++i) {
    em = std::fmax(em, std::fabs(am[i] - am_ref[i]));
    mm = std::fmax(mm, std::fabs(am_ref[i]));
  }
  std::printf("MODLINEAR_FIT_REL_ERR %.3e iterations %zu / %zu\n", em / mm,
              cgm.getNumberIterations(), cgm_ref.getNumberIterations());
  return (err / mx < 1e-12 && ea / ma < 1e-8 && em / mm < 1e-8) ? 0 : 1;
}
"""


def _have_reference():
    return (bool(REF) and os.path.isdir(os.path.join(REF, "base", "src"))
            and os.path.exists(os.path.join(REF_LIB, "libsgpp_ref.so")))


@pytest.mark.skipif(not _have_reference(), reason="reference sources / oracle/_ref not present")
def test_shim_compiles_links_and_fails_loudly_without_gpu(lib, tmp_path):
    src = tmp_path / "driver.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "driver"
    libdir = os.path.join(ROOT, "sgpp_gb300")
    cmd = ["g++", "-std=c++17", "-O1", "-w", "-include", "cstdint", "-include", "memory",
           f"-I{REF}/base/src", f"-I{REF}/solver/src", f"-I{REF}/datadriven/src",
           f"-I{ROOT}/include", str(src), "-o", str(exe),
           f"-L{REF_LIB}", "-lsgpp_ref", f"-Wl,-rpath,{REF_LIB}",
           f"{libdir}/libsgpp_gb300.so", f"-Wl,-rpath,{libdir}", "-fopenmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert "POLY_REJECTED" in run.stdout and "ModLinear" in run.stdout, run.stdout
    if lib.sgmev_device_count() == 0:
        assert run.returncode == 3, run.stdout + run.stderr
        assert "no CUDA device" in run.stdout
    else:
        assert run.returncode == 0, run.stdout + run.stderr

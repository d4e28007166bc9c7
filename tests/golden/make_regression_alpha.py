"""FP64 solution of the regression-fit benchmark workload from the reference's own code.

Writes tests/golden/regression_d10_l5.npz: alpha of the benchmark's regression fit (regular Linear
grid d=10 level 5, N = 13,441; M = 2^20 Gaussian-mixture points from bench.make_workload with
seed 42; lambda = 1e-4) solved by SG++'s own SystemMatrixLeastSquaresIdentity (STREAMING FP64
operator) and ConjugateGradients to epsilon 1e-12
(datadriven/src/sgpp/datadriven/algorithm/SystemMatrixLeastSquaresIdentity.cpp:32-56,
solver/src/sgpp/solver/sle/ConjugateGradients.cpp:22-151), through oracle/_ref/libsgpp_ref.so.
bench.py measures the error of every benchmark fit's alpha against it.

The data are regenerated from the seed wherever the fixture is used; the fixture records checksums
of x and y so that a numpy whose generator streams differ is noticed instead of compared wrongly.

Run where the reference library was built (about 15 minutes on 8 x86 cores):

    make -f oracle/ref.mk -j8 REF=<reference checkout> && python tests/golden/make_regression_alpha.py
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from oracle import REF_STREAMING, Reference  # noqa: E402

SEED, EPSILON, IMAX = 42, 1e-12, 5000


def main():
    ref = Reference()
    ref.set_threads(os.cpu_count() or 1)
    x, y = bench.make_workload(SEED)
    g = ref.grid(bench.DIM, bench.LEVEL)
    lev, idx, _ = g.points()
    t0 = time.time()
    alpha, it, res = g.cg_fit(REF_STREAMING, x, y, bench.LAMBDA, IMAX, EPSILON)
    secs = time.time() - t0
    out = {
        "alpha": alpha, "iterations": np.int64(it), "residual": np.float64(res),
        "seed": np.int64(SEED), "epsilon": np.float64(EPSILON), "lambda": np.float64(bench.LAMBDA),
        "dim": np.int64(bench.DIM), "level": np.int64(bench.LEVEL), "m": np.int64(x.shape[0]),
        "checksums": bench.workload_checksums(x, y), "level_sum": np.int64(lev.sum()),
        "index_sum": np.int64(idx.sum()), "seconds": np.float64(secs),
        "threads": np.int64(ref.max_threads()),
    }
    path = os.path.join(HERE, "regression_d10_l5.npz")
    np.savez_compressed(path, **out)
    print(f"{path}: N={alpha.size} iterations={it} residual={res:.3e} {secs:.0f} s")


if __name__ == "__main__":
    main()

"""Grid sequence and FP64 solution of the adaptive-grid configuration from the reference's own code.

Writes tests/golden/adaptive_d8_l4.npz: the regular Linear grid d=8 level 4 (N = 1,121), data from
sgpp_gb300.adaptive.adaptive_workload (x uniform on [0, 1]^8, M = 2^19, seed 3;
y = prod 4 x_k (1 - x_k) + N(0, 0.01^2)), lambda = 1e-4, then 6 rounds of
SurplusRefinementFunctor(alpha, 40, 0.0) (largest |alpha| first), each followed by a CG solve that
starts from the zero-extended alpha — the loop of LearnerBase::train
(datadriven/src/sgpp/datadriven/application/LearnerBase.cpp:191-245) with the reference's own grid,
HashRefinement, SystemMatrixLeastSquaresIdentity (STREAMING FP64 operator) and ConjugateGradients
(epsilon 1e-12, reuse) through oracle/_ref/libsgpp_ref.so.

Recorded: the grid size after every round, the final grid's points (level/index, the reference's
storage order, which follows its hash map), the final alpha, the CG iterations of every solve and
checksums of x and y (the data are regenerated from the seed where the fixture is used).

    make -f oracle/ref.mk -j8 REF=<reference checkout> && python tests/golden/make_adaptive_fixture.py
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
from sgpp_gb300.adaptive import adaptive_workload  # noqa: E402

SEED, DIM, LEVEL, M, ROUNDS, PER_ROUND, LAM, EPSILON = 3, 8, 4, 1 << 19, 6, 40, 1e-4, 1e-12


def main():
    ref = Reference()
    ref.set_threads(os.cpu_count() or 1)
    x, y = adaptive_workload(SEED, M, DIM)
    g = ref.grid(DIM, LEVEL)
    sizes, iters = [g.size], []
    t0 = time.time()
    alpha, it, _ = g.cg_fit(REF_STREAMING, x, y, LAM, 100000, EPSILON)
    iters.append(it)
    for _ in range(ROUNDS):
        n0 = g.size
        g.refine_surplus(alpha, PER_ROUND, 0.0)
        alpha = np.concatenate([alpha, np.zeros(g.size - n0)])
        alpha, it, _ = g.cg_fit(REF_STREAMING, x, y, LAM, 100000, EPSILON, alpha0=alpha)
        sizes.append(g.size)
        iters.append(it)
        print(f"round {len(sizes) - 1}: N={g.size} iterations={it}", flush=True)
    lev, idx, _ = g.points()
    out = {"level": lev.astype(np.int8), "index": idx.astype(np.int16), "alpha": alpha,
           "sizes": np.array(sizes, np.int64), "iterations": np.array(iters, np.int64),
           "seed": np.int64(SEED), "dim": np.int64(DIM), "start_level": np.int64(LEVEL),
           "m": np.int64(M), "rounds": np.int64(ROUNDS), "per_round": np.int64(PER_ROUND),
           "lambda": np.float64(LAM), "epsilon": np.float64(EPSILON),
           "checksums": bench.workload_checksums(x, y), "seconds": np.float64(time.time() - t0)}
    path = os.path.join(HERE, "adaptive_d8_l4.npz")
    np.savez_compressed(path, **out)
    print(f"{path}: sizes={sizes} iterations={iters} {time.time() - t0:.0f} s")


if __name__ == "__main__":
    main()

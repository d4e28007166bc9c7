"""Adaptive regression loop (refine -> prepare -> warm-started fit) on the GPU operator against
the same loop run entirely by the oracle (FP64 CG, oracle refinement): identical grids round by
round (same points in the same order) and alpha within 1e-6 of the oracle's FP64 solution."""
import numpy as np
import pytest

from conftest import rel_err

import sgpp_gb300 as sg
from sgpp_gb300.adaptive import adaptive_fit

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(lib):
    if lib.sgmev_device_count() < 1:
        pytest.fail("no CUDA device visible")


@pytest.mark.parametrize("mode", [sg.SGMEV_SOLVE_MIXED, sg.SGMEV_SOLVE_PLAIN])
def test_adaptive_loop_matches_oracle(oracle, mode):
    rng = np.random.default_rng(8)
    d, level, m, rounds, per_round, lam = 4, 3, 4000, 3, 10, 1e-4
    X = rng.random((m, d))
    y = np.prod(4.0 * X * (1.0 - X), axis=1) + 0.01 * rng.standard_normal(m)
    grid = sg.Grid.createLinearGrid(d)
    grid.getGenerator().regular(level)
    alpha, records = adaptive_fit(grid, X, y, lam, rounds, per_round, epsilon=1e-11, mode=mode)
    # oracle: the same loop with the oracle's grid code and FP64 CG (warm start)
    lev, idx = oracle.regular_grid(d, level)
    a = None
    st = oracle.stream(X)
    for r in range(rounds + 1):
        lp, ix = oracle.eval_arrays(lev, idx)
        a, _, _ = st.cg_fit(lp, ix, y, lam, 100000, 1e-12, alpha0=a)
        if r < rounds:
            n0 = lev.shape[0]
            lev, idx = oracle.refine_surplus(lev, idx, a, per_round, 0.0)
            a = np.concatenate([a, np.zeros(lev.shape[0] - n0)])
    np.testing.assert_array_equal(grid.getStorage().level, lev)
    np.testing.assert_array_equal(grid.getStorage().index, idx)
    assert rel_err(alpha, a) < 1e-6
    assert [rec["n_grid"] for rec in records][-1] == lev.shape[0]

"""Batched fits (sgmev_batch_*): each problem's alpha against the oracle's FP64 CG fit, multiple
right-hand sides, continuous batching, and the same result alone and in a mix.

Tolerance: 1e-6 relative max error in alpha against the FP64 solution (the mixed-precision
target); alone vs in a mix must agree bit for bit, because every tile of a problem depends only on
that problem's own buffers and sizes.
"""
import numpy as np
import pytest

from conftest import rel_err

import sgpp_gb300 as sg

pytestmark = pytest.mark.gpu

FIT_TOL = 1e-6


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(lib):
    if lib.sgmev_device_count() < 1:
        pytest.fail("no CUDA device visible")


def _problem(seed, d, level, m, k=1, refine=0):
    rng = np.random.default_rng(seed)
    grid = sg.Grid.createLinearGrid(d)
    grid.getGenerator().regular(level)
    for _ in range(refine):
        grid.getGenerator().refine(sg.SurplusRefinementFunctor(rng.standard_normal(grid.getSize()), 5))
    x = rng.random((m, d))
    base = np.sin(3 * x[:, 0]) + x[:, -1] ** 2
    y = base[:, None] + 0.1 * rng.standard_normal((m, k))
    return grid, x, y


def _oracle_fit(oracle, grid, x, y, lam):
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    st = oracle.stream(x)
    cols = [st.cg_fit(lp, ix, y[:, c], lam, 20000, 1e-13)[0] for c in range(y.shape[1])]
    return np.stack(cols, axis=1)


MIX = [(1, 2, 5, 700), (2, 3, 4, 1500), (3, 5, 3, 2048), (4, 4, 4, 999), (5, 7, 2, 3000),
       (6, 1, 6, 257)]


def test_batch_single_rhs_matches_oracle(oracle):
    eng = sg.BatchEngine(max_slots=8, rhs=1)
    probs = {}
    for seed, d, level, m in MIX:
        grid, x, y = _problem(seed, d, level, m)
        slot = eng.add(grid, x, y, 1e-3, epsilon=1e-10)
        probs[slot] = (grid, x, y)
    steps = eng.solve(100000)
    assert steps > 0
    for slot, (grid, x, y) in probs.items():
        alpha, iters, res, phase = eng.result(slot)
        assert phase == eng.PHASE_DONE
        ref = _oracle_fit(oracle, grid, x, y, 1e-3)
        assert rel_err(alpha, ref) < FIT_TOL, (slot, rel_err(alpha, ref))
        assert res <= 1e-19  # (1e-10)^2 relative residual
    eng.close()


def test_batch_sixteen_rhs_matches_oracle(oracle):
    eng = sg.BatchEngine(max_slots=4, rhs=16)
    probs = {}
    for seed, d, level, m in [(11, 3, 4, 1200), (12, 6, 3, 2000), (13, 2, 6, 800)]:
        grid, x, y = _problem(seed, d, level, m, k=16)
        probs[eng.add(grid, x, y, 1e-3, epsilon=1e-10)] = (grid, x, y)
    eng.solve(100000)
    for slot, (grid, x, y) in probs.items():
        alpha, iters, res, phase = eng.result(slot)
        assert phase == eng.PHASE_DONE
        ref = _oracle_fit(oracle, grid, x, y, 1e-3)
        assert rel_err(alpha, ref) < FIT_TOL
    eng.close()


def test_same_result_alone_and_in_the_mix():
    grid, x, y = _problem(21, 4, 4, 1800, k=16)
    eng = sg.BatchEngine(max_slots=1, rhs=16)
    s = eng.add(grid, x, y, 1e-3, epsilon=1e-9)
    eng.solve()
    alone, it_alone, _, _ = eng.result(s)
    eng.close()

    eng = sg.BatchEngine(max_slots=6, rhs=16)
    others = [_problem(30 + k, 2 + k, 3, 500 + 300 * k, k=16) for k in range(4)]
    eng.add(*others[0][:3], 1e-3, epsilon=1e-9)
    eng.add(*others[1][:3], 1e-2, epsilon=1e-7)
    eng.step(3)                                   # others are mid-solve when ours arrives
    s = eng.add(grid, x, y, 1e-3, epsilon=1e-9)
    eng.add(*others[2][:3], 1e-3, epsilon=1e-9)
    eng.step(5)
    eng.add(*others[3][:3], 1e-4, epsilon=1e-8)
    eng.solve()
    mixed, it_mixed, _, _ = eng.result(s)
    eng.close()
    assert it_alone == it_mixed
    assert np.array_equal(alone, mixed)


def test_continuous_batching_refills_slots(oracle):
    """More problems than slots: finished problems are removed and new ones admitted."""
    eng = sg.BatchEngine(max_slots=2, rhs=1)
    queue = [_problem(40 + k, 2 + k % 4, 3 + k % 2, 600 + 100 * k) for k in range(5)]
    done = {}
    active = {}
    k = 0
    while len(done) < len(queue):
        while k < len(queue):
            slot = eng.tryAdd(*queue[k][:3], 1e-3, epsilon=1e-10)
            if slot is None:
                break
            active[slot] = k
            k += 1
        ph = eng.step(1)
        for slot in list(active):
            if ph[slot] == eng.PHASE_DONE:
                done[active.pop(slot)] = eng.result(slot)[0]
                eng.remove(slot)
    for idx, alpha in done.items():
        grid, x, y = queue[idx]
        assert rel_err(alpha, _oracle_fit(oracle, grid, x, y, 1e-3)) < FIT_TOL
    assert eng.info()["free_slots"] == 2
    eng.close()


def test_batch_admission_limits():
    eng = sg.BatchEngine(max_slots=1, rhs=1, grid_capacity=4096, data_capacity=4096)
    grid, x, y = _problem(50, 3, 3, 500)
    s = eng.add(grid, x, y, 1e-3)
    assert eng.tryAdd(grid, x, y, 1e-3) is None  # no free slot
    eng.remove(s)
    big = _problem(51, 8, 4, 5000)  # footprint beyond the pools
    assert eng.tryAdd(*big[:3], 1e-3) is None
    with pytest.raises(sg.OperationException):
        g17 = sg.Grid.createLinearGrid(17)
        g17.getGenerator().regular(1)
        eng.add(g17, np.random.default_rng(0).random((10, 17)), np.zeros(10), 1e-3)
    eng.close()

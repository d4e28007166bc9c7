"""GPU parity at the configurations' own sizes.

* Plain-method configuration (Grid::createLinearGrid(5) regular(6): N = 5,503; M = 65,536 points
  uniform on [0, 1]^5, seed 42; alpha, v ~ N(0, 1)): one mult and one multTranspose of every
  precision and algorithm against the oracle's restatement of the reference's STREAMING operator
  (pinned against the reference's own outputs by test_oracle_golden.py), at 1e-12 relative for the
  FP64-accurate kernels and 1e-4 for FP32.
* Adaptive-grid configuration (d = 8, start level 4, M = 2^19, 6 rounds of 40 refined points,
  lambda = 1e-4): the grid after every round and the final alpha against the reference's own loop
  (tests/golden/adaptive_d8_l4.npz, SG++'s grid, HashRefinement, SystemMatrixLeastSquaresIdentity
  and ConjugateGradients at epsilon 1e-12). The reference appends refined points in its hash map's
  order, so points are matched by (level, index), not by position.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_err

import bench
import sgpp_gb300 as sg
from sgpp_gb300.adaptive import adaptive_fit, adaptive_workload

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(lib):
    if lib.sgmev_device_count() < 1:
        pytest.fail("no CUDA device visible to libsgpp_gb300 (the GPU tests need one)")


def _op(grid, x, precision, algo):
    params = {"precision": precision, "algo": "subspace" if algo == "materialized" else algo}
    if algo in ("subspace", "materialized"):
        params["materialize"] = "on" if algo == "materialized" else "off"
        params["materialize_multt"] = "on" if algo == "materialized" else "off"
    cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                sg.OperationMultipleEvalSubType.CUDA,
                                                parameters=params)
    return sg.createOperationMultipleEval(grid, x, cfg)


@pytest.fixture(scope="module")
def plain_config(oracle):
    rng = np.random.default_rng(42)
    d, level, m = 5, 6, 65536
    x = rng.random((m, d))
    grid = sg.Grid.createLinearGrid(d)
    grid.getGenerator().regular(level)
    assert grid.getSize() == 5503
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    alpha = rng.standard_normal(grid.getSize())
    v = rng.standard_normal(m)
    st = oracle.stream(x)
    ref_m = st.mult(lp, ix, alpha)
    ref_t = st.mult_transpose(lp, ix, v)
    st.close()
    return grid, x, alpha, v, ref_m, ref_t


@pytest.mark.parametrize("precision,tol,algo", [("double", FP64_TOL, "dense"),
                                                ("double", FP64_TOL, "auto"),
                                                ("df64", FP64_TOL, "dense"),
                                                ("df64", FP64_TOL, "subspace"),
                                                ("df64", FP64_TOL, "materialized"),
                                                ("float", FP32_TOL, "dense"),
                                                ("float", FP32_TOL, "subspace"),
                                                ("float", FP32_TOL, "materialized")])
def test_plain_method_configuration_at_full_size(plain_config, precision, tol, algo):
    grid, x, alpha, v, ref_m, ref_t = plain_config
    op = _op(grid, x, precision, algo)
    out = np.zeros(x.shape[0])
    op.mult(alpha, out)
    assert rel_err(out, ref_m) < tol
    outt = np.zeros(grid.getSize())
    op.multTranspose(v, outt)
    assert rel_err(outt, ref_t) < tol
    op.close()


def _keyed(level, index):
    return {(tuple(l), tuple(i)): k for k, (l, i) in
            enumerate(zip(np.asarray(level, np.int64).tolist(), np.asarray(index, np.int64).tolist()))}


@pytest.mark.parametrize("mode,tol", [(sg.SGMEV_SOLVE_PLAIN, 1e-9), (sg.SGMEV_SOLVE_MIXED, 1e-6)])
def test_adaptive_configuration_matches_reference_loop(mode, tol):
    f = np.load(os.path.join(GOLDEN, "adaptive_d8_l4.npz"))
    d, level, m = int(f["dim"]), int(f["start_level"]), int(f["m"])
    x, y = adaptive_workload(int(f["seed"]), m, d)
    np.testing.assert_allclose(bench.workload_checksums(x, y), f["checksums"], rtol=1e-12)
    grid = sg.Grid.createLinearGrid(d)
    grid.getGenerator().regular(level)
    alpha, records = adaptive_fit(grid, x, y, float(f["lambda"]), int(f["rounds"]),
                                  int(f["per_round"]), epsilon=float(f["epsilon"]), mode=mode,
                                  precision="df64")
    assert [r["n_grid"] for r in records] == [int(s) for s in f["sizes"]]
    st = grid.getStorage()
    ours = _keyed(st.level, st.index)
    theirs = _keyed(f["level"], f["index"])
    assert set(ours) == set(theirs)
    order = np.array([ours[k] for k in theirs])  # reference position -> our position
    ref_alpha = f["alpha"][np.array(list(theirs.values()))]
    assert rel_err(alpha[order], ref_alpha) < tol


@pytest.mark.parametrize("batch", ["2", "4"])
def test_multt_batch_gives_the_same_bits(batch):
    """The FP16 multTranspose's batched read-modify-write (multt_batch) adds the same terms in the
    same order as one point at a time, so a mixed fit gives the same bits."""
    rng = np.random.default_rng(31)
    d, level, m = 6, 4, 30000
    grid = sg.Grid.createLinearGrid(d)
    grid.getGenerator().regular(level)
    x = rng.random((m, d))
    y = np.sin(3 * x[:, 0]) + x[:, 1] ** 2 + 0.1 * rng.standard_normal(m)
    out = []
    for b in ("1", batch):
        cfg = sg.OperationMultipleEvalConfiguration(
            sg.OperationMultipleEvalType.STREAMING, sg.OperationMultipleEvalSubType.CUDA,
            parameters={"algo": "subspace", "materialize": "on", "multt_batch": b})
        op = sg.createOperationMultipleEval(grid, x, cfg)
        a, it, _ = op.fit(y, 1e-4, 10000, 1e-10, mode=sg.SGMEV_SOLVE_MIXED)
        out.append((a, it))
        op.close()
    np.testing.assert_array_equal(out[0][0], out[1][0])
    assert out[0][1] == out[1][1]


@pytest.mark.parametrize("knob,value", [("multt_banks", "2"), ("multt_ctas", "3")])
@pytest.mark.parametrize("d,level,m,pin", [(6, 4, 30000, True), (9, 5, 20000, False)])
def test_multt_variants_reach_the_fp64_solution(oracle, knob, value, d, level, m, pin):
    """The FP16 multTranspose's variants add the terms in another order: two banks of cell sums
    (multt_banks = 2) and three CTAs per SM with FP32 cell sums only (multt_ctas = 3). The mixed
    fit still reaches the FP64 solution (the oracle's, d = 6 level 4; the default kernel's to 1e-6,
    d = 9 level 5 with 715 subspaces of 16 cells and 512 owners per CTA), within two inner
    iterations of the default kernel, with the same bits from run to run."""
    rng = np.random.default_rng(37)
    grid = sg.Grid.createLinearGrid(d)
    grid.getGenerator().regular(level)
    x = rng.random((m, d))
    y = np.sin(3 * x[:, 0]) + x[:, 1] ** 2 + 0.1 * rng.standard_normal(m)
    ref = None
    if pin:
        lp, ix = grid.getStorage().getLevelIndexArraysForEval()
        ref, _, _ = oracle.stream(x).cg_fit(lp, ix, y, 1e-4, 20000, 1e-12)
    out = {}
    for v in (None, value, value):
        params = {"algo": "subspace", "materialize": "on"}
        if v is not None:
            params[knob] = v
        cfg = sg.OperationMultipleEvalConfiguration(
            sg.OperationMultipleEvalType.STREAMING, sg.OperationMultipleEvalSubType.CUDA,
            parameters=params)
        op = sg.createOperationMultipleEval(grid, x, cfg)
        a, it, _ = op.fit(y, 1e-4, 10000, 1e-10, mode=sg.SGMEV_SOLVE_MIXED)
        op.close()
        if ref is not None:
            assert rel_err(a, ref) < 1e-6
        if v in out:
            np.testing.assert_array_equal(a, out[v][0])
        out[v] = (a, it)
    assert rel_err(out[value][0], out[None][0]) < 1e-6
    assert abs(out[None][1] - out[value][1]) <= 2


def test_mixed_fit_on_a_grid_whose_coefficients_take_mult_windows():
    """d = 6 level 7: 924 subspaces of up to 64 cells, whose FP32 coefficients (64 x 960) exceed
    the FP16 mult's shared memory; the mult then walks the subspaces in windows (704 + 220 here),
    each launch adding its sums to the output. The mixed fit streams the FP16 products through
    those windows and reaches the plain FP64-accurate fit's solution."""
    rng = np.random.default_rng(43)
    d, level, m = 6, 7, 20000
    grid = sg.Grid.createLinearGrid(d)
    grid.getGenerator().regular(level)
    x = rng.random((m, d))
    y = np.sin(3 * x[:, 0]) + x[:, 1] ** 2 + 0.1 * rng.standard_normal(m)
    cfg = sg.OperationMultipleEvalConfiguration(
        sg.OperationMultipleEvalType.STREAMING, sg.OperationMultipleEvalSubType.CUDA,
        parameters={"algo": "subspace", "materialize": "on"})
    op = sg.createOperationMultipleEval(grid, x, cfg)
    op.profile(True)
    a, it, _ = op.fit(y, 1e-3, 20000, 1e-10, mode=sg.SGMEV_SOLVE_MIXED)
    launches, _ = op.profileRead(sg.SGMEV_KERNEL_MULT_MAT16)
    op.profile(False)
    again, it2, _ = op.fit(y, 1e-3, 20000, 1e-10, mode=sg.SGMEV_SOLVE_MIXED)
    op.close()
    assert launches > 0  # the inner solves ran the FP16 materialised mult
    np.testing.assert_array_equal(a, again)
    assert it == it2
    cfg64 = sg.OperationMultipleEvalConfiguration(
        sg.OperationMultipleEvalType.STREAMING, sg.OperationMultipleEvalSubType.CUDA,
        parameters={"precision": "df64"})
    ref_op = sg.createOperationMultipleEval(grid, x, cfg64)
    ref, _, _ = ref_op.fit(y, 1e-3, 20000, 1e-10, mode=sg.SGMEV_SOLVE_PLAIN)
    ref_op.close()
    assert rel_err(a, ref) < 1e-6, rel_err(a, ref)


def test_fp32_products_on_a_grid_whose_coefficients_take_mult_windows(oracle):
    """The FP32 materialised mult takes the same windows: on the d = 6 level 7 grid its products
    match the oracle to the FP32 tolerance of the other parity tests, and they ran on the
    materialised kernels."""
    rng = np.random.default_rng(44)
    d, level, m = 6, 7, 5000
    grid = sg.Grid.createLinearGrid(d)
    grid.getGenerator().regular(level)
    n = grid.getSize()
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    x = rng.random((m, d))
    alpha = rng.standard_normal(n)
    cfg = sg.OperationMultipleEvalConfiguration(
        sg.OperationMultipleEvalType.STREAMING, sg.OperationMultipleEvalSubType.CUDA,
        parameters={"precision": "float", "algo": "subspace", "materialize": "on"})
    op = sg.createOperationMultipleEval(grid, x, cfg)
    op.profile(True)
    out = np.zeros(m)
    op.mult(alpha, out)
    launches, _ = op.profileRead(sg.SGMEV_KERNEL_MULT_MAT32)
    op.profile(False)
    op.close()
    assert launches > 0
    assert rel_err(out, oracle.mult_naive(lp, ix, x, alpha)) < 1e-4

"""16 right-hand sides on the tensor cores (sgmev_mult_block, sgmev_mult_transpose_block,
sgmev_fit_block) through the C ABI.

With params "block_products": "bf16" the block products round the materialised subspace products
to BF16 (8 significant bits: at most 2^-8 relative) and split the 16 vectors into BF16 high and
low parts (about 2^-16), accumulating in FP32, so column k of B [a_1 .. a_16] may differ from the
FP64 product B a_k by at most about 2^-8 times sum_s |p_s(x_j)| |a_k[c_s(x_j)]|: those tests hold
every entry to 2^-7 times that sum, which the oracle computes exactly as B |a_k| (hats are
non-negative). The default, FP16 operands, has its own bound (below). The block fits refine with
FP64-accurate residuals, so each column's alpha must match the oracle's FP64 CG solution to 1e-6.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_err

import bench
import sgpp_gb300 as sg

pytestmark = pytest.mark.gpu

K = sg.SGMEV_BLOCK_RHS


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(lib):
    if lib.sgmev_device_count() < 1:
        pytest.fail("no CUDA device visible to libsgpp_gb300 (the GPU tests need one)")


def _op(grid, x, **params):
    p = {"algo": "subspace", "materialize": "on"}
    p.update({k: str(v) for k, v in params.items()})
    cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                sg.OperationMultipleEvalSubType.CUDA, parameters=p)
    return sg.createOperationMultipleEval(grid, x, cfg)


def _grid(d, level):
    g = sg.Grid.createLinearGrid(d)
    g.getGenerator().regular(level)
    return g


SHAPES = [(5, 4, 3000), (10, 3, 4097), (2, 8, 2000), (8, 4, 20000), (1, 8, 513)]


@pytest.mark.parametrize("d,level,m", SHAPES)
def test_block_products_within_the_bf16_bound(oracle, d, level, m):
    rng = np.random.default_rng(500 + d * 10 + level)
    grid = _grid(d, level)
    n = grid.getSize()
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    x = rng.random((m, d))
    alpha = rng.standard_normal((K, n))
    v = rng.standard_normal((K, m))
    op = _op(grid, x, block_products="bf16")
    got_m = op.multBlock(alpha)
    got_t = op.multTransposeBlock(v)
    for k in range(K):
        ref = oracle.mult_naive(lp, ix, x, alpha[k])
        bound = 2.0 ** -7 * oracle.mult_naive(lp, ix, x, np.abs(alpha[k])) + 1e-12
        assert np.all(np.abs(got_m[k] - ref) <= bound), (k, np.max(np.abs(got_m[k] - ref) / bound))
        ref_t = oracle.mult_transpose_naive(lp, ix, x, v[k])
        bound_t = 2.0 ** -7 * oracle.mult_transpose_naive(lp, ix, x, np.abs(v[k])) + 1e-12
        assert np.all(np.abs(got_t[k] - ref_t) <= bound_t), (k, np.max(np.abs(got_t[k] - ref_t) / bound_t))
    op.close()


def test_block_products_are_reproducible_and_columns_independent(oracle):
    rng = np.random.default_rng(77)
    grid = _grid(6, 4)
    x = rng.random((5000, 6))
    op = _op(grid, x)
    a = rng.standard_normal((K, grid.getSize()))
    first = op.multBlock(a)
    again = op.multBlock(a)
    np.testing.assert_array_equal(first, again)
    # a column's result does not depend on the other columns
    b = a.copy()
    b[1:] = rng.standard_normal((K - 1, grid.getSize()))
    np.testing.assert_array_equal(op.multBlock(b)[0], first[0])
    op.close()


@pytest.mark.parametrize("d,level,m,lam", [(4, 4, 3000, 1e-3), (6, 3, 2500, 1e-4)])
def test_block_fit_matches_oracle_cg_per_column(oracle, d, level, m, lam):
    rng = np.random.default_rng(900 + d)
    grid = _grid(d, level)
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    x = rng.random((m, d))
    y = np.empty((K, m))
    y[0] = 10 * np.sin(np.pi * x[:, 0] * x[:, 1]) + 20 * (x[:, 2] - 0.5) ** 2 + 10 * x[:, 3]
    y[1:] = rng.standard_normal((K - 1, m))
    op = _op(grid, x, block_products="bf16")
    alpha, its, res = op.fitBlock(y, lam, 100000, 1e-10)
    st = oracle.stream(x)
    for k in range(K):
        ref, _, _ = st.cg_fit(lp, ix, y[k], lam, 100000, 1e-12)
        assert rel_err(alpha[k], ref) < 1e-6, (k, rel_err(alpha[k], ref))
        assert its[k] > 0
    st.close()
    op.close()


def test_block_fit_on_the_regression_workload():
    """The benchmark's regression workload (d=10 level 5, M=2^20): column 0 fits the benchmark's
    y and must match the reference's own FP64 CG solution (fixture) to 1e-6; the other columns
    fit other targets and must match this library's single-vector mixed fit to 1e-6."""
    f = np.load(os.path.join(GOLDEN, "regression_d10_l5.npz"))
    x, y0 = bench.make_workload(int(f["seed"]))
    np.testing.assert_allclose(bench.workload_checksums(x, y0), f["checksums"], rtol=1e-12)
    grid = _grid(bench.DIM, bench.LEVEL)
    rng = np.random.default_rng(5)
    y = np.empty((K, x.shape[0]))
    y[0] = y0
    y[1:] = y0 + rng.standard_normal((K - 1, x.shape[0]))
    op = _op(grid, x)
    alpha, its, res = op.fitBlock(y, bench.LAMBDA, 100000, 1e-8)
    assert rel_err(alpha[0], f["alpha"]) < 1e-6, rel_err(alpha[0], f["alpha"])
    for k in (1, K - 1):
        a1, _, _ = op.fit(y[k], bench.LAMBDA, 100000, 1e-10, mode=sg.SGMEV_SOLVE_MIXED)
        assert rel_err(alpha[k], a1) < 1e-6, (k, rel_err(alpha[k], a1))
    op.close()


def test_block_products_refuse_an_operator_without_materialised_products():
    rng = np.random.default_rng(3)
    grid = _grid(3, 3)
    x = rng.random((100, 3))
    op = _op(grid, x, materialize="off")
    with pytest.raises(sg.OperationException, match="materialised"):
        op.multBlock(np.zeros((K, grid.getSize())))
    op.close()


@pytest.mark.parametrize("d,level,m", [(5, 4, 3000), (2, 8, 2000)])
def test_mult_a_operand_in_tensor_or_shared_memory_gives_the_same_bits(d, level, m):
    """block_mult_a: the mult's A operand (the one-hot tiles of the products) in tensor memory or
    in shared memory feeds the same MMAs with the same values, so the results are identical."""
    rng = np.random.default_rng(60 + d)
    grid = _grid(d, level)
    x = rng.random((m, d))
    a = rng.standard_normal((K, grid.getSize()))
    out = []
    for where in ("tmem", "smem"):
        op = _op(grid, x, block_mult_a=where)
        out.append(op.multBlock(a))
        op.close()
    np.testing.assert_array_equal(out[0], out[1])


@pytest.mark.parametrize("window", ["1", "3"])
def test_interleaved_mma_window_gives_the_same_bits(window):
    """block_window: the MMA thread interleaves the K-steps of neighbouring stages, which feed
    different accumulators, so every accumulator still receives its MMAs in the same order."""
    rng = np.random.default_rng(61)
    grid = _grid(6, 4)
    x = rng.random((20000, 6))
    a = rng.standard_normal((K, grid.getSize()))
    v = rng.standard_normal((K, x.shape[0]))
    out = []
    for w in ("2", window):
        op = _op(grid, x, block_window=w, block_stages=3)
        out.append((op.multBlock(a), op.multTransposeBlock(v)))
        op.close()
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("teams,loads", [("1", "6"), ("3", "6"), ("4", "8")])
def test_producer_teams_give_the_same_bits(teams, loads):
    """block_teams: teams of 4 producer warps write alternate stages; every stage still holds the
    same values and the MMAs consume the stages in the same order, so the results are identical.
    d = 9 level 4 with block_mult_groups 4 runs the mult in several passes over the coefficient
    rows, and 2^15 points give each CTA several hundred stages."""
    rng = np.random.default_rng(62)
    grid = _grid(9, 4)
    x = rng.random((1 << 15, 9))
    a = rng.standard_normal((K, grid.getSize()))
    v = rng.standard_normal((K, x.shape[0]))
    out = []
    for t, nl in (("2", "6"), (teams, loads)):
        for where in ("tmem", "smem"):
            op = _op(grid, x, block_teams=t, block_loads=nl, block_stages=4, block_mult_a=where,
                     block_mult_groups=4)
            out.append((op.multBlock(a), op.multTransposeBlock(v)))
            op.close()
    for o in out[1:]:
        np.testing.assert_array_equal(out[0][0], o[0])
        np.testing.assert_array_equal(out[0][1], o[1])


def test_shapes_whose_load_buffers_would_pass_between_teams_are_refused():
    rng = np.random.default_rng(63)
    grid = _grid(3, 3)
    x = rng.random((300, 3))
    with pytest.raises(sg.OperationException):
        _op(grid, x, block_teams=4, block_loads=6, block_stages=4).multBlock(
            np.zeros((K, grid.getSize())))


# ---- FP16 operands ("block_products": "f16") ------------------------------------------------
# The products keep 11 significant bits (at most 2^-11 relative; FP16 subnormals, below 2^-14,
# keep an absolute 2^-25) and the vectors about 22 (FP16 high and low parts of the column scaled
# by a power of two), accumulating in FP32: every entry is held to 2^-10 times the oracle's
# B |a_k| plus, for the subnormal products, 2^-24 times (subspaces x max |a_k|) for mult and
# 2^-24 times sum |v_k| for multTranspose.

@pytest.mark.parametrize("d,level,m", SHAPES)
def test_f16_block_products_within_the_fp16_bound(oracle, d, level, m):
    rng = np.random.default_rng(700 + d * 10 + level)
    grid = _grid(d, level)
    n = grid.getSize()
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    x = rng.random((m, d))
    alpha = rng.standard_normal((K, n))
    v = rng.standard_normal((K, m))
    # columns far outside FP16's range and a zero column: the per-column scales bring them in
    alpha[1] *= 1e30
    alpha[2] *= 1e-30
    alpha[3] = 0.0
    v[1] *= 1e-25
    v[2] *= 1e25
    v[3] = 0.0
    n_sub = len({tuple(r) for r in np.asarray(lp).tolist()})
    op = _op(grid, x, block_products="f16")
    got_m = op.multBlock(alpha)
    got_t = op.multTransposeBlock(v)
    for k in range(K):
        ref = oracle.mult_naive(lp, ix, x, alpha[k])
        absm = oracle.mult_naive(lp, ix, x, np.abs(alpha[k]))
        bound = 2.0 ** -10 * absm + 2.0 ** -24 * n_sub * np.abs(alpha[k]).max()
        assert np.all(np.abs(got_m[k] - ref) <= bound), (k, np.max(np.abs(got_m[k] - ref) / np.maximum(bound, 1e-300)))
        ref_t = oracle.mult_transpose_naive(lp, ix, x, v[k])
        abst = oracle.mult_transpose_naive(lp, ix, x, np.abs(v[k]))
        bound_t = 2.0 ** -10 * abst + 2.0 ** -24 * np.abs(v[k]).sum()
        assert np.all(np.abs(got_t[k] - ref_t) <= bound_t), (k, np.max(np.abs(got_t[k] - ref_t) / np.maximum(bound_t, 1e-300)))
    op.close()


@pytest.mark.parametrize("d,level,m,lam", [(4, 4, 3000, 1e-3), (6, 3, 2500, 1e-4)])
def test_f16_block_fit_matches_oracle_cg_per_column(oracle, d, level, m, lam):
    rng = np.random.default_rng(910 + d)
    grid = _grid(d, level)
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    x = rng.random((m, d))
    y = np.empty((K, m))
    y[0] = 10 * np.sin(np.pi * x[:, 0] * x[:, 1]) + 20 * (x[:, 2] - 0.5) ** 2 + 10 * x[:, 3]
    y[1:] = rng.standard_normal((K - 1, m))
    y[2] *= 1e6
    op = _op(grid, x, block_products="f16")
    alpha, its, res = op.fitBlock(y, lam, 100000, 1e-10)
    st = oracle.stream(x)
    for k in range(K):
        ref, _, _ = st.cg_fit(lp, ix, y[k], lam, 100000, 1e-12)
        assert rel_err(alpha[k], ref) < 1e-6, (k, rel_err(alpha[k], ref))
    st.close()
    op.close()


def test_block_products_knob_is_checked():
    rng = np.random.default_rng(64)
    grid = _grid(3, 3)
    with pytest.raises(sg.OperationException, match="block_products"):
        _op(grid, rng.random((300, 3)), block_products="fp8")


def test_block_products_on_a_grid_the_materialised_kernels_do_not_take(oracle):
    """d = 6 level 7: 924 subspaces of up to 64 cells, whose coefficients (64 x 928 floats) do not
    fit the materialised kernels' shared memory. The block products still run: the operator builds
    the materialised products only to pack them, then frees them, and its other products stay on
    the on-the-fly kernels. Columns within the BF16 bound against the oracle; a block fit (FP16,
    the default) matches the plain FP64-accurate fit of each column."""
    rng = np.random.default_rng(71)
    d, level, m = 6, 7, 2000
    grid = _grid(d, level)
    n = grid.getSize()
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    x = rng.random((m, d))
    alpha = rng.standard_normal((K, n))
    v = rng.standard_normal((K, m))
    op = _op(grid, x, block_products="bf16")
    got_m = op.multBlock(alpha)
    got_t = op.multTransposeBlock(v)
    for k in (0, K - 1):
        ref = oracle.mult_naive(lp, ix, x, alpha[k])
        bound = 2.0 ** -7 * oracle.mult_naive(lp, ix, x, np.abs(alpha[k])) + 1e-12
        assert np.all(np.abs(got_m[k] - ref) <= bound)
        ref_t = oracle.mult_transpose_naive(lp, ix, x, v[k])
        bound_t = 2.0 ** -7 * oracle.mult_transpose_naive(lp, ix, x, np.abs(v[k])) + 1e-12
        assert np.all(np.abs(got_t[k] - ref_t) <= bound_t)
    # the single-vector products still work (on-the-fly kernels) and agree with the oracle
    out = np.zeros(m)
    op.mult(alpha[0], out)
    assert rel_err(out, oracle.mult_naive(lp, ix, x, alpha[0])) < 1e-12
    y = np.empty((K, m))
    y[0] = np.sin(3 * x[:, 0]) + x[:, 1]
    y[1:] = rng.standard_normal((K - 1, m))
    op.close()
    op = _op(grid, x)
    a_blk, its, _ = op.fitBlock(y, 1e-3, 100000, 1e-10)
    op.close()
    ref_op = _op(grid, x, precision="df64")
    for k in (0, 7, K - 1):
        a1, _, _ = ref_op.fit(y[k], 1e-3, 100000, 1e-10, mode=sg.SGMEV_SOLVE_PLAIN)
        assert rel_err(a_blk[k], a1) < 1e-6, (k, rel_err(a_blk[k], a1))
    ref_op.close()

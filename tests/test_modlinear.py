"""ModLinear grids (the modified linear basis, LinearModifiedBasis.hpp:40-58).

CPU part: the oracle's restatement against the reference's own ModLinear operators
(tests/golden/modlinear.npz, made by tests/golden/make_golden.py from the reference's compiled
OperationMultipleEvalModLinear and OperationMultiEvalModMaskStreaming) and against the golden
B^T matrices of datadriven/tests/testBT.cpp (suite TestOperationBTModLinear).

GPU part (marked gpu): the CUDA path through the C ABI against the same fixtures and the oracle,
with the tolerances of test_parity_gpu.py (FP64 kernels 1e-12, FP32 1e-4, mixed fits 1e-6).
"""
import ctypes
import json

import numpy as np
import pytest

from conftest import load_golden, rel_err

import sgpp_gb300 as sg

FP64_TOL = 1e-12
FP32_TOL = 1e-4

G = load_golden("modlinear.npz")
CASES = [str(c) for c in G["cases"]]


def _lev_idx(name):
    return G[name + "_level"].astype(np.int32), G[name + "_index"].astype(np.int32)


def _it_slack(name):
    # the ModLinear systems are worse conditioned than the Linear ones: near eps = 1e-12 the
    # residual stalls at the rounding floor, where the stopping iteration moves by up to ~6 %
    # between arithmetics (alpha is checked to 1e-9 regardless)
    return max(2, int(0.10 * int(G[name + "_iterations"])))


def _grid(name):
    lev, idx = _lev_idx(name)
    return sg.Grid.fromArrays(lev, idx, sg.GridType.ModLinear)


# ---- CPU: the oracle is the reference's algorithm ----------------------------------------------
@pytest.mark.parametrize("name", CASES)
def test_mask_arrays_match_reference(oracle, name):
    """getLevelIndexMaskArraysForModEval, bit for bit (the mask's sign bits included)."""
    level, index, mask, offset = oracle.mod_arrays(*_lev_idx(name))
    np.testing.assert_array_equal(level, G[name + "_mask_level"])
    np.testing.assert_array_equal(index, G[name + "_mask_index"])
    np.testing.assert_array_equal(mask.view(np.uint64), G[name + "_mask_bits"])
    np.testing.assert_array_equal(offset, G[name + "_mask_offset"])


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_operators(oracle, name):
    lev, idx = _lev_idx(name)
    x = G[name + "_x"]
    st = oracle.stream(x)
    arrays = oracle.mod_arrays(lev, idx)
    assert rel_err(st.mult_mod(arrays, G[name + "_alpha"]), G[name + "_mult_streaming"]) < 1e-14
    assert rel_err(st.mult_transpose_mod(arrays, G[name + "_v"]),
                   G[name + "_multt_streaming"]) < 1e-14
    assert rel_err(oracle.mult_naive_mod(lev, idx, x, G[name + "_alpha"]),
                   G[name + "_mult_default"]) < 1e-14
    assert rel_err(oracle.mult_transpose_naive_mod(lev, idx, x, G[name + "_v"]),
                   G[name + "_multt_default"]) < 1e-14


def test_oracle_extrapolates_outside_the_cube_like_streaming(oracle):
    lev, idx = _lev_idx("outside")
    st = oracle.stream(G["outside_x"])
    arrays = oracle.mod_arrays(lev, idx)
    assert rel_err(st.mult_mod(arrays, G["outside_alpha"]), G["outside_mult_streaming"]) < 1e-14
    assert rel_err(st.mult_transpose_mod(arrays, G["outside_v"]),
                   G["outside_multt_streaming"]) < 1e-14


def test_modified_basis_known_values(oracle):
    """LinearModifiedBasis::eval at a few hand-checked points."""
    e = oracle.modlinear_eval
    assert e(1, 1, 0.0) == 1.0 and e(1, 1, 0.73) == 1.0 and e(1, 1, 1.0) == 1.0
    assert e(2, 1, 0.0) == 2.0 and e(2, 1, 0.25) == 1.0 and e(2, 1, 0.5) == 0.0
    assert e(2, 1, 0.75) == 0.0
    assert e(2, 3, 1.0) == 2.0 and e(2, 3, 0.75) == 1.0 and e(2, 3, 0.5) == 0.0
    assert e(3, 3, 0.375) == 1.0 and e(3, 3, 0.3125) == 0.5 and e(3, 3, 0.5) == 0.0
    assert e(3, 1, 0.0625) == 1.5 and e(3, 7, 0.9375) == 1.5


@pytest.mark.parametrize("key", ["bt_d1_l3", "bt_d1_l5", "bt_d3_l3", "bt_d3_l4"])
def test_bt_golden_matrices_modlinear(oracle, key):
    """datadriven/tests/testBT.cpp (TestOperationBTModLinear): B column by column via mult(e_i);
    row sums in order and sorted column sums within 1e-5 % of the golden files."""
    d, l = int(G[key + "_dim"]), int(G[key + "_level"])
    x = G[key + "_x"]
    lev, idx = oracle.regular_grid(d, l)
    n = lev.shape[0]
    B = np.stack([oracle.mult_naive_mod(lev, idx, x, np.eye(n)[i]) for i in range(n)], axis=1)
    np.testing.assert_allclose(B.sum(axis=1), G[key + "_row_sums"], rtol=1e-7, atol=1e-9)
    np.testing.assert_allclose(np.sort(B.sum(axis=0)), G[key + "_col_sums_sorted"], rtol=1e-7,
                               atol=1e-9)


@pytest.mark.parametrize("name", ["fit_d4_l4", "fit_d6_l3"])
def test_oracle_cg_fit_matches_reference(oracle, name):
    lev, idx = _lev_idx(name)
    st = oracle.stream(G[name + "_x"])
    alpha, it, _ = st.cg_fit_mod(oracle.mod_arrays(lev, idx), G[name + "_y"],
                                 float(G[name + "_lambda"]), 1000, 1e-12)
    assert rel_err(alpha, G[name + "_alpha"]) < 1e-9
    assert abs(it - int(G[name + "_iterations"])) <= _it_slack(name)


def test_grid_type_and_factory_routing():
    g = sg.Grid.createModLinearGrid(3)
    assert g.getType() == sg.GridType.ModLinear
    g.getGenerator().regular(3)
    lin = sg.Grid.createLinearGrid(3)
    lin.getGenerator().regular(3)
    # the same points as the Linear grid of the same level
    np.testing.assert_array_equal(g.getStorage().level, lin.getStorage().level)
    np.testing.assert_array_equal(g.getStorage().index, lin.getStorage().index)


def test_unknown_basis_is_rejected(lib):
    """The basis knob is validated before any device work (no GPU needed)."""
    h = ctypes.c_void_p(None)
    lp = np.array([[2.0]])
    ix = np.array([[1.0]])
    x = np.array([[0.5]])
    rc = lib.sgmev_create(ctypes.byref(h), 1, 1, lp.ctypes.data, ix.ctypes.data, 1,
                          x.ctypes.data, None, None, sg.SGMEV_FP64,
                          json.dumps({"basis": "prewavelet"}).encode())
    assert rc == sg.SGMEV_ERR_INVALID
    assert b"basis" in lib.sgmev_last_error()


# ---- GPU: the CUDA path -----------------------------------------------------------------------
def _op(grid, x, precision="double", algo="auto", **extra):
    params = {"precision": precision, "algo": "subspace" if algo == "materialized" else algo}
    if algo in ("subspace", "materialized"):
        params["materialize"] = "on" if algo == "materialized" else "off"
        params["materialize_multt"] = "on" if algo == "materialized" else "off"
    params.update(extra)
    cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                sg.OperationMultipleEvalSubType.CUDA,
                                                parameters=params)
    return sg.createOperationMultipleEval(grid, x, cfg)


PRECISIONS = [("double", FP64_TOL, "auto"), ("df64", FP64_TOL, "dense"),
              ("df64", FP64_TOL, "materialized"), ("float", FP32_TOL, "dense"),
              ("float", FP32_TOL, "subspace"), ("float", FP32_TOL, "materialized")]


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol,algo", PRECISIONS)
@pytest.mark.parametrize("name", CASES)
def test_gpu_mult_and_transpose_match_reference(name, precision, tol, algo):
    grid = _grid(name)
    x = G[name + "_x"]
    op = _op(grid, x, precision, algo)
    out = np.zeros(x.shape[0])
    op.mult(G[name + "_alpha"], out)
    assert rel_err(out, G[name + "_mult_streaming"]) < tol
    outt = np.zeros(grid.getSize())
    op.multTranspose(G[name + "_v"], outt)
    assert rel_err(outt, G[name + "_multt_streaming"]) < tol


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol,algo", PRECISIONS)
def test_gpu_extrapolation_outside_the_cube(precision, tol, algo):
    """Data outside [0, 1]: the boundary-adjacent functions extrapolate as in the reference's
    STREAMING operator (the materialised products step aside for the dense kernels)."""
    grid = _grid("outside")
    x = G["outside_x"]
    op = _op(grid, x, precision, algo)
    out = np.zeros(x.shape[0])
    op.mult(G["outside_alpha"], out)
    assert rel_err(out, G["outside_mult_streaming"]) < tol
    outt = np.zeros(grid.getSize())
    op.multTranspose(G["outside_v"], outt)
    assert rel_err(outt, G["outside_multt_streaming"]) < tol


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["bt_d1_l3", "bt_d1_l5", "bt_d3_l3", "bt_d3_l4"])
def test_gpu_bt_golden_matrices_modlinear(key):
    d, l = int(G[key + "_dim"]), int(G[key + "_level"])
    x = G[key + "_x"]
    grid = sg.Grid.createModLinearGrid(d)
    grid.getGenerator().regular(l)
    n = grid.getSize()
    op = _op(grid, x)
    B = np.zeros((x.shape[0], n))
    col = np.zeros(x.shape[0])
    for i in range(n):
        op.mult(np.eye(n)[i], col)
        B[:, i] = col
    np.testing.assert_allclose(B.sum(axis=1), G[key + "_row_sums"], rtol=1e-7, atol=1e-9)
    np.testing.assert_allclose(np.sort(B.sum(axis=0)), G[key + "_col_sums_sorted"], rtol=1e-7,
                               atol=1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["double", "df64"])
@pytest.mark.parametrize("name", ["fit_d4_l4", "fit_d6_l3"])
def test_gpu_cg_fit_matches_reference(name, precision):
    grid = _grid(name)
    op = _op(grid, G[name + "_x"], precision)
    alpha, it, _ = op.fit(G[name + "_y"], float(G[name + "_lambda"]), 1000, 1e-12)
    assert rel_err(alpha, G[name + "_alpha"]) < 1e-9
    assert abs(it - int(G[name + "_iterations"])) <= _it_slack(name)


@pytest.mark.gpu
@pytest.mark.parametrize("precond", ["none", "jacobi"])
@pytest.mark.parametrize("products", ["half", "float"])
@pytest.mark.parametrize("name", ["fit_d4_l4", "fit_d6_l3"])
def test_gpu_mixed_fit_within_1e6(name, products, precond):
    grid = _grid(name)
    op = _op(grid, G[name + "_x"], "double", inner_products=products, precond=precond)
    alpha, _, _ = op.fit(G[name + "_y"], float(G[name + "_lambda"]), 5000, 1e-10,
                         mode=sg.SGMEV_SOLVE_MIXED)
    assert rel_err(alpha, G[name + "_alpha"]) < 1e-6


@pytest.mark.gpu
def test_gpu_reference_callers_drive_the_operator_unchanged():
    """SystemMatrixLeastSquaresIdentity + ConjugateGradients on the host, CUDA op inside."""
    name = "fit_d4_l4"
    grid = _grid(name)
    A = sg.SystemMatrixLeastSquaresIdentity(grid, G[name + "_x"], float(G[name + "_lambda"]))
    b = np.zeros(grid.getSize())
    A.generateb(G[name + "_y"], b)
    alpha = np.zeros(grid.getSize())
    cg = sg.ConjugateGradients(1000, 1e-12)
    cg.solve(A, alpha, b, False, False, 0.0)
    assert rel_err(alpha, G[name + "_alpha"]) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("dim,level", [(1, 14), (2, 9), (3, 6), (12, 3)])
@pytest.mark.parametrize("precision,tol,algo", [("float", FP32_TOL, "dense"),
                                                ("float", FP32_TOL, "materialized"),
                                                ("df64", FP64_TOL, "dense"),
                                                ("df64", FP64_TOL, "materialized"),
                                                ("double", FP64_TOL, "dense")])
def test_gpu_shapes_faces_and_cell_boundaries(oracle, dim, level, precision, tol, algo):
    """Deep levels and many narrow subspaces, with points on cell boundaries and on the faces
    x = 0 and x = 1 (where a boundary-adjacent function reaches 2)."""
    rng = np.random.default_rng(dim * 1000 + level)
    grid = sg.Grid.createModLinearGrid(dim)
    grid.getGenerator().regular(level)
    m = 20000
    x = rng.random((m, dim))
    x[:20] = np.round(x[:20] * 2 ** level) / 2 ** level
    x[20:40] = rng.integers(0, 2, size=(20, dim)).astype(np.float64)
    st = grid.getStorage()
    arrays = oracle.mod_arrays(st.level, st.index)
    a = rng.standard_normal(grid.getSize())
    v = rng.standard_normal(m)
    if precision == "float":
        tol = max(tol, 2.0 ** (level - 23))
    elif precision == "df64":
        tol = max(tol, 2.0 ** (level - 47))
    ref = oracle.stream(x)
    op = _op(grid, x, precision, algo)
    out, outt = np.zeros(m), np.zeros(grid.getSize())
    op.mult(a, out)
    op.multTranspose(v, outt)
    assert rel_err(out, ref.mult_mod(arrays, a)) < tol
    assert rel_err(outt, ref.mult_transpose_mod(arrays, v)) < tol


@pytest.mark.gpu
def test_gpu_mixed_fit_at_a_larger_size(oracle):
    """d = 8, level 4 on 60,000 points through the materialised FP16 inner products, against the
    oracle's FP64 CG on the ModLinear streaming layout."""
    rng = np.random.default_rng(2026)
    grid = sg.Grid.createModLinearGrid(8)
    grid.getGenerator().regular(4)
    x = rng.random((60000, 8))
    y = np.sin(3 * x[:, 0]) * x[:, 1] + (x[:, 2] - 0.3) ** 2 + 0.05 * rng.standard_normal(60000)
    op = _op(grid, x)
    alpha, _, _ = op.fit(y, 1e-4, 5000, 1e-10, mode=sg.SGMEV_SOLVE_MIXED)
    st = grid.getStorage()
    ref, _, _ = oracle.stream(x).cg_fit_mod(oracle.mod_arrays(st.level, st.index), y, 1e-4, 5000,
                                            1e-12)
    assert rel_err(alpha, ref) < 1e-6

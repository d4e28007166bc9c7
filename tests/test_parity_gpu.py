"""GPU parity: the CUDA path (through the C ABI) against the reference's own FP64 outputs
(tests/golden, produced by the reference's compiled code) and against the oracle.

Tolerances (max abs error / max abs reference value):
  FP64 kernels   1e-12   (the reference's STREAMING-vs-DEFAULT agreement is ~1e-14), both the
                 native-FP64 ("double") and the float-float ("df64") kernels
  FP32 kernels   1e-4    (x is rounded to float: |dt| <= 2^l * 2^-24 per dimension)
  fits           1e-9 in alpha for the plain FP64 CG, 1e-6 for the mixed-precision fit
"""
import numpy as np
import pytest

from conftest import load_golden, rel_err

import sgpp_gb300 as sg

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(lib):
    if lib.sgmev_device_count() < 1:
        pytest.fail("no CUDA device visible to libsgpp_gb300 (the GPU tests need one)")


def _grid_from(g, name):
    return sg.Grid.fromArrays(g[name + "_level"].astype(np.int32),
                              g[name + "_index"].astype(np.int32))


def _op(grid, x, precision="double", algo="auto"):
    """algo: "auto", "dense", "subspace" (hats evaluated on every call) or "materialized"
    (subspace products kept in device memory, for mult and multTranspose)."""
    params = {"precision": precision, "algo": "subspace" if algo == "materialized" else algo}
    if algo in ("subspace", "materialized"):
        params["materialize"] = "on" if algo == "materialized" else "off"
        params["materialize_multt"] = "on" if algo == "materialized" else "off"
    cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                sg.OperationMultipleEvalSubType.CUDA,
                                                parameters=params)
    return sg.createOperationMultipleEval(grid, x, cfg)


MULTEVAL = [str(c) for c in load_golden("multeval.npz")["cases"]]


@pytest.mark.parametrize("precision,tol,algo", [("double", FP64_TOL, "auto"),
                                                ("df64", FP64_TOL, "dense"),
                                                ("df64", FP64_TOL, "subspace"),
                                                ("df64", FP64_TOL, "materialized"),
                                                ("float", FP32_TOL, "dense"),
                                                ("float", FP32_TOL, "subspace"),
                                                ("float", FP32_TOL, "materialized")])
@pytest.mark.parametrize("name", MULTEVAL)
def test_mult_and_transpose_match_reference(name, precision, tol, algo):
    g = load_golden("multeval.npz")
    grid = _grid_from(g, name)
    x = g[name + "_x"]
    op = _op(grid, x, precision, algo)
    out = np.zeros(x.shape[0])
    op.mult(g[name + "_alpha"], out)
    assert rel_err(out, g[name + "_mult_default"]) < tol
    outt = np.zeros(grid.getSize())
    op.multTranspose(g[name + "_v"], outt)
    assert rel_err(outt, g[name + "_multt_default"]) < tol
    assert op.getDuration() > 0.0


@pytest.mark.parametrize("precision", ["double", "df64"])
@pytest.mark.parametrize("name", ["bb_kat", "bb_rand"])
def test_bounding_box_matches_reference(name, precision):
    g = load_golden("multeval.npz")
    grid = _grid_from(g, name)
    bb = sg.BoundingBox(grid.getDimension())
    for t, (lo, hi) in enumerate(zip(g[name + "_bb_left"], g[name + "_bb_right"])):
        bb.setBoundary(t, sg.BoundingBox1D(lo, hi))
    grid.getStorage().setBoundingBox(bb)
    x = g[name + "_x"]
    op = _op(grid, x, precision)
    out = np.zeros(x.shape[0])
    op.mult(g[name + "_alpha"], out)
    assert rel_err(out, g[name + "_mult_default"]) < FP64_TOL
    outt = np.zeros(grid.getSize())
    op.multTranspose(g[name + "_v"], outt)
    assert rel_err(outt, g[name + "_multt_default"]) < FP64_TOL
    if name == "bb_kat":
        # base/tests/test_OperationMultipleEval.cpp:71-78
        np.testing.assert_allclose(out, [0.0, 2.72, 1.64], rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("name", ["d1_l3", "d1_l5", "d3_l3", "d3_l4"])
def test_bt_golden_matrices(name):
    """datadriven/tests/testBT.cpp (TestOperationBTLinear) through the CUDA operator."""
    g = load_golden("bt_linear.npz")
    d, l = int(g[name + "_dim"]), int(g[name + "_level"])
    grid = sg.Grid.createLinearGrid(d)
    grid.getGenerator().regular(l)
    x = g[name + "_x"]
    op = _op(grid, x)
    n = grid.getSize()
    B = np.zeros((x.shape[0], n))
    col = np.zeros(x.shape[0])
    for i in range(n):
        e = np.zeros(n)
        e[i] = 1.0
        op.mult(e, col)
        B[:, i] = col
    np.testing.assert_allclose(B.sum(axis=1), g[name + "_row_sums"], rtol=1e-7, atol=1e-9)
    np.testing.assert_allclose(np.sort(B.sum(axis=0)), g[name + "_col_sums_sorted"], rtol=1e-7,
                               atol=1e-9)


def test_results_are_bitwise_reproducible():
    g = load_golden("multeval.npz")
    name = "d5_l6_m2000"
    grid = _grid_from(g, name)
    x = g[name + "_x"]
    for prec, algo in (("double", "auto"), ("df64", "auto"), ("float", "dense"),
                       ("float", "subspace"), ("float", "materialized")):
        op = _op(grid, x, prec, algo)
        a = np.zeros(x.shape[0])
        b = np.zeros(x.shape[0])
        op.mult(g[name + "_alpha"], a)
        op.mult(g[name + "_alpha"], b)
        assert np.array_equal(a, b)
        ta = np.zeros(grid.getSize())
        tb = np.zeros(grid.getSize())
        op.multTranspose(g[name + "_v"], ta)
        op.multTranspose(g[name + "_v"], tb)
        assert np.array_equal(ta, tb)


@pytest.mark.parametrize("precision", ["double", "df64"])
def test_ranged_variants(oracle, precision):
    rng = np.random.default_rng(5)
    grid = sg.Grid.createLinearGrid(4)
    grid.getGenerator().regular(5)
    x = rng.random((5000, 4))
    a = rng.standard_normal(grid.getSize())
    v = rng.standard_normal(5000)
    op = _op(grid, x, precision)
    full = np.zeros(5000)
    op.mult(a, full)
    fullt = np.zeros(grid.getSize())
    op.multTranspose(v, fullt)
    for s, e in [(0, 5000), (0, 1), (123, 4321), (4999, 5000), (2048, 2048)]:
        part = np.full(5000, np.nan)
        op.mult(a, part, s, e)
        assert rel_err(part[s:e], full[s:e]) < FP64_TOL if e > s else True
        assert np.isnan(part[:s]).all() and np.isnan(part[e:]).all()
    n = grid.getSize()
    for s, e in [(0, n), (0, 1), (17, n - 5), (n - 1, n)]:
        part = np.full(n, np.nan)
        op.multTranspose(v, part, s, e)
        assert rel_err(part[s:e], fullt[s:e]) < FP64_TOL
        assert np.isnan(part[:s]).all() and np.isnan(part[e:]).all()


def test_edge_sizes(oracle):
    rng = np.random.default_rng(9)
    # single grid point, d = 1
    grid = sg.Grid.createLinearGrid(1)
    grid.getGenerator().regular(1)
    x = np.array([[0.0], [0.25], [0.5], [1.0], [0.75]])
    op = _op(grid, x)
    out = np.zeros(5)
    op.mult(np.array([2.0]), out)
    np.testing.assert_allclose(out, [0.0, 1.0, 2.0, 0.0, 1.0], rtol=0, atol=1e-15)
    # empty data set: mult writes nothing, multTranspose gives zeros
    grid = sg.Grid.createLinearGrid(3)
    grid.getGenerator().regular(3)
    op = _op(grid, np.zeros((0, 3)))
    op.mult(np.ones(grid.getSize()), np.zeros(0))
    outt = np.full(grid.getSize(), 7.0)
    op.multTranspose(np.zeros(0), outt)
    assert not outt.any()
    # high dimension goes through the generic (non-templated) kernels
    d = 20
    grid = sg.Grid.createLinearGrid(d)
    grid.getGenerator().regular(2)
    x = rng.random((333, d))
    a = rng.standard_normal(grid.getSize())
    v = rng.standard_normal(333)
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    for prec, tol in (("double", FP64_TOL), ("df64", FP64_TOL), ("float", FP32_TOL)):
        op = _op(grid, x, prec)
        out = np.zeros(333)
        op.mult(a, out)
        assert rel_err(out, oracle.mult_naive(lp, ix, x, a)) < tol
        outt = np.zeros(grid.getSize())
        op.multTranspose(v, outt)
        assert rel_err(outt, oracle.mult_transpose_naive(lp, ix, x, v)) < tol


def test_wrong_sizes_raise():
    grid = sg.Grid.createLinearGrid(2)
    grid.getGenerator().regular(3)
    op = _op(grid, np.random.default_rng(0).random((10, 2)))
    with pytest.raises(sg.OperationException):
        op.mult(np.ones(grid.getSize() - 1), np.zeros(10))
    with pytest.raises(sg.OperationException):
        op.multTranspose(np.ones(10), np.zeros(grid.getSize() - 1))
    with pytest.raises(sg.OperationException):
        op.mult(np.ones(grid.getSize()), np.zeros(10), 5, 11)


def test_prepare_after_refinement(oracle):
    rng = np.random.default_rng(11)
    grid = sg.Grid.createLinearGrid(6)
    grid.getGenerator().regular(3)
    x = rng.random((3000, 6))
    op = _op(grid, x)
    for _ in range(3):
        grid.getGenerator().refine(sg.SurplusRefinementFunctor(rng.standard_normal(grid.getSize()), 25))
        op.prepare()
        a = rng.standard_normal(grid.getSize())
        out = np.zeros(3000)
        op.mult(a, out)
        lp, ix = grid.getStorage().getLevelIndexArraysForEval()
        assert rel_err(out, oracle.mult_naive(lp, ix, x, a)) < FP64_TOL
        v = rng.standard_normal(3000)
        outt = np.zeros(grid.getSize())
        op.multTranspose(v, outt)
        assert rel_err(outt, oracle.stream(x).mult_transpose(lp, ix, v)) < FP64_TOL


def test_system_apply_matches_oracle(oracle):
    rng = np.random.default_rng(13)
    grid = sg.Grid.createLinearGrid(5)
    grid.getGenerator().regular(4)
    x = rng.random((4000, 5))
    a = rng.standard_normal(grid.getSize())
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    st = oracle.stream(x)
    lam_m = 4000 * 1e-3
    ref = st.mult_transpose(lp, ix, st.mult(lp, ix, a)) + lam_m * a
    op = _op(grid, x)
    out = np.zeros(grid.getSize())
    op.systemApply(a, out, lam_m)
    assert rel_err(out, ref) < FP64_TOL
    opdf = _op(grid, x, "df64")
    opdf.systemApply(a, out, lam_m)
    assert rel_err(out, ref) < FP64_TOL
    for algo in ("dense", "subspace", "materialized"):
        op32 = _op(grid, x, "float", algo)
        op32.systemApply(a, out, lam_m)
        assert rel_err(out, ref) < FP32_TOL


@pytest.mark.parametrize("route", ["separate", "fused"])
def test_system_product_knob(oracle, route):
    """params "system_product": FP32 system products on the materialised products as the mult and
    multTranspose kernels (default) or one fused pass; both match the oracle, and a plain FP32 fit
    through either reaches the FP32 solution. Other values raise."""
    rng = np.random.default_rng(17)
    grid = sg.Grid.createLinearGrid(5)
    grid.getGenerator().regular(4)
    x = rng.random((5000, 5))
    a = rng.standard_normal(grid.getSize())
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    st = oracle.stream(x)
    lam_m = 5000 * 1e-3
    ref = st.mult_transpose(lp, ix, st.mult(lp, ix, a)) + lam_m * a
    cfg = sg.OperationMultipleEvalConfiguration(
        sg.OperationMultipleEvalType.STREAMING, sg.OperationMultipleEvalSubType.CUDA,
        parameters={"precision": "float", "algo": "subspace", "materialize": "on",
                    "system_product": route})
    op = sg.createOperationMultipleEval(grid, x, cfg)
    out = np.zeros(grid.getSize())
    op.systemApply(a, out, lam_m)
    assert rel_err(out, ref) < FP32_TOL
    y = np.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2]
    alpha, _, _ = op.fit(y, 1e-3, 2000, 1e-6)
    want, _, _ = st.cg_fit(lp, ix, y, 1e-3, 2000, 1e-10)
    assert rel_err(alpha, want) < 1e-4
    op.close()
    bad = sg.OperationMultipleEvalConfiguration(
        sg.OperationMultipleEvalType.STREAMING, sg.OperationMultipleEvalSubType.CUDA,
        parameters={"system_product": "both"})
    with pytest.raises(Exception):
        sg.createOperationMultipleEval(grid, x, bad)


@pytest.mark.parametrize("precision", ["double", "df64"])
@pytest.mark.parametrize("name", ["d4_l4", "d6_l3"])
def test_device_cg_fit_matches_reference(name, precision):
    g = load_golden("cgfit.npz")
    grid = _grid_from(g, name)
    op = _op(grid, g[name + "_x"], precision)
    alpha, it, res = op.fit(g[name + "_y"], float(g[name + "_lambda"]), 1000, 1e-12)
    assert rel_err(alpha, g[name + "_alpha"]) < 1e-9
    assert abs(it - int(g[name + "_iterations"])) <= 2


@pytest.mark.parametrize("precond", ["jacobi", "none"])
@pytest.mark.parametrize("mode", [sg.SGMEV_SOLVE_MIXED, sg.SGMEV_SOLVE_MIXED_NATIVE64])
@pytest.mark.parametrize("name", ["d4_l4", "d6_l3"])
def test_mixed_precision_fit_within_1e6(name, mode, precond):
    g = load_golden("cgfit.npz")
    grid = _grid_from(g, name)
    cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                sg.OperationMultipleEvalSubType.CUDA,
                                                parameters={"precond": precond})
    op = sg.createOperationMultipleEval(grid, g[name + "_x"], cfg)
    alpha, it, res = op.fit(g[name + "_y"], float(g[name + "_lambda"]), 5000, 1e-10, mode=mode)
    assert rel_err(alpha, g[name + "_alpha"]) < 1e-6


def test_mixed_fit_after_refinement_uses_fresh_preconditioner(oracle):
    """prepare() after refinement invalidates the cached diagonal: the next mixed fit must still
    reach the FP64 solution (checked against the oracle's FP64 CG)."""
    rng = np.random.default_rng(31)
    grid = sg.Grid.createLinearGrid(4)
    grid.getGenerator().regular(3)
    x = rng.random((3000, 4))
    y = np.sin(4 * x[:, 0]) * x[:, 1] + x[:, 2] ** 2
    op = _op(grid, x)
    a0, _, _ = op.fit(y, 1e-3, 5000, 1e-10, mode=sg.SGMEV_SOLVE_MIXED)
    grid.getGenerator().refine(sg.SurplusRefinementFunctor(a0, 10))
    op.prepare()
    a1, _, _ = op.fit(y, 1e-3, 5000, 1e-10, mode=sg.SGMEV_SOLVE_MIXED)
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    ref, _, _ = oracle.stream(x).cg_fit(lp, ix, y, 1e-3, 5000, 1e-12)
    assert rel_err(a1, ref) < 1e-6


def test_reference_callers_drive_the_operator_unchanged():
    """SystemMatrixLeastSquaresIdentity + ConjugateGradients on the host, CUDA op inside."""
    g = load_golden("cgfit.npz")
    name = "d4_l4"
    grid = _grid_from(g, name)
    A = sg.SystemMatrixLeastSquaresIdentity(grid, g[name + "_x"], float(g[name + "_lambda"]))
    b = np.zeros(grid.getSize())
    A.generateb(g[name + "_y"], b)
    alpha = np.zeros(grid.getSize())
    cg = sg.ConjugateGradients(1000, 1e-12)
    cg.solve(A, alpha, b, False, False, 0.0)
    assert rel_err(alpha, g[name + "_alpha"]) < 1e-9
    assert abs(cg.getNumberIterations() - int(g[name + "_iterations"])) <= 2


@pytest.mark.parametrize("algo", ["dense", "subspace", "materialized"])
def test_df64_at_cell_boundaries_and_outside_the_cube(oracle, algo):
    """Coordinates on dyadic cell boundaries, one double ulp and 1e-9 either side of them, on the
    cube faces and outside [0, 1]: the float-float kernels follow the FP64 value, not its float
    high part, in the choice of cell (checked against the oracle's FP64 evaluation)."""
    rng = np.random.default_rng(41)
    dim, level = 5, 5
    grid = sg.Grid.createLinearGrid(dim)
    grid.getGenerator().regular(level)
    m = 20000
    nodes = rng.integers(0, 2 ** level + 1, (m, dim)) / 2.0 ** level
    shift = rng.choice([0.0, 1e-9, -1e-9, 3e-8, -3e-8, 1e-12], (m, dim))
    x = nodes + shift
    ulp = rng.integers(0, 3, (m, dim))  # 0: as is, 1: next double up, 2: next double down
    x = np.where(ulp == 1, np.nextafter(x, 2.0), np.where(ulp == 2, np.nextafter(x, -1.0), x))
    x[:50, 0] = -1e-9
    x[50:100, 1] = 1.0 + 1e-9
    x[100:200] = rng.random((100, dim))
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    a = rng.standard_normal(grid.getSize())
    ref = oracle.stream(x).mult(lp, ix, a)
    op = _op(grid, x, "df64", algo)
    out = np.zeros(m)
    op.mult(a, out)
    assert rel_err(out, ref) < FP64_TOL


@pytest.mark.parametrize("dim,level", [(1, 14), (2, 9), (3, 6), (12, 3)])
@pytest.mark.parametrize("precision,tol,algo", [("float", FP32_TOL, "subspace"),
                                                ("float", FP32_TOL, "materialized"),
                                                ("df64", FP64_TOL, "subspace"),
                                                ("df64", FP64_TOL, "materialized")])
def test_subspace_shapes_match_oracle(oracle, dim, level, precision, tol, algo):
    """Subspace kernels on grids with few wide subspaces (d=1 level 14: 8192 cells in one
    subspace, beyond the shared-memory sums of the owner-computes multTranspose, so FP32 takes the
    fixed-point scatter and df64 the dense kernel) and with many narrow ones (d=12 level 3)."""
    rng = np.random.default_rng(dim * 100 + level)
    grid = sg.Grid.createLinearGrid(dim)
    grid.getGenerator().regular(level)
    m = 30000
    x = rng.random((m, dim))
    x[:20] = np.round(x[:20] * 2 ** level) / 2 ** level  # on cell boundaries
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    a = rng.standard_normal(grid.getSize())
    v = rng.standard_normal(m)
    if precision == "float":
        # FP32 inputs: rounding x moves 2^l x by up to 2^(l-25), and the hats with it
        tol = max(tol, 2.0 ** (level - 23))
    else:
        # float-float inputs hold 48 of x's 53 bits: 2^l x moves by up to 2^(l-49)
        tol = max(tol, 2.0 ** (level - 47))
    st = oracle.stream(x)
    op = _op(grid, x, precision, algo)
    out, outt = np.zeros(m), np.zeros(grid.getSize())
    op.mult(a, out)
    op.multTranspose(v, outt)
    assert rel_err(out, st.mult(lp, ix, a)) < tol
    assert rel_err(outt, st.mult_transpose(lp, ix, v)) < tol


@pytest.mark.parametrize("dim,level", [(6, 7), (4, 9)])
@pytest.mark.parametrize("precision,tol", [("float", FP32_TOL), ("df64", FP64_TOL)])
def test_large_grids_read_alpha_from_global_memory(oracle, dim, level, precision, tol):
    """Grids with more positions than shared memory holds (40,193 and 65,537 grid points): the
    subspace kernels read alpha from global memory; results match the oracle's FP64 evaluation."""
    rng = np.random.default_rng(dim * 1000 + level)
    grid = sg.Grid.createLinearGrid(dim)
    grid.getGenerator().regular(level)
    m = 4000
    x = rng.random((m, dim))
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    a = rng.standard_normal(grid.getSize())
    v = rng.standard_normal(m)
    if precision == "float":
        tol = max(tol, 2.0 ** (level - 23))
    st = oracle.stream(x)
    op = _op(grid, x, precision, "subspace")
    out, outt = np.zeros(m), np.zeros(grid.getSize())
    op.mult(a, out)
    op.multTranspose(v, outt)
    assert rel_err(out, st.mult(lp, ix, a)) < tol
    assert rel_err(outt, st.mult_transpose(lp, ix, v)) < tol


@pytest.mark.parametrize("products", ["half", "float"])
def test_mixed_fit_inner_products(products):
    """params "inner_products": the inner solves stream the FP16 or the FP32 copy of the
    materialised products; either way the refinement reaches the FP64 solution."""
    g = load_golden("cgfit.npz")
    for name in ("d4_l4", "d6_l3"):
        grid = _grid_from(g, name)
        cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                    sg.OperationMultipleEvalSubType.CUDA,
                                                    parameters={"inner_products": products,
                                                                "algo": "subspace",
                                                                "materialize": "on"})
        op = sg.createOperationMultipleEval(grid, g[name + "_x"], cfg)
        alpha, _, _ = op.fit(g[name + "_y"], float(g[name + "_lambda"]), 5000, 1e-10,
                             mode=sg.SGMEV_SOLVE_MIXED)
        assert rel_err(alpha, g[name + "_alpha"]) < 1e-6
        op.close()
    cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                sg.OperationMultipleEvalSubType.CUDA,
                                                parameters={"inner_products": "bf16"})
    with pytest.raises(Exception):
        sg.createOperationMultipleEval(grid, g[name + "_x"], cfg)


@pytest.mark.parametrize("dim,level", [(2, 7), (3, 6)])
def test_mixed_fit_with_byte_cells(oracle, dim, level):
    """Grids whose subspaces have more than 16 cells keep byte cell indices: the FP16 inner
    products then read two byte-cell words per pair of point groups (the uint2 pair copy). The
    mixed fit on the materialised products still reaches the oracle's FP64 solution."""
    rng = np.random.default_rng(41)
    grid = sg.Grid.createLinearGrid(dim)
    grid.getGenerator().regular(level)
    m = 20000
    x = rng.random((m, dim))
    y = np.sin(5 * x[:, 0]) * np.cos(3 * x[:, 1]) + 0.01 * rng.standard_normal(m)
    cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                sg.OperationMultipleEvalSubType.CUDA,
                                                parameters={"algo": "subspace", "materialize": "on"})
    op = sg.createOperationMultipleEval(grid, x, cfg)
    alpha, _, _ = op.fit(y, 1e-4, 20000, 1e-10, mode=sg.SGMEV_SOLVE_MIXED)
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    ref, _, _ = oracle.stream(x).cg_fit(lp, ix, y, 1e-4, 20000, 1e-12)
    assert rel_err(alpha, ref) < 1e-6
    op.close()


def test_inner_tolerance_knob():
    """params "inner_tol": any value in (0, 1) reaches the same FP64 solution; others raise."""
    g = load_golden("cgfit.npz")
    name = "d4_l4"
    grid = _grid_from(g, name)
    for tol in ("1e-2", "1e-5"):
        cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                    sg.OperationMultipleEvalSubType.CUDA,
                                                    parameters={"inner_tol": tol})
        op = sg.createOperationMultipleEval(grid, g[name + "_x"], cfg)
        alpha, _, _ = op.fit(g[name + "_y"], float(g[name + "_lambda"]), 5000, 1e-10,
                             mode=sg.SGMEV_SOLVE_MIXED)
        assert rel_err(alpha, g[name + "_alpha"]) < 1e-6
        op.close()
    for bad in ("0", "1.5", "x"):
        cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                    sg.OperationMultipleEvalSubType.CUDA,
                                                    parameters={"inner_tol": bad})
        with pytest.raises(Exception):
            sg.createOperationMultipleEval(grid, g[name + "_x"], cfg)


def test_df64_matches_native_fp64_at_full_size():
    """FP64-accurate float-float kernels against the native FP64 kernels at the regression-fit
    workload size (d=10, level 5, 2^20 points)."""
    rng = np.random.default_rng(22)
    grid = sg.Grid.createLinearGrid(10)
    grid.getGenerator().regular(5)
    m = 1 << 20
    x = rng.random((m, 10))
    a = rng.standard_normal(grid.getSize())
    v = rng.standard_normal(m)
    out64, outdf = np.zeros(m), np.zeros(m)
    op64 = _op(grid, x, "double")
    opdf = _op(grid, x, "df64", "dense")
    opsub = _op(grid, x, "df64", "subspace")
    outsub = np.zeros(m)
    opsub.mult(a, outsub)
    op64.mult(a, out64)
    assert rel_err(outsub, out64) < FP64_TOL
    opmat = _op(grid, x, "df64", "materialized")
    outmat = np.zeros(m)
    opmat.mult(a, outmat)
    assert rel_err(outmat, out64) < FP64_TOL
    tmat = np.zeros(grid.getSize())
    opmat.multTranspose(v, tmat)
    op64.mult(a, out64)
    opdf.mult(a, outdf)
    assert rel_err(outdf, out64) < FP64_TOL
    t64, tdf = np.zeros(grid.getSize()), np.zeros(grid.getSize())
    op64.multTranspose(v, t64)
    opdf.multTranspose(v, tdf)
    assert rel_err(tdf, t64) < FP64_TOL
    assert rel_err(tmat, t64) < FP64_TOL


@pytest.mark.parametrize("algo", ["dense", "subspace", "materialized"])
def test_adjoint_and_linearity_at_full_size(algo):
    """Size-independent properties at the regression-fit workload size (d=10, level 5,
    2^20 points): <B a, v> = <a, B^T v>, B is linear, and the FP32 algorithms agree."""
    rng = np.random.default_rng(21)
    grid = sg.Grid.createLinearGrid(10)
    grid.getGenerator().regular(5)
    m = 1 << 20
    x = rng.random((m, 10))
    n = grid.getSize()
    a = rng.standard_normal(n)
    b = rng.standard_normal(n)
    v = rng.standard_normal(m)
    op = _op(grid, x, "float", algo)
    Ba = np.zeros(m)
    Bb = np.zeros(m)
    Bab = np.zeros(m)
    op.mult(a, Ba)
    op.mult(b, Bb)
    op.mult(2.0 * a - 3.0 * b, Bab)
    assert rel_err(Bab, 2.0 * Ba - 3.0 * Bb) < 1e-5
    Btv = np.zeros(n)
    op.multTranspose(v, Btv)
    lhs = float(Ba @ v)
    rhs = float(a @ Btv)
    assert abs(lhs - rhs) <= 1e-5 * (np.abs(Ba).sum() * np.abs(v).max())
    # against the FP64-accurate kernels at full size
    ref = _op(grid, x, "df64", "dense")
    Ba64 = np.zeros(m)
    ref.mult(a, Ba64)
    assert rel_err(Ba, Ba64) < FP32_TOL
    Btv64 = np.zeros(n)
    ref.multTranspose(v, Btv64)
    assert rel_err(Btv, Btv64) < FP32_TOL

"""CPU tests of the product library: it loads without a GPU, exports every entry point that
include/sgmev.h declares, builds grids identical to the reference's, validates arguments, and
fails loudly (no CPU fallback) when no device is present."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT, load_golden

import sgpp_gb300 as sg


def _header_symbols():
    inc = os.path.join(ROOT, "include")
    text = "".join(open(os.path.join(inc, f)).read() for f in sorted(os.listdir(inc))
                   if f.endswith(".h"))
    return sorted(set(re.findall(r"SGMEV_API\s+[\w\s\*]+?\b(sg\w+)\s*\(", text)))


def test_header_symbols_listed(lib):
    declared = _header_symbols()
    assert declared, "no declarations parsed"
    assert sorted(sg.EXPORTED_SYMBOLS) == declared


def test_library_exports_every_declared_symbol(lib):
    for name in _header_symbols():
        assert hasattr(lib, name), name


def test_version_and_error_string(lib):
    assert lib.sgmev_version() >= 10000
    assert lib.sgmev_last_error() is not None


@pytest.mark.parametrize("d,l", [(1, 3), (2, 2), (2, 5), (3, 4), (4, 3), (5, 6), (8, 4), (10, 3),
                                 (10, 5), (12, 3)])
def test_product_regular_grid_equals_reference(lib, oracle, d, l):
    import hashlib
    g = load_golden("grids.npz")
    grid = sg.Grid.createLinearGrid(d)
    grid.getGenerator().regular(l)
    st = grid.getStorage()
    key = f"d{d}_l{l}"
    assert st.getSize() == int(g[key + "_n"])
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a, np.int32).tobytes()).hexdigest()
    assert sha(st.level) == str(g[key + "_sha_level"])
    assert sha(st.index) == str(g[key + "_sha_index"])
    lp, ix = st.getLevelIndexArraysForEval()
    olp, oix = oracle.eval_arrays(*oracle.regular_grid(d, l))
    np.testing.assert_array_equal(lp, olp)
    np.testing.assert_array_equal(ix, oix)


def test_regular_twice_raises(lib):
    grid = sg.Grid.createLinearGrid(2)
    grid.getGenerator().regular(2)
    with pytest.raises(sg.GenerationException):
        grid.getGenerator().regular(2)


@pytest.mark.parametrize("seq", ["small", "adaptive_d8_l4"])
def test_product_refinement_equals_reference_set(lib, seq):
    g = load_golden("refine.npz")
    rows = lambda L, I: set(map(tuple, np.hstack([L, I]).tolist()))
    for r in range(int(g[f"{seq}_rounds"])):
        pre_l = g[f"{seq}_r{r}_pre_level"].astype(np.int32)
        pre_i = g[f"{seq}_r{r}_pre_index"].astype(np.int32)
        grid = sg.Grid.fromArrays(pre_l, pre_i)
        added = []
        grid.getGenerator().refine(
            sg.SurplusRefinementFunctor(g[f"{seq}_r{r}_alpha"], int(g[f"{seq}_npoints"]), 0.0),
            added)
        st = grid.getStorage()
        post_l = g[f"{seq}_r{r}_post_level"].astype(np.int32)
        post_i = g[f"{seq}_r{r}_post_index"].astype(np.int32)
        assert st.getSize() == post_l.shape[0]
        np.testing.assert_array_equal(st.level[: pre_l.shape[0]], pre_l)
        assert rows(st.level, st.index) == rows(post_l, post_i)
        assert added == list(range(pre_l.shape[0], post_l.shape[0]))


def test_product_refinement_equals_oracle_order(lib, oracle):
    rng = np.random.default_rng(3)
    grid = sg.Grid.createLinearGrid(5)
    grid.getGenerator().regular(3)
    lev, idx = oracle.regular_grid(5, 3)
    for _ in range(4):
        a = rng.standard_normal(grid.getSize())
        grid.getGenerator().refine(sg.SurplusRefinementFunctor(a, 17, 0.0))
        lev, idx = oracle.refine_surplus(lev, idx, a, 17, 0.0)
        np.testing.assert_array_equal(grid.getStorage().level, lev)
        np.testing.assert_array_equal(grid.getStorage().index, idx)


def test_refinement_threshold_blocks_small_surpluses(lib):
    grid = sg.Grid.createLinearGrid(2)
    grid.getGenerator().regular(2)
    n0 = grid.getSize()
    grid.getGenerator().refine(sg.SurplusRefinementFunctor(np.full(n0, 0.1), 3, 1.0))
    assert grid.getSize() == n0


def test_factory_rejects_other_combinations(lib):
    grid = sg.Grid.createLinearGrid(2)
    grid.getGenerator().regular(2)
    x = np.random.default_rng(0).random((10, 2))
    cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.SUBSPACELINEAR,
                                                sg.OperationMultipleEvalSubType.COMBINED)
    with pytest.raises(sg.FactoryException):
        sg.createOperationMultipleEval(grid, x, cfg)
    cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                sg.OperationMultipleEvalSubType.OCL)
    with pytest.raises(sg.FactoryException):
        sg.createOperationMultipleEval(grid, x, cfg)


def _create(lib, lp, ix, x, prec=sg.SGMEV_FP64, left=None, right=None):
    import ctypes
    h = ctypes.c_void_p(None)
    vp = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)
    rc = lib.sgmev_create(ctypes.byref(h), lp.shape[1], lp.shape[0], vp(lp), vp(ix), x.shape[0],
                          vp(x), vp(left), vp(right), prec, None)
    return rc, h


def test_create_validates_before_touching_the_device(lib):
    lp = np.array([[2.0, 4.0]])
    ix = np.array([[1.0, 3.0]])
    x = np.zeros((4, 2))
    # index must be odd and inside (0, 2^l)
    rc, _ = _create(lib, lp, np.array([[1.0, 2.0]]), x)
    assert rc == sg.SGMEV_ERR_UNSUPPORTED
    assert b"odd" in lib.sgmev_last_error()
    # level must be a power of two >= 2 (no boundary / level-0 points)
    rc, _ = _create(lib, np.array([[1.0, 4.0]]), ix, x)
    assert rc == sg.SGMEV_ERR_UNSUPPORTED
    rc, _ = _create(lib, np.array([[6.0, 4.0]]), ix, x)
    assert rc == sg.SGMEV_ERR_UNSUPPORTED
    # empty bounding-box interval
    rc, _ = _create(lib, lp, ix, x, left=np.array([0.0, 1.0]), right=np.array([1.0, 1.0]))
    assert rc == sg.SGMEV_ERR_INVALID
    # bad precision
    rc, _ = _create(lib, lp, ix, x, prec=7)
    assert rc == sg.SGMEV_ERR_INVALID


@pytest.mark.parametrize("knob", ["precond", "algo", "materialize", "inner_products",
                                  "system_product", "materialize_multt"])
def test_operator_knobs_are_validated_before_the_device(lib, knob):
    """A bad value of an operator parameter fails sgmev_create with SGMEV_ERR_INVALID and names
    the parameter, before any device work; the Python configuration forwards every parameter of
    OP_KNOBS, so the same value raises there (no GPU needed for either)."""
    import ctypes
    import json
    assert knob in sg.OP_KNOBS
    lp = np.array([[2.0, 4.0]])
    ix = np.array([[1.0, 3.0]])
    x = np.zeros((4, 2))
    h = ctypes.c_void_p(None)
    rc = lib.sgmev_create(ctypes.byref(h), 2, 1, lp.ctypes.data, ix.ctypes.data, 4, x.ctypes.data,
                          None, None, sg.SGMEV_FP64, json.dumps({knob: "bogus"}).encode())
    assert rc == sg.SGMEV_ERR_INVALID
    assert knob.encode() in lib.sgmev_last_error()
    grid = sg.Grid.createLinearGrid(2)
    grid.getGenerator().regular(2)
    cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                sg.OperationMultipleEvalSubType.CUDA,
                                                parameters={knob: "bogus"})
    with pytest.raises(sg.OperationException, match=knob):
        sg.createOperationMultipleEval(grid, np.zeros((3, 2)), cfg)


def test_no_device_fails_loudly(lib):
    if lib.sgmev_device_count() > 0:
        pytest.skip("a GPU is visible; this checks the no-GPU error path")
    grid = sg.Grid.createLinearGrid(2)
    grid.getGenerator().regular(2)
    with pytest.raises(sg.OperationException, match="no CUDA device"):
        sg.createOperationMultipleEval(grid, np.zeros((3, 2)))

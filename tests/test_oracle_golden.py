"""Pin the oracle (oracle/oracle.c) against the reference's own outputs and known answers.

Fixtures come from the reference's compiled FP64 code (tests/golden/make_golden.py). These tests
need no GPU; they establish that the oracle the GPU tests compare against is the reference's
algorithm.
"""
import hashlib

import numpy as np
import pytest

from conftest import load_golden, rel_err


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.int32).tobytes()).hexdigest()


GRID_CASES = [(1, 3), (2, 2), (2, 5), (3, 4), (4, 3), (5, 6), (8, 4), (10, 3), (10, 5), (12, 3)]


@pytest.mark.parametrize("d,l", GRID_CASES)
def test_regular_grid_matches_reference_order(oracle, d, l):
    g = load_golden("grids.npz")
    lev, idx = oracle.regular_grid(d, l)
    key = f"d{d}_l{l}"
    assert lev.shape[0] == int(g[key + "_n"])
    assert _sha(lev) == str(g[key + "_sha_level"])
    assert _sha(idx) == str(g[key + "_sha_index"])
    if key + "_level" in g:
        np.testing.assert_array_equal(lev, g[key + "_level"])
        np.testing.assert_array_equal(idx, g[key + "_index"])


def test_regular_grid_sizes_match_the_reference_counts(oracle):
    # sizes of the reference's regular grids (d=5 l=6, d=10 l=5, d=8 l=4, d=12 l=7)
    assert oracle.lib.orc_regular_grid_size(5, 6) == 5503
    assert oracle.lib.orc_regular_grid_size(10, 5) == 13441
    assert oracle.lib.orc_regular_grid_size(8, 4) == 1121
    assert oracle.lib.orc_regular_grid_size(12, 7) == 956929


def _rows(lev, idx):
    return set(map(tuple, np.hstack([lev, idx]).tolist()))


@pytest.mark.parametrize("seq", ["small", "adaptive_d8_l4"])
def test_refinement_point_sets_match_reference(oracle, seq):
    g = load_golden("refine.npz")
    rounds = int(g[f"{seq}_rounds"])
    npts = int(g[f"{seq}_npoints"])
    for r in range(rounds):
        pre_l = g[f"{seq}_r{r}_pre_level"].astype(np.int32)
        pre_i = g[f"{seq}_r{r}_pre_index"].astype(np.int32)
        alpha = g[f"{seq}_r{r}_alpha"]
        lev, idx = oracle.refine_surplus(pre_l, pre_i, alpha, npts, 0.0)
        post_l = g[f"{seq}_r{r}_post_level"].astype(np.int32)
        post_i = g[f"{seq}_r{r}_post_index"].astype(np.int32)
        assert lev.shape[0] == post_l.shape[0]
        # existing points keep their positions; the appended set equals the reference's
        np.testing.assert_array_equal(lev[: pre_l.shape[0]], pre_l)
        assert _rows(lev, idx) == _rows(post_l, post_i)


def _case(g, name):
    lev = g[name + "_level"].astype(np.int32)
    idx = g[name + "_index"].astype(np.int32)
    lp = np.left_shift(1, lev.astype(np.int64)).astype(np.float64)
    return lp, idx.astype(np.float64)


def test_multeval_oracle_matches_reference(oracle):
    g = load_golden("multeval.npz")
    for name in g["cases"]:
        name = str(name)
        lp, ix = _case(g, name)
        x, a, v = g[name + "_x"], g[name + "_alpha"], g[name + "_v"]
        ref_m = g[name + "_mult_default"]
        ref_t = g[name + "_multt_default"]
        # STREAMING and DEFAULT agree with each other (the reference's own harness check)
        assert rel_err(g[name + "_mult_streaming"], ref_m) < 1e-12, name
        assert rel_err(g[name + "_multt_streaming"], ref_t) < 1e-12, name
        assert rel_err(oracle.mult_naive(lp, ix, x, a), ref_m) < 1e-12, name
        assert rel_err(oracle.mult_transpose_naive(lp, ix, x, v), ref_t) < 1e-12, name
        st = oracle.stream(x)
        assert rel_err(st.mult(lp, ix, a), ref_m) < 1e-12, name
        assert rel_err(st.mult_transpose(lp, ix, v), ref_t) < 1e-12, name


def test_bounding_box_known_answer(oracle):
    """base/tests/test_OperationMultipleEval.cpp:24-79: d=2 level 2, box [3,5]x[-2,2],
    alpha_i = i+1, three points -> mult = {0.0, 2.72, 1.64} (BOOST_CHECK_CLOSE 1e-7 %)."""
    g = load_golden("multeval.npz")
    lp, ix = _case(g, "bb_kat")
    x = g["bb_kat_x"]
    xu = oracle.bb_to_unit(x, g["bb_kat_bb_left"], g["bb_kat_bb_right"])
    out = oracle.mult_naive(lp, ix, xu, g["bb_kat_alpha"])
    np.testing.assert_allclose(out, [0.0, 2.72, 1.64], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(out, g["bb_kat_mult_default"], rtol=1e-12, atol=1e-14)


def test_bounding_box_random_matches_reference(oracle):
    g = load_golden("multeval.npz")
    lp, ix = _case(g, "bb_rand")
    xu = oracle.bb_to_unit(g["bb_rand_x"], g["bb_rand_bb_left"], g["bb_rand_bb_right"])
    assert rel_err(oracle.mult_naive(lp, ix, xu, g["bb_rand_alpha"]), g["bb_rand_mult_default"]) < 1e-12
    assert rel_err(oracle.mult_transpose_naive(lp, ix, xu, g["bb_rand_v"]),
                   g["bb_rand_multt_default"]) < 1e-12


@pytest.mark.parametrize("name", ["d1_l3", "d1_l5", "d3_l3", "d3_l4"])
def test_bt_golden_matrices(oracle, name):
    """datadriven/tests/testBT.cpp (TestOperationBTLinear): B built column by column via
    mult(e_i); row sums in order and sorted column sums within 1e-5 % of the golden files."""
    g = load_golden("bt_linear.npz")
    d, l = int(g[name + "_dim"]), int(g[name + "_level"])
    x = g[name + "_x"]
    lev, idx = oracle.regular_grid(d, l)
    lp, ix = oracle.eval_arrays(lev, idx)
    n = lev.shape[0]
    B = np.zeros((x.shape[0], n))
    for i in range(n):
        e = np.zeros(n)
        e[i] = 1.0
        B[:, i] = oracle.mult_naive(lp, ix, x, e)
    np.testing.assert_allclose(B.sum(axis=1), g[name + "_row_sums"], rtol=1e-7, atol=1e-9)
    np.testing.assert_allclose(np.sort(B.sum(axis=0)), g[name + "_col_sums_sorted"], rtol=1e-7,
                               atol=1e-9)


@pytest.mark.parametrize("name", ["d4_l4", "d6_l3"])
def test_cg_fit_matches_reference(oracle, name):
    g = load_golden("cgfit.npz")
    lp, ix = _case(g, name)
    st = oracle.stream(g[name + "_x"])
    alpha, it, res = st.cg_fit(lp, ix, g[name + "_y"], float(g[name + "_lambda"]), 1000, 1e-12)
    ref = g[name + "_alpha"]
    assert rel_err(alpha, ref) < 1e-9
    assert abs(it - int(g[name + "_iterations"])) <= 2


def test_planted_mistake_is_caught(oracle):
    """The comparison machinery catches a wrong hat: shift one grid index in the oracle input."""
    g = load_golden("multeval.npz")
    lp, ix = _case(g, "d3_l4_m512")
    ix = ix.copy()
    ix[5, 1] += 2.0
    out = oracle.mult_naive(lp, ix, g["d3_l4_m512_x"], g["d3_l4_m512_alpha"])
    assert rel_err(out, g["d3_l4_m512_mult_default"]) > 1e-6

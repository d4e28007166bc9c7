"""Generate the golden fixtures in this folder from the reference's own compiled code.

Run where the reference sources exist (they are read only by oracle/ref.mk at build time):

    make -f oracle/ref.mk -j8 && make -C oracle && python tests/golden/make_golden.py

Every fixture comes from SG++'s own FP64 implementation (oracle/_ref/libsgpp_ref.so, built
from the unmodified reference sources plus oracle/ref_harness.cpp), on seeded inputs:

  grids.npz     regular Linear grids (HashGenerator::regular_iter order) — full arrays for
                small grids, SHA-256 of the int32 level/index arrays for large ones
  refine.npz    surplus-refinement sequences (SurplusRefinementFunctor + HashRefinement::free_refine)
  multeval.npz  mult / multTranspose outputs of the DEFAULT (OperationMultipleEvalLinear) and
                STREAMING (OperationMultiEvalStreaming) operators, with their inputs
  cgfit.npz     regression fits through SystemMatrixLeastSquaresIdentity + ConjugateGradients
  bt_linear.npz the reference's golden B^T matrices for the hat basis
                (datadriven/datasets/BT_BBT/BT_phi_li_hut_*), reduced to the row sums and sorted
                column sums that datadriven/tests/testBT.cpp compares, plus their data points
  datasets.npz  ARFF / CSV text through the reference's ARFFTools::readARFF and CSVTools::readCSV:
                seeded synthetic texts (written by this script) under every reading option, the
                reference's own reader fixtures datadriven/datasets/dataread/simple.{arff,csv}
                (their SHA-256 and parsed outputs only, for the cases test_readARFF.cpp and
                test_readCSV.cpp check), and a regression data set as ARFF text
  fit_adapt.npz ModelFittingLeastSquares::fit followed by adapt() rounds, replayed with the
                reference's own classes (grid, SurplusRefinementFunctor,
                SystemMatrixLeastSquaresIdentity, ConjugateGradients with reuse): final grid,
                alpha and the CG iterations of every solve
  modlinear.npz ModLinear grids: the streaming layout (getLevelIndexMaskArraysForModEval),
                mult / multTranspose of the DEFAULT (OperationMultipleEvalModLinear) and STREAMING
                (OperationMultiEvalModMaskStreaming) operators, regression fits, and the golden
                B^T matrices of the modified basis (BT_phi_li_ausgeklappt_*, testBT.cpp suite
                TestOperationBTModLinear) reduced like bt_linear.npz
"""
from __future__ import annotations

import gzip
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import REF_DEFAULT, REF_STREAMING, Reference, reference_source  # noqa: E402

REF_SRC = reference_source() or ""


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, np.int32).tobytes()).hexdigest()


def edge_points(rng, m, d):
    """Uniform points with a share of exact hat nodes / support edges / cube faces mixed in."""
    x = rng.random((m, d))
    k = max(1, m // 8)
    nodes = rng.integers(0, 65, size=(k, d)) / 64.0  # exact dyadic grid nodes incl. 0 and 1
    x[:k] = nodes
    return x


def make_grids(ref: Reference):
    out = {}
    cases = [(1, 3), (2, 2), (2, 5), (3, 4), (4, 3), (5, 6), (8, 4), (10, 3), (10, 5), (12, 3)]
    for d, l in cases:
        g = ref.grid(d, l)
        lev, idx, leaf = g.points()
        key = f"d{d}_l{l}"
        out[key + "_n"] = np.int64(lev.shape[0])
        out[key + "_sha_level"] = np.array(sha(lev))
        out[key + "_sha_index"] = np.array(sha(idx))
        if lev.shape[0] <= 400:
            out[key + "_level"] = lev.astype(np.int8)
            out[key + "_index"] = idx.astype(np.int16)
            out[key + "_leaf"] = leaf.astype(np.int8)
    np.savez_compressed(os.path.join(HERE, "grids.npz"), **out)


def make_refine(ref: Reference):
    out = {}
    seqs = [("small", 4, 3, 3, 10, 11), ("adaptive_d8_l4", 8, 4, 6, 40, 12)]
    for name, d, l, rounds, npts, seed in seqs:
        rng = np.random.default_rng(seed)
        g = ref.grid(d, l)
        out[f"{name}_dim"] = np.int64(d)
        out[f"{name}_level"] = np.int64(l)
        out[f"{name}_rounds"] = np.int64(rounds)
        out[f"{name}_npoints"] = np.int64(npts)
        for r in range(rounds):
            lev, idx, _ = g.points()
            out[f"{name}_r{r}_pre_level"] = lev.astype(np.int8)
            out[f"{name}_r{r}_pre_index"] = idx.astype(np.int16)
            alpha = rng.standard_normal(g.size)
            out[f"{name}_r{r}_alpha"] = alpha
            g.refine_surplus(alpha, npts, 0.0)
            lev, idx, _ = g.points()
            out[f"{name}_r{r}_post_level"] = lev.astype(np.int8)
            out[f"{name}_r{r}_post_index"] = idx.astype(np.int16)
    np.savez_compressed(os.path.join(HERE, "refine.npz"), **out)


def make_multeval(ref: Reference):
    out = {}
    cases = [
        ("d1_l3_m8", 1, 3, 8, 0),
        ("d2_l5_m300", 2, 5, 300, 0),
        ("d3_l4_m512", 3, 4, 512, 0),
        ("d5_l4_m1000", 5, 4, 1000, 0),
        ("d5_l6_m2000", 5, 6, 2000, 0),       # the plain FP64 d=5 level 6 grid, fewer points
        ("d10_l3_m777", 10, 3, 777, 0),       # ragged M (not a multiple of any chunk)
        ("d10_l5_m300", 10, 5, 300, 0),       # the regression-fit grid
        ("d8_l4_ad2_m1000", 8, 4, 1000, 2),   # adaptive: 2 surplus-refinement rounds of 40
        ("d12_l3_m257", 12, 3, 257, 0),
        ("d4_l3_m1", 4, 3, 1, 0),             # single data point
    ]
    rng = np.random.default_rng(20261203)
    names = []
    for name, d, l, m, rounds in cases:
        g = ref.grid(d, l)
        for _ in range(rounds):
            g.refine_surplus(rng.standard_normal(g.size), 40, 0.0)
        lev, idx, _ = g.points()
        x = edge_points(rng, m, d)
        alpha = rng.standard_normal(g.size)
        v = rng.standard_normal(m)
        out[name + "_level"] = lev.astype(np.int8)
        out[name + "_index"] = idx.astype(np.int16)
        out[name + "_x"] = x
        out[name + "_alpha"] = alpha
        out[name + "_v"] = v
        out[name + "_mult_default"] = g.mult(REF_DEFAULT, x, alpha)
        out[name + "_mult_streaming"] = g.mult(REF_STREAMING, x, alpha)
        out[name + "_multt_default"] = g.mult_transpose(REF_DEFAULT, x, v)
        out[name + "_multt_streaming"] = g.mult_transpose(REF_STREAMING, x, v)
        names.append(name)
    # bounding box: reference KAT layout (base/tests/test_OperationMultipleEval.cpp:24-79) and a
    # random box, both through the DEFAULT operator which applies BoundingBox::transformPointToUnitCube
    for name, d, l, m, left, right in [
        ("bb_kat", 2, 2, 3, [3.0, -2.0], [5.0, 2.0]),
        ("bb_rand", 3, 4, 400, [-1.0, 0.5, 2.0], [1.0, 2.5, 2.25]),
    ]:
        g = ref.grid(d, l)
        g.set_bounding_box(left, right)
        lev, idx, _ = g.points()
        if name == "bb_kat":
            x = np.array([[4.0, 2.0], [3.6, -0.4], [4.8, 0.8]])
            alpha = np.arange(1, g.size + 1, dtype=np.float64)
        else:
            lo, hi = np.array(left), np.array(right)
            x = lo + (hi - lo) * (rng.random((m, d)) * 1.2 - 0.1)  # some points outside the box
            alpha = rng.standard_normal(g.size)
        v = rng.standard_normal(x.shape[0])
        out[name + "_level"] = lev.astype(np.int8)
        out[name + "_index"] = idx.astype(np.int16)
        out[name + "_x"] = x
        out[name + "_alpha"] = alpha
        out[name + "_v"] = v
        out[name + "_bb_left"] = np.array(left)
        out[name + "_bb_right"] = np.array(right)
        out[name + "_mult_default"] = g.mult(REF_DEFAULT, x, alpha)
        out[name + "_multt_default"] = g.mult_transpose(REF_DEFAULT, x, v)
    out["cases"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "multeval.npz"), **out)


def make_cgfit(ref: Reference):
    out = {}
    rng = np.random.default_rng(7)
    cases = [("d4_l4", 4, 4, 3000, 1e-3), ("d6_l3", 6, 3, 2500, 1e-4)]
    for name, d, l, m, lam in cases:
        g = ref.grid(d, l)
        x = rng.random((m, d))
        y = (10 * np.sin(np.pi * x[:, 0] * x[:, 1]) + 20 * (x[:, 2] - 0.5) ** 2 + 10 * x[:, 3]
             + 0.1 * rng.standard_normal(m))
        lev, idx, _ = g.points()
        alpha, it, res = g.cg_fit(REF_STREAMING, x, y, lam, 1000, 1e-12)
        out[name + "_level"] = lev.astype(np.int8)
        out[name + "_index"] = idx.astype(np.int16)
        out[name + "_x"] = x
        out[name + "_y"] = y
        out[name + "_lambda"] = np.float64(lam)
        out[name + "_alpha"] = alpha
        out[name + "_iterations"] = np.int64(it)
        out[name + "_residual"] = np.float64(res)
    np.savez_compressed(os.path.join(HERE, "cgfit.npz"), **out)


def read_arff(path):
    rows = []
    with gzip.open(path, "rt") as f:
        data = False
        for line in f:
            s = line.strip()
            if not s:
                continue
            if data:
                rows.append([float(v) for v in s.split(",")])
            elif s.upper().startswith("@DATA"):
                data = True
    return np.array(rows)


def read_matrix(path):
    rows = []
    with gzip.open(path, "rt") as f:
        for line in f:
            s = line.strip()
            if not s:
                break
            rows.append([float(v) for v in s.split()])
    return np.array(rows)


def make_bt(ref: Reference):
    """datadriven/tests/testBT.cpp, suite TestOperationBTLinear: regular Linear grid, B built
    column by column with mult(e_i); row sums compared in order, column sums sorted, 1e-5 %."""
    base = os.path.join(REF_SRC, "datadriven", "datasets", "BT_BBT")
    cases = [("d1_l3", 1, 3, "data_dim_1_nops_8_float.arff.gz", "BT_phi_li_hut_dim_1_nopsgrid_7_float.dat.gz"),
             ("d1_l5", 1, 5, "data_dim_1_nops_8_float.arff.gz", "BT_phi_li_hut_dim_1_nopsgrid_31_float.dat.gz"),
             ("d3_l3", 3, 3, "data_dim_3_nops_512_float.arff.gz", "BT_phi_li_hut_dim_3_nopsgrid_31_float.dat.gz"),
             ("d3_l4", 3, 4, "data_dim_3_nops_512_float.arff.gz", "BT_phi_li_hut_dim_3_nopsgrid_111_float.dat.gz")]
    out = {}
    for name, d, l, data_file, mat_file in cases:
        x = read_arff(os.path.join(base, data_file))
        mat = read_matrix(os.path.join(base, mat_file))
        g = ref.grid(d, l)
        assert mat.shape == (x.shape[0], g.size), (name, mat.shape, x.shape, g.size)
        out[name + "_x"] = x
        out[name + "_row_sums"] = mat.sum(axis=1)
        out[name + "_col_sums_sorted"] = np.sort(mat.sum(axis=0))
        out[name + "_dim"] = np.int64(d)
        out[name + "_level"] = np.int64(l)
    np.savez_compressed(os.path.join(HERE, "bt_linear.npz"), **out)


def make_modlinear(ref: Reference):
    out = {}
    rng = np.random.default_rng(20261204)
    cases = [
        ("d1_l4_m40", 1, 4, 40, 0),
        ("d2_l5_m300", 2, 5, 300, 0),
        ("d3_l4_m512", 3, 4, 512, 0),
        ("d5_l4_m777", 5, 4, 777, 0),          # ragged M
        ("d10_l3_m300", 10, 3, 300, 0),
        ("d6_l4_ad2_m600", 6, 4, 600, 2),      # adaptive: 2 surplus-refinement rounds of 30
        ("d4_l3_m1", 4, 3, 1, 0),              # single data point
    ]
    names = []
    for name, d, l, m, rounds in cases:
        g = ref.grid(d, l, "modlinear")
        for _ in range(rounds):
            g.refine_surplus(rng.standard_normal(g.size), 30, 0.0)
        lev, idx, _ = g.points()
        x = edge_points(rng, m, d)            # nodes on the faces 0 and 1 included
        alpha = rng.standard_normal(g.size)
        v = rng.standard_normal(m)
        level, index, mask, offset = g.mask_arrays()
        out[name + "_level"] = lev.astype(np.int8)
        out[name + "_index"] = idx.astype(np.int16)
        out[name + "_mask_level"] = level
        out[name + "_mask_index"] = index
        out[name + "_mask_bits"] = mask.view(np.uint64)
        out[name + "_mask_offset"] = offset
        out[name + "_x"] = x
        out[name + "_alpha"] = alpha
        out[name + "_v"] = v
        out[name + "_mult_default"] = g.mult(REF_DEFAULT, x, alpha)
        out[name + "_mult_streaming"] = g.mult(REF_STREAMING, x, alpha)
        out[name + "_multt_default"] = g.mult_transpose(REF_DEFAULT, x, v)
        out[name + "_multt_streaming"] = g.mult_transpose(REF_STREAMING, x, v)
        names.append(name)
    out["cases"] = np.array(names)
    # points outside the cube: the STREAMING operator extrapolates the boundary-adjacent functions
    g = ref.grid(3, 4, "modlinear")
    lev, idx, _ = g.points()
    x = rng.random((200, 3)) * 1.4 - 0.2
    alpha = rng.standard_normal(g.size)
    v = rng.standard_normal(200)
    out["outside_level"] = lev.astype(np.int8)
    out["outside_index"] = idx.astype(np.int16)
    out["outside_x"] = x
    out["outside_alpha"] = alpha
    out["outside_v"] = v
    out["outside_mult_streaming"] = g.mult(REF_STREAMING, x, alpha)
    out["outside_multt_streaming"] = g.mult_transpose(REF_STREAMING, x, v)
    # regression fits through SystemMatrixLeastSquaresIdentity (STREAMING -> ModMaskStreaming)
    for name, d, l, m, lam in [("fit_d4_l4", 4, 4, 3000, 1e-3), ("fit_d6_l3", 6, 3, 2500, 1e-4)]:
        g = ref.grid(d, l, "modlinear")
        x = rng.random((m, d))
        y = (10 * np.sin(np.pi * x[:, 0] * x[:, 1]) + 20 * (x[:, 2] - 0.5) ** 2 + 10 * x[:, 3]
             + 0.1 * rng.standard_normal(m))
        lev, idx, _ = g.points()
        a, it, res = g.cg_fit(REF_STREAMING, x, y, lam, 1000, 1e-12)
        out[name + "_level"] = lev.astype(np.int8)
        out[name + "_index"] = idx.astype(np.int16)
        out[name + "_x"] = x
        out[name + "_y"] = y
        out[name + "_lambda"] = np.float64(lam)
        out[name + "_alpha"] = a
        out[name + "_iterations"] = np.int64(it)
        out[name + "_residual"] = np.float64(res)
    # golden B^T matrices of the modified basis (testBT.cpp, TestOperationBTModLinear)
    base = os.path.join(REF_SRC, "datadriven", "datasets", "BT_BBT")
    for key, d, l, data_file, mat_file in [
            ("bt_d1_l3", 1, 3, "data_dim_1_nops_8_float.arff.gz", "BT_phi_li_ausgeklappt_dim_1_nopsgrid_7_float.dat.gz"),
            ("bt_d1_l5", 1, 5, "data_dim_1_nops_8_float.arff.gz", "BT_phi_li_ausgeklappt_dim_1_nopsgrid_31_float.dat.gz"),
            ("bt_d3_l3", 3, 3, "data_dim_3_nops_512_float.arff.gz", "BT_phi_li_ausgeklappt_dim_3_nopsgrid_31_float.dat.gz"),
            ("bt_d3_l4", 3, 4, "data_dim_3_nops_512_float.arff.gz", "BT_phi_li_ausgeklappt_dim_3_nopsgrid_111_float.dat.gz")]:
        x = read_arff(os.path.join(base, data_file))
        mat = read_matrix(os.path.join(base, mat_file))
        g = ref.grid(d, l, "modlinear")
        assert mat.shape == (x.shape[0], g.size), (key, mat.shape, x.shape, g.size)
        out[key + "_x"] = x
        out[key + "_row_sums"] = mat.sum(axis=1)
        out[key + "_col_sums_sorted"] = np.sort(mat.sum(axis=0))
        out[key + "_dim"] = np.int64(d)
        out[key + "_level"] = np.int64(l)
    np.savez_compressed(os.path.join(HERE, "modlinear.npz"), **out)


def synthetic_texts(rng):
    """Seeded ARFF / CSV texts that exercise the readers' rules (this script's own inputs)."""
    def num(v, style):
        return {0: f"{v:.6f}", 1: f"{v:.3e}", 2: f" {v:g} ", 3: f"{v:.17g}", 4: f"{int(round(v))}"}[style]

    texts = []
    for k in range(12):
        rows, cols = int(rng.integers(1, 9)), int(rng.integers(1, 6))
        vals = rng.standard_normal((rows, cols)) * 10.0 ** int(rng.integers(-3, 4))
        targets = rng.choice([0.0, 1.0, 7.0, 42.42, -5.0], size=rows)
        lines = []
        arff = k % 2 == 0
        if arff:
            lines += ["% generated", "@RELATION synthetic"]
            lines += [f"@ATTRIBUTE x{t} NUMERIC" for t in range(cols)] + ["@ATTRIBUTE y NUMERIC", "",
                                                                          "@DATA"]
        elif k % 4 == 1:
            lines.append(",".join(f"h{t}" for t in range(cols + 1)))
        for r in range(rows):
            style = int(rng.integers(0, 5))
            lines.append(",".join(num(v, style) for v in vals[r]) + "," + num(targets[r], 0))
            if rng.random() < 0.2:
                lines.append("")
            if arff and rng.random() < 0.2:
                lines.append("% a comment line")
        sep = "\r\n" if k % 3 == 2 else "\n"
        text = sep.join(lines) + (sep if k % 5 != 4 else "")
        texts.append((("arff" if arff else "csv"), text, k % 4 == 1))
    # rules at the edges
    texts.append(("arff", "1\n2,3\n4,5\n", False))               # first data line without commas
    texts.append(("arff", "1,2,3\n1,2\n", False))                  # ragged line: an error
    texts.append(("arff", "@DATA\n0.5,0.25,1\n\n0.75,,2\n", False))  # an empty field
    texts.append(("csv", "\nx,y,t\n1,2,3\n4,5,6\n", True))         # empty first line + header
    texts.append(("csv", "1,2,3", False))                             # no trailing newline
    texts.append(("arff", "", False))                                 # empty text
    return texts


# (has_targets, cutoff, cols, targets). A cutoff of 0 is left out: the reference then writes row
# 0 of an empty matrix (ARFFTools.cpp readARFF, CSVTools.cpp readCSV) and crashes.
OPTIONS = [
    (True, -1, None, None), (False, -1, None, None), (True, 2, None, None),
    (True, -1, [1, 0], None), (True, -1, None, [7.0, 42.42]),
]


def make_datasets(ref: Reference):
    out = {}
    rng = np.random.default_rng(20261205)
    texts = synthetic_texts(rng)
    keys = []
    for i, (fmt, text, header) in enumerate(texts):
        out[f"t{i}_text"] = np.array(text)
        out[f"t{i}_format"] = np.int64(0 if fmt == "arff" else 1)
        out[f"t{i}_header"] = np.int64(int(header))
        for j, (ht, cut, cols, tg) in enumerate(OPTIONS):
            key = f"t{i}_o{j}"
            try:
                data, y = ref.read_dataset(0 if fmt == "arff" else 1, text.encode(), ht, header,
                                           cut, cols, tg)
                out[key + "_data"] = data
                out[key + "_y"] = y
                out[key + "_error"] = np.array("")
            except RuntimeError:
                # the reference's file_exception keeps a pointer into a freed string, so only
                # the failure itself is recorded
                out[key + "_error"] = np.array("error")
            keys.append(key)
    out["cases"] = np.array(keys)
    out["options"] = np.array([json_opt(o) for o in OPTIONS])
    # the reference's own reader fixtures, as test_readARFF.cpp / test_readCSV.cpp read them
    base = os.path.join(REF_SRC, "datadriven", "datasets", "dataread")
    for fmt, name in ((0, "simple.arff"), (1, "simple.csv")):
        raw = open(os.path.join(base, name), "rb").read()
        tag = name.replace(".", "_")
        out[tag + "_sha256"] = np.array(hashlib.sha256(raw).hexdigest())
        for j, (ht, cut, cols, tg) in enumerate([(True, -1, None, None), (False, -1, None, None),
                                                 (True, 2, None, None), (True, -1, [4, 2, 0], None),
                                                 (True, -1, None, [7.0, 42.42])]):
            data, y = ref.read_dataset(fmt, raw, ht, fmt == 1, cut, cols, tg)
            out[f"{tag}_c{j}_data"] = data
            out[f"{tag}_c{j}_y"] = y
    # a regression data set as ARFF text, for the end-to-end fit (read -> device -> fit)
    x = rng.random((1500, 4)) * 2.0 - 0.5       # outside the unit cube: a bounding box maps it
    y = np.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2] - 0.5 * x[:, 3] + 0.01 * rng.standard_normal(1500)
    lines = ["@RELATION regression", *[f"@ATTRIBUTE x{t} NUMERIC" for t in range(4)],
             "@ATTRIBUTE y NUMERIC", "@DATA"]
    lines += [",".join(f"{v:.17g}" for v in row) + f",{t:.17g}" for row, t in zip(x, y)]
    text = "\n".join(lines) + "\n"
    data, yy = ref.read_dataset(0, text.encode(), True, False, -1, None, None, n_cap=2000, dim_cap=8)
    out["fit_text"] = np.array(text)
    out["fit_data"] = data
    out["fit_y"] = yy
    np.savez_compressed(os.path.join(HERE, "datasets.npz"), **out)


FIT_ADAPT_CASES = [
    # name, basis, dim, level, m, lambda, final (eps, maxit), refine (eps, maxit), rounds, points
    ("lin_d2_l3", 0, 2, 3, 500, 1e-4, (1e-10, 1000), (1e-10, 1000), 3, 5),
    ("mod_d3_l2", 1, 3, 2, 800, 1e-3, (1e-10, 1000), (1e-10, 1000), 2, 3),
    ("defaults_d4_l3", 0, 4, 3, 600, 0.01, (1e-12, 100), (1e-12, 100), 1, 1),
]


def make_fit_adapt(ref: Reference):
    out = {}
    rng = np.random.default_rng(20261206)
    for name, basis, d, l, m, lam, fin, refi, rounds, pts in FIT_ADAPT_CASES:
        x = rng.random((m, d))
        y = np.sin(3 * x[:, 0]) * (1 + x[:, 1]) + 0.5 * x[:, d - 1] ** 2 + 0.01 * rng.standard_normal(m)
        lev, idx, alpha, iters = ref.fit_adapt(basis, x, y, l, lam, fin[0], fin[1], refi[0],
                                               refi[1], rounds, pts)
        out[name + "_x"] = x
        out[name + "_y"] = y
        out[name + "_level"] = lev.astype(np.int8)
        out[name + "_index"] = idx.astype(np.int16)
        out[name + "_alpha"] = alpha
        out[name + "_iterations"] = iters
    np.savez_compressed(os.path.join(HERE, "fit_adapt.npz"), **out)


def json_opt(o):
    import json
    return json.dumps({"has_targets": o[0], "cutoff": o[1], "cols": o[2], "targets": o[3]})


def main():
    ref = Reference()
    ref.set_threads(os.cpu_count() or 1)
    make_grids(ref)
    make_refine(ref)
    make_multeval(ref)
    make_cgfit(ref)
    make_bt(ref)
    make_modlinear(ref)
    make_datasets(ref)
    make_fit_adapt(ref)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()

"""Dataset ingest (sgdata_* in the library; Python ARFFTools / CSVTools / Dataset).

CPU part: the library's readers against the reference's own ARFFTools::readARFF and
CSVTools::readCSV (tests/golden/datasets.npz, made by tests/golden/make_golden.py from the
reference's compiled readers): every synthetic text under every reading option, bit for bit, and
the reference's reader fixtures datadriven/datasets/dataread/simple.{arff,csv} under the options
that datadriven/tests/test_readARFF.cpp and test_readCSV.cpp check (when the reference's sources
are present).

GPU part (marked gpu): ARFF text -> reader -> operator (bounding box applied on the device) ->
regression fit, against the oracle's FP64 CG on the same rows.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import load_golden, rel_err
from oracle import reference_source

import sgpp_gb300 as sg

G = load_golden("datasets.npz")
CASES = [str(c) for c in G["cases"]]
OPTIONS = [json.loads(str(o)) for o in G["options"]]
REF_SRC = reference_source() or ""


def _read(fmt, text, header, opt):
    kw = dict(hasTargets=opt["has_targets"], instanceCutoff=opt["cutoff"],
              selectedCols=opt["cols"], selectedTargets=opt["targets"])
    if fmt == 0:
        return sg.ARFFTools.readARFFFromString(text, **kw)
    return sg.CSVTools.readCSVFromString(text, skipFirstLine=header, **kw)


@pytest.mark.parametrize("case", CASES)
def test_reader_matches_reference(lib, case):
    t, o = case.split("_")
    text = str(G[t + "_text"])
    fmt = int(G[t + "_format"])
    header = bool(int(G[t + "_header"]))
    opt = OPTIONS[int(o[1:])]
    if str(G[case + "_error"]):
        with pytest.raises(sg.FileException):
            _read(fmt, text, header, opt)
        return
    d = _read(fmt, text, header, opt)
    want = G[case + "_data"]
    assert d.getData().shape == want.shape
    np.testing.assert_array_equal(d.getData(), want)  # the same strtod, bit for bit
    if opt["has_targets"]:
        np.testing.assert_array_equal(d.getTargets(), G[case + "_y"])
    assert d.getNumberInstances() == want.shape[0]


@pytest.mark.parametrize("name,fmt", [("simple.arff", 0), ("simple.csv", 1)])
def test_reference_reader_fixtures(lib, name, fmt):
    """test_readARFF.cpp / test_readCSV.cpp: full read with and without targets, cutoff 2,
    columns (4, 2, 0), targets {7, 42.42}."""
    path = os.path.join(REF_SRC, "datadriven", "datasets", "dataread", name)
    if not os.path.exists(path):
        pytest.skip("the reference's reader fixtures are not present")
    raw = open(path, "rb").read()
    tag = name.replace(".", "_")
    assert hashlib.sha256(raw).hexdigest() == str(G[tag + "_sha256"])
    cases = [dict(hasTargets=True), dict(hasTargets=False), dict(hasTargets=True, instanceCutoff=2),
             dict(hasTargets=True, selectedCols=[4, 2, 0]),
             dict(hasTargets=True, selectedTargets=[7.0, 42.42])]
    for j, kw in enumerate(cases):
        if fmt == 0:
            d = sg.ARFFTools.readARFFFromString(raw, **kw)
        else:
            d = sg.CSVTools.readCSVFromString(raw, skipFirstLine=True, **kw)
        np.testing.assert_array_equal(d.getData(), G[f"{tag}_c{j}_data"])
        if kw["hasTargets"]:
            np.testing.assert_array_equal(d.getTargets(), G[f"{tag}_c{j}_y"])


def test_sizes_and_errors(lib, tmp_path):
    text = "@RELATION r\n@ATTRIBUTE a NUMERIC\n@DATA\n1,2,3\n4,5,6\n% c\n7,8,9\n"
    assert sg.ARFFTools.readARFFSizeFromString(text) == (3, 2)
    assert sg.ARFFTools.readARFFSizeFromString(text, False) == (3, 3)
    assert sg.ARFFTools.readARFFSizeFromString(text, True, [6.0]) == (1, 2)
    # a cutoff of 0 gives an empty data set (the reference writes into an empty matrix there)
    d = sg.ARFFTools.readARFFFromString(text, instanceCutoff=0)
    assert d.getNumberInstances() == 0
    with pytest.raises(sg.FileException, match="Columns missing"):
        sg.ARFFTools.readARFFFromString("1,2,3\n4,5\n")
    with pytest.raises(sg.FileException, match="col selection"):
        sg.ARFFTools.readARFFFromString(text, selectedCols=[2])
    # files, plain and gzip-compressed
    import gzip
    p = tmp_path / "d.arff"
    p.write_text(text)
    pz = tmp_path / "d.arff.gz"
    with gzip.open(pz, "wt") as f:
        f.write(text)
    a = sg.ARFFTools.readARFFFromFile(str(p))
    b = sg.ARFFTools.readARFFFromFile(str(pz))
    np.testing.assert_array_equal(a.getData(), b.getData())
    np.testing.assert_array_equal(a.getTargets(), [3.0, 6.0, 9.0])
    with pytest.raises(sg.FileException):
        sg.ARFFTools.readARFFFromFile(str(tmp_path / "missing.arff"))


def test_regression_text_parses_like_the_reference(lib):
    d = sg.ARFFTools.readARFFFromString(str(G["fit_text"]))
    np.testing.assert_array_equal(d.getData(), G["fit_data"])
    np.testing.assert_array_equal(d.getTargets(), G["fit_y"])


@pytest.mark.gpu
def test_gpu_fit_from_arff_text(oracle):
    """ARFF text -> reader -> operator with a bounding box (mapped on the device) -> fit."""
    d = sg.ARFFTools.readARFFFromString(str(G["fit_text"]))
    x, y = d.getData(), d.getTargets()
    grid = sg.Grid.createLinearGrid(4)
    grid.getGenerator().regular(4)
    bb = grid.getBoundingBox()
    for t in range(4):
        bb.setBoundary(t, sg.BoundingBox1D(-0.5, 1.5))
    cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                sg.OperationMultipleEvalSubType.CUDA)
    op = sg.createOperationMultipleEval(grid, x, cfg)
    alpha, _, _ = op.fit(y, 1e-4, 2000, 1e-12)
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    xu = oracle.bb_to_unit(x, [-0.5] * 4, [1.5] * 4)
    ref, _, _ = oracle.stream(xu).cg_fit(lp, ix, y, 1e-4, 2000, 1e-12)
    assert rel_err(alpha, ref) < 1e-9

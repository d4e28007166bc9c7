"""The benchmark's byte model and peak lookup (bench.py), on the CPU.

The roofline fraction bench.py reports is algorithmic bytes per launch over the launch time and the
measured HBM copy bandwidth; these tests pin the byte model to the storage the kernels stream.
"""
import json
import os

import numpy as np

import bench
import sgpp_gb300 as sg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _lp(dim, level):
    g = sg.Grid.createLinearGrid(dim)
    g.getGenerator().regular(level)
    return g.getStorage().getLevelIndexArraysForEval()[0], g.getSize()


def test_benchmark_grid_sizes():
    grid, lp, _ = bench.grid_arrays()
    assert grid.getSize() == 13441
    assert bench.subspace_count(lp) == 1001  # level vectors with |l|_1 <= 14 in 10 dimensions
    assert bench.cell_bytes(lp) == 0.5       # at most 2^(14 - 10) = 16 cells: nibbles


def test_cell_bytes_switch_to_bytes_above_16_cells():
    lp, _ = _lp(2, 7)  # up to 2^6 = 64 cells per subspace
    assert bench.cell_bytes(lp) == 1.0
    lp, _ = _lp(3, 5)  # up to 2^4 = 16 cells
    assert bench.cell_bytes(lp) == 0.5


def test_bytes_per_launch_match_the_stored_entries():
    _, lp, _ = bench.grid_arrays()
    m, n = 1 << 20, 13441
    entries = m * 1024  # padded points x padded subspaces
    vec32 = 4 * m + 8 * n
    # FP16 products (2 B) + nibble cells (0.5 B): the FP16 kernels' pair layout holds the same bytes
    assert bench.mat_bytes_per_launch("multT_mat16", lp, m, n) == entries * 2.5 + vec32
    assert bench.mat_bytes_per_launch("mult_mat16", lp, m, n) == entries * 2.5 + vec32
    # FP32 products (4 B) + nibble cells; float-float products (8 B) + nibble cells
    assert bench.mat_bytes_per_launch("multT_mat32", lp, m, n) == entries * 4.5 + vec32
    assert bench.mat_bytes_per_launch("multT_matdf64", lp, m, n) == entries * 8.5 + 8 * m + 8 * n
    # padding: points to a multiple of 1024, subspaces to a multiple of 32
    assert bench.mat_bytes_per_launch("mult_mat16", lp, 1000, n) == 1024 * 1024 * 2.5 + 4 * 1000 + 8 * n


def test_peak_comes_from_the_measured_file():
    gbs, src = bench.hbm_peak_gbs()
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        assert gbs == float(json.load(open(path))["hbm_gbs"])
        assert "of measured" in src
    else:
        assert gbs == 6800.0 and "of fallback" in src
    assert np.isfinite(gbs) and gbs > 0


def test_reference_arm_grid_matches_the_library_grid():
    """The reference arm builds the grid with the oracle; it must be the benchmark grid in the
    same point order as the library's (alpha indices line up)."""
    _, lp, ix = bench.grid_arrays()
    lp2, ix2 = bench.oracle_grid_arrays()
    np.testing.assert_array_equal(lp, lp2)
    np.testing.assert_array_equal(ix, ix2)


def test_reference_arm_loads_nothing_of_the_library():
    """bench.py --impl reference times the reference's CPU path only: its grid, data and timing
    helpers import no module of this library (checked in a fresh interpreter)."""
    import subprocess
    import sys

    code = ("import sys, numpy as np, bench\n"
            "lp, ix = bench.oracle_grid_arrays()\n"
            "x, y = bench.make_workload(42, m=2048)\n"
            "ref = bench.CpuReference(x, lp, ix, 2)\n"
            "ref.warm(); ref.apply_seconds(); ref.close()\n"
            "bad = [k for k in sys.modules if k.startswith('sgpp_gb300')]\n"
            "assert not bad, bad\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_both_arms_print_the_same_config():
    a = bench.bench_config("linear", 13441, 1 << 20, 1e-8, 1)
    b = bench.bench_config("linear", 13441, 1 << 20, 1e-8, 1)
    assert a == b and "13441" in a["workload"] and "1e-08" in a["workload"]
    assert "mixed" not in a["workload"]  # the precision scheme is a key of its own


def test_cpu_operator_count_per_fit():
    # ConjugateGradients.cpp:22-151: one B^T B per iteration, a true residual every 50, b = B^T y
    assert bench.cg_operator_applications(75) == 75 + 1 + 0.5

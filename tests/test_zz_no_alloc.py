"""sgmev_mult_transpose_noalloc: B^T v for callers that cannot allocate GPU memory.

Such callers — an application whose own memory manager owns the whole device budget, or a
latency-critical loop that cannot afford the implicit synchronisation of cudaMalloc / cudaFree —
pass device buffers they already own; the entry point keeps its scratch in a fixed array inside
the library. This test calls it through the C ABI and compares it with the existing entry point
(sgmev_mult_transpose on an operator) and with the oracle's FP64 multTranspose, at the FP64
tolerance of the other parity tests, on two calls in a row with different inputs (the shared
scratch must not leak between calls), and checks that an empty data set gives zeros.

The file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

import sgpp_gb300 as sg
from oracle import Oracle

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("dim,level,m", [(5, 4, 3000), (10, 3, 4097), (20, 2, 777), (2, 6, 1)])
def test_noalloc_matches_existing_entry_point_on_two_calls(lib, dim, level, m):
    torch = pytest.importorskip("torch")
    if lib.sgmev_device_count() < 1:
        pytest.fail("no CUDA device visible")
    orc = Oracle()
    rng = np.random.default_rng(100 + dim)
    grid = sg.Grid.createLinearGrid(dim)
    grid.getGenerator().regular(level)
    n = grid.getSize()
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    x = rng.random((m, dim))
    op = sg.createOperationMultipleEval(grid, x)  # the existing entry point
    dev = torch.device("cuda:0")
    d_lp = torch.from_numpy(np.ascontiguousarray(lp)).to(dev)
    d_ix = torch.from_numpy(np.ascontiguousarray(ix)).to(dev)
    d_x = torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    vp = ctypes.c_void_p
    for call in range(2):
        v = rng.standard_normal(m)
        expected = np.zeros(n)
        op.multTranspose(v, expected)
        d_v = torch.from_numpy(v).to(dev)
        d_out = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
        rc = lib.sgmev_mult_transpose_noalloc(dim, n, vp(d_lp.data_ptr()), vp(d_ix.data_ptr()),
                                              m, vp(d_x.data_ptr()), vp(d_v.data_ptr()),
                                              vp(d_out.data_ptr()), vp(stream or None))
        assert rc == sg.SGMEV_OK, lib.sgmev_last_error()
        torch.cuda.synchronize(dev)
        got = d_out.cpu().numpy()
        assert np.isfinite(got).all()
        assert _rel(got, expected) < FP64_TOL, (call, _rel(got, expected))
        ref = orc.mult_transpose_naive(lp, ix, x, v)
        assert _rel(got, ref) < FP64_TOL, (call, _rel(got, ref))
    op.close()


def test_noalloc_empty_data_gives_zeros(lib):
    torch = pytest.importorskip("torch")
    if lib.sgmev_device_count() < 1:
        pytest.fail("no CUDA device visible")
    grid = sg.Grid.createLinearGrid(4)
    grid.getGenerator().regular(3)
    n = grid.getSize()
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    dev = torch.device("cuda:0")
    d_lp = torch.from_numpy(np.ascontiguousarray(lp)).to(dev)
    d_ix = torch.from_numpy(np.ascontiguousarray(ix)).to(dev)
    d_out = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
    vp = ctypes.c_void_p
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = lib.sgmev_mult_transpose_noalloc(4, n, vp(d_lp.data_ptr()), vp(d_ix.data_ptr()), 0, None,
                                          None, vp(d_out.data_ptr()), vp(stream or None))
    assert rc == sg.SGMEV_OK, lib.sgmev_last_error()
    torch.cuda.synchronize(dev)
    assert (d_out.cpu().numpy() == 0.0).all()


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    if lib.sgmev_device_count() < 1:
        pytest.fail("no CUDA device visible")
    vp = ctypes.c_void_p
    rc = lib.sgmev_mult_transpose_noalloc(3, (1 << 21) + 1, vp(8), vp(8), 10, vp(8), vp(8), vp(8),
                                          None)
    assert rc == sg.SGMEV_ERR_INVALID
    assert b"exceeds the no-alloc scratch capacity" in lib.sgmev_last_error()
    rc = lib.sgmev_mult_transpose_noalloc(65, 10, vp(8), vp(8), 10, vp(8), vp(8), vp(8), None)
    assert rc == sg.SGMEV_ERR_INVALID

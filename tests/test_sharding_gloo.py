"""Data-parallel split over two gloo ranks on CPU: the sharded system matrix and the replicated CG
give the single-process oracle's result, and both ranks hold bit-identical alpha.

The per-shard operator here is a small dense-matrix stand-in built from the oracle (CPU test
infrastructure); on a GPU host each rank uses the CUDA operator on its shard."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT, rel_err

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


class _DenseShardOp:
    def __init__(self, B):
        self.B = B

    def mult(self, a, out):
        out[:] = self.B @ a

    def multTranspose(self, v, out):
        out[:] = self.B.T @ v


def _worker(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    from oracle import Oracle

    import sgpp_gb300 as sg
    from sgpp_gb300.sharding import ShardedSystemMatrix

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    orc = Oracle()
    rng = np.random.default_rng(17)
    d, level, m = 3, 4, 1001
    lev, idx = orc.regular_grid(d, level)
    lp, ix = orc.eval_arrays(lev, idx)
    X = rng.random((m, d))
    y = np.sin(2 * X[:, 0]) + X[:, 1] * X[:, 2]
    n = lp.shape[0]

    def make_op(Xs):
        B = np.zeros((Xs.shape[0], n))
        for i in range(n):
            e = np.zeros(n)
            e[i] = 1.0
            B[:, i] = orc.mult_naive(lp, ix, Xs, e)
        return _DenseShardOp(B)

    A = ShardedSystemMatrix(n, X, 1e-3, make_op)
    b = np.zeros(n)
    A.generateb(y, b)
    alpha = np.zeros(n)
    cg = sg.ConjugateGradients(1000, 1e-12)
    cg.solve(A, alpha, b, False, False, 0.0)
    np.save(os.path.join(out_dir, f"alpha_{rank}.npy"), alpha)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharded_fit(tmp_path, oracle):
    import socket

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    a0 = np.load(tmp_path / "alpha_0.npy")
    a1 = np.load(tmp_path / "alpha_1.npy")
    assert np.array_equal(a0, a1)
    rng = np.random.default_rng(17)
    d, level, m = 3, 4, 1001
    lev, idx = oracle.regular_grid(d, level)
    lp, ix = oracle.eval_arrays(lev, idx)
    X = rng.random((m, d))
    y = np.sin(2 * X[:, 0]) + X[:, 1] * X[:, 2]
    ref, _, _ = oracle.stream(X).cg_fit(lp, ix, y, 1e-3, 1000, 1e-12)
    assert rel_err(a0, ref) < 1e-8


def test_shard_ranges_cover_exactly():
    from sgpp_gb300.sharding import shard_range

    for m in (0, 1, 7, 1000, 1001):
        for world in (1, 2, 3, 8):
            rs = [shard_range(m, r, world) for r in range(world)]
            assert rs[0][0] == 0 and rs[-1][1] == m
            assert all(rs[k][1] == rs[k + 1][0] for k in range(world - 1))
            assert max(e - s for s, e in rs) - min(e - s for s, e in rs) <= 1

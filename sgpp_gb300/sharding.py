"""Data-parallel split of the least-squares system over ranks (one GPU per rank).

Each rank owns the contiguous data range [start, end) of its rank in a balanced split (the
shape of the reference's master/worker multi-evaluation, OperationMultiEvalMPI.cpp:53-164, and of
the ranged interface OperationMultipleEval::mult(alpha, result, start, end),
OperationMultipleEval.hpp:70-73). mult needs no communication (alpha is replicated); B^T v and the
system product B^T(B a) + lambda M a need one sum of N-vectors over ranks, done as an all-gather
followed by a sum in rank order, so every rank gets bit-identical results independent of the
communication library's reduction order. The CG loop then runs replicated on every rank.

The local operator is any object with mult(alpha, out) / multTranspose(v, out) over the rank's
data shard — on a GPU host the CUDA operator built on that shard.
"""
from __future__ import annotations

from typing import Callable

import numpy as np


def shard_range(m: int, rank: int, world: int):
    """Balanced contiguous split of m data points (first m % world ranks get one more)."""
    base, extra = divmod(m, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


class ShardedSystemMatrix:
    """(B^T B + lambda*M*I) over data split across torch.distributed ranks."""

    def __init__(self, n_grid: int, data, lam: float, make_op: Callable, group=None):
        import torch.distributed as dist

        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        self.m_total = int(data.shape[0])
        self.start, self.end = shard_range(self.m_total, self.rank, self.world)
        self.local = make_op(np.ascontiguousarray(data[self.start:self.end]))
        self.n = int(n_grid)
        self.lam = float(lam)

    def _sum_ranks(self, vec: np.ndarray) -> np.ndarray:
        import torch

        t = torch.from_numpy(np.ascontiguousarray(vec, np.float64))
        parts = [torch.empty_like(t) for _ in range(self.world)]
        self.dist.all_gather(parts, t, group=self.group)
        out = np.zeros_like(vec)
        for p in parts:  # fixed rank order: deterministic on every rank
            out += p.numpy()
        return out

    def multLocal(self, alpha, out_local) -> None:
        self.local.mult(alpha, out_local)

    def multTranspose(self, v_local, out) -> None:
        part = np.zeros(self.n)
        self.local.multTranspose(v_local, part)
        out[:] = self._sum_ranks(part)

    def mult(self, alpha, result) -> None:
        """OperationMatrix::mult: result = sum_ranks B_r^T (B_r alpha) + lambda*M*alpha."""
        tmp = np.zeros(self.end - self.start)
        self.local.mult(alpha, tmp)
        part = np.zeros(self.n)
        self.local.multTranspose(tmp, part)
        result[:] = self._sum_ranks(part) + self.lam * self.m_total * np.asarray(alpha)

    def generateb(self, y_full, b) -> None:
        self.multTranspose(np.ascontiguousarray(y_full[self.start:self.end]), b)

"""Regression-fit servers: continuous batching over the batch engine (sgmev_batch_*), or a pool
of worker threads that each fit one request at a time with its own operator (subspace and
materialised products, own CUDA stream).

Requests (grid, X, Y, lambda, epsilon) arrive over time. The loop admits waiting requests in
arrival order while a slot and pool space are free (admission by device-memory footprint: the
engine's pools are sized once and a problem is admitted only if its padded grid, data and vector
blocks fit), advances every resident problem by a few steps, hands finished results back and
frees their slots. Grids, data and CG state stay on the device for a request's whole life; work of
requests that arrive while others run overlaps with theirs in the same launches.

    python -m sgpp_gb300.serving --rate 200 --duration 20 --max-work 2e10 [--engine pool|batch]

The pool server (default): a request is admitted in arrival order when a worker is free and its
device-memory footprint (staged data, grid, CG vectors and the materialised products the library
would build for it) fits what the fits in flight leave of the memory budget (by default 80 % of
the device memory free when the run starts; a request larger than the whole budget runs alone);
the worker creates the operator for the request's grid and data (algo and materialisation chosen
by the library), runs the device-resident mixed-precision fit and frees the operator. Workers
overlap on the GPU through their streams; the host waits of one fit (its CG scalars) are hidden
by the other workers' launches. The library call releases the GIL.

prints one JSON line: completed fits/s, offered load, p50/p99 latency, queue depth.
Synthetic requests follow the batched-fit size mix (d uniform in 2..12, level in 3..7, data size
log-uniform in [1e3, 2^20], uniform data), optionally truncated to N*M*d <= --max-work.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import sys
import time
import weakref
from typing import Callable, Dict, List, Optional

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import sgpp_gb300 as sg  # noqa: E402


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float          # seconds after the start of the run
    grid: "sg.Grid"
    X: np.ndarray
    Y: np.ndarray
    lam: float
    epsilon: float = 1e-8
    # filled in by the server
    admitted: Optional[float] = None
    finished: Optional[float] = None
    alpha: Optional[np.ndarray] = None
    iterations: int = 0
    residual: float = 0.0
    footprint: int = 0      # device bytes the pool server reserved for the request


# subspace count per live grid object (with the size it was counted at: grids can grow)
_SUBSPACES: "weakref.WeakKeyDictionary" = weakref.WeakKeyDictionary()


def _keep(keep_alpha, r: "Request") -> bool:
    """keep_alpha: True / False for every request, or a predicate of the request."""
    return bool(keep_alpha(r)) if callable(keep_alpha) else bool(keep_alpha)


def request_footprint(grid: "sg.Grid", m: int) -> int:
    """Device bytes one request's operator and fit hold, as the pool server budgets them: the data
    staged dim-major in FP64, FP32 and FP32 low parts (points padded to 1024), the grid arrays,
    the CG vectors, and the materialised subspace products (P_hi, P_lo, the FP16 copy and the
    cells, 12 bytes per padded point and padded subspace while they are built, at most 64 GiB, the
    library's own cap)."""
    d, n = grid.getDimension(), grid.getSize()
    mpad = -(-max(m, 1) // 1024) * 1024
    npad = -(-max(n, 1) // 512) * 512
    try:
        cached = _SUBSPACES.get(grid)
    except TypeError:  # an object without weak references: count every time
        cached = None
    if cached is not None and cached[0] == n:
        n_sub = cached[1]
    else:
        lp, _ = grid.getStorage().getLevelIndexArraysForEval()
        n_sub = len(np.unique(np.asarray(lp), axis=0)) if n else 0
        try:
            _SUBSPACES[grid] = (n, n_sub)
        except TypeError:
            pass
    s_pad = -(-n_sub // 32) * 32
    products = min(mpad * s_pad * 12, 64 << 30)
    return int(mpad * d * 16 + npad * d * 32 + 12 * npad * 8 + 4 * mpad * 8 + products)


class FitServer:
    def __init__(self, max_slots: int = 64, rhs: int = 1, grid_capacity: int = 1 << 24,
                 data_capacity: int = 1 << 26, steps_per_poll: int = 4):
        self.engine = sg.BatchEngine(max_slots, rhs, grid_capacity, data_capacity)
        self.steps_per_poll = steps_per_poll
        self.queue_depths: List[int] = []

    def close(self) -> None:
        self.engine.close()

    def run(self, requests: List[Request], clock: Callable[[], float] = time.perf_counter,
            keep_alpha: bool = True, max_seconds: float = 1e9) -> List[Request]:
        """Serve `requests` (sorted by arrival) in real time; returns the completed ones."""
        pending = sorted(requests, key=lambda r: r.arrival)
        waiting: List[Request] = []
        resident: Dict[int, Request] = {}
        done: List[Request] = []
        t0 = clock()
        k = 0
        while (k < len(pending) or waiting or resident) and clock() - t0 < max_seconds:
            now = clock() - t0
            while k < len(pending) and pending[k].arrival <= now:
                waiting.append(pending[k])
                k += 1
            # FIFO admission while a slot and pool space are free
            while waiting:
                r = waiting[0]
                slot = self.engine.tryAdd(r.grid, r.X, r.Y, r.lam, r.epsilon)
                if slot is None:
                    if not resident:
                        raise sg.OperationException(
                            f"request {r.rid} does not fit into an empty engine")
                    break
                r.admitted = clock() - t0
                resident[slot] = r
                waiting.pop(0)
            self.queue_depths.append(len(waiting))
            if not resident:
                # idle until the next arrival
                if k < len(pending):
                    time.sleep(max(0.0, min(0.001, pending[k].arrival - (clock() - t0))))
                continue
            phases = self.engine.step(self.steps_per_poll)
            for slot in list(resident):
                if phases[slot] == sg.BatchEngine.PHASE_DONE:
                    r = resident.pop(slot)
                    alpha, r.iterations, r.residual, _ = self.engine.result(slot)
                    r.alpha = alpha if _keep(keep_alpha, r) else None
                    r.finished = clock() - t0
                    self.engine.remove(slot)
                    done.append(r)
        return done


class PoolServer:
    """Worker threads, each fitting one request at a time with its own operator."""

    def __init__(self, workers: int = 8, params: Optional[dict] = None,
                 memory_budget: Optional[int] = None):
        self.workers = workers
        self.params = dict(params or {})
        self.memory_budget = memory_budget  # bytes; None: 80 % of the free device memory
        self.queue_depths: List[int] = []
        self.phase_seconds = {"create": 0.0, "fit": 0.0, "close": 0.0}
        self.peak_reserved = 0
        self.budget_used: Optional[int] = None  # the budget of the last run

    def footprint(self, r: Request) -> int:
        return request_footprint(r.grid, r.X.shape[0])

    def _budget(self) -> int:
        if self.memory_budget is not None:
            return int(self.memory_budget)
        import torch

        free, _ = torch.cuda.mem_get_info()
        return int(0.8 * free)

    def close(self) -> None:
        pass

    def _fit(self, r: Request, keep_alpha: bool) -> None:
        cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                    sg.OperationMultipleEvalSubType.CUDA,
                                                    parameters=self.params)
        t0 = time.perf_counter()
        op = sg.createOperationMultipleEval(r.grid, r.X, cfg)
        t1 = time.perf_counter()
        try:
            alpha, r.iterations, r.residual = op.fit(np.ascontiguousarray(r.Y[:, 0]), r.lam,
                                                     100000, r.epsilon,
                                                     mode=sg.SGMEV_SOLVE_MIXED)
        finally:
            t2 = time.perf_counter()
            op.close()
        t3 = time.perf_counter()
        self.phase_seconds["create"] += t1 - t0  # (unsynchronised sums: a rough split)
        self.phase_seconds["fit"] += t2 - t1
        self.phase_seconds["close"] += t3 - t2
        r.alpha = alpha if _keep(keep_alpha, r) else None

    def run(self, requests: List[Request], clock: Callable[[], float] = time.perf_counter,
            keep_alpha: bool = True, max_seconds: float = 1e9) -> List[Request]:
        """Serve `requests` (sorted by arrival) in real time; returns the completed ones."""
        import queue
        import threading

        pending = sorted(requests, key=lambda r: r.arrival)
        work: "queue.Queue[Optional[Request]]" = queue.Queue()
        done: List[Request] = []
        lock = threading.Lock()
        errors: List[BaseException] = []
        budget = self._budget()
        self.budget_used = budget
        # admission in arrival order: ticket k is admitted once tickets 0 .. k-1 are and its
        # footprint fits next to the fits in flight (alone if it exceeds the whole budget)
        mem = threading.Condition()
        state = {"next": 0, "reserved": 0, "running": 0}
        t0 = clock()

        def admit(r: Request, ticket: int) -> None:
            with mem:
                mem.wait_for(lambda: state["next"] == ticket and (
                    state["running"] == 0 or state["reserved"] + r.footprint <= budget))
                state["next"] += 1
                state["reserved"] += r.footprint
                state["running"] += 1
                self.peak_reserved = max(self.peak_reserved, state["reserved"])
                mem.notify_all()

        def release(r: Request) -> None:
            with mem:
                state["reserved"] -= r.footprint
                state["running"] -= 1
                mem.notify_all()

        def worker():
            while True:
                item = work.get()
                if item is None:
                    return
                ticket, r = item
                if clock() - t0 > max_seconds:
                    with mem:  # past the deadline: drop it, in its turn
                        mem.wait_for(lambda: state["next"] == ticket)
                        state["next"] += 1
                        mem.notify_all()
                    continue
                try:
                    r.footprint = self.footprint(r)
                except BaseException as e:  # reported after the run; the ticket still passes
                    with lock:
                        errors.append(e)
                    r.footprint = 0
                admit(r, ticket)
                r.admitted = clock() - t0
                try:
                    self._fit(r, keep_alpha)
                except BaseException as e:  # reported after the run
                    with lock:
                        errors.append(e)
                    continue
                finally:
                    release(r)
                r.finished = clock() - t0
                with lock:
                    done.append(r)

        threads = [threading.Thread(target=worker, daemon=True) for _ in range(self.workers)]
        for t in threads:
            t.start()
        for k, r in enumerate(pending):
            wait = r.arrival - (clock() - t0)
            if wait > 0:
                time.sleep(wait)
            work.put((k, r))
            self.queue_depths.append(work.qsize())
        for _ in threads:
            work.put(None)
        for t in threads:
            t.join()
        if errors:
            raise errors[0]
        return done


def percentile(values: List[float], q: float) -> float:
    if not values:
        return float("nan")
    v = sorted(values)
    return v[min(len(v) - 1, int(round(q * (len(v) - 1))))]


class MixGenerator:
    """Synthetic requests of the batched-fit size mix; grids are cached per (d, level) and the
    data of a request is drawn from a pool of pre-generated matrices (per dimension)."""

    def __init__(self, seed: int = 0, max_work: float = float("inf"), pool: int = 8,
                 max_points: int = 1 << 20, pinned: bool = False):
        self.pinned = pinned
        self._keep = []  # pinned tensors backing the pooled matrices
        self.rng = np.random.default_rng(seed)
        self.max_work = max_work
        self.max_points = max_points
        self.grids: Dict[tuple, sg.Grid] = {}
        self.pool = pool
        self.data: Dict[int, List[np.ndarray]] = {}

    def grid(self, d: int, level: int) -> "sg.Grid":
        key = (d, level)
        if key not in self.grids:
            g = sg.Grid.createLinearGrid(d)
            g.getGenerator().regular(level)
            self.grids[key] = g
        return self.grids[key]

    def _x(self, d: int, m: int) -> np.ndarray:
        lst = self.data.setdefault(d, [])
        if len(lst) < self.pool:
            a = self.rng.random((self.max_points, d))
            if self.pinned:  # request data in page-locked host memory, as a server's receive
                import torch  # buffers would be; host-to-device copies then run at full speed

                t = torch.from_numpy(a).pin_memory()
                self._keep.append(t)
                a = t.numpy()
            lst.append(a)
        base = lst[int(self.rng.integers(0, len(lst)))]
        off = int(self.rng.integers(0, self.max_points - m + 1))
        return base[off:off + m]

    def draw(self, rhs: int = 1):
        for _ in range(1000):
            d = int(self.rng.integers(2, 13))
            level = int(self.rng.integers(3, 8))
            m = int(np.exp(self.rng.uniform(np.log(1e3), np.log(self.max_points))))
            n = sg.Grid.regularSize(d, level)
            if n * m * d <= self.max_work:
                break
        X = self._x(d, m)
        Y = self.rng.standard_normal((m, rhs))
        return self.grid(d, level), X, Y


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--rate", type=float, default=200.0, help="mean arrivals per second")
    ap.add_argument("--duration", type=float, default=20.0, help="arrival window in seconds")
    ap.add_argument("--max-work", type=float, default=2e10, help="cap on N*M*d per request")
    ap.add_argument("--max-slots", type=int, default=64)
    ap.add_argument("--epsilon", type=float, default=1e-8)
    ap.add_argument("--lam", type=float, default=1e-4)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--drain-seconds", type=float, default=60.0)
    ap.add_argument("--engine", choices=["pool", "batch"], default="pool")
    ap.add_argument("--workers", type=int, default=8, help="pool server: concurrent fits")
    ap.add_argument("--check-every", type=int, default=500,
                    help="keep alpha of every n-th request for the FP64 check")
    ap.add_argument("--checks", type=int, default=6, help="served requests checked against FP64")
    ap.add_argument("--pinned", action="store_true",
                    help="request data in page-locked host memory (receive buffers)")
    args = ap.parse_args()

    gen = MixGenerator(args.seed, args.max_work, pinned=args.pinned)
    rng = np.random.default_rng(args.seed + 1)
    t, reqs = 0.0, []
    while True:
        t += rng.exponential(1.0 / args.rate)
        if t > args.duration:
            break
        g, X, Y = gen.draw()
        reqs.append(Request(len(reqs), t, g, X, Y, args.lam, args.epsilon))
    if args.engine == "pool":
        server = PoolServer(workers=args.workers)
    else:
        server = FitServer(max_slots=args.max_slots, grid_capacity=1 << 25,
                           data_capacity=1 << 27)
    t0 = time.perf_counter()
    # alpha is kept for every check_every-th request only (checked against FP64 afterwards)
    done = server.run(reqs, keep_alpha=lambda r: r.rid % args.check_every == 0,
                      max_seconds=args.duration + args.drain_seconds)
    wall = time.perf_counter() - t0
    # the served alphas against FP64 solutions of the same requests (df64-refined fits to 1e-12)
    errs = []
    for r in sorted((r for r in done if r.alpha is not None), key=lambda r: r.rid)[:args.checks]:
        op = sg.createOperationMultipleEval(r.grid, r.X)
        ref, _, _ = op.fit(np.ascontiguousarray(r.Y[:, 0]), r.lam, 100000, 1e-12,
                           mode=sg.SGMEV_SOLVE_MIXED)
        op.close()
        errs.append(float(np.abs(r.alpha - ref).max() / max(np.abs(ref).max(), 1e-300)))
    lat = [r.finished - r.arrival for r in done]
    line = {
        "metric": "served_fits_per_sec", "value": len(done) / wall, "unit": "fits/s",
        "offered_rate": args.rate, "requests": len(reqs), "completed": len(done),
        "wall_s": wall, "latency_ms": {"p50": 1e3 * percentile(lat, 0.5),
                                        "p99": 1e3 * percentile(lat, 0.99)},
        "alpha_rel_err_vs_fp64": {"max": max(errs) if errs else None, "checked": len(errs)},
        "queue_depth": {"max": max(server.queue_depths or [0]),
                        "mean": float(np.mean(server.queue_depths or [0]))},
        "config": {"mix": "d in 2..12, level 3..7, M log-uniform [1e3, 2^20], uniform data",
                   "max_work_NMd": args.max_work, "epsilon": args.epsilon, "lambda": args.lam,
                   "engine": args.engine, "pinned_request_data": args.pinned,
                   **({"workers": args.workers} if args.engine == "pool" else
                      {"slots": args.max_slots, "engine_steps": server.engine.info()["steps"]})},
    }
    if args.engine == "pool":
        line["worker_seconds"] = server.phase_seconds
        line["memory"] = {"budget_bytes": server.budget_used,
                          "peak_reserved_bytes": server.peak_reserved}
    print(json.dumps(line))
    server.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())

"""Host logic of the fit servers (sgpp_gb300/serving.py), on the CPU.

The servers' scheduling is plain Python around the GPU work: FitServer admits requests in arrival
order into the batch engine's slots and retires them when their phase is done; PoolServer hands
requests to worker threads. Here the GPU parts are replaced by fakes, so the order of admission,
the bookkeeping of times, the deadline and the error paths are checked without a device.
"""
import threading
import time

import numpy as np
import pytest

import sgpp_gb300 as sg
from sgpp_gb300 import serving


def _requests(n, gap=0.0, y_cols=1):
    return [serving.Request(rid=k, arrival=k * gap, grid=None, X=np.zeros((4, 2)),
                            Y=np.full((4, y_cols), float(k)), lam=1e-3)
            for k in range(n)]


class FakeEngine:
    """The BatchEngine calls FitServer makes: tryAdd / step / result / remove."""
    PHASE_DONE = sg.BatchEngine.PHASE_DONE

    def __init__(self, slots, steps_to_finish=2):
        self.slots = [None] * slots
        self.left = {}
        self.steps_to_finish = steps_to_finish
        self.added = []

    def tryAdd(self, grid, X, Y, lam, eps):
        for s, occupant in enumerate(self.slots):
            if occupant is None:
                self.slots[s] = float(Y[0, 0])
                self.left[s] = self.steps_to_finish
                self.added.append(int(Y[0, 0]))
                return s
        return None

    def step(self, n):
        phases = [0] * len(self.slots)
        for s in list(self.left):
            self.left[s] -= 1
            if self.left[s] <= 0:
                phases[s] = self.PHASE_DONE
        return phases

    def result(self, slot):
        return np.array([self.slots[slot]]), 7, 1e-9, 0

    def remove(self, slot):
        self.slots[slot] = None
        del self.left[slot]


def _fit_server(engine):
    srv = serving.FitServer.__new__(serving.FitServer)
    srv.engine = engine
    srv.steps_per_poll = 1
    srv.queue_depths = []
    return srv


def test_fit_server_admits_in_arrival_order_and_retires_every_request():
    engine = FakeEngine(slots=3)
    srv = _fit_server(engine)
    reqs = _requests(10, gap=1e-4)
    done = srv.run(list(reversed(reqs)))  # the server sorts by arrival
    assert sorted(r.rid for r in done) == list(range(10))
    assert engine.added == list(range(10))  # FIFO admission
    for r in done:
        assert r.alpha[0] == float(r.rid)  # each slot's own result
        assert r.iterations == 7 and r.residual == 1e-9
        assert r.arrival <= r.admitted <= r.finished
    assert max(srv.queue_depths) <= 10 and all(s is None for s in engine.slots)


def test_fit_server_rejects_a_request_that_does_not_fit_an_empty_engine():
    srv = _fit_server(FakeEngine(slots=0))
    with pytest.raises(sg.OperationException, match="does not fit into an empty engine"):
        srv.run(_requests(1))


class FakePool(serving.PoolServer):
    def __init__(self, workers, fail_rid=None, delay=0.002):
        super().__init__(workers=workers, memory_budget=1 << 40)
        self.fail_rid = fail_rid
        self.delay = delay
        self.concurrent = 0
        self.peak = 0
        self._lock = threading.Lock()

    def footprint(self, r):
        return 0

    def _fit(self, r, keep_alpha):
        with self._lock:
            self.concurrent += 1
            self.peak = max(self.peak, self.concurrent)
        try:
            time.sleep(self.delay)
            if r.rid == self.fail_rid:
                raise sg.OperationException(f"fit of request {r.rid} failed")
            r.iterations = 3
            r.alpha = np.array([float(r.rid)]) if keep_alpha else None
        finally:
            with self._lock:
                self.concurrent -= 1


def test_pool_server_serves_every_request_with_bounded_concurrency():
    srv = FakePool(workers=3)
    done = srv.run(_requests(12, gap=0.0005))
    assert sorted(r.rid for r in done) == list(range(12))
    assert 1 <= srv.peak <= 3
    for r in done:
        assert r.arrival <= r.admitted + 1e-3 and r.admitted <= r.finished
        assert r.alpha[0] == float(r.rid)
    assert len(srv.queue_depths) == 12


def test_pool_server_reports_a_failed_fit_after_the_run():
    srv = FakePool(workers=2, fail_rid=4)
    with pytest.raises(sg.OperationException, match="request 4 failed"):
        srv.run(_requests(8))


def test_pool_server_drops_queued_requests_past_the_deadline():
    srv = FakePool(workers=1, delay=0.02)
    done = srv.run(_requests(20), max_seconds=0.05)
    assert len(done) < 20  # the rest were dropped (none at all if the worker started late)
    assert sorted(r.rid for r in done) == list(range(len(done)))  # served in arrival order


def test_percentile():
    assert np.isnan(serving.percentile([], 0.5))
    v = [5.0, 1.0, 3.0, 2.0, 4.0]
    assert serving.percentile(v, 0.0) == 1.0
    assert serving.percentile(v, 0.5) == 3.0
    assert serving.percentile(v, 1.0) == 5.0


class BudgetPool(FakePool):
    """FakePool with a fixed footprint per request and a memory budget."""

    def __init__(self, workers, budget, sizes, delay=0.003):
        super().__init__(workers=workers, delay=delay)
        self.memory_budget = budget
        self.sizes = sizes
        self.order = []
        self.live = 0
        self.peak_live = 0

    def footprint(self, r):
        return self.sizes[r.rid]

    def _fit(self, r, keep_alpha):
        with self._lock:
            self.order.append(r.rid)
            self.live += r.footprint
            self.peak_live = max(self.peak_live, self.live)
        try:
            super()._fit(r, keep_alpha)
        finally:
            with self._lock:
                self.live -= r.footprint


def test_pool_server_admits_by_memory_footprint_in_arrival_order():
    sizes = [6, 6, 6, 3, 3, 6, 12, 1]  # the 12 exceeds the budget: it runs alone
    srv = BudgetPool(workers=4, budget=10, sizes=sizes)
    done = srv.run(_requests(len(sizes)))
    assert sorted(r.rid for r in done) == list(range(len(sizes)))
    assert srv.order == list(range(len(sizes)))  # admitted in arrival order
    # never more than the budget in flight, except the oversized request alone
    assert srv.peak_live <= 12 and srv.peak_reserved <= 12
    assert all(r.footprint == sizes[r.rid] for r in done)
    assert srv.budget_used == 10


def test_pool_server_runs_side_by_side_what_fits():
    srv = BudgetPool(workers=4, budget=100, sizes=[10] * 8, delay=0.02)
    srv.run(_requests(8))
    assert srv.peak >= 2  # the budget does not serialise requests that fit together


def test_request_footprint_counts_the_materialised_products():
    grid = sg.Grid.createLinearGrid(3)
    grid.getGenerator().regular(3)
    small = serving.request_footprint(grid, 1000)
    big = serving.request_footprint(grid, 100000)
    n_sub = 10  # level sums 3..5 in 3 dimensions: 1 + 3 + 6
    assert big - small >= (100352 - 1024) * 32 * 12  # products: 12 bytes per point and subspace
    assert small > 1024 * 32 * 12 and n_sub <= 32


def test_pool_server_keeps_admitting_after_a_footprint_error():
    class BadFootprint(BudgetPool):
        def footprint(self, r):
            if r.rid == 2:
                raise ValueError("no footprint for request 2")
            return super().footprint(r)

    srv = BadFootprint(workers=3, budget=10, sizes=[4] * 6)
    with pytest.raises(ValueError, match="request 2"):
        srv.run(_requests(6))
    assert sorted(srv.order) == list(range(6))  # every request still ran, in order


def test_request_footprint_recounts_a_grid_that_grew():
    grid = sg.Grid.createLinearGrid(2)
    grid.getGenerator().regular(2)
    before = serving.request_footprint(grid, 5000)
    n_sub_before = serving._SUBSPACES[grid][1]
    for _ in range(3):  # the same object, more points and subspaces
        alpha = np.ones(grid.getSize())
        grid.getGenerator().refine(sg.SurplusRefinementFunctor(alpha, grid.getSize(), 0.0))
    after = serving.request_footprint(grid, 5000)
    assert serving._SUBSPACES[grid] == (grid.getSize(), serving._SUBSPACES[grid][1])
    # the count was redone (3 -> 15 subspaces; both pad to 32, so the bytes may stay the same)
    assert serving._SUBSPACES[grid][1] > n_sub_before and after >= before

"""Continuous-batching server: every request completes, latency is measured from arrival, and
each result is bit-for-bit the result the same problem gets alone in an empty engine."""
import numpy as np
import pytest

import sgpp_gb300 as sg
from sgpp_gb300.serving import FitServer, MixGenerator, Request, percentile

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu(lib):
    if lib.sgmev_device_count() < 1:
        pytest.fail("no CUDA device visible")


def test_server_results_equal_alone_results():
    gen = MixGenerator(seed=3, max_work=2e7, max_points=4096)
    rng = np.random.default_rng(4)
    reqs, t = [], 0.0
    for rid in range(24):
        t += rng.exponential(1.0 / 500.0)  # arrivals faster than service: requests queue up
        g, X, Y = gen.draw()
        reqs.append(Request(rid, t, g, X, Y, 1e-3, 1e-9))
    server = FitServer(max_slots=6, grid_capacity=1 << 20, data_capacity=1 << 21, steps_per_poll=2)
    done = server.run(reqs)
    server.close()
    assert len(done) == len(reqs)
    assert max(server.queue_depths) > 0  # some requests had to wait for a slot
    lat = [r.finished - r.arrival for r in done]
    assert all(v > 0 for v in lat) and percentile(lat, 0.99) >= percentile(lat, 0.5)
    for r in done[:8]:
        eng = sg.BatchEngine(max_slots=1, rhs=1, grid_capacity=1 << 20, data_capacity=1 << 21)
        s = eng.add(r.grid, r.X, r.Y, r.lam, r.epsilon)
        eng.solve()
        alone, it, _, phase = eng.result(s)
        eng.close()
        assert phase == sg.BatchEngine.PHASE_DONE
        assert it == r.iterations
        assert np.array_equal(alone, r.alpha)


def test_pool_server_results_equal_alone_fits():
    """Worker-pool server: every request completes with the same alpha, bit for bit, as the same
    fit run alone (the operator's results do not depend on what else runs on the GPU)."""
    from sgpp_gb300.serving import PoolServer

    gen = MixGenerator(seed=6, max_work=5e7, max_points=8192)
    rng = np.random.default_rng(7)
    reqs, t = [], 0.0
    for rid in range(20):
        t += rng.exponential(1.0 / 500.0)
        g, X, Y = gen.draw()
        reqs.append(Request(rid, t, g, X, Y, 1e-3, 1e-9))
    server = PoolServer(workers=4)
    done = server.run(reqs)
    assert len(done) == len(reqs)
    lat = [r.finished - r.arrival for r in done]
    assert all(v > 0 for v in lat)
    for r in done[:6]:
        op = sg.createOperationMultipleEval(r.grid, r.X)
        alone, it, _ = op.fit(np.ascontiguousarray(r.Y[:, 0]), r.lam, 100000, r.epsilon,
                              mode=sg.SGMEV_SOLVE_MIXED)
        op.close()
        assert it == r.iterations
        assert np.array_equal(alone, r.alpha)

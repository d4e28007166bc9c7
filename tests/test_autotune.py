"""The launch-shape autotuner's host logic (no GPU): the enumeration of combinations, the cache
and its keys, and that the search keeps the fastest combination and skips failing ones (with a
fake operator whose timings are given)."""
import json

import numpy as np
import pytest

import sgpp_gb300 as sg
from sgpp_gb300 import autotune


def test_combinations_enumerate_every_value_first_parameter_fastest():
    params = [autotune.TunableParameter("a", [1, 2]), autotune.TunableParameter("b", [7, 8, 9])]
    got = list(autotune.combinations(params))
    assert len(got) == 6
    assert got[0] == {"a": "1", "b": "7"} and got[1] == {"a": "2", "b": "7"}
    assert got[-1] == {"a": "2", "b": "9"}
    assert len({json.dumps(c, sort_keys=True) for c in got}) == 6


def test_cache_round_trip(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("SGPP_GB300_TUNE_CACHE", str(path))
    assert autotune.cache_path() == str(path)
    assert autotune.load_cache() == {}
    autotune.store_cache({"k": {"params": {"multt_batch": "2"}, "ms": 0.5}})
    assert autotune.load_cache()["k"]["params"] == {"multt_batch": "2"}


def test_shape_key_rounds_the_data_size_to_a_power_of_two():
    g = sg.Grid.createLinearGrid(3)
    g.getGenerator().regular(3)
    k1 = autotune.shape_key("block", g, 1000)
    k2 = autotune.shape_key("block", g, 1024)
    k3 = autotune.shape_key("block", g, 1025)
    assert k1 == k2 != k3
    assert "|d3|" in k1 and f"|n{g.getSize()}|" in k1


class _FakeOp:
    """Times per combination; raises for shapes that do not fit."""

    def __init__(self, times):
        self.times = times
        self.params = {}

    def setParams(self, p):
        if p.get("multt_banks") == "2" and p.get("multt_ctas") == "3":
            raise sg.OperationException("does not fit")
        self.params = dict(p)


def test_tune_keeps_the_fastest_and_skips_failures(monkeypatch):
    times = {"2": 0.5e-3, "3": 0.4e-3}
    op = _FakeOp(times)
    # two banks cost 0.05 ms more here, so one bank with three CTAs per SM wins
    monkeypatch.setattr(autotune, "_evaluate",
                        lambda o, kernel, m, n, repeats: times[o.params["multt_ctas"]]
                        + (0.05e-3 if o.params.get("multt_banks") == "2" else 0.0))
    g = sg.Grid.createLinearGrid(2)
    g.getGenerator().regular(2)
    log = []
    best, t = autotune.tune(op, g, 100, "multT16", log=log.append)
    assert best == {"multt_banks": "1", "multt_ctas": "3"} and t == pytest.approx(0.4e-3)
    assert op.params == best  # left set on the operator
    assert any("error" in rec for rec in log)


def test_tune_and_cache_reuses_the_cached_choice(tmp_path, monkeypatch):
    path = str(tmp_path / "c.json")
    calls = []
    monkeypatch.setattr(autotune, "_evaluate",
                        lambda o, kernel, m, n, repeats: calls.append(1) or 1e-3)
    g = sg.Grid.createLinearGrid(2)
    g.getGenerator().regular(2)
    op = _FakeOp({})
    first = autotune.tune_and_cache(op, g, 64, ["multT16"], path=path)
    n_calls = len(calls)
    again = autotune.tune_and_cache(op, g, 64, ["multT16"], path=path)
    assert again == first and len(calls) == n_calls
    assert autotune.tuned_params(g, 64, ["multT16"], path=path) == first

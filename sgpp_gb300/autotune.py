"""Launch-shape autotuner: grid search over the tunable knobs of an operator's kernels, scored by
measured kernel time, with the choices cached per device and problem shape.

It follows the reference's StaticParameterTuner
(datadriven/src/sgpp/datadriven/application/StaticParameterTuner.cpp:297-417): every combination
of the tunable parameters' values is enumerated (the first parameter varies fastest), each is
evaluated by running the operation it affects, and the combination with the shortest duration is
kept and written back as the operator's parameters. Here the evaluation times the kernels
themselves with CUDA events (sgmev_profile), and the parameters are set on the live operator
(sgmev_set_params) instead of rebuilding it, so a search costs a few seconds.

Tunables:
  multT16   "multt_banks"            banks of cell sums per owner of the FP16 multTranspose (2: two
                                     independent read-modify-write chains)
            "multt_ctas"             its CTAs per SM (3: FP32 cell sums only, two loads in flight)
  block     "block_window", "block_mult_a", "block_mult_tiles", "block_stages",
            "block_multt_groups"
                                      the tensor-core products with 16 right-hand sides

    python -m sgpp_gb300.autotune --dim 10 --level 5 --points 1048576 --kernel all

prints one JSON line per combination and the best per kernel. The cache is a JSON file
($SGPP_GB300_TUNE_CACHE, else ~/.cache/sgpp_gb300/tune.json) keyed by device name, kernel, grid
(dimension, grid points, subspace count) and the data size rounded to a power of two.
"""
from __future__ import annotations

import argparse
import itertools
import json
import os
import sys
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import sgpp_gb300 as sg  # noqa: E402


class TunableParameter:
    """A knob and the values the search tries (StaticParameterTuner's TunableParameter)."""

    def __init__(self, name: str, values: Sequence):
        self.name = name
        self.values = [str(v) for v in values]


TUNABLES: Dict[str, List[TunableParameter]] = {
    "multT16": [TunableParameter("multt_banks", [1, 2]),
                TunableParameter("multt_ctas", [2, 3])],
    "block": [TunableParameter("block_window", [1, 2]),
              TunableParameter("block_mult_a", ["tmem", "smem"]),
              TunableParameter("block_mult_tiles", [4, 8]),
              TunableParameter("block_stages", [3, 4]),
              TunableParameter("block_multt_groups", [8, 16])],
}


def combinations(params: Sequence[TunableParameter]):
    """Every combination, the first parameter varying fastest (the reference's enumeration)."""
    for vals in itertools.product(*[p.values for p in reversed(params)]):
        yield {p.name: v for p, v in zip(params, reversed(vals))}


def cache_path() -> str:
    return os.environ.get("SGPP_GB300_TUNE_CACHE") or os.path.join(
        os.path.expanduser("~"), ".cache", "sgpp_gb300", "tune.json")


def shape_key(kernel: str, grid, m: int) -> str:
    st = grid.getStorage()
    lp, _ = st.getLevelIndexArraysForEval()
    n_sub = len({tuple(r) for r in np.asarray(lp, np.int64).tolist()}) if st.getSize() else 0
    mb = 1 << max(0, int(np.ceil(np.log2(max(m, 1)))))
    return f"{device_name()}|{kernel}|d{st.getDimension()}|n{st.getSize()}|s{n_sub}|m{mb}"


def device_name() -> str:
    try:
        import torch

        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except Exception:
        pass
    return "cuda"


def load_cache(path: Optional[str] = None) -> dict:
    path = path or cache_path()
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def store_cache(cache: dict, path: Optional[str] = None) -> None:
    path = path or cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _evaluate(op, kernel: str, m: int, n: int, repeats: int) -> float:
    """Median seconds of the operation the kernel serves, on the live operator."""
    rng = np.random.default_rng(11)
    if kernel == "multT16":
        # the FP16 multTranspose runs inside the inner solves of a mixed fit: time those launches
        y = rng.standard_normal(m)
        op.fit(y, 1e-4, 8, 1e-30, mode=sg.SGMEV_SOLVE_MIXED)  # warm-up (builds the products)
        op.profile(True)
        op.fit(y, 1e-4, 8 * repeats, 1e-30, mode=sg.SGMEV_SOLVE_MIXED)
        cnt, sec = op.profileRead(sg.SGMEV_KERNEL_MULTT_MAT16)
        op.profile(False)
        return sec / max(cnt, 1)
    a = rng.standard_normal((sg.SGMEV_BLOCK_RHS, n))
    v = rng.standard_normal((sg.SGMEV_BLOCK_RHS, m))
    op.multBlock(a)
    op.multTransposeBlock(v)
    op.profile(True)
    for _ in range(repeats):
        op.multBlock(a)
        op.multTransposeBlock(v)
    c1, s1 = op.profileRead(sg.SGMEV_KERNEL_BLOCK_MULT)
    c2, s2 = op.profileRead(sg.SGMEV_KERNEL_BLOCK_MULTT)
    op.profile(False)
    return s1 / max(c1, 1) + s2 / max(c2, 1)


def tune(op, grid, m: int, kernel: str, repeats: int = 3, log=None) -> Tuple[dict, float]:
    """Grid search of `kernel`'s tunables on the live operator; leaves the best combination set
    on it and returns (params, seconds)."""
    best, best_t = None, float("inf")
    for combo in combinations(TUNABLES[kernel]):
        try:
            op.setParams(combo)
            t = _evaluate(op, kernel, m, grid.getSize(), repeats)
        except sg.OperationException as e:
            if log:
                log({"kernel": kernel, "params": combo, "error": str(e)})
            continue
        if log:
            log({"kernel": kernel, "params": combo, "ms": t * 1e3})
        if t < best_t:
            best, best_t = combo, t
    if best is None:
        raise sg.OperationException(f"autotune: no combination of {kernel} ran")
    op.setParams(best)
    return best, best_t


def tuned_params(grid, m: int, kernels: Sequence[str] = ("multT16", "block"),
                 path: Optional[str] = None) -> dict:
    """The cached choices for this device and problem shape (empty where none was tuned)."""
    cache = load_cache(path)
    out = {}
    for k in kernels:
        out.update(cache.get(shape_key(k, grid, m), {}).get("params", {}))
    return out


def tune_and_cache(op, grid, m: int, kernels: Sequence[str] = ("multT16", "block"),
                   path: Optional[str] = None, log=None, force: bool = False) -> dict:
    """Tune the kernels not yet cached for this shape (all of them with force), set the choices on
    the operator and store them; returns the parameters set."""
    cache = load_cache(path)
    chosen = {}
    for k in kernels:
        key = shape_key(k, grid, m)
        if key in cache and not force:
            params = cache[key]["params"]
            op.setParams(params)
        else:
            params, t = tune(op, grid, m, k, log=log)
            cache[key] = {"params": params, "ms": t * 1e3}
        chosen.update(params)
    store_cache(cache, path)
    return chosen


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--dim", type=int, default=10)
    ap.add_argument("--level", type=int, default=5)
    ap.add_argument("--points", type=int, default=1 << 20)
    ap.add_argument("--kernel", choices=["multT16", "block", "all"], default="all")
    ap.add_argument("--force", action="store_true", help="search again even when cached")
    args = ap.parse_args()
    rng = np.random.default_rng(7)
    grid = sg.Grid.createLinearGrid(args.dim)
    grid.getGenerator().regular(args.level)
    x = rng.random((args.points, args.dim))
    cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                sg.OperationMultipleEvalSubType.CUDA,
                                                parameters={"algo": "subspace",
                                                            "materialize": "on"})
    op = sg.createOperationMultipleEval(grid, x, cfg)
    kernels = ["multT16", "block"] if args.kernel == "all" else [args.kernel]
    chosen = tune_and_cache(op, grid, args.points, kernels, force=args.force,
                            log=lambda rec: print(json.dumps(rec), flush=True))
    print(json.dumps({"best": chosen, "cache": cache_path()}), flush=True)
    op.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())

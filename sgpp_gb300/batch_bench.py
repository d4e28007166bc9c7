"""Batched multi-problem, multi-right-hand-side fits: solves/s of the batch engine against
sequential per-problem fits.

    python -m sgpp_gb300.batch_bench --problems 96 --rhs 16 --max-work 2e9

Problems follow the batched-fit size mix (d uniform in 2..12, level in 3..7, data size
log-uniform in [1e3, 2^20], uniform data, Y ~ N(0,1) with `rhs` columns), truncated to
N*M*d <= --max-work so that the run ends in minutes with the dense kernels. One "solve" is one
right-hand side of one problem fitted to the relative FP64 residual --epsilon.

Reported: batched solves/s (all problems resident, one engine), the error of a subset's alpha
against FP64 solutions (single-problem df64-refined fits to 1e-12), and sequential solves/s of
the plain FP64 CUDA path (native FP64 kernels, CG per right-hand side) and of the single-problem
mixed path, both timed on the first --sequential problems (one right-hand side each).
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import sgpp_gb300 as sg  # noqa: E402
from sgpp_gb300.serving import MixGenerator  # noqa: E402


def block_pool(probs, lam: float, epsilon: float, workers: int, params=None):
    """Every problem's 16 right-hand sides as one block fit (sgmev_fit_block: tensor-core
    inner solves, df64 residuals) on its own operator and stream, `workers` problems at a time.
    A problem the block products do not take (a subspace above 128 cells, or products too large
    to materialise) runs its right-hand sides as single mixed fits. Returns
    (seconds, alphas, paths, inner steps per problem, seconds per problem, why single)."""
    import queue
    import threading

    work = queue.Queue()
    for k in range(len(probs)):
        work.put(k)
    alphas = [None] * len(probs)
    paths = [None] * len(probs)
    steps = [0] * len(probs)
    secs = [0.0] * len(probs)
    why = [None] * len(probs)
    errors = []

    def run():
        while True:
            try:
                k = work.get_nowait()
            except queue.Empty:
                return
            g, X, Y = probs[k]
            t_k = time.perf_counter()
            try:
                cfg = sg.OperationMultipleEvalConfiguration(
                    sg.OperationMultipleEvalType.STREAMING, sg.OperationMultipleEvalSubType.CUDA,
                    parameters=dict(params or {}))
                op = sg.createOperationMultipleEval(g, X, cfg)
                try:
                    a, its, _ = op.fitBlock(np.ascontiguousarray(Y.T), lam, 100000, epsilon)
                    alphas[k], paths[k], steps[k] = a.T, "block", int(max(its))
                except sg.OperationException as e:
                    why[k] = str(e)
                    cols = []
                    for c in range(Y.shape[1]):
                        a, it, _ = op.fit(np.ascontiguousarray(Y[:, c]), lam, 100000, epsilon,
                                          mode=sg.SGMEV_SOLVE_MIXED)
                        cols.append(a)
                        steps[k] += it
                    alphas[k], paths[k] = np.stack(cols, axis=1), "single"
                op.close()
                secs[k] = time.perf_counter() - t_k
            except BaseException as e:  # reported after the run
                errors.append(e)

    threads = [threading.Thread(target=run, daemon=True) for _ in range(workers)]
    t0 = time.perf_counter()
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    sec = time.perf_counter() - t0
    if errors:
        raise errors[0]
    return sec, alphas, paths, steps, secs, why


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--problems", type=int, default=96)
    ap.add_argument("--rhs", type=int, default=16)
    ap.add_argument("--max-work", type=float, default=2e9)
    ap.add_argument("--epsilon", type=float, default=1e-8)
    ap.add_argument("--lam", type=float, default=1e-4)
    ap.add_argument("--check", type=int, default=4, help="problems checked against FP64 fits")
    ap.add_argument("--sequential", type=int, default=4, help="problems timed sequentially")
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--engine", choices=["batch", "block"], default="batch",
                    help="batch: the batch engine (dense kernels, one persistent launch per "
                         "phase); block: per-problem block fits on the tensor cores")
    ap.add_argument("--workers", type=int, default=4, help="block engine: problems in flight")
    ap.add_argument("--plain", type=int, default=1,
                    help="block engine: time the plain FP64 path on every problem (0: skip)")
    ap.add_argument("--param", action="append", default=[], metavar="KEY=VALUE",
                    help="block engine: operator knob of the block fits (repeatable)")
    args = ap.parse_args()
    if args.engine == "block":
        return main_block(args)

    gen = MixGenerator(args.seed, args.max_work, pool=4)
    probs = [gen.draw(args.rhs) for _ in range(args.problems)]
    grid_elems = sum(sg.BatchEngine.footprint(g.getDimension(), g.getSize(), X.shape[0], args.rhs)[0]
                     for g, X, _ in probs)
    data_elems = sum(sg.BatchEngine.footprint(g.getDimension(), g.getSize(), X.shape[0], args.rhs)[1]
                     for g, X, _ in probs)
    eng = sg.BatchEngine(max_slots=args.problems, rhs=args.rhs, grid_capacity=grid_elems + 4096,
                         data_capacity=data_elems + 4096)
    slots = [eng.add(g, X, Y, args.lam, args.epsilon) for g, X, Y in probs]
    # the first step captures the graph; time from there on
    eng.step(1)
    t0 = time.perf_counter()
    steps = eng.solve()
    t_batch = time.perf_counter() - t0
    solves = args.problems * args.rhs
    iters = [eng.result(s)[1] for s in slots]

    errs = []
    for k in range(min(args.check, args.problems)):
        g, X, Y = probs[k]
        alpha = eng.result(slots[k])[0]
        op = sg.createOperationMultipleEval(g, X)
        for c in range(args.rhs):
            ref, _, _ = op.fit(Y[:, c], args.lam, 100000, 1e-12, mode=sg.SGMEV_SOLVE_MIXED)
            errs.append(float(np.abs(alpha[:, c] - ref).max() / np.abs(ref).max()))
        op.close()
    eng.close()

    seq_plain, seq_mixed = [], []
    for k in range(min(args.sequential, args.problems)):
        g, X, Y = probs[k]
        op = sg.createOperationMultipleEval(g, X)
        t1 = time.perf_counter()
        op.fit(Y[:, 0], args.lam, 100000, args.epsilon, mode=sg.SGMEV_SOLVE_PLAIN)
        seq_plain.append(time.perf_counter() - t1)
        t1 = time.perf_counter()
        op.fit(Y[:, 0], args.lam, 100000, args.epsilon, mode=sg.SGMEV_SOLVE_MIXED)
        seq_mixed.append(time.perf_counter() - t1)
        op.close()
    # the sequential subset's share of the batch work, to put both on the same footing
    work = np.array([g.getSize() * X.shape[0] * g.getDimension() for g, X, _ in probs], float)
    share = work[: len(seq_plain)].sum() / work.sum()
    line = {
        "metric": "batched_solves_per_sec", "value": solves / t_batch, "unit": "solves/s",
        "problems": args.problems, "rhs": args.rhs, "steps": steps, "seconds": t_batch,
        "inner_iterations": {"min": int(min(iters)), "max": int(max(iters))},
        "alpha_rel_err_vs_fp64": {"max": max(errs) if errs else None, "checked_solves": len(errs)},
        # all problems x all right-hand sides sequentially: sum(subset times) / share per column
        "sequential_plain_fp64_solves_per_sec_est": (
            args.problems * share / sum(seq_plain) if seq_plain else None),
        "sequential_mixed_solves_per_sec_est": (
            args.problems * share / sum(seq_mixed) if seq_mixed else None),
        "sequential_note": (f"timed on the first {len(seq_plain)} problems x 1 right-hand side, "
                            "rescaled by their share of the batch's N*M*d work"),
        "config": {"mix": "d 2..12, level 3..7, M log-uniform [1e3, 2^20], uniform data",
                   "max_work_NMd": args.max_work, "epsilon": args.epsilon, "lambda": args.lam},
    }
    print(json.dumps(line))
    return 0


def main_block(args) -> int:
    print(json.dumps(measure_block(args)))
    return 0


def measure_block(args) -> dict:
    """The block engine on the mix (see main): returns the JSON line as a dict."""
    gen = MixGenerator(args.seed, args.max_work, pool=4)
    probs = [gen.draw(args.rhs) for _ in range(args.problems)]
    if args.rhs != sg.SGMEV_BLOCK_RHS:
        raise SystemExit(f"--engine block takes --rhs {sg.SGMEV_BLOCK_RHS}")
    params = dict(kv.split("=", 1) for kv in args.param)
    block_pool(probs[:2], args.lam, args.epsilon, 1, params)  # warm-up (library, kernels)
    sec, alphas, paths, steps, secs, why = block_pool(probs, args.lam, args.epsilon, args.workers,
                                                      params)
    errs = []
    for k in range(min(args.check, args.problems)):
        g, X, Y = probs[k]
        op = sg.createOperationMultipleEval(g, X)
        for c in (0, args.rhs - 1):
            ref, _, _ = op.fit(np.ascontiguousarray(Y[:, c]), args.lam, 100000, 1e-12,
                               mode=sg.SGMEV_SOLVE_MIXED)
            errs.append(float(np.abs(alphas[k][:, c] - ref).max() / np.abs(ref).max()))
        op.close()
    solves = args.problems * args.rhs
    # the plain per-problem FP64 path: every problem's first right-hand side as a plain
    # FP64-accurate CG fit (the reference's algorithm) on a df64 operator, products built before
    # the clock starts; its right-hand sides are independent fits of the same cost, so all
    # problems x all right-hand sides take rhs x the summed time
    plain = None
    t_plain_k = [None] * len(probs)
    if args.plain:
        t_plain = 0.0
        for k, (g, X, Y) in enumerate(probs):
            cfg = sg.OperationMultipleEvalConfiguration(
                sg.OperationMultipleEvalType.STREAMING, sg.OperationMultipleEvalSubType.CUDA,
                parameters={"precision": "df64"})
            op = sg.createOperationMultipleEval(g, X, cfg)
            y0 = np.ascontiguousarray(Y[:, 0])
            op.fit(y0, args.lam, 8, args.epsilon, mode=sg.SGMEV_SOLVE_PLAIN)  # builds the products
            t1 = time.perf_counter()
            op.fit(y0, args.lam, 100000, args.epsilon, mode=sg.SGMEV_SOLVE_PLAIN)
            t_plain_k[k] = time.perf_counter() - t1
            t_plain += t_plain_k[k]
            op.close()
        plain = {"solves_per_sec": solves / (args.rhs * t_plain),
                 "seconds_all_problems_one_rhs": t_plain,
                 "what": "plain FP64-accurate CG (SGMEV_SOLVE_PLAIN) on a df64 operator per "
                         "problem and right-hand side, one after another; every problem timed "
                         "on its first right-hand side"}
    line = {
        "metric": "batched_solves_per_sec", "value": solves / sec, "unit": "solves/s",
        "engine": "block", "params": params, "problems": args.problems, "rhs": args.rhs,
        "seconds": sec,
        "workers": args.workers,
        "paths": {p: paths.count(p) for p in set(paths)},
        "inner_steps": {"min": int(min(steps)), "max": int(max(steps))},
        "alpha_rel_err_vs_fp64": {"max": max(errs) if errs else None, "checked_solves": len(errs)},
        "plain_fp64_path": plain,
        "speedup_vs_plain_fp64": (solves / sec) / plain["solves_per_sec"] if plain else None,
        "why_single": sorted({w for w in why if w}),
        # per problem: d, level, grid points, data points, path, inner steps, seconds in the pool
        # (workers overlap), seconds of one plain FP64 fit
        "problems_detail": [[g.getDimension(), int(round(np.log2(max(g.getStorage().getLevelIndexArraysForEval()[0].max(), 2)))),
                             g.getSize(), X.shape[0], paths[k], int(steps[k]), round(secs[k], 4),
                             None if t_plain_k[k] is None else round(t_plain_k[k], 4)]
                            for k, (g, X, _) in enumerate(probs)],
        "config": {"mix": "d 2..12, level 3..7, M log-uniform [1e3, 2^20], uniform data",
                   "max_work_NMd": args.max_work, "epsilon": args.epsilon, "lambda": args.lam},
    }
    return line


if __name__ == "__main__":
    sys.exit(main())

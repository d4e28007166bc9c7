"""Spatially adaptive regression: refine -> prepare -> warm-started fit, on the GPU operator.

The loop of LearnerBase::train (datadriven/src/sgpp/datadriven/application/LearnerBase.cpp:
113-260): after each solve, SurplusRefinementFunctor refines the `points_per_round` grid points
with the largest |alpha| (HashRefinement::free_refine appends the new points), the operator is
re-staged (prepare(), SystemMatrixLeastSquaresIdentity::prepareGrid), alpha is extended with zeros
(resizeZero) and the next CG solve starts from it (reuse). The data stay resident on the GPU for
the whole loop; only the grid is re-staged.

    python -m sgpp_gb300.adaptive        # the adaptive-grid configuration, one JSON line per round

--engine fitter (default) runs the loop as ModelFittingLeastSquares fit() + adapt() on the
device-resident fitter (sgpp_gb300.fitting: y and alpha stay on the GPU, one operator for all
rounds); --engine operator runs adaptive_fit() below on the Python-level operator (alpha and y
cross to the host every round). --throughput adds per-round kernel throughputs (extra operators,
outside the fit timing).
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


def adaptive_workload(seed: int = 3, m: int = 524288, dim: int = 8):
    """The adaptive-grid configuration's data: x uniform on [0, 1]^dim (seeded),
    y = prod_k 4 x_k (1 - x_k) + N(0, 0.01^2)."""
    rng = np.random.default_rng(seed)
    X = rng.random((m, dim))
    y = np.prod(4.0 * X * (1.0 - X), axis=1) + 0.01 * rng.standard_normal(m)
    return X, y


def adaptive_fit(grid, X, y, lam: float, rounds: int, points_per_round: int,
                 epsilon: float = 1e-8, mode: int = sg.SGMEV_SOLVE_MIXED, precision="double",
                 on_round=None):
    """Returns (alpha, per-round records). `grid` is refined in place."""
    cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                sg.OperationMultipleEvalSubType.CUDA,
                                                parameters={"precision": precision})
    op = sg.createOperationMultipleEval(grid, X, cfg)
    alpha = None
    records = []
    for r in range(rounds + 1):
        t0 = time.perf_counter()
        alpha, iters, res = op.fit(y, lam, 100000, epsilon, alpha=alpha, mode=mode)
        rec = {"round": r, "n_grid": grid.getSize(), "cg_iterations": iters,
               "fit_seconds": time.perf_counter() - t0, "residual": res}
        if on_round is not None:
            on_round(op, rec)
        records.append(rec)
        if r < rounds:
            n0 = grid.getSize()
            grid.getGenerator().refine(sg.SurplusRefinementFunctor(alpha, points_per_round, 0.0))
            op.prepare()
            alpha = np.concatenate([alpha, np.zeros(grid.getSize() - n0)])
    op.close()
    return alpha, records


def _throughput(op, grid, m, d):
    """Event-timed mult / multT of the op's precision, reference-count TFLOP/s."""
    n = grid.getSize()
    a = np.random.default_rng(0).standard_normal(n)
    v = np.random.default_rng(1).standard_normal(m)
    om, ot = np.zeros(m), np.zeros(n)
    op.mult(a, om)
    op.multTranspose(v, ot)
    op.profile(True)
    for _ in range(3):
        op.mult(a, om)
        op.multTranspose(v, ot)
    out = {}
    flop = 6.0 * n * m * d
    kinds = {sg.SGMEV_FP32: (sg.SGMEV_KERNEL_MULT_FP32, sg.SGMEV_KERNEL_MULTT_FP32),
             sg.SGMEV_FP64: (sg.SGMEV_KERNEL_MULT_FP64, sg.SGMEV_KERNEL_MULTT_FP64),
             sg.SGMEV_DF64: (sg.SGMEV_KERNEL_MULT_DF64, sg.SGMEV_KERNEL_MULTT_DF64)}[op.precision]
    for name, kind in zip(("mult", "multT"), kinds):
        c, s = op.profileRead(kind)
        out[name + "_tflops"] = flop / (s / c) / 1e12 if c else None
    op.profile(False)
    return out


def fitter_rounds(grid_dim, X, y, level, lam, rounds, per_round, epsilon, mode="mixed"):
    """The loop on the device-resident fitter: (model, per-round records)."""
    from . import fitting

    c = fitting.FitterConfigurationLeastSquares()
    c.getGridConfig().level_ = level
    c.getRegularizationConfig().lambda_ = lam
    for sc in (c.getSolverFinalConfig(), c.getSolverRefineConfig()):
        sc.eps_, sc.maxIterations_ = epsilon, 100000
    c.getRefinementConfig().numRefinements_ = rounds
    c.getRefinementConfig().numRefinementPoints_ = per_round
    c.getMultipleEvalConfig().getParameters()["solve"] = mode
    model = fitting.ModelFittingLeastSquares(c)
    records = []
    t0 = time.perf_counter()
    model.fit(sg.Dataset(X, y))
    st = model.stats()
    records.append({"round": 0, "n_grid": model.getGrid().getSize(),
                    "cg_iterations": st["cg_iterations"], "seconds": time.perf_counter() - t0})
    for r in range(rounds):
        t0 = time.perf_counter()
        grew = model.adapt()
        st = model.stats()
        records.append({"round": r + 1, "n_grid": model.getGrid().getSize(),
                        "cg_iterations": st["cg_iterations"] if grew else 0,
                        "seconds": time.perf_counter() - t0})
        if not grew:
            break
    return model, records


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--dim", type=int, default=8)
    ap.add_argument("--level", type=int, default=4)
    ap.add_argument("--points", type=int, default=524288)
    ap.add_argument("--rounds", type=int, default=6)
    ap.add_argument("--per-round", type=int, default=40)
    ap.add_argument("--lam", type=float, default=1e-4)
    ap.add_argument("--epsilon", type=float, default=1e-8)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--engine", choices=["fitter", "operator"], default="fitter")
    ap.add_argument("--throughput", action="store_true")
    args = ap.parse_args()
    X, y = adaptive_workload(args.seed, args.points, args.dim)

    if args.engine == "fitter":
        t0 = time.perf_counter()
        model, records = fitter_rounds(args.dim, X, y, args.level, args.lam, args.rounds,
                                       args.per_round, args.epsilon)
        total = time.perf_counter() - t0
        for rec in records:
            print(json.dumps(rec), flush=True)
        n_final = model.getGrid().getSize()
        model.close()
    else:
        grid = sg.Grid.createLinearGrid(args.dim)
        grid.getGenerator().regular(args.level)
        timing = {"measure": 0.0}

        def on_round(op, rec):
            if args.throughput:
                t_m = time.perf_counter()
                for prec, name in ((sg.SGMEV_FP32, "fp32"), (sg.SGMEV_FP64, "fp64"),
                                   (sg.SGMEV_DF64, "df64")):
                    cfg = sg.OperationMultipleEvalConfiguration(
                        sg.OperationMultipleEvalType.STREAMING, sg.OperationMultipleEvalSubType.CUDA,
                        parameters={"precision": {sg.SGMEV_FP32: "float", sg.SGMEV_FP64: "double",
                                                  sg.SGMEV_DF64: "df64"}[prec]})
                    o2 = sg.createOperationMultipleEval(grid, X, cfg)
                    rec[name] = _throughput(o2, grid, args.points, args.dim)
                    o2.close()
                timing["measure"] += time.perf_counter() - t_m
            print(json.dumps(rec), flush=True)

        t0 = time.perf_counter()
        _, records = adaptive_fit(grid, X, y, args.lam, args.rounds, args.per_round,
                                  args.epsilon, on_round=on_round)
        total = time.perf_counter() - t0 - timing["measure"]
        n_final = grid.getSize()
    print(json.dumps({"metric": "adaptive_fit_seconds", "value": total, "engine": args.engine,
                      "final_n_grid": n_final,
                      "total_cg_iterations": sum(r["cg_iterations"] for r in records),
                      "config": vars(args)}))
    return 0


if __name__ == "__main__":
    sys.exit(main())

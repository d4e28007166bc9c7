"""Run a few launches of one tile kernel on a synthetic case, for profilers (ncu) and timing.

    python profile_case.py --kernel mult --precision float --dim 10 --level 5 \
        --points 4194304 --launches 3

Data are uniform on [0, 1]^d (seeded); the grid is the regular Linear grid of the given level.
Prints one JSON line with the per-launch CUDA-event times of the tile kernel (sgmev_profile).
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import sgpp_gb300 as sg  # noqa: E402

KINDS = {("mult", "float", "dense"): sg.SGMEV_KERNEL_MULT_FP32,
         ("multT", "float", "dense"): sg.SGMEV_KERNEL_MULTT_FP32,
         ("mult", "float", "subspace"): sg.SGMEV_KERNEL_MULT_SUB32,
         ("multT", "float", "subspace"): sg.SGMEV_KERNEL_MULTT_SUB32,
         ("mult", "float", "materialized"): sg.SGMEV_KERNEL_MULT_MAT32,
         ("multT", "float", "materialized"): sg.SGMEV_KERNEL_MULTT_MAT32,
         ("system", "float", "materialized"): sg.SGMEV_KERNEL_SYSTEM_MAT32,
         ("mult", "df64", "materialized"): sg.SGMEV_KERNEL_MULT_MATDF,
         ("multT", "df64", "materialized"): sg.SGMEV_KERNEL_MULTT_MATDF,
         ("mult", "double", "dense"): sg.SGMEV_KERNEL_MULT_FP64,
         ("multT", "double", "dense"): sg.SGMEV_KERNEL_MULTT_FP64,
         ("mult", "df64", "dense"): sg.SGMEV_KERNEL_MULT_DF64,
         ("multT", "df64", "dense"): sg.SGMEV_KERNEL_MULTT_DF64,
         ("mult", "df64", "subspace"): sg.SGMEV_KERNEL_MULT_SUBDF,
         ("multT", "df64", "subspace"): sg.SGMEV_KERNEL_MULTT_SUBDF}


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--kernel", choices=["mult", "multT", "system", "fit", "block_mult",
                                         "block_multT"], default="mult",
                    help="system: B^T (B a) + lambda M a (systemApply; with materialized "
                         "products the fused kernel, system_product=fused); fit: one "
                         "mixed-precision fit (its inner solves stream the FP16 products); "
                         "reports the kernel given by --report; block_mult / block_multT: the "
                         "BF16 tensor-core products with 16 right-hand sides")
    ap.add_argument("--report", choices=["mult16", "multT16"], default="mult16",
                    help="with --kernel fit: which kernel's launches to report")
    ap.add_argument("--precision", choices=["float", "double", "df64"], default="float")
    ap.add_argument("--algo", choices=["dense", "subspace", "materialized"], default="dense",
                    help="materialized: subspace products kept in device memory (float-float, "
                         "with an FP16 copy for the inner solves of --kernel fit)")
    ap.add_argument("--dim", type=int, default=10)
    ap.add_argument("--level", type=int, default=5)
    ap.add_argument("--points", type=int, default=1 << 22)
    ap.add_argument("--launches", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--param", action="append", default=[], metavar="KEY=VALUE",
                    help="operator knob (repeatable), e.g. multt_batch=2")
    args = ap.parse_args()

    mat = args.algo == "materialized"
    rng = np.random.default_rng(7)
    grid = sg.Grid.createLinearGrid(args.dim)
    grid.getGenerator().regular(args.level)
    n = grid.getSize()
    x = rng.random((args.points, args.dim))
    cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                sg.OperationMultipleEvalSubType.CUDA,
                                                parameters={
                                                    "precision": args.precision,
                                                    "algo": "subspace" if mat else args.algo,
                                                    "materialize": "on" if mat else "off",
                                                    "materialize_multt": "on" if mat else "off",
                                                    "system_product": "fused",
                                                    **dict(kv.split("=", 1) for kv in args.param)})
    op = sg.createOperationMultipleEval(grid, x, cfg)
    a = rng.standard_normal(n)
    v = rng.standard_normal(args.points)
    out_m = np.zeros(args.points)
    out_t = np.zeros(n)

    ab = rng.standard_normal((sg.SGMEV_BLOCK_RHS, n))
    vb = rng.standard_normal((sg.SGMEV_BLOCK_RHS, args.points))

    def run():
        if args.kernel == "block_mult":
            op.multBlock(ab)
        elif args.kernel == "block_multT":
            op.multTransposeBlock(vb)
        elif args.kernel == "fit":
            op.fit(v, 1e-4, 100000, 1e-8, mode=sg.SGMEV_SOLVE_MIXED)
        elif args.kernel == "system":
            op.systemApply(a, out_t, 1e-4 * args.points)
        elif args.kernel == "mult":
            op.mult(a, out_m)
        else:
            op.multTranspose(v, out_t)

    for _ in range(args.warmup):
        run()
    op.profile(True)
    for _ in range(args.launches):
        run()
    algo = "dense" if args.precision == "double" else args.algo
    if args.kernel == "fit":
        kind = sg.SGMEV_KERNEL_MULT_MAT16 if args.report == "mult16" else sg.SGMEV_KERNEL_MULTT_MAT16
    elif args.kernel.startswith("block"):
        kind = sg.SGMEV_KERNEL_BLOCK_MULT if args.kernel == "block_mult" else sg.SGMEV_KERNEL_BLOCK_MULTT
    else:
        kind = KINDS[(args.kernel, args.precision, algo)]
    cnt, sec = op.profileRead(kind)
    op.profile(False)
    flop = 6.0 * n * args.points * args.dim
    avg = sec / cnt if cnt else None
    print(json.dumps({"kernel": args.kernel, "precision": args.precision, "algo": algo,
                      "dim": args.dim,
                      "level": args.level, "n_grid": n, "points": args.points, "launches": cnt,
                      "avg_ms": avg * 1e3 if avg else None,
                      "tflops_ref_count": flop / avg / 1e12 if avg else None}))
    if not cnt:
        print(f"no launches of the reported kernel kind {kind}", file=sys.stderr)
        op.close()
        return 1
    op.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())

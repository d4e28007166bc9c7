#!/usr/bin/env python3
"""Headline benchmark: regression fits per second on the GB300.

Workload (the regression-fit configuration): regular Linear sparse grid d=10, level 5
(N = 13,441 grid points); M = 2^20 data points from an 8-component Gaussian mixture (means
uniform in [0.2, 0.8]^10, diagonal sigma 0.08, equal weights) clipped to [0, 1]^10;
y = 10 sin(pi x1 x2) + 20 (x3 - 0.5)^2 + 10 x4 + 5 x5 + N(0, 0.1^2); lambda = 1e-4.
Synthetic, seeded data of that shape (no dataset files are read).

One step = one regression fit: b = B^T y, then CG on (B^T B + lambda M I) alpha = b to the
relative FP64 residual `epsilon`, mixed precision (inside CG, FP32 arithmetic on the FP16 copy of
the materialised subspace products; the outer iterative-refinement residual b - A alpha with the
FP64-accurate float-float "df64" products), all state resident on the GPU. Each fit's alpha is
checked against the reference's own FP64 CG solution of this workload (SG++'s
SystemMatrixLeastSquaresIdentity + ConjugateGradients at epsilon 1e-12, the fixture
tests/golden/regression_d10_l5.npz).

value   fits/s with the data resident in HBM (device pointers for y and alpha)
e2e     fits/s through the public API from pinned host buffers: create the operator from the
        host data matrix (H2D copy inside the timed region), fit with host y, read alpha back
roofline  the kernel with the most device time in the fits. When it streams the materialised
        subspace products (the default), it is HBM-bound: achieved = its algorithmic bytes per
        launch (FP16 2 B, FP32 4 B, df64 8 B per padded point and padded subspace, plus the cell
        index, and the vectors) over its CUDA-event duration, against MEASURED_PEAKS.json's copy
        bandwidth. A kernel that evaluates hats is reported against the FP32/FP64 FMA peak
        measured in the same run, with the reference's count of 6 N M d FLOP per launch
        (LearnerVectorizedPerformanceCalculator.cpp:91-93).
mult_gflops  one launch each of the dense FP32 and FP64 mult kernels (STREAMING's algorithm) on
        this workload: GFLOP/s by the reference's count and the fraction of the FMA peaks
        measured in this run
plain_fp64_path  whole plain FP64-accurate CG fits (the reference's algorithm) on a df64
        operator, and the mixed fits' speed-up over them
cpu_baseline  the oracle port of the reference's STREAMING FP64 path on the host cores: one
        B^T(B a) on all points (median of 3), times the operator applications of one CG fit
batched  one run of the batched configuration (96 problems of the size mix, 16 targets each,
        as block fits on the tensor cores) against the plain per-problem FP64 path: solves/s of
        both and their ratio (sgpp_gb300.batch_bench --engine block; --batched-probe 0 skips it)

--impl reference prints the same line for the reference's CPU implementation of the path
(the oracle port: the compiled reference needs its sources, which do not travel); its steps are
single B^T(B a) applications on all points, and it loads nothing of this library.

--basis modlinear runs the same workload on a ModLinear grid (the same points with the modified
linear basis; the reference streams it with OperationMultiEvalModMaskStreaming), with the oracle's
port of that operator as the CPU baseline. --count-iterations prints the plain CG iteration count
of one fit (FP64-accurate df64 products, untimed), the figure REFERENCE_ITERATIONS holds.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

DIM, LEVEL, M_POINTS, LAMBDA = 10, 5, 1 << 20, 1e-4
FLOP_PER_PAIR_DIM = 6.0  # reference's count per (grid point, data point, dimension)


def make_workload(seed: int, m: int = M_POINTS, d: int = DIM):
    """Seeded Gaussian-mixture data and the benchmark's target function."""
    rng = np.random.default_rng(seed)
    means = rng.uniform(0.2, 0.8, size=(8, d))
    comp = rng.integers(0, 8, size=m)
    x = np.clip(means[comp] + 0.08 * rng.standard_normal((m, d)), 0.0, 1.0)
    y = (10.0 * np.sin(np.pi * x[:, 0] * x[:, 1]) + 20.0 * (x[:, 2] - 0.5) ** 2 + 10.0 * x[:, 3]
         + 5.0 * x[:, 4] + 0.1 * rng.standard_normal(m))
    return x, y


def env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu_index = gpu_index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.gpu_index), "-lms", "200"], stdout=self.file,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        rows = list(csv.reader(io.StringIO(self.file.read())))
        self.file.close()
        os.unlink(self.file.name)
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                power.append(float(r[3]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


class CpuReference:
    """Oracle port of the reference's STREAMING FP64 path on the host cores
    (OperationMultiEvalStreaming, or OperationMultiEvalModMaskStreaming for ModLinear): one
    application of the system's data term B^T (B a) on ALL points per call, the operation a
    ConjugateGradients iteration performs (SystemMatrixLeastSquaresIdentity.cpp:32-47)."""

    def __init__(self, x, grid_lp, grid_ix, threads: int, basis: str = "linear"):
        from oracle import Oracle

        self.orc = Oracle()
        self.orc.set_threads(threads)
        self.threads = threads
        self.x = x
        self.basis = basis
        self.lp, self.ix = grid_lp, grid_ix
        self.a = np.random.default_rng(0).standard_normal(grid_lp.shape[0])
        if basis == "modlinear":
            lev = np.rint(np.log2(grid_lp)).astype(np.int32)
            self.arrays = self.orc.mod_arrays(lev, grid_ix.astype(np.int32))
        self.full = self.orc.stream(x)
        self.sample = None

    def _apply(self, st):
        if self.basis == "modlinear":
            st.mult_transpose_mod(self.arrays, st.mult_mod(self.arrays, self.a))
        else:
            st.mult_transpose(self.lp, self.ix, st.mult(self.lp, self.ix, self.a))

    def warm(self):
        """One application on 1/16 of the points (threads and code paths warm; seconds)."""
        if self.sample is None:
            self.sample = self.orc.stream(self.x[: max(1, self.x.shape[0] // 16)])
        self._apply(self.sample)

    def apply_seconds(self) -> float:
        t0 = time.perf_counter()
        self._apply(self.full)
        return time.perf_counter() - t0

    def close(self):
        self.full.close()
        if self.sample is not None:
            self.sample.close()

    def describe(self, reps: int, cg_ops: float) -> str:
        return (f"one B^T(B a) (mult + multTranspose, FP64) on all {self.x.shape[0]} points per "
                f"sample, median of {reps} after a warm-up on 1/16 of the points, {self.threads} "
                f"OpenMP threads, x{cg_ops:g} operator applications per fit "
                f"(ConjugateGradients.cpp:22-151)")


def cpu_fit_seconds(x, grid_lp, grid_ix, cg_ops: float, threads: int, basis: str = "linear",
                    reps: int = 3):
    """Seconds per fit of the reference's CPU path: the median of `reps` applications of
    B^T (B a) on all points (after a warm-up), times the operator applications of one CG fit.
    Returns (seconds per fit, sample description)."""
    ref = CpuReference(x, grid_lp, grid_ix, threads, basis)
    ref.warm()
    ts = [ref.apply_seconds() for _ in range(reps)]
    ref.close()
    return statistics.median(ts) * cg_ops, ref.describe(reps, cg_ops)


def cg_operator_applications(iterations: int) -> float:
    """B^T B applications of one fit as ConjugateGradients.cpp:22-151 performs them: one per
    iteration, one extra every 50 iterations (true residual), plus b = B^T y (half)."""
    return iterations + iterations // 50 + 0.5


def grid_arrays(basis: str = "linear"):
    import sgpp_gb300 as sg

    grid = (sg.Grid.createModLinearGrid(DIM) if basis == "modlinear"
            else sg.Grid.createLinearGrid(DIM))
    grid.getGenerator().regular(LEVEL)
    lp, ix = grid.getStorage().getLevelIndexArraysForEval()
    return grid, lp, ix


def oracle_grid_arrays():
    """The benchmark grid's eval arrays from the oracle's restatement of the reference's
    regular-grid generator (the same point order; a ModLinear grid has the same points). The
    reference arm uses these, so that it loads nothing of this library."""
    from oracle import Oracle

    lev, idx = Oracle().regular_grid(DIM, LEVEL)
    return Oracle.eval_arrays(lev, idx)


def bench_config(basis: str, n: int, m: int, epsilon: float, world: int) -> dict:
    """The `config` object of both arms' lines (the same workload, so the same dict)."""
    return {"workload": f"regression fit, regular {grid_name(basis)} grid d={DIM} level {LEVEL} "
                        f"(N={n}), M={m} Gaussian-mixture points, lambda={LAMBDA}, CG to "
                        f"relative residual {epsilon}",
            "l2_policy": "inputs larger than L2: every system product streams the data term "
                         "(GPU: the materialised subspace products, 5.4 GB at M=2^20) from memory",
            "parallelism": "replicas" if world > 1 else "single GPU"}


# Plain CG iterations of one fit to relative residual 1e-8 on this seeded workload, per basis
# (bench.py --count-iterations: SGMEV_SOLVE_PLAIN with the FP64-accurate df64 products); they
# scale the per-application CPU timings of the reference path to one fit.
REFERENCE_ITERATIONS = {"linear": 75, "modlinear": 768}


def subspace_count(lp):
    """Distinct level vectors of the grid (its subspaces), from the eval arrays (2^l)."""
    return len({tuple(row) for row in np.asarray(lp, dtype=np.int64).tolist()})


def cell_bytes(lp) -> float:
    """Bytes per stored cell index: a nibble when no subspace has more than 16 cells."""
    levels = np.rint(np.log2(np.asarray(lp, dtype=np.float64))).astype(np.int64)
    cmax = int(2 ** int((levels - 1).sum(axis=1).max()))
    return 0.5 if cmax <= 16 else 1.0


def mat_bytes_per_launch(kernel: str, lp, m: int, n: int) -> float:
    """Algorithmic HBM bytes of one launch of a kernel streaming the materialised products."""
    mpad = -(-m // 1024) * 1024
    s_pad = -(-subspace_count(lp) // 32) * 32
    per_entry = (8 if "df64" in kernel else (2 if "mat16" in kernel else 4)) + cell_bytes(lp)
    vec = (8 if "df64" in kernel else 4) * m + 8 * n
    return float(mpad) * s_pad * per_entry + vec


def hbm_peak_gbs():
    """(GB/s, source): the measured HBM copy bandwidth of these GB300s (MEASURED_PEAKS.json),
    else the 6.8 TB/s fallback of an earlier GB300 measurement."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(path))["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (of measured)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback 6.8 TB/s (of fallback)"




def run_reference(args):
    """The reference's CPU implementation of the path (the oracle port of its STREAMING FP64
    operator, all host cores): each step is one B^T (B a) on all points, the work of one CG
    iteration; fits/s = 1 / (median step time x the operator applications of one fit). Warm-up
    steps run on 1/16 of the points. Imports nothing of this library."""
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    x, _ = make_workload(args.seed)
    lp, ix = oracle_grid_arrays()
    n, m = lp.shape[0], x.shape[0]
    iters = args.reference_iterations or REFERENCE_ITERATIONS[args.basis]
    cg_ops = cg_operator_applications(iters)
    ref = CpuReference(x, lp, ix, threads, args.basis)
    for _ in range(args.warmup):
        ref.warm()
    times = [ref.apply_seconds() for _ in range(args.steps)]
    ref.close()
    step = statistics.median(times)
    value = 1.0 / (step * cg_ops)
    line = {
        "impl": "reference", "metric": "fits_per_sec", "value": value, "unit": "fits/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sum(times) * 1e3 / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(args.basis, n, m, args.epsilon, world),
        "precision": "FP64 (the reference's STREAMING operator and ConjugateGradients)",
        "step": "one B^T(B a) on all points (one CG iteration's operator work); fits/s = 1 / "
                f"(median step x {cg_ops:g} operator applications per fit)",
        "seconds_per_fit": step * cg_ops,
        "cpu_baseline": {"value": value, "unit": "fits/s", "cores": threads, "kind": "port",
                         "sample": ref.describe(args.steps, cg_ops),
                         "cg_iterations_per_fit": iters, "host": os.uname().machine},
        "e2e": {"value": value, "unit": "fits/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def grid_name(basis: str) -> str:
    return "ModLinear" if basis == "modlinear" else "Linear"


def count_iterations(args):
    """Plain CG iterations of one fit with the FP64-accurate df64 products (untimed)."""
    import sgpp_gb300 as sg

    x, y = make_workload(args.seed)
    grid, _, _ = grid_arrays(args.basis)
    params = {"precision": "df64"}
    params.update(dict(kv.split("=", 1) for kv in args.param))
    cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                sg.OperationMultipleEvalSubType.CUDA,
                                                parameters=params)
    op = sg.createOperationMultipleEval(grid, x, cfg)
    t0 = time.perf_counter()
    _, it, res = op.fit(y, LAMBDA, 20000, args.epsilon, mode=sg.SGMEV_SOLVE_PLAIN)
    print(json.dumps({"basis": args.basis, "plain_cg_iterations": it, "residual": res,
                      "epsilon": args.epsilon, "seconds": time.perf_counter() - t0}), flush=True)
    op.close()
    return 0


REGRESSION_FIXTURE = os.path.join(ROOT, "tests", "golden", "regression_d10_l5.npz")


def workload_checksums(x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """Sums, sums of squares and a few entries of x and y; the regression fixture records them
    (tests/golden/make_regression_alpha.py) so that a numpy whose generator streams differ is
    noticed."""
    return np.array([x.sum(), (x * x).sum(), y.sum(), (y * y).sum(), x[0, 0], x[-1, -1],
                     y[0], y[-1]], dtype=np.float64)


def reference_alpha(args, x, y):
    """(alpha, note): the reference's own FP64 CG solution of this workload (SG++'s
    SystemMatrixLeastSquaresIdentity + ConjugateGradients at epsilon 1e-12, committed as a
    fixture), or (None, why not) when the run's workload is not the fixture's."""
    if args.basis != "linear" or not os.path.exists(REGRESSION_FIXTURE):
        return None, "no reference fixture for this workload"
    f = np.load(REGRESSION_FIXTURE)
    if int(f["seed"]) != args.seed or int(f["m"]) != x.shape[0]:
        return None, "no reference fixture for this seed"
    want = f["checksums"]
    got = workload_checksums(x, y)
    if not np.allclose(got, want, rtol=1e-12, atol=0.0):
        return None, "the regenerated workload differs from the fixture's (numpy streams)"
    return (f["alpha"], f"the reference's FP64 ConjugateGradients solution (epsilon "
                        f"{float(f['epsilon']):g}, {int(f['iterations'])} iterations, "
                        "tests/golden/regression_d10_l5.npz)")


def dense_mult_gflops(args, grid, x, work_per_op, peak32, peak64):
    """One launch each of the dense FP32 and native FP64 mult kernels (the STREAMING algorithm)
    on the benchmark workload, untimed by the fits: GFLOP/s by the reference's count
    (LearnerVectorizedPerformanceCalculator.cpp:89-109, 6 N M d per op) and the fraction of the
    FP32 / FP64 FMA peak measured in this run (sgmev_fma_peak, 2 FLOP per FMA)."""
    import sgpp_gb300 as sg

    out = {}
    for name, prec, kind, peak in (("fp32_dense", "float", sg.SGMEV_KERNEL_MULT_FP32, peak32),
                                   ("fp64_dense", "double", sg.SGMEV_KERNEL_MULT_FP64, peak64)):
        cfg = sg.OperationMultipleEvalConfiguration(
            sg.OperationMultipleEvalType.STREAMING, sg.OperationMultipleEvalSubType.CUDA,
            parameters={"precision": prec, "algo": "dense", "materialize": "off"})
        op = sg.createOperationMultipleEval(grid, x, cfg)
        a = np.random.default_rng(3).standard_normal(grid.getSize())
        out_m = np.zeros(x.shape[0])
        op.mult(a, out_m)  # warm-up
        op.profile(True)
        for _ in range(args.dense_probe):
            op.mult(a, out_m)
        cnt, sec = op.profileRead(kind)
        op.profile(False)
        op.close()
        if not cnt:
            out[name] = None
            continue
        avg = sec / cnt
        gflops = work_per_op / avg / 1e9
        out[name] = {"gflops_ref_count": gflops, "ms_per_launch": avg * 1e3, "launches": cnt,
                     "peak_gflops_measured": peak / 1e9, "frac_of_peak": gflops / (peak / 1e9)}
    return out


def plain_fp64_fit(args, grid, x, d_y, stream, mixed_fits_per_sec, local_rank):
    """The plain per-problem FP64 path: one FP64-accurate CG fit (SGMEV_SOLVE_PLAIN, the
    reference's algorithm) on a df64 operator, whose products stream the materialised
    float-float subspace products, timed whole on the device after one warm-up fit."""
    import torch

    import sgpp_gb300 as sg

    params = dict(kv.split("=", 1) for kv in args.param)
    params["precision"] = "df64"
    cfg = sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                sg.OperationMultipleEvalSubType.CUDA,
                                                parameters=params)
    op = sg.createOperationMultipleEval(grid, x, cfg)
    op.setStream(stream.cuda_stream)
    n = grid.getSize()
    d_a = torch.zeros(n, dtype=torch.float64, device=f"cuda:{local_rank}")
    op.fitDevice(d_y.data_ptr(), d_a.data_ptr(), LAMBDA, 20000, args.epsilon,
                 mode=sg.SGMEV_SOLVE_PLAIN)  # warm-up (builds the products)
    times, its = [], []
    for _ in range(args.plain_fp64_probe):
        d_a.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        it, _ = op.fitDevice(d_y.data_ptr(), d_a.data_ptr(), LAMBDA, 20000, args.epsilon,
                             mode=sg.SGMEV_SOLVE_PLAIN)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
        its.append(it)
    op.close()
    t = statistics.median(times)
    return {"fits_per_sec": 1.0 / t, "ms_per_fit": t * 1e3, "cg_iterations": its,
            "what": "SGMEV_SOLVE_PLAIN on a df64 operator (FP64-accurate float-float products "
                    "streamed from the materialised subspace products), the reference's CG",
            "speedup_mixed_vs_plain_fp64": mixed_fits_per_sec * t}


def batched_probe(args):
    """One run of the batched configuration: 96 problems of the size mix (d uniform in 2..12,
    level in 3..7, M log-uniform in [1e3, 2^20], N*M*d <= 1e12), 16 targets each, as block fits
    on the tensor cores with 4 problems in flight, against the plain per-problem FP64 path
    (sgpp_gb300.batch_bench --engine block); a summary of its line."""
    import types

    from sgpp_gb300 import batch_bench

    a = types.SimpleNamespace(problems=96, rhs=16, max_work=1e12, epsilon=args.epsilon, lam=1e-4,
                              check=2, seed=11, workers=4, plain=1, param=[])
    line = batch_bench.measure_block(a)
    return {"metric": "batched_solves_per_sec", "value": line["value"], "unit": "solves/s",
            "seconds": line["seconds"], "problems": a.problems, "rhs": a.rhs,
            "plain_fp64_solves_per_sec": line["plain_fp64_path"]["solves_per_sec"],
            "speedup_vs_plain_fp64": line["speedup_vs_plain_fp64"], "paths": line["paths"],
            "alpha_rel_err_vs_fp64": line["alpha_rel_err_vs_fp64"],
            "workload": "96 problems, d uniform in 2..12, level in 3..7, M log-uniform in "
                        "[1e3, 2^20], uniform data, N*M*d <= 1e12, 16 targets each; block fits "
                        "on the tensor cores (FP16 products), 4 problems in flight; plain FP64 = "
                        "SGMEV_SOLVE_PLAIN on a df64 operator per problem and target"}


def op_config(args):
    """Operator configuration: the CUDA subtype with its default knobs, plus --inner-tol."""
    import sgpp_gb300 as sg

    params = dict(kv.split("=", 1) for kv in args.param)
    if args.inner_tol is not None:
        params["inner_tol"] = repr(args.inner_tol)
    return sg.OperationMultipleEvalConfiguration(sg.OperationMultipleEvalType.STREAMING,
                                                 sg.OperationMultipleEvalSubType.CUDA,
                                                 parameters=params)


def run_ours(args):
    import torch

    import sgpp_gb300 as sg

    rank, world, local_rank = env_rank()
    dist = None
    if world > 1:
        import torch.distributed as dist_mod

        dist = dist_mod
        dist.init_process_group("nccl")
    torch.cuda.set_device(local_rank)
    if sg.device_count() < 1:
        raise RuntimeError("bench.py needs a CUDA device")

    x, y = make_workload(args.seed + rank)
    grid, lp, ix = grid_arrays(args.basis)
    n, m = grid.getSize(), x.shape[0]
    work_per_op = FLOP_PER_PAIR_DIM * n * m * DIM

    stream = torch.cuda.Stream()
    op = sg.createOperationMultipleEval(grid, x, op_config(args))  # FP64 op + FP32 copies
    op.setStream(stream.cuda_stream)
    tuned = None
    if args.autotune:
        from sgpp_gb300 import autotune

        # launch shapes of the inner solves' kernels, searched once per device and shape (untimed)
        tuned = autotune.tune_and_cache(op, grid, m, ["multT16"])
    d_y = torch.from_numpy(y).to(f"cuda:{local_rank}")
    d_alpha = torch.zeros(n, dtype=torch.float64, device=f"cuda:{local_rank}")
    d_ref = torch.zeros(n, dtype=torch.float64, device=f"cuda:{local_rank}")

    # FP64 solutions for the error check (untimed): the reference's own CG solution of this
    # workload (fixture) and this library's refinement to a tight FP64 residual
    it_ref, _ = op.fitDevice(d_y.data_ptr(), d_ref.data_ptr(), LAMBDA, 20000, args.ref_epsilon,
                             mode=sg.SGMEV_SOLVE_MIXED)
    alpha_ref = d_ref.cpu().numpy()
    alpha_fixture, fixture_note = reference_alpha(args, x, y)

    def one_fit():
        return op.fitDevice(d_y.data_ptr(), d_alpha.data_ptr(), LAMBDA, 20000, args.epsilon,
                            mode=sg.SGMEV_SOLVE_MIXED)

    for _ in range(args.warmup):
        one_fit()
    peak32, clock_khz = sg.fma_peak(sg.SGMEV_FP32)
    peak64, _ = sg.fma_peak(sg.SGMEV_FP64)

    gpu_index = int(os.environ.get("CUDA_VISIBLE_DEVICES", str(local_rank)).split(",")[local_rank]) \
        if os.environ.get("CUDA_VISIBLE_DEVICES") else local_rank
    sampler = ClockSampler(gpu_index)
    launches0 = op.kernelLaunches()
    op.profile(True)
    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
    iters = []
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    for k in range(args.steps):
        events[k][0].record(stream)
        it, _ = one_fit()
        events[k][1].record(stream)
        iters.append(it)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    if dist:
        dist.barrier()
    step_ms = [a.elapsed_time(b) for a, b in events]
    total_s = sum(step_ms) * 1e-3
    launches = op.kernelLaunches() - launches0
    kstats = {name: op.profileRead(kind) for name, kind in
              (("mult_fp32", sg.SGMEV_KERNEL_MULT_FP32), ("multT_fp32", sg.SGMEV_KERNEL_MULTT_FP32),
               ("mult_fp64", sg.SGMEV_KERNEL_MULT_FP64), ("multT_fp64", sg.SGMEV_KERNEL_MULTT_FP64),
               ("mult_df64", sg.SGMEV_KERNEL_MULT_DF64), ("multT_df64", sg.SGMEV_KERNEL_MULTT_DF64),
               ("mult_sub32", sg.SGMEV_KERNEL_MULT_SUB32),
               ("multT_sub32", sg.SGMEV_KERNEL_MULTT_SUB32),
               ("mult_subdf64", sg.SGMEV_KERNEL_MULT_SUBDF),
               ("multT_subdf64", sg.SGMEV_KERNEL_MULTT_SUBDF),
               ("mult_mat32", sg.SGMEV_KERNEL_MULT_MAT32),
               ("multT_mat32", sg.SGMEV_KERNEL_MULTT_MAT32),
               ("mult_matdf64", sg.SGMEV_KERNEL_MULT_MATDF),
               ("multT_matdf64", sg.SGMEV_KERNEL_MULTT_MATDF),
               ("system_mat32", sg.SGMEV_KERNEL_SYSTEM_MAT32),
               ("mult_mat16", sg.SGMEV_KERNEL_MULT_MAT16),
               ("multT_mat16", sg.SGMEV_KERNEL_MULTT_MAT16))}
    op.profile(False)
    alpha = d_alpha.cpu().numpy()
    err = float(np.abs(alpha - alpha_ref).max() / np.abs(alpha_ref).max())
    err_ref = (float(np.abs(alpha - alpha_fixture).max() / np.abs(alpha_fixture).max())
               if alpha_fixture is not None else None)

    if dist:
        t = torch.tensor([total_s], device=f"cuda:{local_rank}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_s = float(t.item())
    value = args.steps * world / total_s

    # roofline of the dominant tile kernel: HBM-bound for the kernels that stream the
    # materialised products, FMA-bound for the ones that evaluate the hats
    dom = max(kstats, key=lambda k: kstats[k][1])
    cnt, sec = kstats[dom]
    avg = sec / max(cnt, 1)
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        traffic = json.load(open(tpath)).get(dom)
    if "_mat" in dom:
        by = mat_bytes_per_launch(dom, lp, m, n)
        achieved = by / avg / 1e9
        peak, peak_src = hbm_peak_gbs()
        roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                    "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                    "launches_timed": cnt, "avg_launch_ms": avg * 1e3,
                    "peak_source": peak_src,
                    "bytes_per_launch": by,
                    "bytes_model": "materialised products read once per launch (FP16: 2 B, FP32: "
                                   "4 B, df64: 8 B per product, plus its cell index: a nibble when "
                                   "no subspace has more than 16 cells, else a byte) per padded "
                                   "point and padded subspace, plus the input and output vectors"}
    else:
        achieved = work_per_op / avg / 1e12
        is64 = dom.endswith("fp64") and not dom.endswith("df64")
        peak = (peak64 if is64 else peak32) / 1e12
        roofline = {"bound": "fp64-vector" if is64 else "fp32-vector", "kernel": dom,
                    "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak, "traffic": traffic, "launches_timed": cnt,
                    "avg_launch_ms": avg * 1e3,
                    "peak_source": "measured in this run: FMA chains on every SM (sgmev_fma_peak)",
                    "peaks_measured_tflops": {"fp32": peak32 / 1e12, "fp64": peak64 / 1e12},
                    "flop_per_launch": work_per_op}

    # mult GFLOP/s by the reference's count (6 N M d per op) of the dense kernels (the
    # STREAMING algorithm: every grid point for every data point), against the FMA peaks
    # measured in this run
    mult_gflops = dense_mult_gflops(args, grid, x, work_per_op, peak32, peak64) \
        if args.dense_probe else None
    # end to end through the public API from pinned host buffers
    e2e = None
    if args.e2e_steps > 0:
        x_pin = torch.from_numpy(x).pin_memory()
        y_pin = torch.from_numpy(y).pin_memory()
        xs = x_pin.numpy()
        ys = y_pin.numpy()
        e2e_times = []
        for k in range(args.e2e_steps + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            op2 = sg.createOperationMultipleEval(grid, xs, op_config(args))
            a_host, _, _ = op2.fit(ys, LAMBDA, 20000, args.epsilon, mode=sg.SGMEV_SOLVE_MIXED)
            op2.close()
            torch.cuda.synchronize()
            if k > 0:  # first call is a warm-up
                e2e_times.append(time.perf_counter() - t0)
        h2d = x.nbytes + y.nbytes + lp.nbytes + ix.nbytes
        e2e = {"value": len(e2e_times) / sum(e2e_times), "unit": "fits/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(n * 8),
               "steps": len(e2e_times),
               "what": "createOperationMultipleEval(host X) + fit(host y) + alpha to host + close"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        iters_fit = args.reference_iterations or REFERENCE_ITERATIONS[args.basis]
        t_fit, sample = cpu_fit_seconds(x, lp, ix, cg_operator_applications(iters_fit), threads,
                                        args.basis)
        cpu = {"value": 1.0 / t_fit, "unit": "fits/s", "cores": threads, "kind": "port",
               "sample": sample, "cg_iterations_per_fit": iters_fit,
               "host": os.uname().machine}

    # plain FP64 path: one FP64-accurate plain CG fit (SGMEV_SOLVE_PLAIN) on the df64
    # materialised products, the fastest FP64-accurate operator here, timed whole on the device
    plain = plain_fp64_fit(args, grid, x, d_y, stream, value / world, local_rank) \
        if args.plain_fp64_probe else None

    # the batched configuration (96 problems x 16 targets on the tensor cores against the plain
    # per-problem FP64 path), one run on one GPU, outside the timed region
    batched = None
    if args.batched_probe and world == 1:
        try:
            batched = batched_probe(args)
        except Exception as e:  # the line itself does not depend on this probe
            batched = {"error": f"{type(e).__name__}: {e}"}

    if rank == 0:
        lat = sorted(step_ms)
        p = lambda q: lat[min(len(lat) - 1, int(round(q * (len(lat) - 1))))]
        line = {
            "metric": "fits_per_sec", "value": value, "unit": "fits/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_s * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f16+f32+df64", "data": "synthetic",
            "config": bench_config(args.basis, n, m, args.epsilon, world),
            "precision": "mixed: inner CG in FP32 arithmetic on FP16 copies of the materialised "
                         "subspace products (2^-11 relative per product) with FP64 vectors; "
                         "outer iterative-refinement residual with FP64-accurate float-float "
                         "(df64) products",
            "latency_ms": {"p50": p(0.5), "p99": p(0.99)},
            "alpha_rel_err_vs_fp64": err_ref if err_ref is not None else err,
            "alpha_rel_err_vs_fp64_source": (fixture_note if err_ref is not None else
                                             "this library's df64 refinement to relative "
                                             f"residual {args.ref_epsilon} ({fixture_note})"),
            "alpha_rel_err_vs_df64_refinement": err,
            "cg_iterations": iters, "fp64_solution_iterations": it_ref,
            "mult_gflops": mult_gflops,
            "kernel_stats": {k: {"launches": c, "ms_total": s * 1e3} for k, (c, s) in kstats.items()},
            "roofline": roofline, "clocks": clocks, "gpu_launches": int(launches),
            "launch_shape": tuned,
            "e2e": e2e, "cpu_baseline": cpu, "plain_fp64_path": plain,
            "batched": batched,
        }
        print(json.dumps(line), flush=True)
    op.close()
    if dist:
        dist.destroy_process_group()
    return 0


def run_block(args):
    """16 regression fits sharing the benchmark's grid and data (targets y and y + N(0, 1) noise)
    through sgmev_fit_block: tensor-core inner solves over the 16 columns, df64 outer
    residuals. value = fits/s (16 per step); compared with 16 single-target mixed fits."""
    import torch

    import sgpp_gb300 as sg
    from sgpp_gb300 import autotune

    blk = dict(kv.split("=", 1) for kv in args.param).get("block_products", "f16")
    torch.cuda.set_device(0)
    x, y = make_workload(args.seed)
    grid, lp, ix = grid_arrays(args.basis)
    n, m = grid.getSize(), x.shape[0]
    K = sg.SGMEV_BLOCK_RHS
    rng = np.random.default_rng(args.seed + 1)
    Y = np.empty((K, m))
    Y[0] = y
    Y[1:] = y + rng.standard_normal((K - 1, m))
    stream = torch.cuda.Stream()
    op = sg.createOperationMultipleEval(grid, x, op_config(args))
    op.setStream(stream.cuda_stream)
    tuned = None
    if args.autotune:
        tuned = autotune.tune_and_cache(op, grid, m, ["block"])
    d_y = torch.from_numpy(Y).cuda()
    d_a = torch.zeros((K, n), dtype=torch.float64, device="cuda")
    for _ in range(args.warmup):
        op.fitBlockDevice(d_y.data_ptr(), d_a.data_ptr(), LAMBDA, 100000, args.epsilon)
    op.profile(True)
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    ms, its = [], None
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        its, res = op.fitBlockDevice(d_y.data_ptr(), d_a.data_ptr(), LAMBDA, 100000, args.epsilon)
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    clocks = sampler.stop()
    kst = {k: op.profileRead(kind) for k, kind in (("block_mult", sg.SGMEV_KERNEL_BLOCK_MULT),
                                                   ("block_multT", sg.SGMEV_KERNEL_BLOCK_MULTT),
                                                   ("mult_matdf64", sg.SGMEV_KERNEL_MULT_MATDF),
                                                   ("multT_matdf64", sg.SGMEV_KERNEL_MULTT_MATDF))}
    op.profile(False)
    alpha = d_a.cpu().numpy()
    ref, note = reference_alpha(args, x, y)
    err0 = float(np.abs(alpha[0] - ref).max() / np.abs(ref).max()) if ref is not None else None
    # one single-target mixed fit (the per-problem path), timed, and its alpha for column K-1
    d_y1 = torch.from_numpy(Y[K - 1].copy()).cuda()
    d_a1 = torch.zeros(n, dtype=torch.float64, device="cuda")
    op.fitDevice(d_y1.data_ptr(), d_a1.data_ptr(), LAMBDA, 100000, args.epsilon,
                 mode=sg.SGMEV_SOLVE_MIXED)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    it1, _ = op.fitDevice(d_y1.data_ptr(), d_a1.data_ptr(), LAMBDA, 100000, args.epsilon,
                          mode=sg.SGMEV_SOLVE_MIXED)
    e1.record(stream)
    torch.cuda.synchronize()
    single_ms = e0.elapsed_time(e1)
    a1 = d_a1.cpu().numpy()
    err_last = float(np.abs(alpha[K - 1] - a1).max() / np.abs(a1).max())
    op.close()
    step = statistics.median(ms)
    value = K / (step * 1e-3)
    bm = kst["block_mult"]
    bt = kst["block_multT"]
    line = {
        "metric": "fits_per_sec", "value": value, "unit": "fits/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step,
        "higher_is_better": True, "workload": "block",
        "config": {"workload": f"16 regression fits sharing one grid and data set: "
                               f"{bench_config(args.basis, n, m, args.epsilon, 1)['workload']}; "
                               "targets y and y + N(0, 1)"},
        "dtype": f"{blk} (tensor cores, FP32 accumulation) + df64",
        "precision": f"inner block CG on {blk.upper()} tcgen05 products (products rounded to "
                     f"{blk.upper()}, vectors as {blk.upper()} high + low parts, FP32 accumulation "
                     "in tensor memory), FP64 vectors; "
                     "outer residuals with FP64-accurate float-float products per column",
        "inner_cg_steps_per_column": [int(v) for v in its],
        "alpha_rel_err_vs_fp64_column0": err0, "alpha_rel_err_source": note,
        "alpha_rel_err_vs_single_mixed_fit_column15": err_last,
        "single_target_mixed_fit_ms": single_ms, "single_target_iterations": it1,
        "speedup_vs_16_single_fits": 16 * single_ms / step,
        "block_kernels": {"mult": {"launches": bm[0], "ms_avg": bm[1] / max(bm[0], 1) * 1e3},
                          "multT": {"launches": bt[0], "ms_avg": bt[1] / max(bt[0], 1) * 1e3}},
        "df64_residual_ms": (kst["mult_matdf64"][1] + kst["multT_matdf64"][1]) * 1e3 / args.steps,
        "launch_shape": tuned, "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    return 0


def run_module_workload(args):
    """The other configurations' benchmarks, each printing its own JSON line: the adaptive-grid
    loop (d=8 level 4, M=2^19, 6 rounds of 40 points), the batched mix (96 problems x 16 targets
    on block fits) and the serving loop (Poisson arrivals, 200 req/s for 60 s)."""
    argv = {"adaptive": ["--engine", "fitter"],
            "batched": ["--engine", "block", "--problems", "96", "--rhs", "16",
                        "--max-work", "1e12"],
            "serving": ["--rate", "200", "--duration", "60", "--max-work", "1e12"]}[args.workload]
    module = {"adaptive": "sgpp_gb300.adaptive", "batched": "sgpp_gb300.batch_bench",
              "serving": "sgpp_gb300.serving"}[args.workload]
    import importlib

    mod = importlib.import_module(module)
    saved = sys.argv
    sys.argv = [module] + argv
    try:
        return mod.main()
    finally:
        sys.argv = saved


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--seed", type=int, default=42)
    ap.add_argument("--epsilon", type=float, default=1e-8)
    ap.add_argument("--ref-epsilon", type=float, default=1e-12)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--reference-iterations", type=int, default=0,
                    help="plain CG iterations per fit for the CPU scaling (0: REFERENCE_ITERATIONS)")
    ap.add_argument("--basis", default="linear", choices=["linear", "modlinear"])
    ap.add_argument("--count-iterations", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--plain-fp64-probe", type=int, default=2,
                    help="timed plain FP64-accurate fits on a df64 operator (0: skip)")
    ap.add_argument("--batched-probe", type=int, default=1,
                    help="one run of the batched configuration beside the line (0: skip)")
    ap.add_argument("--dense-probe", type=int, default=1,
                    help="timed launches of the dense FP32 and FP64 mult kernels (0: skip)")
    ap.add_argument("--inner-tol", type=float, default=None,
                    help="inner tolerance of the mixed fits (library default when omitted)")
    ap.add_argument("--workload", default="regression",
                    choices=["regression", "block", "adaptive", "batched", "serving"],
                    help="block: 16 fits sharing the data (tensor-core block fits); adaptive: "
                         "the adaptive-grid loop (sgpp_gb300.adaptive); batched: 96 problems x "
                         "16 targets (sgpp_gb300.batch_bench --engine block); serving: Poisson "
                         "arrivals at 200 req/s (sgpp_gb300.serving)")
    ap.add_argument("--autotune", type=int, default=1,
                    help="pick launch shapes with sgpp_gb300.autotune before timing (cached)")
    ap.add_argument("--param", action="append", default=[], metavar="KEY=VALUE",
                    help="operator knob passed to createOperationMultipleEval (repeatable)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.count_iterations:
        return count_iterations(args)
    if args.workload == "block":
        return run_block(args)
    if args.workload in ("adaptive", "batched", "serving"):
        return run_module_workload(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())

"""Least-squares fitting with spatial adaptivity on the GPU (sgfit_* in the library).

Mirrors the reference's datamining fitting module
(datadriven/src/sgpp/datadriven/datamining/modules/fitting/ModelFittingLeastSquares.cpp and
FitterConfigurationLeastSquares, with the configuration structures and defaults of
FitterConfiguration::setupDefaults): fit(dataset), adapt(), update(dataset), evaluate(samples).
The operator, y and alpha stay on the device between solves; adapt() re-stages only the grid.
"""
from __future__ import annotations

import ctypes
import json
from typing import Optional

import numpy as np

from . import (SGMEV_DF64, SGMEV_FP32, SGMEV_FP64, SGMEV_SOLVE_MIXED, SGMEV_SOLVE_PLAIN, Dataset,
               OP_KNOBS, Grid, GridType, OperationException, OperationMultipleEvalConfiguration,
               OperationMultipleEvalSubType, OperationMultipleEvalType, _as_matrix, _check,
               _precision_of, _vp, load_library)


class sgfit_config(ctypes.Structure):
    _fields_ = [("level", ctypes.c_int), ("basis", ctypes.c_int), ("lambda_", ctypes.c_double),
                ("final_eps", ctypes.c_double), ("final_max_iterations", ctypes.c_int64),
                ("refine_eps", ctypes.c_double), ("refine_max_iterations", ctypes.c_int64),
                ("num_refinements", ctypes.c_int64), ("num_refinement_points", ctypes.c_int64),
                ("refinement_threshold", ctypes.c_double), ("mode", ctypes.c_int),
                ("precision", ctypes.c_int)]


def _lib():
    L = load_library()
    if not getattr(L, "_sgfit_bound", False):
        vp, i64, c_int, dbl = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
        pi64 = ctypes.POINTER(i64)
        for name, res, args in (
                ("sgfit_config_defaults", None, [ctypes.POINTER(sgfit_config)]),
                ("sgfit_create", c_int, [ctypes.POINTER(vp), ctypes.POINTER(sgfit_config),
                                         ctypes.c_char_p]),
                ("sgfit_destroy", c_int, [vp]),
                ("sgfit_fit", c_int, [vp, i64, c_int, vp, vp]),
                ("sgfit_adapt", c_int, [vp, ctypes.POINTER(c_int)]),
                ("sgfit_update", c_int, [vp, i64, c_int, vp, vp]),
                ("sgfit_evaluate", c_int, [vp, i64, vp, vp]),
                ("sgfit_grid", c_int, [vp, ctypes.POINTER(c_int), pi64, vp, vp]),
                ("sgfit_alpha", c_int, [vp, vp]),
                ("sgfit_stats", c_int, [vp, pi64, ctypes.POINTER(dbl), pi64])):
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        L._sgfit_bound = True
    return L


# ---- configuration (the reference's structures, FitterConfiguration.cpp:143-218 defaults) ----
class RegularGridConfiguration:
    def __init__(self):
        self.type_ = GridType.Linear
        self.dim_ = 0
        self.level_ = 3


class AdaptivityConfiguration:
    def __init__(self):
        self.numRefinements_ = 1
        self.refinementThreshold_ = 0.0
        self.numRefinementPoints_ = 1


class SLESolverConfiguration:
    def __init__(self):
        self.eps_ = 1e-12
        self.maxIterations_ = 100
        self.threshold_ = 1e-12


class RegularizationConfiguration:
    def __init__(self):
        self.lambda_ = 0.01


class FitterConfigurationLeastSquares:
    """Grid, adaptivity, solver (refine / final), regularization and multiple-eval configuration.
    The multiple-eval configuration's parameters are the CUDA operator's knobs ("precision",
    "algo", ...) plus "solve": "plain" (default, the reference's CG) or "mixed"."""

    def __init__(self):
        self.setupDefaults()

    def setupDefaults(self) -> None:
        self.gridConfig = RegularGridConfiguration()
        self.adaptivityConfig = AdaptivityConfiguration()
        self.solverRefineConfig = SLESolverConfiguration()
        self.solverFinalConfig = SLESolverConfiguration()
        self.regularizationConfig = RegularizationConfiguration()
        self.multipleEvalConfig = OperationMultipleEvalConfiguration(
            OperationMultipleEvalType.STREAMING, OperationMultipleEvalSubType.CUDA)

    def getGridConfig(self) -> RegularGridConfiguration:
        return self.gridConfig

    def getRefinementConfig(self) -> AdaptivityConfiguration:
        return self.adaptivityConfig

    def getSolverRefineConfig(self) -> SLESolverConfiguration:
        return self.solverRefineConfig

    def getSolverFinalConfig(self) -> SLESolverConfiguration:
        return self.solverFinalConfig

    def getRegularizationConfig(self) -> RegularizationConfiguration:
        return self.regularizationConfig

    def getMultipleEvalConfig(self) -> OperationMultipleEvalConfiguration:
        return self.multipleEvalConfig


_OP_KNOBS = OP_KNOBS


class ModelFittingLeastSquares:
    """ModelFittingLeastSquares over one device-resident GPU operator."""

    def __init__(self, config: Optional[FitterConfigurationLeastSquares] = None):
        self.config = config or FitterConfigurationLeastSquares()
        c = self.config
        params = dict(c.getMultipleEvalConfig().getParameters())
        cfg = sgfit_config()
        L = _lib()
        L.sgfit_config_defaults(ctypes.byref(cfg))
        cfg.level = int(c.getGridConfig().level_)
        gt = GridType(c.getGridConfig().type_)
        if gt not in (GridType.Linear, GridType.ModLinear):
            raise OperationException("ModelFittingLeastSquares on the GPU: Linear and ModLinear grids")
        cfg.basis = 1 if gt == GridType.ModLinear else 0
        cfg.lambda_ = float(c.getRegularizationConfig().lambda_)
        cfg.final_eps = float(c.getSolverFinalConfig().eps_)
        cfg.final_max_iterations = int(c.getSolverFinalConfig().maxIterations_)
        cfg.refine_eps = float(c.getSolverRefineConfig().eps_)
        cfg.refine_max_iterations = int(c.getSolverRefineConfig().maxIterations_)
        cfg.num_refinements = int(c.getRefinementConfig().numRefinements_)
        cfg.num_refinement_points = int(c.getRefinementConfig().numRefinementPoints_)
        cfg.refinement_threshold = float(c.getRefinementConfig().refinementThreshold_)
        solve = str(params.get("solve", "plain")).lower()
        if solve not in ("plain", "mixed"):
            raise OperationException('parameter "solve" must be "plain" or "mixed"')
        cfg.mode = SGMEV_SOLVE_MIXED if solve == "mixed" else SGMEV_SOLVE_PLAIN
        cfg.precision = _precision_of(params)
        knobs = {k: str(v) for k, v in params.items() if k in _OP_KNOBS}
        h = ctypes.c_void_p(None)
        _check(L.sgfit_create(ctypes.byref(h), ctypes.byref(cfg),
                              json.dumps(knobs).encode() if knobs else None))
        self._h = h
        self._cfg = cfg
        self.dataset = None

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib().sgfit_destroy(self._h)
            self._h = ctypes.c_void_p(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _data(dataset: Dataset):
        x = _as_matrix(dataset.getData())
        y = np.ascontiguousarray(dataset.getTargets(), np.float64)
        if y.shape[0] != x.shape[0]:
            raise OperationException("dataset targets and rows differ in number")
        return x, y

    def fit(self, dataset: Dataset) -> None:
        x, y = self._data(dataset)
        self.dataset = dataset
        self.config.getGridConfig().dim_ = x.shape[1]
        _check(_lib().sgfit_fit(self._h, x.shape[0], x.shape[1], _vp(x), _vp(y)))

    def adapt(self) -> bool:
        refined = ctypes.c_int(0)
        _check(_lib().sgfit_adapt(self._h, ctypes.byref(refined)))
        return bool(refined.value)

    def update(self, dataset: Dataset) -> None:
        x, y = self._data(dataset)
        self.dataset = dataset
        _check(_lib().sgfit_update(self._h, x.shape[0], x.shape[1], _vp(x), _vp(y)))

    def evaluate(self, samples, results: Optional[np.ndarray] = None) -> np.ndarray:
        x = _as_matrix(samples)
        out = np.zeros(x.shape[0]) if results is None else results
        if out.shape[0] != x.shape[0] or out.dtype != np.float64 or not out.flags.c_contiguous:
            raise OperationException("results must be a contiguous float64 vector of len(samples)")
        _check(_lib().sgfit_evaluate(self._h, x.shape[0], _vp(x), _vp(out)))
        return out

    def getGrid(self) -> Grid:
        d = ctypes.c_int(0)
        n = ctypes.c_int64(0)
        L = _lib()
        _check(L.sgfit_grid(self._h, ctypes.byref(d), ctypes.byref(n), None, None))
        lev = np.zeros((n.value, max(d.value, 1)), np.int32)
        idx = np.zeros_like(lev)
        _check(L.sgfit_grid(self._h, None, None, _vp(lev), _vp(idx)))
        gt = GridType.ModLinear if self._cfg.basis == 1 else GridType.Linear
        return Grid.fromArrays(lev, idx, gt)

    def getSurpluses(self) -> np.ndarray:
        n = ctypes.c_int64(0)
        L = _lib()
        _check(L.sgfit_grid(self._h, None, ctypes.byref(n), None, None))
        a = np.zeros(max(n.value, 1))
        _check(L.sgfit_alpha(self._h, _vp(a)))
        return a[:n.value]

    def stats(self):
        it = ctypes.c_int64(0)
        res = ctypes.c_double(0.0)
        ref = ctypes.c_int64(0)
        _check(_lib().sgfit_stats(self._h, ctypes.byref(it), ctypes.byref(res), ctypes.byref(ref)))
        return {"cg_iterations": int(it.value), "residual": float(res.value),
                "refinements": int(ref.value)}

    @property
    def refinementsPerformed(self) -> int:
        return self.stats()["refinements"]


__all__ = ["ModelFittingLeastSquares", "FitterConfigurationLeastSquares",
           "RegularGridConfiguration", "AdaptivityConfiguration", "SLESolverConfiguration",
           "RegularizationConfiguration", "SGMEV_FP64", "SGMEV_FP32", "SGMEV_DF64"]

"""sgpp_gb300 — GB300 (sm_103a) multi-evaluation for SG++'s hat-basis sparse grids.

Host-side mirror of the reference interface for this path, over the C ABI of
``libsgpp_gb300.so`` (``include/sgmev.h``). Names, argument meaning and error behaviour follow
the reference (pysgpp) so that callers and tests read like the reference's own:

  Grid.createLinearGrid(d); grid.getGenerator().regular(l); .refine(SurplusRefinementFunctor)
      base/src/sgpp/base/grid/Grid.cpp:73, StandardGridGenerator.cpp:27-30,64-68
  createOperationMultipleEval(grid, dataset, OperationMultipleEvalConfiguration(...))
      datadriven/src/sgpp/datadriven/DatadrivenOpFactory.cpp:409-552 — the (Linear, STREAMING,
      CUDA) branch returns OperationMultiEvalCuda; other combinations raise FactoryException
  op.mult(alpha, result) / op.multTranspose(source, result) / ranged variants / prepare() /
      getDuration() / getImplementationName()
      base/src/sgpp/base/operation/hash/OperationMultipleEval.hpp:27-130
  SystemMatrixLeastSquaresIdentity(grid, data, lambda)
      datadriven/src/sgpp/datadriven/algorithm/SystemMatrixLeastSquaresIdentity.cpp:18-65
  ConjugateGradients(imax, epsilon).solve(A, alpha, b, reuse, verbose, max_threshold)
      solver/src/sgpp/solver/sle/ConjugateGradients.cpp:22-151

DataVector / DataMatrix are numpy float64 arrays (1-D, and 2-D row-major [rows x dim]); result
arrays are written in place, as the reference writes into its DataVector arguments.

The compute path is the CUDA library only: importing works without a GPU, but creating an
operator raises OperationException when the library or a CUDA device is missing. There is no
CPU fallback.
"""
from __future__ import annotations

import ctypes
import enum
import json
import os
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBRARY_PATH = os.path.join(_HERE, "libsgpp_gb300.so")

SGMEV_OK = 0
SGMEV_ERR_INVALID = -1
SGMEV_ERR_CUDA = -2
SGMEV_ERR_NO_DEVICE = -3
SGMEV_ERR_UNSUPPORTED = -4
SGMEV_ERR_NOT_CONVERGED = -5
SGMEV_ERR_OOM = -6

SGMEV_FP64 = 0
SGMEV_FP32 = 1
SGMEV_DF64 = 2
SGMEV_SOLVE_PLAIN = 0
SGMEV_SOLVE_MIXED = 1
SGMEV_SOLVE_MIXED_NATIVE64 = 2

# every entry point declared in include/sgmev.h
EXPORTED_SYMBOLS = (
    "sgmev_last_error", "sgmev_version", "sgmev_device_count", "sgmev_create", "sgmev_destroy",
    "sgmev_prepare", "sgmev_get_sizes", "sgmev_mult", "sgmev_mult_transpose", "sgmev_mult_range",
    "sgmev_mult_transpose_range", "sgmev_mult_device", "sgmev_mult_transpose_device",
    "sgmev_system_apply", "sgmev_system_apply_device", "sgmev_fit", "sgmev_get_duration",
    "sgmev_set_stream", "sgmev_synchronize", "sgmev_kernel_launches", "sggrid_regular",
    "sggrid_refine_surplus", "sggrid_level_index_for_eval", "sgmev_fma_peak", "sgmev_profile",
    "sgmev_profile_read", "sgmev_fit_device", "sgmev_mult_transpose_noalloc",
    "sgmev_batch_create", "sgmev_batch_destroy", "sgmev_batch_footprint", "sgmev_batch_add",
    "sgmev_batch_remove", "sgmev_batch_step", "sgmev_batch_solve", "sgmev_batch_result",
    "sgmev_batch_info", "sgdata_size", "sgdata_read", "sgfit_config_defaults", "sgfit_create",
    "sgfit_destroy", "sgfit_fit", "sgfit_adapt", "sgfit_update", "sgfit_evaluate", "sgfit_grid",
    "sgfit_alpha", "sgfit_stats", "sgmev_mult_block", "sgmev_mult_transpose_block",
    "sgmev_fit_block", "sgmev_fit_block_device", "sgmev_set_params",
)

SGMEV_KERNEL_MULT_FP32 = 0
SGMEV_KERNEL_MULTT_FP32 = 1
SGMEV_KERNEL_MULT_FP64 = 2
SGMEV_KERNEL_MULTT_FP64 = 3
SGMEV_KERNEL_MULT_DF64 = 4
SGMEV_KERNEL_MULTT_DF64 = 5
SGMEV_KERNEL_MULT_SUB32 = 6
SGMEV_KERNEL_MULTT_SUB32 = 7
SGMEV_KERNEL_MULT_SUBDF = 8
SGMEV_KERNEL_MULTT_SUBDF = 9
SGMEV_KERNEL_MULT_MAT32 = 10
SGMEV_KERNEL_MULTT_MAT32 = 11
SGMEV_KERNEL_MULT_MATDF = 12
SGMEV_KERNEL_MULTT_MATDF = 13
SGMEV_KERNEL_SYSTEM_MAT32 = 14
SGMEV_KERNEL_MULT_MAT16 = 15
SGMEV_KERNEL_MULTT_MAT16 = 16
SGMEV_KERNEL_BLOCK_MULT = 17
SGMEV_KERNEL_BLOCK_MULTT = 18
SGMEV_BLOCK_RHS = 16


# ---- exceptions (base/src/sgpp/base/exception/) --------------------------------------------
class SGppException(RuntimeError):
    pass


class OperationException(SGppException):
    """operation_exception"""


class FactoryException(SGppException):
    """factory_exception"""


class NotImplementedException(SGppException):
    """not_implemented_exception"""


class FileException(SGppException):
    """base::file_exception: unreadable or malformed dataset text."""


class GenerationException(SGppException):
    """generation_exception"""


# ---- library loading ----------------------------------------------------------------------
_lib = None


def _vp(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


# operator parameters passed to sgmev_create (the other configuration parameters, such as
# "precision", are read by the Python side)
OP_KNOBS = ("precond", "algo", "inner_tol", "materialize", "materialize_multt", "inner_products",
            "system_product", "block_inner_tol", "block_mult_tiles", "block_mult_groups",
            "block_multt_groups", "block_stages", "block_loads", "block_mult_a", "block_window",
            "block_teams", "multt_batch", "multt_banks", "multt_ctas",
            "block_products")


def load_library(path: str = LIBRARY_PATH):
    """Load libsgpp_gb300.so (built by sgpp_gb300.build). Raises OperationException if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OperationException(
            f"{path} is missing: build it with `python -m sgpp_gb300.build` (no CPU fallback)")
    L = ctypes.CDLL(path)
    i64, c_int, dbl, vp = ctypes.c_int64, ctypes.c_int, ctypes.c_double, ctypes.c_void_p
    pi64, pdbl = ctypes.POINTER(i64), ctypes.POINTER(dbl)
    sig = {
        "sgmev_last_error": (ctypes.c_char_p, []),
        "sgmev_version": (c_int, []),
        "sgmev_device_count": (c_int, []),
        "sgmev_create": (c_int, [ctypes.POINTER(vp), c_int, i64, vp, vp, i64, vp, vp, vp, c_int,
                                 ctypes.c_char_p]),
        "sgmev_destroy": (c_int, [vp]),
        "sgmev_prepare": (c_int, [vp, i64, vp, vp]),
        "sgmev_get_sizes": (c_int, [vp, ctypes.POINTER(c_int), pi64, pi64]),
        "sgmev_mult": (c_int, [vp, vp, vp]),
        "sgmev_mult_transpose": (c_int, [vp, vp, vp]),
        "sgmev_mult_range": (c_int, [vp, vp, vp, i64, i64]),
        "sgmev_mult_transpose_range": (c_int, [vp, vp, vp, i64, i64]),
        "sgmev_mult_device": (c_int, [vp, vp, vp]),
        "sgmev_mult_transpose_device": (c_int, [vp, vp, vp]),
        "sgmev_system_apply": (c_int, [vp, vp, vp, dbl]),
        "sgmev_system_apply_device": (c_int, [vp, vp, vp, dbl]),
        "sgmev_fit": (c_int, [vp, c_int, vp, dbl, i64, dbl, c_int, vp, pi64, pdbl]),
        "sgmev_get_duration": (dbl, [vp]),
        "sgmev_set_stream": (c_int, [vp, vp]),
        "sgmev_synchronize": (c_int, [vp]),
        "sgmev_kernel_launches": (i64, [vp]),
        "sggrid_regular": (c_int, [c_int, c_int, pi64, vp, vp]),
        "sggrid_refine_surplus": (c_int, [c_int, i64, i64, vp, vp, vp, i64, dbl, pi64]),
        "sggrid_level_index_for_eval": (c_int, [c_int, i64, vp, vp, vp, vp]),
        "sgmev_fma_peak": (c_int, [c_int, pdbl, ctypes.POINTER(c_int)]),
        "sgmev_fit_device": (c_int, [vp, c_int, vp, dbl, i64, dbl, c_int, vp, pi64, pdbl]),
        "sgmev_mult_block": (c_int, [vp, vp, vp]),
        "sgmev_set_params": (c_int, [vp, ctypes.c_char_p]),
        "sgmev_mult_transpose_block": (c_int, [vp, vp, vp]),
        "sgmev_fit_block": (c_int, [vp, vp, dbl, i64, dbl, vp, vp, vp]),
        "sgmev_fit_block_device": (c_int, [vp, vp, dbl, i64, dbl, vp, vp, vp]),
        "sgmev_mult_transpose_noalloc": (c_int, [c_int, i64, vp, vp, i64, vp, vp, vp, vp]),
        "sgmev_batch_create": (c_int, [ctypes.POINTER(vp), c_int, c_int, i64, i64, ctypes.c_char_p]),
        "sgmev_batch_destroy": (c_int, [vp]),
        "sgmev_batch_footprint": (c_int, [c_int, i64, i64, c_int, pi64, pi64]),
        "sgmev_batch_add": (c_int, [vp, c_int, i64, vp, vp, i64, vp, vp, dbl, dbl, i64,
                                    ctypes.POINTER(c_int)]),
        "sgmev_batch_remove": (c_int, [vp, c_int]),
        "sgmev_batch_step": (c_int, [vp, c_int, vp]),
        "sgmev_batch_solve": (c_int, [vp, i64, pi64]),
        "sgmev_batch_result": (c_int, [vp, c_int, vp, pi64, pdbl, ctypes.POINTER(c_int)]),
        "sgmev_batch_info": (c_int, [vp, pi64, pi64, ctypes.POINTER(c_int)]),
        "sgmev_profile": (c_int, [vp, c_int]),
        "sgmev_profile_read": (c_int, [vp, c_int, pi64, pdbl]),
        "sgdata_size": (c_int, [c_int, ctypes.c_char_p, i64, c_int, c_int, vp, c_int, pi64, pi64]),
        "sgdata_read": (c_int, [c_int, ctypes.c_char_p, i64, c_int, c_int, i64, vp, c_int, vp,
                                c_int, vp, vp, i64, pi64, pi64]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(rc: int, exc=OperationException):
    if rc != SGMEV_OK:
        msg = load_library().sgmev_last_error().decode(errors="replace")
        raise exc(f"libsgpp_gb300 error {rc}: {msg}")


def device_count() -> int:
    return int(load_library().sgmev_device_count())


def fma_peak(precision: int = SGMEV_FP32):
    """Measured vector FMA throughput (FLOP/s, FMA = 2) and the reported SM clock (kHz)."""
    f = ctypes.c_double(0.0)
    k = ctypes.c_int(0)
    _check(load_library().sgmev_fma_peak(int(precision), ctypes.byref(f), ctypes.byref(k)))
    return float(f.value), int(k.value)


# ---- grids --------------------------------------------------------------------------------
class GridType(enum.IntEnum):
    Linear = 0
    ModLinear = 1


class BoundingBox1D:
    def __init__(self, leftBoundary: float = 0.0, rightBoundary: float = 1.0):
        self.leftBoundary = float(leftBoundary)
        self.rightBoundary = float(rightBoundary)


class BoundingBox:
    """base/src/sgpp/base/grid/common/BoundingBox.hpp — per-dimension [left, right]."""

    def __init__(self, dim: int):
        self._b = [BoundingBox1D() for _ in range(dim)]

    def setBoundary(self, d: int, bb: BoundingBox1D) -> None:
        self._b[d] = BoundingBox1D(bb.leftBoundary, bb.rightBoundary)

    def getBoundary(self, d: int) -> BoundingBox1D:
        return self._b[d]

    def getDimension(self) -> int:
        return len(self._b)

    def isUnitCube(self) -> bool:
        return all(b.leftBoundary == 0.0 and b.rightBoundary == 1.0 for b in self._b)

    def arrays(self):
        return (np.array([b.leftBoundary for b in self._b]),
                np.array([b.rightBoundary for b in self._b]))


class GridStorage:
    """Hash-grid storage view: raw (level, index) rows in sequence order."""

    def __init__(self, dim: int):
        self.dim = dim
        self.level = np.zeros((0, dim), np.int32)
        self.index = np.zeros((0, dim), np.int32)
        self.boundingBox = BoundingBox(dim)

    def getSize(self) -> int:
        return int(self.level.shape[0])

    def getDimension(self) -> int:
        return self.dim

    def getBoundingBox(self) -> BoundingBox:
        return self.boundingBox

    def setBoundingBox(self, bb: BoundingBox) -> None:
        self.boundingBox = bb

    def getLevelIndexArraysForEval(self, level: Optional[np.ndarray] = None,
                                   index: Optional[np.ndarray] = None):
        """(2^l, i) as [N x d] doubles (HashGridStorage.cpp:433-450)."""
        n = self.getSize()
        lp = np.empty((n, self.dim)) if level is None else level
        ix = np.empty((n, self.dim)) if index is None else index
        if n:
            L = np.ascontiguousarray(self.level)
            I = np.ascontiguousarray(self.index)
            _check(load_library().sggrid_level_index_for_eval(self.dim, n, _vp(L), _vp(I),
                                                               _vp(lp), _vp(ix)))
        return lp, ix


class SurplusRefinementFunctor:
    """base/src/sgpp/base/grid/generation/functors/SurplusRefinementFunctor.cpp:14-44"""

    def __init__(self, alpha, refinements_num: int = 1, threshold: float = 0.0):
        self.alpha = np.ascontiguousarray(alpha, np.float64)
        self.refinements_num = int(refinements_num)
        self.threshold = float(threshold)

    def getRefinementsNum(self) -> int:
        return self.refinements_num

    def getRefinementThreshold(self) -> float:
        return self.threshold


class GridGenerator:
    def __init__(self, grid: "Grid"):
        self.grid = grid

    def regular(self, level: int) -> None:
        """HashGenerator::regular (HashGenerator.hpp:53-58): storage must be empty."""
        st = self.grid.getStorage()
        if st.getSize() > 0:
            raise GenerationException("storage not empty")
        L = load_library()
        n = ctypes.c_int64(0)
        _check(L.sggrid_regular(st.dim, int(level), ctypes.byref(n), None, None),
               GenerationException)
        lev = np.zeros((n.value, st.dim), np.int32)
        idx = np.zeros((n.value, st.dim), np.int32)
        _check(L.sggrid_regular(st.dim, int(level), ctypes.byref(n), _vp(lev), _vp(idx)),
               GenerationException)
        st.level, st.index = lev, idx

    def refine(self, functor: SurplusRefinementFunctor, addedPoints: Optional[list] = None) -> None:
        """HashRefinement::free_refine (HashRefinement.cpp:124-147); new points are appended."""
        st = self.grid.getStorage()
        n = st.getSize()
        if n == 0:
            raise GenerationException("storage empty")
        if functor.alpha.size < n:
            raise GenerationException("alpha shorter than the grid")
        k = functor.getRefinementsNum()
        cap = n + max(k, 0) * 2 * st.dim * (2 + int(st.level.max(initial=1))) * st.dim + 16
        lev = np.zeros((cap, st.dim), np.int32)
        idx = np.zeros((cap, st.dim), np.int32)
        lev[:n] = st.level
        idx[:n] = st.index
        out = ctypes.c_int64(0)
        _check(load_library().sggrid_refine_surplus(st.dim, n, cap, _vp(lev), _vp(idx),
                                                    _vp(functor.alpha), k,
                                                    functor.getRefinementThreshold(),
                                                    ctypes.byref(out)), GenerationException)
        st.level, st.index = lev[:out.value].copy(), idx[:out.value].copy()
        if addedPoints is not None:
            addedPoints.extend(range(n, out.value))


class Grid:
    """A sparse grid without boundary points: Linear (hat basis, Grid::createLinearGrid,
    Grid.cpp:73) or ModLinear (the same points with the modified linear basis,
    Grid::createModLinearGrid; LinearModifiedBasis.hpp:40-58)."""

    def __init__(self, dim: int, gridType: GridType = GridType.Linear):
        self._storage = GridStorage(dim)
        self._generator = GridGenerator(self)
        self._type = GridType(gridType)

    @staticmethod
    def createLinearGrid(dim: int) -> "Grid":
        if dim < 1:
            raise GenerationException("dimension must be >= 1")
        return Grid(int(dim))

    @staticmethod
    def createModLinearGrid(dim: int) -> "Grid":
        if dim < 1:
            raise GenerationException("dimension must be >= 1")
        return Grid(int(dim), GridType.ModLinear)

    @staticmethod
    def regularSize(dim: int, level: int) -> int:
        """Number of points of the regular Linear grid of this dimension and level."""
        n = ctypes.c_int64(0)
        _check(load_library().sggrid_regular(int(dim), int(level), ctypes.byref(n), None, None),
               GenerationException)
        return int(n.value)

    @staticmethod
    def fromArrays(level, index, gridType: GridType = GridType.Linear) -> "Grid":
        """A grid from raw [N x d] level / index rows (e.g. exported from an SG++ storage)."""
        level = np.ascontiguousarray(level, np.int32)
        g = Grid(level.shape[1], gridType)
        g._storage.level = level.copy()
        g._storage.index = np.ascontiguousarray(index, np.int32).copy()
        return g

    def getStorage(self) -> GridStorage:
        return self._storage

    def getGenerator(self) -> GridGenerator:
        return self._generator

    def getBoundingBox(self) -> BoundingBox:
        return self._storage.getBoundingBox()

    def getSize(self) -> int:
        return self._storage.getSize()

    def getDimension(self) -> int:
        return self._storage.getDimension()

    def getType(self) -> GridType:
        return self._type


# ---- operator configuration (DatadrivenOperationCommon.hpp:17-95) ---------------------------
class OperationMultipleEvalType(enum.IntEnum):
    DEFAULT = 0
    STREAMING = 1
    SUBSPACELINEAR = 2
    ADAPTIVE = 3
    MORTONORDER = 4
    SCALAPACK = 5


class OperationMultipleEvalSubType(enum.IntEnum):
    DEFAULT = 0
    SIMPLE = 1
    COMBINED = 2
    OCL = 3
    OCLFASTMP = 4
    OCLMP = 5
    OCLMASKMP = 6
    OCLOPT = 7
    OCLUNIFIED = 8
    CUDA = 9


class OperationMultipleEvalMPIType(enum.IntEnum):
    NONE = 0
    MASTERSLAVE = 1
    HPX = 2


class OperationMultipleEvalConfiguration:
    """Operator selection plus a parameters tree. Parameters understood by the CUDA operator:
    ``precision``: "double" (default, native FP64), "df64" (FP64-accurate float-float on the
    FP32 pipes) or "float"; ``precond``: "none" (default) or "jacobi" for the inner solves of
    mixed-precision fits; ``algo``: "auto" (default), "dense" or "subspace" for the FP32 products
    (subspace = one basis function per subspace and data point)."""

    def __init__(self, type=OperationMultipleEvalType.DEFAULT,
                 subType=OperationMultipleEvalSubType.DEFAULT,
                 mpiType=OperationMultipleEvalMPIType.NONE, parameters: Optional[dict] = None,
                 name: str = "unnamed"):
        self.type = OperationMultipleEvalType(type)
        self.subType = OperationMultipleEvalSubType(subType)
        self.mpiType = OperationMultipleEvalMPIType(mpiType)
        self.parameters = dict(parameters or {})
        self.name = name

    def getType(self):
        return self.type

    def getSubType(self):
        return self.subType

    def getMPIType(self):
        return self.mpiType

    def getParameters(self):
        return self.parameters

    def getName(self):
        return self.name


def _as_matrix(data) -> np.ndarray:
    a = np.ascontiguousarray(data, np.float64)
    if a.ndim == 1:
        a = a.reshape(-1, 1)
    if a.ndim != 2:
        raise OperationException("dataset must be a [rows x dim] matrix")
    return a


def _precision_of(params: dict) -> int:
    p = str(params.get("precision", "double")).lower()
    if p in ("double", "fp64", "f64"):
        return SGMEV_FP64
    if p in ("float", "fp32", "f32", "single"):
        return SGMEV_FP32
    if p in ("df64", "float-float", "double-float"):
        return SGMEV_DF64
    raise OperationException(f"unknown precision {p!r}")


class OperationMultiEvalCuda:
    """B / B^T on the GPU for a Linear or ModLinear grid (OperationMultipleEval interface)."""

    def __init__(self, grid: Grid, dataset, precision: int = SGMEV_FP64,
                 params: Optional[dict] = None):
        self.grid = grid
        self.dataset = _as_matrix(dataset)
        self.precision = precision
        st = grid.getStorage()
        if self.dataset.shape[1] != st.getDimension() and self.dataset.shape[0] > 0:
            raise OperationException("dataset dimension does not match the grid")
        L = load_library()
        lp, ix = st.getLevelIndexArraysForEval()
        bb = st.getBoundingBox()
        left = right = None
        if not bb.isUnitCube():
            left, right = bb.arrays()
        h = ctypes.c_void_p(None)
        knobs = {k: str(v) for k, v in (params or {}).items() if k in OP_KNOBS}
        if grid.getType() == GridType.ModLinear:
            knobs["basis"] = "modlinear"
        pj = json.dumps(knobs).encode() if knobs else None
        _check(L.sgmev_create(ctypes.byref(h), st.getDimension(), st.getSize(), _vp(lp), _vp(ix),
                              self.dataset.shape[0], _vp(self.dataset), _vp(left), _vp(right),
                              precision, pj))
        self._h = h
        self._n = st.getSize()
        self._m = self.dataset.shape[0]

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            load_library().sgmev_destroy(self._h)
            self._h = ctypes.c_void_p(None)

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def _vec(self, v, n: int, what: str) -> np.ndarray:
        a = np.ascontiguousarray(v, np.float64)
        if a.ndim != 1 or a.size < n:
            raise OperationException(f"{what} has size {a.size}, expected {n}")
        return a

    @staticmethod
    def _out(v, n: int, what: str) -> np.ndarray:
        if not isinstance(v, np.ndarray) or v.dtype != np.float64 or not v.flags.c_contiguous:
            raise OperationException(f"{what} must be a contiguous float64 numpy array")
        if v.ndim != 1 or v.size < n:
            raise OperationException(f"{what} has size {v.size}, expected {n}")
        return v

    def mult(self, alpha, result, startIndexData: Optional[int] = None,
             endIndexData: Optional[int] = None) -> None:
        a = self._vec(alpha, self._n, "alpha")
        r = self._out(result, self._m, "result")
        L = load_library()
        if startIndexData is None:
            _check(L.sgmev_mult(self._h, _vp(a), _vp(r)))
        else:
            _check(L.sgmev_mult_range(self._h, _vp(a), _vp(r), int(startIndexData),
                                      int(endIndexData)))

    def eval(self, alpha, result) -> None:
        self.mult(alpha, result)

    def multTranspose(self, source, result, startIndexGrid: Optional[int] = None,
                      endIndexGrid: Optional[int] = None) -> None:
        s = self._vec(source, self._m, "source")
        r = self._out(result, self._n, "result")
        L = load_library()
        if startIndexGrid is None:
            _check(L.sgmev_mult_transpose(self._h, _vp(s), _vp(r)))
        else:
            _check(L.sgmev_mult_transpose_range(self._h, _vp(s), _vp(r), int(startIndexGrid),
                                                int(endIndexGrid)))

    def prepare(self) -> None:
        """Re-stage the (refined) grid (OperationMultipleEval::prepare)."""
        st = self.grid.getStorage()
        lp, ix = st.getLevelIndexArraysForEval()
        _check(load_library().sgmev_prepare(self._h, st.getSize(), _vp(lp), _vp(ix)))
        self._n = st.getSize()

    def getDuration(self) -> float:
        return float(load_library().sgmev_get_duration(self._h))

    def getImplementationName(self) -> str:
        return {SGMEV_FP64: "CUDA_LINEAR_FP64", SGMEV_FP32: "CUDA_LINEAR_FP32",
                SGMEV_DF64: "CUDA_LINEAR_DF64"}[self.precision]

    def kernelLaunches(self) -> int:
        return int(load_library().sgmev_kernel_launches(self._h))

    def setStream(self, stream_ptr: int) -> None:
        """Run this op's work on an external cudaStream_t (0 restores the op's own stream)."""
        _check(load_library().sgmev_set_stream(self._h, ctypes.c_void_p(int(stream_ptr) or None)))

    def synchronize(self) -> None:
        _check(load_library().sgmev_synchronize(self._h))

    def profile(self, enable: bool = True) -> None:
        """Reset and enable (or disable) per-kernel event timing of the tile kernels."""
        _check(load_library().sgmev_profile(self._h, 1 if enable else 0))

    def profileRead(self, kind: int):
        """(launches, seconds) of one tile-kernel kind since the last profile() call."""
        n = ctypes.c_int64(0)
        t = ctypes.c_double(0.0)
        _check(load_library().sgmev_profile_read(self._h, int(kind), ctypes.byref(n),
                                                 ctypes.byref(t)))
        return int(n.value), float(t.value)

    def fitDevice(self, d_y: int, d_alpha: int, lam: float, imax: int, epsilon: float,
                  reuse: bool = False, mode: int = SGMEV_SOLVE_PLAIN):
        """fit() on device pointers (y [n_data], alpha [n_grid] float64); (iterations, residual)."""
        it = ctypes.c_int64(0)
        res = ctypes.c_double(0.0)
        _check(load_library().sgmev_fit_device(self._h, int(mode), ctypes.c_void_p(d_y),
                                               float(lam), int(imax), float(epsilon),
                                               1 if reuse else 0, ctypes.c_void_p(d_alpha),
                                               ctypes.byref(it), ctypes.byref(res)))
        return int(it.value), float(res.value)

    def multDevice(self, d_alpha: int, d_result: int) -> None:
        """mult on device pointers (float64, n_grid / n_data), enqueued on the op's stream."""
        _check(load_library().sgmev_mult_device(self._h, ctypes.c_void_p(d_alpha),
                                                ctypes.c_void_p(d_result)))

    def multTransposeDevice(self, d_source: int, d_result: int) -> None:
        _check(load_library().sgmev_mult_transpose_device(self._h, ctypes.c_void_p(d_source),
                                                          ctypes.c_void_p(d_result)))

    def systemApplyDevice(self, d_alpha: int, d_result: int, lambda_times_m: float) -> None:
        _check(load_library().sgmev_system_apply_device(self._h, ctypes.c_void_p(d_alpha),
                                                        ctypes.c_void_p(d_result),
                                                        float(lambda_times_m)))

    def systemApply(self, alpha, result, lambda_times_m: float) -> None:
        a = self._vec(alpha, self._n, "alpha")
        r = self._out(result, self._n, "result")
        _check(load_library().sgmev_system_apply(self._h, _vp(a), _vp(r), float(lambda_times_m)))

    def fit(self, y, lam: float, imax: int, epsilon: float, alpha=None, mode: int = SGMEV_SOLVE_PLAIN):
        """Device-resident regression fit; returns (alpha, iterations, residual)."""
        yv = self._vec(y, self._m, "y")
        alpha_out = (np.zeros(self._n) if alpha is None
                     else np.array(alpha, np.float64, copy=True))
        it = ctypes.c_int64(0)
        res = ctypes.c_double(0.0)
        _check(load_library().sgmev_fit(self._h, int(mode), _vp(yv), float(lam), int(imax),
                                        float(epsilon), 0 if alpha is None else 1,
                                        _vp(alpha_out), ctypes.byref(it), ctypes.byref(res)))
        return alpha_out, int(it.value), float(res.value)

    def setParams(self, params: dict) -> None:
        """Change launch-shape knobs (multt_batch, block_*) of this live operator."""
        pj = json.dumps({k: str(v) for k, v in params.items()}).encode()
        _check(load_library().sgmev_set_params(self._h, pj))

    # ---- 16 right-hand sides on the tensor cores (no counterpart in the reference) -----------
    def _block(self, a, rows: int, name: str):
        a = np.ascontiguousarray(a, np.float64)
        if a.shape != (SGMEV_BLOCK_RHS, rows):
            raise OperationException(f"{name} must be [{SGMEV_BLOCK_RHS} x {rows}] (one row per vector)")
        return a

    def multBlock(self, alpha):
        """[16 x n_data] = the mult of each of the 16 rows of alpha [16 x n_grid] (tensor cores:
        products rounded to FP16, vectors to about 2^-22, FP32 accumulation; with params
        "block_products": "bf16" products rounded to BF16, vectors to about 2^-16)."""
        a = self._block(alpha, self._n, "alpha")
        out = np.zeros((SGMEV_BLOCK_RHS, self._m))
        _check(load_library().sgmev_mult_block(self._h, _vp(a), _vp(out)))
        return out

    def multTransposeBlock(self, source):
        """[16 x n_grid] = the multTranspose of each of the 16 rows of source [16 x n_data]."""
        v = self._block(source, self._m, "source")
        out = np.zeros((SGMEV_BLOCK_RHS, self._n))
        _check(load_library().sgmev_mult_transpose_block(self._h, _vp(v), _vp(out)))
        return out

    def fitBlock(self, y, lam: float, imax: int, epsilon: float):
        """16 regression fits sharing this operator: y [16 x n_data] -> (alpha [16 x n_grid],
        inner CG steps per column, final ||b - A alpha||^2 per column)."""
        yv = self._block(y, self._m, "y")
        alpha = np.zeros((SGMEV_BLOCK_RHS, self._n))
        its = np.zeros(SGMEV_BLOCK_RHS, np.int64)
        res = np.zeros(SGMEV_BLOCK_RHS)
        _check(load_library().sgmev_fit_block(self._h, _vp(yv), float(lam), int(imax),
                                              float(epsilon), _vp(alpha), _vp(its), _vp(res)))
        return alpha, its, res

    def fitBlockDevice(self, d_y: int, d_alpha: int, lam: float, imax: int, epsilon: float):
        """fitBlock on device pointers (column-major float64 [16][n_data] and [16][n_grid])."""
        its = np.zeros(SGMEV_BLOCK_RHS, np.int64)
        res = np.zeros(SGMEV_BLOCK_RHS)
        _check(load_library().sgmev_fit_block_device(self._h, ctypes.c_void_p(d_y), float(lam),
                                                     int(imax), float(epsilon),
                                                     ctypes.c_void_p(d_alpha), _vp(its),
                                                     _vp(res)))
        return its, res


class BatchEngine:
    """Many independent regression fits advanced together on the GPU (sgmev_batch_*).

    Every problem is a (grid, data X [M x d], Y [M x rhs], lambda) fit; add() stages it and
    computes b = B^T Y, step()/solve() advance all unfinished problems (continuous batching:
    problems may be added while others run), result() returns alpha [N x rhs]."""

    PHASE_EMPTY, PHASE_OUTER, PHASE_INNER, PHASE_DONE = 0, 1, 2, 3

    def __init__(self, max_slots: int, rhs: int = 1, grid_capacity: int = 1 << 24,
                 data_capacity: int = 1 << 26):
        L = load_library()
        h = ctypes.c_void_p(None)
        _check(L.sgmev_batch_create(ctypes.byref(h), int(max_slots), int(rhs), int(grid_capacity),
                                    int(data_capacity), None))
        self._h = h
        self.max_slots = int(max_slots)
        self.rhs = int(rhs)
        self.sizes = {}

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            load_library().sgmev_batch_destroy(self._h)
            self._h = ctypes.c_void_p(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def footprint(dim: int, n_grid: int, n_data: int, rhs: int = 1):
        g = ctypes.c_int64(0)
        d = ctypes.c_int64(0)
        _check(load_library().sgmev_batch_footprint(int(dim), int(n_grid), int(n_data), int(rhs),
                                                    ctypes.byref(g), ctypes.byref(d)))
        return int(g.value), int(d.value)

    def add(self, grid: Grid, X, Y, lam: float, epsilon: float = 1e-8,
            max_iterations: int = 100000) -> int:
        if grid.getType() != GridType.Linear:
            raise FactoryException("the batch engine serves Linear grids")
        st = grid.getStorage()
        lp, ix = st.getLevelIndexArraysForEval()
        X = _as_matrix(X)
        Y = np.ascontiguousarray(np.asarray(Y, np.float64).reshape(X.shape[0], self.rhs))
        slot = ctypes.c_int(-1)
        _check(load_library().sgmev_batch_add(self._h, st.getDimension(), st.getSize(), _vp(lp),
                                              _vp(ix), X.shape[0], _vp(X), _vp(Y), float(lam),
                                              float(epsilon), int(max_iterations),
                                              ctypes.byref(slot)))
        self.sizes[slot.value] = st.getSize()
        return int(slot.value)

    def tryAdd(self, grid: Grid, X, Y, lam: float, epsilon: float = 1e-8,
               max_iterations: int = 100000):
        """add() that returns None instead of raising when no slot or pool space is free."""
        try:
            return self.add(grid, X, Y, lam, epsilon, max_iterations)
        except OperationException as e:
            if f"error {SGMEV_ERR_OOM}" in str(e):
                return None
            raise

    def remove(self, slot: int) -> None:
        _check(load_library().sgmev_batch_remove(self._h, int(slot)))
        self.sizes.pop(slot, None)

    def step(self, steps: int = 1) -> np.ndarray:
        ph = np.zeros(self.max_slots, np.int32)
        _check(load_library().sgmev_batch_step(self._h, int(steps), _vp(ph)))
        return ph

    def solve(self, max_steps: int = 1000000) -> int:
        n = ctypes.c_int64(0)
        _check(load_library().sgmev_batch_solve(self._h, int(max_steps), ctypes.byref(n)))
        return int(n.value)

    def result(self, slot: int):
        n = self.sizes[slot]
        a = np.zeros((n, self.rhs))
        it = ctypes.c_int64(0)
        res = ctypes.c_double(0.0)
        ph = ctypes.c_int(0)
        _check(load_library().sgmev_batch_result(self._h, int(slot), _vp(a), ctypes.byref(it),
                                                 ctypes.byref(res), ctypes.byref(ph)))
        return a, int(it.value), float(res.value), int(ph.value)

    def info(self):
        s = ctypes.c_int64(0)
        l = ctypes.c_int64(0)
        f = ctypes.c_int(0)
        _check(load_library().sgmev_batch_info(self._h, ctypes.byref(s), ctypes.byref(l),
                                               ctypes.byref(f)))
        return {"steps": int(s.value), "launches": int(l.value), "free_slots": int(f.value)}


def createOperationMultipleEval(grid: Grid, dataset,
                                configuration: Optional[OperationMultipleEvalConfiguration] = None):
    """op_factory::createOperationMultipleEval with the new CUDA branch for Linear and ModLinear
    grids (DatadrivenOpFactory.cpp:439-452 and :479-483).

    (Linear or ModLinear, STREAMING, CUDA) and, when no configuration is given, the default route
    give the GPU operator; every other combination raises FactoryException, as the reference does
    for combinations it was not built with (DatadrivenOpFactory.cpp:551)."""
    if configuration is None:
        configuration = OperationMultipleEvalConfiguration(
            OperationMultipleEvalType.STREAMING, OperationMultipleEvalSubType.CUDA)
    if grid.getType() not in (GridType.Linear, GridType.ModLinear):
        raise FactoryException("OperationMultipleEval is not implemented for this grid type.")
    if (configuration.getType() == OperationMultipleEvalType.STREAMING
            and configuration.getSubType() == OperationMultipleEvalSubType.CUDA
            and configuration.getMPIType() == OperationMultipleEvalMPIType.NONE):
        return OperationMultiEvalCuda(grid, dataset, _precision_of(configuration.getParameters()),
                                      configuration.getParameters())
    raise FactoryException("OperationMultipleEval is not implemented for this combination of "
                           "type, subtype and MPI type (the CUDA subtype: STREAMING, no MPI).")


# ---- least-squares system and CG (the callers that drive the operator unchanged) -----------
class SystemMatrixLeastSquaresIdentity:
    """(B^T B + lambda*M*I) alpha, b = B^T y  (SystemMatrixLeastSquaresIdentity.cpp:18-65)."""

    def __init__(self, grid: Grid, trainData, lambdaRegression: float):
        self.grid = grid
        self.dataset = _as_matrix(trainData)
        self.lambda_ = float(lambdaRegression)
        self.instances = self.dataset.shape[0]
        self.implementationConfiguration = OperationMultipleEvalConfiguration(
            OperationMultipleEvalType.STREAMING, OperationMultipleEvalSubType.CUDA)
        self.B = createOperationMultipleEval(grid, self.dataset, self.implementationConfiguration)
        self.completeTimeMult = 0.0
        self.computeTimeMult = 0.0
        self.completeTimeMultTrans = 0.0
        self.computeTimeMultTrans = 0.0

    def mult(self, alpha, result) -> None:
        temp = np.zeros(self.instances)
        self.B.mult(alpha, temp)
        self.computeTimeMult += self.B.getDuration()
        self.B.multTranspose(temp, result)
        self.computeTimeMultTrans += self.B.getDuration()
        result += float(self.instances) * self.lambda_ * np.asarray(alpha, np.float64)

    def generateb(self, classes, b) -> None:
        self.B.multTranspose(np.array(classes, np.float64, copy=True), b)
        self.computeTimeMultTrans += self.B.getDuration()

    def prepareGrid(self) -> None:
        self.B.prepare()

    def setImplementation(self, operationConfiguration: OperationMultipleEvalConfiguration) -> None:
        self.implementationConfiguration = operationConfiguration
        if hasattr(self.B, "close"):
            self.B.close()
        self.B = createOperationMultipleEval(self.grid, self.dataset, operationConfiguration)

    def getLambda(self) -> float:
        return self.lambda_


class ConjugateGradients:
    """FP64 CG on the host driving any OperationMatrix-like `mult` (ConjugateGradients.cpp:22-151)."""

    def __init__(self, imax: int, epsilon: float):
        self.nMaxIterations = int(imax)
        self.myEpsilon = float(epsilon)
        self.nIterations = 0
        self.residuum = 0.0

    def solve(self, SystemMatrix, alpha: np.ndarray, b, reuse: bool = False,
              verbose: bool = False, max_threshold: float = 0.0) -> None:
        eps2 = self.myEpsilon * self.myEpsilon
        self.nIterations = 0
        n = alpha.size
        temp = np.zeros(n)
        q = np.zeros(n)
        r = np.array(b, np.float64, copy=True)
        delta_0 = 0.0
        if reuse:
            q[:] = 0.0
            SystemMatrix.mult(q, temp)
            r -= temp
            delta_0 = float(r @ r) * eps2
        else:
            alpha[:] = 0.0
        SystemMatrix.mult(alpha, temp)
        r -= temp
        d = r.copy()
        delta_new = float(r @ r)
        if not reuse:
            delta_0 = delta_new * eps2
        self.residuum = delta_0 / eps2 if eps2 > 0 else delta_new
        while (self.nIterations < self.nMaxIterations and delta_new > delta_0
               and delta_new > max_threshold):
            SystemMatrix.mult(d, q)
            dq = float(d @ q)
            if dq == 0.0:
                break
            a = delta_new / dq
            alpha += a * d
            if self.nIterations % 50 == 0 and self.nIterations > 0:
                SystemMatrix.mult(alpha, temp)
                r[:] = np.asarray(b, np.float64) - temp
            else:
                r -= a * q
            delta_old = delta_new
            delta_new = float(r @ r)
            beta = delta_new / delta_old
            self.residuum = delta_new
            if verbose:
                print(f"delta: {delta_new}")
            d *= beta
            d += r
            self.nIterations += 1
        self.residuum = delta_new

    def getNumberIterations(self) -> int:
        return self.nIterations

    def getResiduum(self) -> float:
        return self.residuum


__all__ = [
    "Grid", "GridStorage", "GridGenerator", "GridType", "BoundingBox", "BoundingBox1D",
    "SurplusRefinementFunctor", "OperationMultipleEvalType", "OperationMultipleEvalSubType",
    "OperationMultipleEvalMPIType", "OperationMultipleEvalConfiguration",
    "createOperationMultipleEval", "OperationMultiEvalCuda", "SystemMatrixLeastSquaresIdentity",
    "ConjugateGradients", "BatchEngine", "OperationException", "FactoryException", "NotImplementedException",
    "GenerationException", "load_library", "device_count", "EXPORTED_SYMBOLS", "SGMEV_FP64",
    "SGMEV_FP32", "SGMEV_DF64", "SGMEV_SOLVE_PLAIN", "SGMEV_SOLVE_MIXED",
    "SGMEV_SOLVE_MIXED_NATIVE64", "Dataset", "ARFFTools", "CSVTools", "FileException",
    "SGDATA_ARFF", "SGDATA_CSV",
]


# ---- datasets (datadriven/src/sgpp/datadriven/tools/{Dataset,ARFFTools,CSVTools}.cpp) ------
SGDATA_ARFF, SGDATA_CSV = 0, 1


class Dataset:
    """Data matrix [instances x dimension] and targets (datadriven/.../tools/Dataset.hpp)."""

    def __init__(self, data=None, targets=None):
        self._data = np.zeros((0, 0)) if data is None else np.ascontiguousarray(data, np.float64)
        n = self._data.shape[0]
        self._targets = (np.zeros(n) if targets is None
                         else np.ascontiguousarray(targets, np.float64))

    def getData(self) -> np.ndarray:
        return self._data

    def getTargets(self) -> np.ndarray:
        return self._targets

    def getNumberInstances(self) -> int:
        return int(self._data.shape[0])

    def getDimension(self) -> int:
        return int(self._data.shape[1]) if self._data.ndim == 2 else 0


def _text_bytes(content) -> bytes:
    return content.encode() if isinstance(content, str) else bytes(content)


def _file_bytes(filename: str) -> bytes:
    """A dataset file's bytes (gzip-compressed files, *.gz, are expanded)."""
    import gzip
    try:
        if filename.endswith(".gz"):
            with gzip.open(filename, "rb") as f:
                return f.read()
        with open(filename, "rb") as f:
            return f.read()
    except OSError as e:
        raise FileException(f"Unable to open file: {filename} ({e})") from e


def _data_size(fmt, text: bytes, has_targets, skip_first, targets):
    t = np.ascontiguousarray(targets if targets is not None else [], np.float64)
    n = ctypes.c_int64(0)
    d = ctypes.c_int64(0)
    _check(load_library().sgdata_size(fmt, text, len(text), int(bool(has_targets)),
                                      int(bool(skip_first)), _vp(t) if t.size else None,
                                      int(t.size), ctypes.byref(n), ctypes.byref(d)),
           FileException)
    return int(n.value), int(d.value)


def _data_read(fmt, text: bytes, has_targets, skip_first, cutoff, cols, targets) -> Dataset:
    n, dim = _data_size(fmt, text, has_targets, skip_first, targets)
    c = np.ascontiguousarray(cols if cols else [], np.int64)
    t = np.ascontiguousarray(targets if targets is not None else [], np.float64)
    ncap = n if cutoff is None or cutoff < 0 else min(n, int(cutoff))
    width = c.size if c.size else dim
    data = np.zeros((max(ncap, 1), max(width, 1)))
    y = np.zeros(max(ncap, 1))
    nr = ctypes.c_int64(0)
    dout = ctypes.c_int64(0)
    _check(load_library().sgdata_read(fmt, text, len(text), int(bool(has_targets)),
                                      int(bool(skip_first)),
                                      -1 if cutoff is None or cutoff < 0 else int(cutoff),
                                      _vp(c) if c.size else None, int(c.size),
                                      _vp(t) if t.size else None, int(t.size), _vp(data), _vp(y),
                                      int(ncap), ctypes.byref(nr), ctypes.byref(dout)),
           FileException)
    rows = int(nr.value)
    return Dataset(data[:rows, :int(dout.value)].copy(),
                   y[:rows].copy() if has_targets else np.zeros(rows))


class ARFFTools:
    """ARFF reading as datadriven/.../tools/ARFFTools.cpp (sgdata_* in the library)."""

    @staticmethod
    def readARFFSizeFromString(content, hasTargets: bool = True, selectedTargets=None):
        return _data_size(SGDATA_ARFF, _text_bytes(content), hasTargets, False, selectedTargets)

    @staticmethod
    def readARFFSizeFromFile(filename: str, hasTargets: bool = True, selectedTargets=None):
        return _data_size(SGDATA_ARFF, _file_bytes(filename), hasTargets, False, selectedTargets)

    @staticmethod
    def readARFFFromString(content, hasTargets: bool = True, instanceCutoff: int = -1,
                           selectedCols=None, selectedTargets=None) -> Dataset:
        return _data_read(SGDATA_ARFF, _text_bytes(content), hasTargets, False, instanceCutoff,
                          selectedCols, selectedTargets)

    @staticmethod
    def readARFFFromFile(filename: str, hasTargets: bool = True, instanceCutoff: int = -1,
                         selectedCols=None, selectedTargets=None) -> Dataset:
        return _data_read(SGDATA_ARFF, _file_bytes(filename), hasTargets, False, instanceCutoff,
                          selectedCols, selectedTargets)


class CSVTools:
    """CSV reading as datadriven/.../tools/CSVTools.cpp (sgdata_* in the library)."""

    @staticmethod
    def readCSVSizeFromString(content, skipFirstLine: bool = False, hasTargets: bool = True,
                              selectedTargets=None):
        return _data_size(SGDATA_CSV, _text_bytes(content), hasTargets, skipFirstLine,
                          selectedTargets)

    @staticmethod
    def readCSVSizeFromFile(filename: str, skipFirstLine: bool = False, hasTargets: bool = True,
                            selectedTargets=None):
        return _data_size(SGDATA_CSV, _file_bytes(filename), hasTargets, skipFirstLine,
                          selectedTargets)

    @staticmethod
    def readCSVFromString(content, skipFirstLine: bool = False, hasTargets: bool = True,
                          instanceCutoff: int = -1, selectedCols=None,
                          selectedTargets=None) -> Dataset:
        return _data_read(SGDATA_CSV, _text_bytes(content), hasTargets, skipFirstLine,
                          instanceCutoff, selectedCols, selectedTargets)

    @staticmethod
    def readCSVFromFile(filename: str, skipFirstLine: bool = False, hasTargets: bool = True,
                        instanceCutoff: int = -1, selectedCols=None,
                        selectedTargets=None) -> Dataset:
        return _data_read(SGDATA_CSV, _file_bytes(filename), hasTargets, skipFirstLine,
                          instanceCutoff, selectedCols, selectedTargets)

"""ORACLE — test infrastructure only.

ctypes bindings for
  * ``liboracle.so``  — the plain-C FP64 restatement of SG++'s multi-evaluation path
    (``oracle/oracle.c``; every function there cites the reference file:line it restates);
  * ``_ref/libsgpp_ref.so`` — the reference's own FP64 code compiled from its sources by
    ``oracle/ref.mk`` (only where the reference sources exist; absent on hosts without them).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import this package, and only as the reference results of the tests or the timed CPU baseline. The product
(``sgpp_gb300``) never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_REF_LIB = os.path.join(_HERE, "_ref", "libsgpp_ref.so")

_c_i64 = ctypes.c_int64
_c_int = ctypes.c_int
_c_dbl = ctypes.c_double
_vp = ctypes.c_void_p


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_vp)


def reference_source() -> str | None:
    """The reference checkout that the build recipe (oracle/ref.mk) and the fixture scripts read:
    $SGPP_REFERENCE_SRC when set, else the build container's checkout; None when the sources are
    not there (a machine without the reference checkout; nothing the GPU tests or the benchmark
    run needs them)."""
    path = os.environ.get("SGPP_REFERENCE_SRC") or "/root/reference"
    return path if os.path.isdir(os.path.join(path, "base", "src")) else None


def build() -> None:
    """Compile liboracle.so (gcc, seconds)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


class Oracle:
    """FP64 restatement of the reference (see oracle/oracle.c for the citations)."""

    def __init__(self, path: str = _LIB):
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        self.lib = L
        L.orc_regular_grid.restype = _c_i64
        L.orc_regular_grid.argtypes = [_c_int, _c_int, _c_i64, _vp, _vp]
        L.orc_regular_grid_size.restype = _c_i64
        L.orc_regular_grid_size.argtypes = [_c_int, _c_int]
        L.orc_refine_surplus.restype = _c_i64
        L.orc_refine_surplus.argtypes = [_c_int, _c_i64, _c_i64, _vp, _vp, _vp, _c_i64, _c_dbl]
        L.orc_level_index_for_eval.restype = None
        L.orc_level_index_for_eval.argtypes = [_c_int, _c_i64, _vp, _vp, _vp, _vp]
        L.orc_bb_to_unit.restype = None
        L.orc_bb_to_unit.argtypes = [_c_int, _c_i64, _vp, _vp, _vp, _vp]
        for name in ("orc_mult_naive", "orc_mult_transpose_naive"):
            f = getattr(L, name)
            f.restype = None
            f.argtypes = [_c_int, _c_i64, _vp, _vp, _c_i64, _vp, _vp, _vp]
        L.orc_stream_prepare.restype = _vp
        L.orc_stream_prepare.argtypes = [_c_int, _c_i64, _vp]
        L.orc_stream_release.restype = None
        L.orc_stream_release.argtypes = [_vp]
        for name in ("orc_stream_mult", "orc_stream_mult_transpose"):
            f = getattr(L, name)
            f.restype = None
            f.argtypes = [_vp, _c_i64, _vp, _vp, _vp, _vp]
        L.orc_cg_fit.restype = _c_int
        L.orc_cg_fit.argtypes = [_vp, _c_i64, _vp, _vp, _vp, _c_dbl, _c_i64, _c_dbl, _c_int,
                                 _vp, ctypes.POINTER(_c_i64), ctypes.POINTER(_c_dbl)]
        L.orc_max_threads.restype = _c_int
        L.orc_set_threads.argtypes = [_c_int]
        L.orc_modlinear_eval.restype = _c_dbl
        L.orc_modlinear_eval.argtypes = [_c_int, _c_int, _c_dbl]
        for name in ("orc_mult_naive_mod", "orc_mult_transpose_naive_mod"):
            f = getattr(L, name)
            f.restype = None
            f.argtypes = [_c_int, _c_i64, _vp, _vp, _c_i64, _vp, _vp, _vp]
        L.orc_mod_mask_arrays.restype = None
        L.orc_mod_mask_arrays.argtypes = [_c_int, _c_i64, _vp, _vp, _vp, _vp, _vp, _vp]
        for name in ("orc_stream_mult_mod", "orc_stream_mult_transpose_mod"):
            f = getattr(L, name)
            f.restype = None
            f.argtypes = [_vp, _c_i64, _vp, _vp, _vp, _vp, _vp, _vp]
        L.orc_cg_fit_mod.restype = _c_int
        L.orc_cg_fit_mod.argtypes = [_vp, _c_i64, _vp, _vp, _vp, _vp, _vp, _c_dbl, _c_i64,
                                     _c_dbl, _c_int, _vp, ctypes.POINTER(_c_i64),
                                     ctypes.POINTER(_c_dbl)]

    # ---- grids -------------------------------------------------------------------------
    def regular_grid(self, dim: int, level: int):
        """(level, index) int32 [N x d] in the reference's regular-grid storage order."""
        n = int(self.lib.orc_regular_grid_size(dim, level))
        lev = np.zeros((max(n, 1), dim), np.int32)
        idx = np.zeros((max(n, 1), dim), np.int32)
        got = int(self.lib.orc_regular_grid(dim, level, n, _ptr(lev), _ptr(idx)))
        assert got == n, (got, n)
        return lev[:n].copy(), idx[:n].copy()

    def refine_surplus(self, lev, idx, alpha, n_points: int, threshold: float = 0.0):
        n, dim = lev.shape
        cap = n + int(n_points) * (2 * dim) * 8 + 1024
        L = np.zeros((cap, dim), np.int32)
        I = np.zeros((cap, dim), np.int32)
        L[:n] = lev
        I[:n] = idx
        a = np.ascontiguousarray(alpha, np.float64)
        got = int(self.lib.orc_refine_surplus(dim, n, cap, _ptr(L), _ptr(I), _ptr(a),
                                              int(n_points), float(threshold)))
        assert got >= n
        return L[:got].copy(), I[:got].copy()

    @staticmethod
    def eval_arrays(lev, idx):
        """(2^l, i) as doubles, the reference's getLevelIndexArraysForEval layout."""
        return (np.left_shift(1, lev.astype(np.int64)).astype(np.float64),
                idx.astype(np.float64))

    def mod_arrays(self, lev, idx):
        """ModLinear streaming layout (level, index, mask, offset), each [N x d] doubles; mask
        holds raw 64-bit sign masks (getLevelIndexMaskArraysForModEval)."""
        lev = np.ascontiguousarray(lev, np.int32)
        idx = np.ascontiguousarray(idx, np.int32)
        n, dim = lev.shape
        out = [np.zeros((n, dim), np.float64) for _ in range(4)]
        self.lib.orc_mod_mask_arrays(dim, n, _ptr(lev), _ptr(idx), *(_ptr(a) for a in out))
        return tuple(out)

    def modlinear_eval(self, l: int, i: int, x: float) -> float:
        return float(self.lib.orc_modlinear_eval(int(l), int(i), float(x)))

    def mult_naive_mod(self, lev, idx, data, alpha):
        lev, idx = (np.ascontiguousarray(a, np.int32) for a in (lev, idx))
        data, alpha = (np.ascontiguousarray(a, np.float64) for a in (data, alpha))
        n, dim = lev.shape
        out = np.zeros(data.shape[0], np.float64)
        self.lib.orc_mult_naive_mod(dim, n, _ptr(lev), _ptr(idx), data.shape[0], _ptr(data),
                                    _ptr(alpha), _ptr(out))
        return out

    def mult_transpose_naive_mod(self, lev, idx, data, source):
        lev, idx = (np.ascontiguousarray(a, np.int32) for a in (lev, idx))
        data, source = (np.ascontiguousarray(a, np.float64) for a in (data, source))
        n, dim = lev.shape
        out = np.zeros(n, np.float64)
        self.lib.orc_mult_transpose_naive_mod(dim, n, _ptr(lev), _ptr(idx), data.shape[0],
                                              _ptr(data), _ptr(source), _ptr(out))
        return out

    def bb_to_unit(self, data, left, right):
        data = np.ascontiguousarray(data, np.float64)
        out = np.empty_like(data)
        m, dim = data.shape
        l = np.ascontiguousarray(left, np.float64)
        r = np.ascontiguousarray(right, np.float64)
        self.lib.orc_bb_to_unit(dim, m, _ptr(l), _ptr(r), _ptr(data), _ptr(out))
        return out

    # ---- evaluation --------------------------------------------------------------------
    def mult_naive(self, lp, ix, data, alpha):
        lp, ix, data, alpha = (np.ascontiguousarray(a, np.float64) for a in (lp, ix, data, alpha))
        n, dim = lp.shape
        m = data.shape[0]
        out = np.zeros(m, np.float64)
        self.lib.orc_mult_naive(dim, n, _ptr(lp), _ptr(ix), m, _ptr(data), _ptr(alpha), _ptr(out))
        return out

    def mult_transpose_naive(self, lp, ix, data, source):
        lp, ix, data, source = (np.ascontiguousarray(a, np.float64)
                                for a in (lp, ix, data, source))
        n, dim = lp.shape
        m = data.shape[0]
        out = np.zeros(n, np.float64)
        self.lib.orc_mult_transpose_naive(dim, n, _ptr(lp), _ptr(ix), m, _ptr(data),
                                          _ptr(source), _ptr(out))
        return out

    def stream(self, data):
        return OracleStream(self, data)

    def set_threads(self, n: int) -> None:
        self.lib.orc_set_threads(int(n))

    def max_threads(self) -> int:
        return int(self.lib.orc_max_threads())


class OracleStream:
    """STREAMING-shaped OpenMP kernels over one prepared (dim-major, padded) data set."""

    def __init__(self, orc: Oracle, data):
        self.orc = orc
        self.data = np.ascontiguousarray(data, np.float64)
        self.m, self.dim = self.data.shape
        self.h = orc.lib.orc_stream_prepare(self.dim, self.m, _ptr(self.data))

    def close(self):
        if self.h:
            self.orc.lib.orc_stream_release(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def mult(self, lp, ix, alpha):
        lp, ix, alpha = (np.ascontiguousarray(a, np.float64) for a in (lp, ix, alpha))
        out = np.zeros(self.m, np.float64)
        self.orc.lib.orc_stream_mult(self.h, lp.shape[0], _ptr(lp), _ptr(ix), _ptr(alpha),
                                     _ptr(out))
        return out

    def mult_transpose(self, lp, ix, source):
        lp, ix, source = (np.ascontiguousarray(a, np.float64) for a in (lp, ix, source))
        out = np.zeros(lp.shape[0], np.float64)
        self.orc.lib.orc_stream_mult_transpose(self.h, lp.shape[0], _ptr(lp), _ptr(ix),
                                               _ptr(source), _ptr(out))
        return out

    def cg_fit(self, lp, ix, y, lam, imax, eps, alpha0=None):
        lp, ix = (np.ascontiguousarray(a, np.float64) for a in (lp, ix))
        y = np.ascontiguousarray(y, np.float64)
        n = lp.shape[0]
        alpha = (np.zeros(n) if alpha0 is None else np.array(alpha0, np.float64, copy=True))
        it = _c_i64(0)
        res = _c_dbl(0.0)
        self.orc.lib.orc_cg_fit(self.h, n, _ptr(lp), _ptr(ix), _ptr(y), float(lam), int(imax),
                                float(eps), 0 if alpha0 is None else 1, _ptr(alpha),
                                ctypes.byref(it), ctypes.byref(res))
        return alpha, int(it.value), float(res.value)

    # ---- ModLinear (arrays from Oracle.mod_arrays) ---------------------------------------
    def mult_mod(self, arrays, alpha):
        arrays = [np.ascontiguousarray(a, np.float64) for a in arrays]
        alpha = np.ascontiguousarray(alpha, np.float64)
        out = np.zeros(self.m, np.float64)
        self.orc.lib.orc_stream_mult_mod(self.h, arrays[0].shape[0], *(_ptr(a) for a in arrays),
                                         _ptr(alpha), _ptr(out))
        return out

    def mult_transpose_mod(self, arrays, source):
        arrays = [np.ascontiguousarray(a, np.float64) for a in arrays]
        source = np.ascontiguousarray(source, np.float64)
        out = np.zeros(arrays[0].shape[0], np.float64)
        self.orc.lib.orc_stream_mult_transpose_mod(self.h, arrays[0].shape[0],
                                                   *(_ptr(a) for a in arrays), _ptr(source),
                                                   _ptr(out))
        return out

    def cg_fit_mod(self, arrays, y, lam, imax, eps, alpha0=None):
        arrays = [np.ascontiguousarray(a, np.float64) for a in arrays]
        y = np.ascontiguousarray(y, np.float64)
        n = arrays[0].shape[0]
        alpha = (np.zeros(n) if alpha0 is None else np.array(alpha0, np.float64, copy=True))
        it = _c_i64(0)
        res = _c_dbl(0.0)
        self.orc.lib.orc_cg_fit_mod(self.h, n, *(_ptr(a) for a in arrays), _ptr(y), float(lam),
                                    int(imax), float(eps), 0 if alpha0 is None else 1,
                                    _ptr(alpha), ctypes.byref(it), ctypes.byref(res))
        return alpha, int(it.value), float(res.value)


REF_DEFAULT, REF_STREAMING, REF_NAIVE = 0, 1, 2


def reference_available() -> bool:
    return os.path.exists(_REF_LIB)


class Reference:
    """The reference's own compiled FP64 code (oracle/_ref), where it could be built."""

    def __init__(self, path: str = _REF_LIB):
        L = ctypes.CDLL(path)
        self.lib = L
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_grid_create_linear.restype = _vp
        L.ref_grid_create_linear.argtypes = [_c_int]
        L.ref_grid_create_modlinear.restype = _vp
        L.ref_grid_create_modlinear.argtypes = [_c_int]
        L.ref_grid_mask_arrays.argtypes = [_vp, _vp, _vp, _vp, _vp]
        L.ref_grid_destroy.argtypes = [_vp]
        L.ref_grid_regular.argtypes = [_vp, _c_int]
        L.ref_grid_size.restype = _c_i64
        L.ref_grid_size.argtypes = [_vp]
        L.ref_grid_dim.argtypes = [_vp]
        L.ref_grid_level_index.argtypes = [_vp, _vp, _vp]
        L.ref_grid_points.argtypes = [_vp, _vp, _vp, _vp]
        L.ref_grid_set_bounding_box.argtypes = [_vp, _vp, _vp]
        L.ref_grid_refine_surplus.argtypes = [_vp, _vp, _c_i64, _c_i64, _c_dbl]
        L.ref_grid_serialize.argtypes = [_vp, ctypes.c_char_p, _c_i64, ctypes.POINTER(_c_i64)]
        for name in ("ref_mult", "ref_mult_transpose"):
            f = getattr(L, name)
            f.argtypes = [_vp, _c_int, _vp, _c_i64, _vp, _vp, ctypes.POINTER(_c_dbl)]
        L.ref_streaming_time.argtypes = [_vp, _vp, _c_i64, _vp, _vp, _c_int, _vp, _vp]
        L.ref_cg_fit.argtypes = [_vp, _c_int, _vp, _c_i64, _vp, _c_dbl, _c_i64, _c_dbl, _c_int,
                                 _vp, ctypes.POINTER(_c_i64), ctypes.POINTER(_c_dbl)]
        L.ref_max_threads.restype = _c_int
        L.ref_set_threads.argtypes = [_c_int]
        L.ref_fit_adapt.argtypes = [_c_int, _c_int, _c_int, _vp, _c_i64, _vp, _c_dbl, _c_dbl,
                                    _c_i64, _c_dbl, _c_i64, _c_i64, _c_i64, _c_dbl, _c_i64, _vp,
                                    _vp, _vp, ctypes.POINTER(_c_i64), _vp]
        L.ref_read_dataset.argtypes = [_c_int, ctypes.c_char_p, _c_i64, _c_int, _c_int, _c_i64,
                                       _vp, _c_int, _vp, _c_int, _vp, _vp, _c_i64, _c_i64,
                                       ctypes.POINTER(_c_i64), ctypes.POINTER(_c_i64)]

    def fit_adapt(self, basis: int, x, y, level: int, lam: float, final_eps: float,
                  final_maxit: int, refine_eps: float, refine_maxit: int, rounds: int,
                  points: int, threshold: float = 0.0, cap: int = 100000):
        """ModelFittingLeastSquares::fit + adapt() rounds through the reference's classes:
        (level [n x d], index [n x d], alpha [n], CG iterations per solve)."""
        x = np.ascontiguousarray(x, np.float64)
        y = np.ascontiguousarray(y, np.float64)
        m, d = x.shape
        lev = np.zeros((cap, d), np.int32)
        idx = np.zeros((cap, d), np.int32)
        alpha = np.zeros(cap)
        n = _c_i64(0)
        iters = np.zeros(rounds + 1, np.int64)
        self._check(self.lib.ref_fit_adapt(basis, d, level, _ptr(x), m, _ptr(y), float(lam),
                                           float(final_eps), int(final_maxit), float(refine_eps),
                                           int(refine_maxit), int(rounds), int(points),
                                           float(threshold), cap, _ptr(lev), _ptr(idx),
                                           _ptr(alpha), ctypes.byref(n), _ptr(iters)))
        k = int(n.value)
        return lev[:k].copy(), idx[:k].copy(), alpha[:k].copy(), iters

    def read_dataset(self, fmt: int, text: bytes, has_targets=True, skip_first=False, cutoff=-1,
                     cols=None, targets=None, n_cap=1 << 16, dim_cap=64):
        """The reference's ARFFTools::readARFF (fmt 0) / CSVTools::readCSV (fmt 1) on `text`:
        (data, y) or raises RuntimeError with the reference's message."""
        c = np.ascontiguousarray(cols or [], np.int64)
        t = np.ascontiguousarray(targets or [], np.float64)
        data = np.zeros((n_cap, dim_cap))
        y = np.zeros(n_cap)
        n = _c_i64(0)
        d = _c_i64(0)
        self._check(self.lib.ref_read_dataset(fmt, text, len(text), int(has_targets),
                                              int(skip_first), int(cutoff),
                                              _ptr(c) if c.size else None, int(c.size),
                                              _ptr(t) if t.size else None, int(t.size),
                                              _ptr(data), _ptr(y), n_cap, dim_cap,
                                              ctypes.byref(n), ctypes.byref(d)))
        nn, dd = int(n.value), int(d.value)
        assert nn <= n_cap and dd <= dim_cap
        return data[:nn, :dd].copy(), y[:nn].copy()

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(self.lib.ref_last_error().decode(errors="replace"))

    def grid(self, dim: int, level: int | None = None, basis: str = "linear"):
        return RefGrid(self, dim, level, basis)

    def set_threads(self, n: int) -> None:
        self.lib.ref_set_threads(int(n))

    def max_threads(self) -> int:
        return int(self.lib.ref_max_threads())


class RefGrid:
    def __init__(self, ref: Reference, dim: int, level: int | None, basis: str = "linear"):
        self.ref = ref
        self.dim = dim
        self.basis = basis
        if basis == "linear":
            self.h = ref.lib.ref_grid_create_linear(dim)
        elif basis == "modlinear":
            self.h = ref.lib.ref_grid_create_modlinear(dim)
        else:
            raise ValueError(f"unknown basis {basis!r}")
        if level is not None:
            ref._check(ref.lib.ref_grid_regular(self.h, level))

    def __del__(self):
        try:
            if self.h:
                self.ref.lib.ref_grid_destroy(self.h)
        except Exception:
            pass

    @property
    def size(self) -> int:
        return int(self.ref.lib.ref_grid_size(self.h))

    def points(self):
        n = self.size
        lev = np.zeros((n, self.dim), np.int32)
        idx = np.zeros((n, self.dim), np.int32)
        leaf = np.zeros(n, np.int32)
        self.ref._check(self.ref.lib.ref_grid_points(self.h, _ptr(lev), _ptr(idx), _ptr(leaf)))
        return lev, idx, leaf

    def eval_arrays(self):
        n = self.size
        lp = np.zeros((n, self.dim))
        ix = np.zeros((n, self.dim))
        self.ref._check(self.ref.lib.ref_grid_level_index(self.h, _ptr(lp), _ptr(ix)))
        return lp, ix

    def mask_arrays(self):
        n = self.size
        out = [np.zeros((n, self.dim)) for _ in range(4)]
        self.ref._check(self.ref.lib.ref_grid_mask_arrays(self.h, *(_ptr(a) for a in out)))
        return tuple(out)

    def set_bounding_box(self, left, right):
        l = np.ascontiguousarray(left, np.float64)
        r = np.ascontiguousarray(right, np.float64)
        self.ref._check(self.ref.lib.ref_grid_set_bounding_box(self.h, _ptr(l), _ptr(r)))

    def refine_surplus(self, alpha, n_points: int, threshold: float = 0.0):
        a = np.ascontiguousarray(alpha, np.float64)
        self.ref._check(self.ref.lib.ref_grid_refine_surplus(self.h, _ptr(a), a.size,
                                                             int(n_points), float(threshold)))

    def serialize(self) -> str:
        need = _c_i64(0)
        self.ref._check(self.ref.lib.ref_grid_serialize(self.h, None, 0, ctypes.byref(need)))
        buf = ctypes.create_string_buffer(int(need.value))
        self.ref._check(self.ref.lib.ref_grid_serialize(self.h, buf, need.value,
                                                        ctypes.byref(need)))
        return buf.value.decode()

    def mult(self, kind: int, data, alpha):
        data = np.ascontiguousarray(data, np.float64)
        alpha = np.ascontiguousarray(alpha, np.float64)
        out = np.zeros(data.shape[0])
        sec = _c_dbl(0)
        self.ref._check(self.ref.lib.ref_mult(self.h, kind, _ptr(data), data.shape[0],
                                              _ptr(alpha), _ptr(out), ctypes.byref(sec)))
        return out

    def mult_transpose(self, kind: int, data, source):
        data = np.ascontiguousarray(data, np.float64)
        source = np.ascontiguousarray(source, np.float64)
        out = np.zeros(self.size)
        sec = _c_dbl(0)
        self.ref._check(self.ref.lib.ref_mult_transpose(self.h, kind, _ptr(data), data.shape[0],
                                                        _ptr(source), _ptr(out),
                                                        ctypes.byref(sec)))
        return out

    def streaming_time(self, data, alpha, source, reps: int):
        data = np.ascontiguousarray(data, np.float64)
        alpha = np.ascontiguousarray(alpha, np.float64)
        source = np.ascontiguousarray(source, np.float64)
        tm = np.zeros(reps)
        tt = np.zeros(reps)
        self.ref._check(self.ref.lib.ref_streaming_time(self.h, _ptr(data), data.shape[0],
                                                        _ptr(alpha), _ptr(source), reps,
                                                        _ptr(tm), _ptr(tt)))
        return tm, tt

    def cg_fit(self, kind: int, data, y, lam, imax, eps, alpha0=None):
        data = np.ascontiguousarray(data, np.float64)
        y = np.ascontiguousarray(y, np.float64)
        alpha = np.zeros(self.size) if alpha0 is None else np.array(alpha0, np.float64, copy=True)
        it = _c_i64(0)
        res = _c_dbl(0)
        self.ref._check(self.ref.lib.ref_cg_fit(self.h, kind, _ptr(data), data.shape[0], _ptr(y),
                                                float(lam), int(imax), float(eps),
                                                0 if alpha0 is None else 1, _ptr(alpha),
                                                ctypes.byref(it), ctypes.byref(res)))
        return alpha, int(it.value), float(res.value)

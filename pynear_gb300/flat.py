"""Exact flat indexes (GPU exhaustive scan) behind PyNear's index API.

Two families share one engine (gn_flat_* in libgpunear.so):

* ``FlatL2Index`` / ``FlatL1Index`` / ``FlatChebyshevIndex`` /
  ``FlatHammingIndex`` return results nearest-first, ties to the lower row
  index.
* ``VPTreeL2Index`` / ``VPTreeL1Index`` / ``VPTreeChebyshevIndex`` /
  ``VPTreeBinaryIndex`` are drop-ins for the reference classes of the same
  names (pynear/src/PythonBindings.cpp:344-408, pynear/__init__.py:56-104): same
  methods, same argument checks, and results farthest-first as the reference's
  fillSearchResult produces them (pynear/include/VPTree.hpp:621-631).

Distances are the reference's values bit for bit: Euclidean (sqrt) for L2,
float32 L1 / L-inf, int64 Hamming counts.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _as_float2d(a, what: str) -> np.ndarray:
    arr = np.ascontiguousarray(np.asarray(a), dtype=np.float32)
    if arr.ndim != 2:
        raise RuntimeError(f"{what}() expects a 2D float32 array of shape (n, d)")
    return arr


class _FlatBase:
    _metric = _lib.METRIC_L2
    _binary = False

    def __init__(self) -> None:
        self._h = _lib.Handle("gn_flat_create", self._metric)
        self._n = 0
        self._dim = 0
        self._host = None  # host copy kept for pickling

    # ── data in ────────────────────────────────────────────────────────────
    def _prep(self, a, what: str) -> np.ndarray:
        if self._binary:
            arr = np.ascontiguousarray(a)
            if arr.ndim != 2:
                raise ValueError("invalid data shape: binary indexes must be 2D")
            if arr.dtype != np.uint8:
                raise TypeError("invalid data type: binary indexes must be uint8")
            return arr
        return _as_float2d(a, what)

    def set(self, vectors) -> None:
        arr = self._prep(vectors, "set")
        n, d = arr.shape
        _lib.call("gn_flat_set", self._h.h, _lib.ptr(arr), n, d if n else 0)
        self._n, self._dim = n, (d if n else 0)
        self._host = arr.copy() if n else None

    def _queries(self, queries, what: str) -> np.ndarray:
        q = self._prep(queries, what)
        if self._n and q.shape[0] and q.shape[1] != self._dim:
            raise ValueError(
                f"invalid data dimension: index built data and query data dimensions must agree, index built data "
                f"dimension is {self._dim}")
        return q

    # ── raw arrays (nearest-first) ────────────────────────────────────────
    def search_knn_arrays(self, queries, k: int):
        """(nq, min(k, n)) int64 indices and distances, nearest-first."""
        q = self._queries(queries, "searchKNN")
        k = int(k)
        if k <= 0:
            raise ValueError("k must be positive")
        nq = q.shape[0]
        idx = np.empty((nq, k), np.int64)
        dist = np.empty((nq, k), np.int64 if self._binary else np.float32)
        if nq or self._n == 0:  # an empty index raises even for zero queries
            _lib.call("gn_flat_search_knn", self._h.h, _lib.ptr(q), nq, k, _lib.ptr(idx), _lib.ptr(dist))
        kk = min(k, self._n)
        return idx[:, :kk], dist[:, :kk]

    def search_1nn_arrays(self, queries):
        idx, dist = self.search_knn_arrays(queries, 1)
        return idx[:, 0], dist[:, 0]

    # ── pickling: the host copy of the rows is the whole state ─────────────
    def __getstate__(self):
        return {"data": self._host}

    def __setstate__(self, state):
        self.__init__()
        if state.get("data") is not None:
            self.set(state["data"])

    def to_string(self) -> str:
        kind = type(self).__name__
        return (f"####################\n# [{kind} state]\nNum Data Points: {self._n}\nDimension: {self._dim}\n"
                f"Engine: GPU exhaustive scan\n####################\n")


class _NearestFirst(_FlatBase):
    def searchKNN(self, queries, k: int):
        idx, dist = self.search_knn_arrays(queries, k)
        return idx.tolist(), dist.tolist()

    def search1NN(self, queries):
        idx, dist = self.search_1nn_arrays(queries)
        return idx.tolist(), dist.tolist()


class FlatL2Index(_NearestFirst):
    """Exact Euclidean k-NN; nearest-first."""
    _metric = _lib.METRIC_L2


class FlatL1Index(_NearestFirst):
    """Exact Manhattan k-NN; nearest-first."""
    _metric = _lib.METRIC_L1


class FlatChebyshevIndex(_NearestFirst):
    """Exact Chebyshev (L-inf) k-NN; nearest-first."""
    _metric = _lib.METRIC_LINF


class FlatHammingIndex(_NearestFirst):
    """Exact Hamming k-NN over uint8 rows of any width; nearest-first."""
    _metric = _lib.METRIC_HAMMING
    _binary = True


class FlatL2TCIndex:
    """Exact Euclidean k-NN for large batches: tensor-core shortlist of
    `shortlist` rows per query (tcgen05 GEMM, FP32 accumulation), re-ranked with
    the reference's FP32 L2 distance.  Results are nearest-first and equal the
    exact scan whenever the true k nearest rows are in the shortlist; k <= 32.

    ``precision``: "bf16" (default) or "fp8" (E4M3 operands with one FP32 scale
    per row; shortlist 16, 32, 40, 48 or 56 -- FP8 scores are coarser, so
    a longer shortlist keeps the same recall).
    """

    _PRECISIONS = {"bf16": 0, "fp8": 1}

    def __init__(self, shortlist: int = 40, precision: str = "bf16") -> None:
        if precision not in self._PRECISIONS:
            raise ValueError("precision must be 'bf16' or 'fp8'")
        self._h = _lib.Handle("gn_tcflat_create", int(shortlist))
        self._n = 0
        self._dim = 0
        self._host = None
        self.shortlist = int(shortlist)
        self.precision = precision
        if precision != "bf16":
            _lib.call("gn_tcflat_set_precision", self._h.h, self._PRECISIONS[precision])

    def set(self, vectors) -> None:
        arr = _as_float2d(vectors, "set")
        _lib.call("gn_tcflat_set", self._h.h, _lib.ptr(arr), arr.shape[0], arr.shape[1])
        self._n, self._dim = arr.shape
        self._host = arr.copy()

    # ── pickling: the configuration and the host copy of the rows ──────────
    def __getstate__(self):
        return {"shortlist": self.shortlist, "precision": self.precision, "data": self._host}

    def __setstate__(self, state):
        self.__init__(state["shortlist"], state["precision"])
        if state.get("data") is not None:
            self.set(state["data"])

    def search_knn_arrays(self, queries, k: int):
        q = _as_float2d(queries, "searchKNN")
        if self._n and q.shape[1] != self._dim:
            raise ValueError("invalid data dimension: index and query dimensions must agree")
        k = int(k)
        nq = q.shape[0]
        idx = np.empty((nq, k), np.int64)
        dist = np.empty((nq, k), np.float32)
        if nq or self._n == 0:
            _lib.call("gn_tcflat_search_knn", self._h.h, _lib.ptr(q), nq, k, _lib.ptr(idx), _lib.ptr(dist))
        return idx, dist

    def searchKNN(self, queries, k: int):
        idx, dist = self.search_knn_arrays(queries, k)
        return idx.tolist(), dist.tolist()

    def search1NN(self, queries):
        idx, dist = self.search_knn_arrays(queries, 1)
        return idx[:, 0].tolist(), dist[:, 0].tolist()


class _VPTreeCompat(_FlatBase):
    """Reference-compatible surface: searchKNN returns farthest-first."""

    def searchKNN(self, vectors, k: int):
        idx, dist = self.search_knn_arrays(vectors, k)
        return idx[:, ::-1].tolist(), dist[:, ::-1].tolist()

    def search1NN(self, vectors):
        idx, dist = self.search_1nn_arrays(vectors)
        return idx.tolist(), dist.tolist()


class VPTreeL2Index(_VPTreeCompat):
    """Drop-in for pynear.VPTreeL2Index (exact; GPU scan instead of a VP-tree)."""
    _metric = _lib.METRIC_L2


class VPTreeL1Index(_VPTreeCompat):
    """Drop-in for pynear.VPTreeL1Index."""
    _metric = _lib.METRIC_L1


class VPTreeChebyshevIndex(_VPTreeCompat):
    """Drop-in for pynear.VPTreeChebyshevIndex."""
    _metric = _lib.METRIC_LINF


class VPTreeBinaryIndex:
    """Drop-in for pynear.VPTreeBinaryIndex (pynear/__init__.py:56-104).

    Mirrors the reference wrapper: validation raises ValueError / TypeError,
    a search before set() returns ([], []), and k-NN results are
    farthest-first.
    """

    def __init__(self) -> None:
        self._index = None
        self._dimension = None

    def set(self, data: np.ndarray) -> None:
        self._validate(data)
        self._index = _VPTreeBinaryEngine()
        self._dimension = data.shape[1]
        self._index.set(data)

    def searchKNN(self, queries: np.ndarray, k: int):
        dim = queries.shape[1]
        if dim != self._dimension:
            raise ValueError(
                f"invalid data dimension: index built data and query data dimensions must agree, index built data "
                f"dimension is {dim}")
        if self._index is None:
            return [], []
        self._validate(queries)
        return self._index.searchKNN(queries, k)

    def search1NN(self, queries: np.ndarray):
        if self._index is None:
            return [], []
        self._validate(queries)
        return self._index.search1NN(queries)

    def _validate(self, data: np.ndarray) -> None:
        if len(data.shape) != 2:
            raise ValueError("invalid data shape: binary indexes must be 2D")
        if data.dtype != "uint8":
            raise TypeError("invalid data type: binary indexes must be uint8")

    def __getstate__(self):
        return {"dim": self._dimension, "index": self._index}

    def __setstate__(self, st):
        self._dimension = st["dim"]
        self._index = st["index"]


class _VPTreeBinaryEngine(_VPTreeCompat):
    _metric = _lib.METRIC_HAMMING
    _binary = True


# ── single-pair distances (pynear/__init__.py:40-53, PythonBindings.cpp:283-303) ─
def _pair(metric, binary, a, b):
    """One pair's distance on the GPU (gn_dist: one small kernel per call)."""
    dt = np.uint8 if binary else np.float32
    a = np.ascontiguousarray(a, dtype=dt).reshape(-1)
    b = np.ascontiguousarray(b, dtype=dt).reshape(-1)
    if a.size != b.size:
        raise ValueError("invalid data dimension: a and b dimensions must agree.")
    out = ctypes.c_double()
    rc = _lib.load().gn_dist(metric, a.ctypes.data, b.ctypes.data, a.size, ctypes.byref(out))
    if rc:
        _lib.check(rc, "gn_dist")
    return out.value


def dist_l2(a, b) -> float:
    return _pair(_lib.METRIC_L2, False, a, b)


def dist_l1(a, b) -> float:
    return _pair(_lib.METRIC_L1, False, a, b)


def dist_chebyshev(a, b) -> float:
    return _pair(_lib.METRIC_LINF, False, a, b)


def dist_hamming(a, b) -> int:
    if len(a) != len(b):
        raise ValueError("invalid data dimension: a and b dimensions must agree.")
    return int(_pair(_lib.METRIC_HAMMING, True, a, b))

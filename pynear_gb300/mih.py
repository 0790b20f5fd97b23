"""``MIHBinaryIndex``: multi-index hashing for binary descriptors.

Drop-in for the reference binding (pynear/src/PythonBindings.cpp:468-481,
pynear/include/MIH.hpp:58-175): constructor ``(m=8)``, ``set(vectors)``,
``searchKNN(vectors, k, radius=8)`` returning ``(indices, distances)`` lists
of lists nearest-first (int Hamming distances, possibly fewer than k per
query), ``m()``, ``n()``, ``nbytes()``.  The hash-table lookup runs on the host,
the candidates' verification (exact Hamming + top-k) on the GPU; ties go to
the lower row index.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _u8_2d(a, what: str) -> np.ndarray:
    arr = np.ascontiguousarray(a)
    if arr.ndim != 2:
        raise ValueError(f"invalid data shape: {what} must be 2D")
    if arr.dtype != np.uint8:
        raise TypeError(f"invalid data type: {what} must be uint8")
    return arr


class MIHBinaryIndex:
    def __init__(self, m: int = 8):
        self._m = int(m)
        self._h = _lib.Handle("gn_mih_create", self._m)
        self._data = None

    def set(self, vectors) -> None:
        arr = _u8_2d(vectors, "vectors")
        n = arr.shape[0]
        _lib.call("gn_mih_set", self._h.h, _lib.ptr(arr) if n else None, n, arr.shape[1] if n else 0)
        self._data = arr.copy() if n else None

    def search_knn_arrays(self, vectors, k: int, radius: int = 8):
        """(indices (nq,k) int64, distances (nq,k) int64, counts (nq,) int64), nearest-first."""
        q = _u8_2d(vectors, "vectors")
        k = int(k)
        nq = q.shape[0]
        if self._data is not None and nq and q.shape[1] != self._data.shape[1]:
            raise ValueError("invalid data dimension: query width must equal the indexed width")
        idx = np.empty((nq, k), np.int64)
        dist = np.empty((nq, k), np.int64)
        cnt = np.zeros(nq, np.int64)
        if nq:
            _lib.call("gn_mih_search_knn", self._h.h, _lib.ptr(q), nq, k, int(radius), _lib.ptr(idx), _lib.ptr(dist),
                      _lib.ptr(cnt))
        return idx, dist, cnt

    def searchKNN(self, vectors, k: int, radius: int = 8):
        idx, dist, cnt = self.search_knn_arrays(vectors, k, radius)
        return ([idx[i, :cnt[i]].tolist() for i in range(len(cnt))],
                [dist[i, :cnt[i]].tolist() for i in range(len(cnt))])

    def m(self) -> int:
        return self._m

    def n(self) -> int:
        return 0 if self._data is None else int(self._data.shape[0])

    def nbytes(self) -> int:
        return 0 if self._data is None else int(self._data.shape[1])

    def __getstate__(self):
        return {"m": self._m, "data": self._data}

    def __setstate__(self, st):
        self.__init__(st["m"])
        if st["data"] is not None:
            self.set(st["data"])

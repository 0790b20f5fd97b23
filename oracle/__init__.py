"""CPU oracle for the search path (test infrastructure only).

Wraps ``oracle.cpp`` (a C++ restatement of the reference's distance, k-NN,
k-means and IVF routines; see the citations there) through ctypes.  Only the
tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use
this package, always as the expected answer or the timed CPU baseline -- never as the
thing measured or shipped.
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile oracle.cpp into oracle/_build/liboracle.so (g++, OpenMP)."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    flags = ["-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags += ["-mfma", "-mpopcnt"]  # hardware fma / popcount; results are identical
    tmp = LIB + ".tmp"
    subprocess.check_call(["g++", *flags, SRC, "-o", tmp])
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        I64 = ctypes.c_int64
        L.or_hamming.restype = I64
        L.or_hamming.argtypes = [P, P, I64]
        L.or_hamming_ref_dispatch.restype = I64
        L.or_hamming_ref_dispatch.argtypes = [P, P, I64]
        for name in ("or_l2", "or_l1", "or_linf"):
            getattr(L, name).restype = ctypes.c_float
            getattr(L, name).argtypes = [P, P, I64]
        L.or_knn_float.argtypes = [ctypes.c_int, P, I64, I64, P, I64, I64, P, P, ctypes.c_int]
        L.or_knn_hamming.argtypes = [P, I64, I64, P, I64, I64, P, P, ctypes.c_int]
        L.or_kmeans_l2.argtypes = [P, I64, I64, I64, I64, ctypes.c_uint32, P, P, P, ctypes.c_int]
        L.or_ivfbin_build.argtypes = [P, I64, I64, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint32, P, P, P, ctypes.c_int]
        L.or_ivfbin_search.argtypes = [P, I64, I64, P, ctypes.c_int32, P, P, I64, I64, ctypes.c_int32, ctypes.c_int,
                                       P, P, P, ctypes.c_int]
        L.or_ivfl2_search.argtypes = [P, I64, I64, P, ctypes.c_int32, P, P, I64, I64, ctypes.c_int32, P, P, P, ctypes.c_int]
        L.or_knn_l2sq_f64.argtypes = [P, I64, I64, P, I64, I64, P, P, ctypes.c_int]
        L.or_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


METRICS = {"l2": 0, "l1": 1, "linf": 2, "chebyshev": 2}


def num_threads() -> int:
    return lib().or_num_threads()


def dist(metric: str, a, b) -> float:
    a = np.ascontiguousarray(a, dtype=np.float32).ravel()
    b = np.ascontiguousarray(b, dtype=np.float32).ravel()
    fn = {"l2": lib().or_l2, "l1": lib().or_l1, "linf": lib().or_linf, "chebyshev": lib().or_linf}[metric]
    return float(np.float32(fn(_p(a), _p(b), a.size)))


def hamming(a, b, ref_dispatch: bool = False) -> int:
    a = np.ascontiguousarray(a, dtype=np.uint8).ravel()
    b = np.ascontiguousarray(b, dtype=np.uint8).ravel()
    fn = lib().or_hamming_ref_dispatch if ref_dispatch else lib().or_hamming
    return int(fn(_p(a), _p(b), a.size))


def knn_float(metric: str, db, q, k: int, threads: int = 0):
    db = np.ascontiguousarray(db, dtype=np.float32)
    q = np.ascontiguousarray(q, dtype=np.float32)
    nq = q.shape[0]
    idx = np.empty((nq, k), np.int64)
    dist_ = np.empty((nq, k), np.float32)
    rc = lib().or_knn_float(METRICS[metric], _p(db), db.shape[0], db.shape[1], _p(q), nq, k, _p(idx), _p(dist_), threads)
    if rc:
        raise RuntimeError("oracle knn_float failed")
    return idx, dist_


def knn_hamming(db, q, k: int, threads: int = 0):
    db = np.ascontiguousarray(db, dtype=np.uint8)
    q = np.ascontiguousarray(q, dtype=np.uint8)
    nq = q.shape[0]
    idx = np.empty((nq, k), np.int64)
    dist_ = np.empty((nq, k), np.int64)
    rc = lib().or_knn_hamming(_p(db), db.shape[0], db.shape[1], _p(q), nq, k, _p(idx), _p(dist_), threads)
    if rc:
        raise RuntimeError("oracle knn_hamming failed")
    return idx, dist_


def knn_l2sq_f64(db, q, k: int, threads: int = 0):
    db = np.ascontiguousarray(db, dtype=np.float32)
    q = np.ascontiguousarray(q, dtype=np.float32)
    nq = q.shape[0]
    idx = np.empty((nq, k), np.int64)
    dist_ = np.empty((nq, k), np.float64)
    lib().or_knn_l2sq_f64(_p(db), db.shape[0], db.shape[1], _p(q), nq, k, _p(idx), _p(dist_), threads)
    return idx, dist_


def kmeans_l2(data, k: int, max_iter: int = 100, seed: int = 42, threads: int = 0):
    data = np.ascontiguousarray(data, dtype=np.float32)
    n, d = data.shape
    labels = np.empty(n, np.int32)
    cent = np.empty((k, d), np.float32)
    iters = np.zeros(1, np.int64)
    rc = lib().or_kmeans_l2(_p(data), n, d, k, max_iter, seed, _p(labels), _p(cent), _p(iters), threads)
    if rc:
        raise RuntimeError("oracle kmeans_l2: k must be between 1 and N")
    return labels, cent, int(iters[0])


def ivfbin_build(db, nlist: int, max_iter: int = 20, seed: int = 42, threads: int = 0):
    db = np.ascontiguousarray(db, dtype=np.uint8)
    n, nb = db.shape
    kk = min(nlist, n)
    cent = np.empty((kk, nb), np.uint8)
    labels = np.empty(n, np.int32)
    kout = np.zeros(1, np.int32)
    lib().or_ivfbin_build(_p(db), n, nb, nlist, max_iter, seed, _p(cent), _p(labels), _p(kout), threads)
    return cent[: int(kout[0])], labels


def ivfbin_search(db, cent, labels, q, k: int, nprobe: int, tie_mode: int = 1, threads: int = 0):
    db = np.ascontiguousarray(db, dtype=np.uint8)
    cent = np.ascontiguousarray(cent, dtype=np.uint8)
    labels = np.ascontiguousarray(labels, dtype=np.int32)
    q = np.ascontiguousarray(q, dtype=np.uint8)
    nq = q.shape[0]
    idx = np.empty((nq, k), np.int64)
    dist_ = np.empty((nq, k), np.int64)
    cnt = np.empty(nq, np.int64)
    lib().or_ivfbin_search(_p(db), db.shape[0], db.shape[1], _p(cent), cent.shape[0], _p(labels), _p(q), nq, k,
                           nprobe, tie_mode, _p(idx), _p(dist_), _p(cnt), threads)
    return idx, dist_, cnt


def ivfl2_search(db, cent, labels, q, k: int, nprobe: int, threads: int = 0):
    db = np.ascontiguousarray(db, dtype=np.float32)
    cent = np.ascontiguousarray(cent, dtype=np.float32)
    labels = np.ascontiguousarray(labels, dtype=np.int32)
    q = np.ascontiguousarray(q, dtype=np.float32)
    nq = q.shape[0]
    idx = np.empty((nq, k), np.int64)
    dist_ = np.empty((nq, k), np.float32)
    cnt = np.empty(nq, np.int64)
    lib().or_ivfl2_search(_p(db), db.shape[0], db.shape[1], _p(cent), cent.shape[0], _p(labels), _p(q), nq, k,
                          nprobe, _p(idx), _p(dist_), _p(cnt), threads)
    return idx, dist_, cnt


def mih_search(db, q, k: int, m: int, radius: int):
    """Multi-index hashing search restated in NumPy (pynear/include/MIH.hpp:96-152):
    a row is a candidate when one of its m sub-strings (nbytes/m bytes) is within
    radius // m bits of the query's; the k nearest candidates by exact Hamming
    distance, ties to the lower row index.  Returns (idx, dist, cnt) padded with
    -1 / 0.  For small cases (dense n x nq x nbytes work)."""
    db = np.ascontiguousarray(db, dtype=np.uint8)
    q = np.ascontiguousarray(q, dtype=np.uint8)
    n, nbytes = db.shape
    sub = nbytes // m
    r_sub = radius // m
    pc = np.unpackbits(np.arange(256, dtype=np.uint8)[:, None], axis=1).sum(1)
    x = pc[np.bitwise_xor(q[:, None, :], db[None, :, :])]  # (nq, n, nbytes) bit counts
    full = x.sum(-1)
    part = x.reshape(len(q), n, m, sub).sum(-1)  # (nq, n, m)
    cand = (part <= r_sub).any(-1)
    idx = np.full((len(q), k), -1, np.int64)
    dist = np.zeros((len(q), k), np.int64)
    cnt = np.zeros(len(q), np.int64)
    for i in range(len(q)):
        rows = np.nonzero(cand[i])[0]
        order = np.lexsort((rows, full[i, rows]))[:k]
        c = len(order)
        idx[i, :c] = rows[order]
        dist[i, :c] = full[i, rows[order]]
        cnt[i] = c
    return idx, dist, cnt


def voronoi_raster(seeds, xs, ys):
    """Voronoi raster restated in NumPy (demo/voronoi.py:93-110, a search1NN of
    every pixel (xs[c], ys[r]) against the seeds): float32 arithmetic in the
    reference's L2 order for d = 2 (pynear/include/DistanceFunctions.hpp:185-195,
    sqrt(rn(rn(dx*dx) + rn(dy*dy))), dx = pixel - seed), nearest seed with ties
    to the lower index.  Returns (ids int32 (h, w), dist float32 (h, w))."""
    seeds = np.ascontiguousarray(seeds, dtype=np.float32)
    xs = np.asarray(xs, np.float32)
    ys = np.asarray(ys, np.float32)
    ids = np.empty((len(ys), len(xs)), np.int32)
    dist = np.empty((len(ys), len(xs)), np.float32)
    for r, py in enumerate(ys):
        dx = xs[:, None] - seeds[None, :, 0]
        dy = py - seeds[:, 1]
        d = np.sqrt(dx * dx + (dy * dy)[None, :])
        ids[r] = np.argmin(d, axis=1)
        dist[r] = d[np.arange(len(xs)), ids[r]]
    return ids, dist

"""IVF-flat indexes and the k-means coarse quantiser on the GPU.

``IVFFlatL2Index`` mirrors pynear.IVFFlatL2Index (pynear/forest.py:167-194):
constructor ``(n_clusters=100, n_probe=10)``, ``set``, ``searchKNN``,
``search1NN``, properties ``n_clusters`` (clusters actually built, empty ones
dropped) and ``n_probe``; distances are squared L2, nearest-first; a 1-D query
is treated as one row; a query may get fewer than k results.

``IVFFlatBinaryIndex`` mirrors the reference binding
(pynear/src/PythonBindings.cpp:454-466): ``(nlist=256, nprobe=8, max_iter=20,
seed=42)``, ``set``, ``searchKNN``, ``nlist()``, ``nprobe()``,
``set_nprobe()``; Hamming distances as int64, ascending.

``kmeans_l2(data, k, max_iter=100, seed=42)`` mirrors _pynear.kmeans_l2
(pynear/src/PythonBindings.cpp:305-329) and returns (labels int32, centroids
float32).
"""
from __future__ import annotations

import numpy as np

from . import _lib


def _f32_2d(a, what: str) -> np.ndarray:
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if arr.ndim != 2:
        raise ValueError(f"{what} must be a 2-D array of shape (N, D)")
    return arr


def kmeans_l2(data, k: int, max_iter: int = 100, seed: int = 42):
    """Lloyd k-means with k-means++ seeding on the GPU -> (labels, centroids)."""
    arr = np.ascontiguousarray(np.asarray(data), dtype=np.float32)
    if arr.ndim != 2:
        raise RuntimeError("kmeans_l2: data must be a 2D float32 array (N, D)")
    n, d = arr.shape
    if k <= 0 or k > n:
        raise RuntimeError("kmeans_l2: k must be between 1 and N")
    labels = np.empty(n, np.int32)
    cent = np.empty((k, d), np.float32)
    iters = np.zeros(1, np.int64)
    _lib.call("gn_kmeans_l2", _lib.ptr(arr), n, d, int(k), int(max_iter), int(seed) & 0xffffffff,
              _lib.ptr(labels), _lib.ptr(cent), _lib.ptr(iters))
    return labels, cent


def _rows_to_lists(idx: np.ndarray, dist: np.ndarray, cnt: np.ndarray, as_int: bool):
    out_i, out_d = [], []
    for i in range(idx.shape[0]):
        c = int(cnt[i])
        out_i.append(idx[i, :c].tolist())
        out_d.append(dist[i, :c].tolist())
    return out_i, out_d


class IVFFlatL2Index:
    """GPU IVF-flat over squared L2 (drop-in for pynear.IVFFlatL2Index)."""

    def __init__(self, n_clusters: int = 100, n_probe: int = 10, engine: str = "fp32", shortlist: int = 40):
        """engine "fp32": CUDA-core scan with the reference's |q|^2+|x|^2-2q.x
        distances; engine "tc": BF16 tensor-core shortlist of `shortlist`
        candidates per query, re-ranked with exact FP32 squared L2 (k <= 32)."""
        self._n_clusters_req = int(n_clusters)
        self._n_probe = min(int(n_probe), int(n_clusters))
        self._h = _lib.Handle("gn_ivfl2_create", self._n_clusters_req, self._n_probe)
        self._built = False
        self._state = None  # host copy for pickling: (data, centroids, labels)
        self.set_engine(engine, shortlist)

    def set_engine(self, engine: str, shortlist: int = 40) -> None:
        if engine not in ("fp32", "tc"):
            raise ValueError('engine must be "fp32" or "tc"')
        _lib.call("gn_ivfl2_set_mode", self._h.h, 0 if engine == "fp32" else 1, int(shortlist))
        self._engine, self._shortlist = engine, int(shortlist)

    def set(self, data) -> None:
        arr = _f32_2d(data, "data")
        n, d = arr.shape
        _lib.call("gn_ivfl2_set", self._h.h, _lib.ptr(arr), n, d)
        self._built = n > 0
        self._state = None
        self._data = arr

    def set_prober(self, prober, threshold: float = 0.5) -> None:
        """Probe adaptively with a trained LearnedProber (probability threshold),
        or with prober=None go back to the fixed n_probe."""
        from .prober import prob_to_logit
        self._prober = prober  # keeps the model alive while attached
        self._prober_threshold = float(threshold)
        _lib.call("gn_ivfl2_set_prober", self._h.h, None if prober is None else prober._h.h,
                  prob_to_logit(threshold))

    def enable_graphs(self, max_batch: int, k: int) -> None:
        """Replay searches of 1..max_batch queries at this k as captured CUDA
        graphs (one per batch size); max_batch 0 turns it off.  Results are
        those of the uncaptured pipeline."""
        _lib.call("gn_ivfl2_enable_graphs", self._h.h, int(max_batch), int(k))

    def graph_info(self) -> dict:
        out = np.zeros(4, np.int64)
        _lib.call("gn_ivfl2_graph_info", self._h.h, _lib.ptr(out))
        return {"max_batch": int(out[0]), "graphs": int(out[1]), "replays": int(out[2]),
                "capture_failures": int(out[3])}

    def autotune(self, sample_queries, k: int, reps: int = 3) -> np.ndarray:
        """Time the tensor-core engine's launch choices on sample queries for
        every batch-size bucket the sample reaches and keep the fastest; returns
        the (7, 4) table of (rows per work unit, most blocks per query
        selection, selector threads, queries per list-scan work unit) per
        bucket.  Results are unchanged."""
        q = _f32_2d(sample_queries, "sample_queries")
        table = np.zeros((7, 4), np.int32)
        _lib.call("gn_ivfl2_autotune", self._h.h, _lib.ptr(q), q.shape[0], int(k), int(reps), _lib.ptr(table))
        return table

    @property
    def tuning(self) -> np.ndarray:
        table = np.zeros((7, 4), np.int32)
        _lib.call("gn_ivfl2_get_tuning", self._h.h, _lib.ptr(table))
        return table

    @tuning.setter
    def tuning(self, table) -> None:
        t = np.ascontiguousarray(table, dtype=np.int32).reshape(7, -1)
        if t.shape[1] < 4:  # a table saved without the tile column: the built-in tile
            t = np.concatenate([t, np.zeros((7, 4 - t.shape[1]), np.int32)], axis=1)
        t = np.ascontiguousarray(t.reshape(7, 4))
        _lib.call("gn_ivfl2_set_tuning", self._h.h, _lib.ptr(t))

    def last_lists_probed(self, nq: int) -> np.ndarray:
        """Lists probed per query by the last search with a prober."""
        out = np.empty(nq, np.int32)
        _lib.call("gn_ivfl2_last_nprobed", self._h.h, nq, _lib.ptr(out))
        return out

    def set_assigned(self, data, centroids, labels) -> None:
        """Build the lists from given centroids and labels (no k-means)."""
        arr = _f32_2d(data, "data")
        cent = _f32_2d(centroids, "centroids")
        lab = np.ascontiguousarray(labels, dtype=np.int32)
        _lib.call("gn_ivfl2_set_assigned", self._h.h, _lib.ptr(arr), arr.shape[0], arr.shape[1], _lib.ptr(cent),
                  cent.shape[0], _lib.ptr(lab))
        self._built = arr.shape[0] > 0
        self._data = arr

    def fork(self) -> "IVFFlatL2Index":
        """A second search context over this index's lists.  It shares the
        device data (centroids, lists, rows: nothing is copied) and owns its
        scratch, stream and captured graphs, so searches on the index and on
        its forks can run at the same time, each fork on its own stream.
        n_probe, engine, prober and tuning start as this index's and are the
        fork's own afterwards.  While forks are alive the index cannot be
        rebuilt (set / set_assigned raise)."""
        if not self._built:
            raise RuntimeError("Index is empty — call set() first")
        f = IVFFlatL2Index.__new__(IVFFlatL2Index)
        f._n_clusters_req, f._n_probe = self._n_clusters_req, self._n_probe
        f._h = _lib.Handle("gn_ivfl2_fork", self._h.h)
        f._built, f._state, f._data = True, None, self._data
        f._engine, f._shortlist = self._engine, self._shortlist
        f._parent = self  # the lists' owner
        if getattr(self, "_prober", None) is not None:
            f._prober, f._prober_threshold = self._prober, self._prober_threshold
        return f

    def search_knn_device(self, queries, k: int, out_idx, out_dist, out_cnt, stream=None) -> None:
        """Search device-resident queries (a contiguous float32 CUDA tensor
        (nq, d)) into device tensors idx (nq, k) int64, dist (nq, k) float32
        and count (nq,) int64, in the order of `stream` (a torch.cuda.Stream;
        default: the current stream), without synchronising."""
        import torch
        if not self._built:
            raise RuntimeError("Index is empty — call set() first")
        if queries.dtype != torch.float32 or not queries.is_cuda or not queries.is_contiguous() or queries.dim() != 2:
            raise ValueError("queries must be a contiguous 2-D float32 CUDA tensor")
        nq, k = int(queries.shape[0]), int(k)
        for t, dt, shape in ((out_idx, torch.int64, (nq, k)), (out_dist, torch.float32, (nq, k)),
                             (out_cnt, torch.int64, (nq,))):
            if t.dtype != dt or not t.is_cuda or not t.is_contiguous() or tuple(t.shape[:len(shape)]) != shape:
                raise ValueError(f"output tensors must be contiguous CUDA tensors of shape {shape} and {dt}")
        if stream is None:
            stream = torch.cuda.current_stream(queries.device)
        if nq:
            _lib.call("gn_ivfl2_search_knn_device", self._h.h, queries.data_ptr(), nq, k, out_idx.data_ptr(),
                      out_dist.data_ptr(), out_cnt.data_ptr(), stream.cuda_stream)

    def search_knn_arrays(self, queries, k: int):
        """(idx (nq,k) int64, dist (nq,k) float32, count (nq,) int64), nearest-first."""
        q = np.asarray(queries, dtype=np.float32)
        if q.ndim == 1:
            q = q[np.newaxis]
        q = np.ascontiguousarray(q)
        if not self._built:
            raise RuntimeError("Index is empty — call set() first")
        k = int(k)
        nq = q.shape[0]
        idx = np.empty((nq, k), np.int64)
        dist = np.empty((nq, k), np.float32)
        cnt = np.empty(nq, np.int64)
        if nq:
            _lib.call("gn_ivfl2_search_knn", self._h.h, _lib.ptr(q), nq, k, _lib.ptr(idx), _lib.ptr(dist),
                      _lib.ptr(cnt))
        return idx, dist, cnt

    def searchKNN(self, queries, k: int):
        idx, dist, cnt = self.search_knn_arrays(queries, k)
        return _rows_to_lists(idx, dist, cnt, False)

    def search1NN(self, queries):
        return self.searchKNN(queries, 1)

    @property
    def n_clusters(self) -> int:
        if not self._built:
            return 0
        nc = np.zeros(1, np.int32)
        _lib.call("gn_ivfl2_info", self._h.h, _lib.ptr(nc), None, None, None)
        return int(nc[0])

    @property
    def n_probe(self) -> int:
        return self._n_probe

    @n_probe.setter
    def n_probe(self, value: int) -> None:
        self._n_probe = int(value)
        _lib.call("gn_ivfl2_set_n_probe", self._h.h, self._n_probe)

    def export(self):
        """(centroids (C,D), offsets (C+1,), ids in list order (N,)) of the built CSR lists."""
        nc = self.n_clusters
        d = self._data.shape[1]
        cent = np.empty((nc, d), np.float32)
        offs = np.empty(nc + 1, np.int64)
        ids = np.empty(self._data.shape[0], np.int64)
        _lib.call("gn_ivfl2_export", self._h.h, _lib.ptr(cent), _lib.ptr(offs), _lib.ptr(ids))
        return cent, offs, ids

    def __getstate__(self):
        st = {"n_clusters": self._n_clusters_req, "n_probe": self._n_probe, "built": self._built,
              "engine": self._engine, "shortlist": self._shortlist, "tuning": self.tuning}
        if self._built:
            cent, offs, ids = self.export()
            labels = np.empty(self._data.shape[0], np.int32)
            for c in range(len(offs) - 1):
                labels[ids[offs[c]:offs[c + 1]]] = c
            st.update(data=self._data, centroids=cent, labels=labels)
            prober = getattr(self, "_prober", None)
            if prober is not None:  # the attached learned prober: weights and threshold
                st["prober"] = {"params": prober.get_params(), "threshold": self._prober_threshold}
        return st

    def __setstate__(self, st):
        self.__init__(st["n_clusters"], st["n_probe"], st.get("engine", "fp32"), st.get("shortlist", 40))
        if "tuning" in st:
            self.tuning = st["tuning"]
        if st["built"]:
            self.set_assigned(st["data"], st["centroids"], st["labels"])
            if "prober" in st:
                from .prober import LearnedProber
                pr = LearnedProber(self)
                pr.set_params(st["prober"]["params"])
                self.set_prober(pr, st["prober"]["threshold"])


class IVFFlatBinaryIndex:
    """GPU IVF-flat over Hamming distance (drop-in for pynear.IVFFlatBinaryIndex)."""

    def __init__(self, nlist: int = 256, nprobe: int = 8, max_iter: int = 20, seed: int = 42):
        self._args = (int(nlist), int(nprobe), int(max_iter), int(seed) & 0xffffffff)
        self._h = _lib.Handle("gn_ivfbin_create", *self._args)
        self._n = 0
        self._nbytes = 0

    def set(self, vectors) -> None:
        arr = np.ascontiguousarray(vectors)
        if arr.ndim != 2:
            raise ValueError("invalid data shape: binary indexes must be 2D")
        if arr.dtype != np.uint8:
            arr = arr.astype(np.uint8)
        n, nb = arr.shape
        _lib.call("gn_ivfbin_set", self._h.h, _lib.ptr(arr), n, nb)
        self._n, self._nbytes = n, nb
        self._data = arr.copy() if n else None  # host copy for pickling

    def search_knn_arrays(self, queries, k: int):
        q = np.ascontiguousarray(queries)
        if q.ndim != 2:
            raise ValueError("invalid data shape: binary indexes must be 2D")
        if q.dtype != np.uint8:
            q = q.astype(np.uint8)
        k = int(k)
        nq = q.shape[0]
        idx = np.empty((nq, k), np.int64)
        dist = np.empty((nq, k), np.int64)
        cnt = np.zeros(nq, np.int64)
        if nq and self._n:
            _lib.call("gn_ivfbin_search_knn", self._h.h, _lib.ptr(q), nq, k, _lib.ptr(idx), _lib.ptr(dist),
                      _lib.ptr(cnt))
        return idx, dist, cnt

    def searchKNN(self, vectors, k: int):
        idx, dist, cnt = self.search_knn_arrays(vectors, k)
        return _rows_to_lists(idx, dist, cnt, True)

    def nlist(self) -> int:
        return self._args[0]

    def nprobe(self) -> int:
        a = np.zeros(2, np.int32)
        _lib.call("gn_ivfbin_get_params", self._h.h, _lib.ptr(a[:1]), _lib.ptr(a[1:]))
        return int(a[1])

    def set_nprobe(self, nprobe: int) -> None:
        _lib.call("gn_ivfbin_set_nprobe", self._h.h, int(nprobe))

    # Pickling (the reference's binary IVF has none): the rows and parameters;
    # the binary k-means is deterministic, so unpickling rebuilds the same
    # centroids and lists.
    def __getstate__(self):
        return {"args": self._args, "data": getattr(self, "_data", None), "nprobe": self.nprobe()}

    def __setstate__(self, st):
        self.__init__(*st["args"])
        if st["data"] is not None:
            self.set(st["data"])
        self.set_nprobe(st["nprobe"])

    def export(self):
        """(centroids (k, nbytes) uint8, labels (n,) int32) of the built index."""
        kk = min(self._args[0], self._n)
        cent = np.empty((kk, self._nbytes), np.uint8)
        labels = np.empty(self._n, np.int32)
        kout = np.zeros(1, np.int32)
        _lib.call("gn_ivfbin_export", self._h.h, _lib.ptr(cent), _lib.ptr(labels), _lib.ptr(kout))
        return cent[: int(kout[0])], labels

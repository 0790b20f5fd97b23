"""Learned probe selection for IVFFlatL2Index (GPU-trained MLP).

    prober = LearnedProber(index)              # index: a built IVFFlatL2Index
    prober.train(train_queries, exact_ids)     # exact ids: (nq, k) from exact search
    index.set_prober(prober, prob_threshold)   # searches now probe adaptively
    index.set_prober(None)                     # back to fixed n_probe

For each query the network reads the 64 nearest lists and their squared
centroid distances and predicts which of them hold one of the query's exact
k nearest neighbours; the index probes those with probability >= threshold
(and always the nearest list).  Training, inference and the gradient all run in
the library's own CUDA kernels.
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib

CAND, HIDDEN = 64, 256


def prob_to_logit(p: float) -> float:
    p = min(max(float(p), 1e-7), 1 - 1e-7)
    return math.log(p / (1 - p))


class LearnedProber:
    def __init__(self, index, seed: int = 1):
        nl = index.n_clusters
        if nl < CAND:
            raise ValueError("learned probing needs an index with at least 64 lists")
        self.n_lists = nl
        self._h = _lib.Handle("gn_prober_create", nl, int(seed) & 0xffffffff)
        self._index = index

    @property
    def num_params(self) -> int:
        n = np.zeros(1, np.int64)
        _lib.call("gn_prober_num_params", self._h.h, _lib.ptr(n))
        return int(n[0])

    def get_params(self) -> np.ndarray:
        out = np.empty(self.num_params, np.float32)
        _lib.call("gn_prober_get_params", self._h.h, _lib.ptr(out))
        return out

    def set_params(self, params) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != self.num_params:
            raise ValueError("parameter vector has the wrong size")
        _lib.call("gn_prober_set_params", self._h.h, _lib.ptr(p))

    def split(self, params: np.ndarray):
        """Views (W1, b1, W2, b2, W3, b3) of a flat parameter vector."""
        L, H = self.n_lists, HIDDEN
        o = np.cumsum([0, L * H, H, H * H, H, L * H, L])
        return (params[o[0]:o[1]].reshape(L, H), params[o[1]:o[2]], params[o[2]:o[3]].reshape(H, H),
                params[o[3]:o[4]], params[o[4]:o[5]].reshape(L, H), params[o[5]:o[6]])

    def loss_and_grad(self, cand, feat, lab):
        cand = np.ascontiguousarray(cand, dtype=np.int32)
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        lab = np.ascontiguousarray(lab, dtype=np.float32)
        B = cand.shape[0]
        loss = np.zeros(1, np.float32)
        grads = np.empty(self.num_params, np.float32)
        _lib.call("gn_prober_loss_grad", self._h.h, B, _lib.ptr(cand), _lib.ptr(feat), _lib.ptr(lab),
                  _lib.ptr(loss), _lib.ptr(grads))
        return float(loss[0]), grads

    def train(self, queries, exact_ids, epochs: int = 4, batch: int = 1024, lr: float = 1e-3):
        q = np.ascontiguousarray(queries, dtype=np.float32)
        gt = np.ascontiguousarray(exact_ids, dtype=np.int64)
        losses = np.zeros(epochs, np.float32)
        _lib.call("gn_prober_train", self._h.h, self._index._h.h, _lib.ptr(q), q.shape[0], _lib.ptr(gt),
                  gt.shape[1], int(epochs), int(batch), float(lr), _lib.ptr(losses))
        return losses

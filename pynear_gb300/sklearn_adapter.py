"""scikit-learn style estimators over the GPU exact flat indexes.

Same classes, parameters and methods as the reference's adapters
(pynear/sklearn_adapter.py:111-374): ``PyNearNearestNeighbors``
(``fit`` / ``kneighbors`` / ``kneighbors_graph``), ``PyNearKNeighborsClassifier``
(``fit`` / ``predict`` / ``predict_proba`` / ``score``) and
``PyNearKNeighborsRegressor`` (``fit`` / ``predict`` / ``score``), metrics
``euclidean`` / ``l2``, ``manhattan`` / ``l1``, ``chebyshev`` / ``linf`` and
``hamming``, weights ``uniform`` / ``distance``.

The searches run on the GPU flat indexes, which return results nearest-first
as arrays (ties to the lower row index), so no list-of-lists conversion or
re-sort is needed; votes and weighted means are vectorised.  scikit-learn is
optional: when it is installed the estimators derive from its base classes
(``clone``, pipelines, ``get_params``); otherwise small stand-ins give the
same ``get_params`` / ``set_params`` / ``score``.
"""
from __future__ import annotations

import inspect

import numpy as np

from .flat import FlatChebyshevIndex, FlatHammingIndex, FlatL1Index, FlatL2Index

try:  # pragma: no cover - depends on the environment
    from sklearn.base import BaseEstimator, ClassifierMixin, RegressorMixin
except ImportError:  # pragma: no cover
    class BaseEstimator:
        """get_params / set_params from the constructor's keyword arguments."""

        @classmethod
        def _param_names(cls):
            sig = inspect.signature(cls.__init__)
            return [p for p in sig.parameters if p != "self"]

        def get_params(self, deep=True):
            return {p: getattr(self, p) for p in self._param_names()}

        def set_params(self, **params):
            for key, value in params.items():
                if key not in self._param_names():
                    raise ValueError(f"Invalid parameter {key!r} for estimator {type(self).__name__}")
                setattr(self, key, value)
            return self

        def __repr__(self):
            args = ", ".join(f"{k}={v!r}" for k, v in self.get_params().items())
            return f"{type(self).__name__}({args})"

    class ClassifierMixin:
        def score(self, X, y, sample_weight=None):
            return float(np.average(self.predict(X) == np.asarray(y), weights=sample_weight))

    class RegressorMixin:
        def score(self, X, y, sample_weight=None):
            y = np.asarray(y, dtype=np.float64)
            pred = np.asarray(self.predict(X), dtype=np.float64)
            w = np.ones(len(y)) if sample_weight is None else np.asarray(sample_weight, dtype=np.float64)
            w = w.reshape((-1,) + (1,) * (y.ndim - 1))
            num = (w * (y - pred) ** 2).sum(axis=0)
            den = (w * (y - np.average(y, axis=0, weights=w.ravel())) ** 2).sum(axis=0)
            r2 = np.where(den > 0, 1.0 - num / np.where(den > 0, den, 1.0), 0.0)
            return float(np.mean(r2))


_METRICS = {
    "euclidean": FlatL2Index, "l2": FlatL2Index,
    "manhattan": FlatL1Index, "l1": FlatL1Index,
    "chebyshev": FlatChebyshevIndex, "linf": FlatChebyshevIndex,
    "hamming": FlatHammingIndex,
}


def _index_class(metric: str):
    cls = _METRICS.get(str(metric).lower())
    if cls is None:
        raise ValueError(f"Unsupported metric '{metric}'. Supported values: {sorted(_METRICS)}")
    return cls


def _check_X(X, metric: str) -> np.ndarray:
    binary = _index_class(metric) is FlatHammingIndex
    arr = np.asarray(X)
    if arr.ndim != 2:
        raise ValueError(f"Expected a 2D array, got an array of shape {arr.shape}")
    if arr.shape[0] == 0:
        raise ValueError("Found array with 0 sample(s)")
    return np.ascontiguousarray(arr, dtype=np.uint8 if binary else np.float32)


def _check_fitted(est) -> None:
    if not hasattr(est, "_index"):
        try:  # the exception type scikit-learn callers catch
            from sklearn.exceptions import NotFittedError
        except ImportError:  # pragma: no cover
            class NotFittedError(ValueError, AttributeError):
                pass
        raise NotFittedError(f"This {type(est).__name__} instance is not fitted yet. Call 'fit' first.")


def _weights(dist: np.ndarray, weights: str) -> np.ndarray:
    """(nq, k) neighbour weights; 'distance' gives an exact match all the
    weight of its query (the reference's and scikit-learn's convention)."""
    if weights == "uniform":
        return np.ones_like(dist, dtype=np.float64)
    if weights == "distance":
        d = dist.astype(np.float64)
        with np.errstate(divide="ignore"):
            w = 1.0 / d
        zero = d == 0.0
        rows = zero.any(axis=1)
        w[rows] = zero[rows].astype(np.float64)
        return w
    raise ValueError(f"weights must be 'uniform' or 'distance', got '{weights}'")


def _search(index, X, k: int):
    """(distances float64, indices intp), nearest-first."""
    idx, dist = index.search_knn_arrays(X, k)
    return dist.astype(np.float64), idx.astype(np.intp)


class PyNearNearestNeighbors(BaseEstimator):
    """Unsupervised nearest-neighbour lookup (``sklearn.neighbors.NearestNeighbors``)."""

    def __init__(self, n_neighbors: int = 5, metric: str = "euclidean"):
        self.n_neighbors = n_neighbors
        self.metric = metric

    def fit(self, X, y=None):
        X = _check_X(X, self.metric)
        index = _index_class(self.metric)()
        index.set(X)
        self._index, self._fit_X = index, X
        self.n_samples_fit_ = X.shape[0]
        return self

    def kneighbors(self, X=None, n_neighbors=None, return_distance=True):
        """(distances, indices) of shape (n_queries, n_neighbors), nearest first;
        without X, the neighbours of every training point other than itself."""
        _check_fitted(self)
        k = self.n_neighbors if n_neighbors is None else int(n_neighbors)
        exclude_self = X is None
        Xq = self._fit_X if exclude_self else _check_X(X, self.metric)
        dst, ind = _search(self._index, Xq, k + 1 if exclude_self else k)
        if exclude_self:
            # drop each point itself (distance 0); a duplicate of it may rank first
            own = ind == np.arange(len(ind))[:, None]
            keep = ~own
            keep[~own.any(axis=1), -1] = False  # self not found: drop the farthest
            dst = dst[keep].reshape(len(ind), k)
            ind = ind[keep].reshape(len(ind), k)
        return (dst, ind) if return_distance else ind

    def kneighbors_graph(self, X=None, n_neighbors=None, mode="connectivity"):
        """Sparse (n_queries, n_samples_fit) matrix of the k-NN edges."""
        from scipy.sparse import csr_matrix

        k = self.n_neighbors if n_neighbors is None else int(n_neighbors)
        dst, ind = self.kneighbors(X, n_neighbors=k, return_distance=True)
        nq = ind.shape[0]
        rows = np.repeat(np.arange(nq), ind.shape[1])
        if mode == "connectivity":
            data = np.ones(rows.size)
        elif mode == "distance":
            data = dst.ravel()
        else:
            raise ValueError(f"mode must be 'connectivity' or 'distance', got '{mode}'")
        return csr_matrix((data, (rows, ind.ravel())), shape=(nq, self.n_samples_fit_))


class PyNearKNeighborsClassifier(ClassifierMixin, BaseEstimator):
    """k-NN classifier (``sklearn.neighbors.KNeighborsClassifier``)."""

    def __init__(self, n_neighbors: int = 5, metric: str = "euclidean", weights: str = "uniform"):
        self.n_neighbors = n_neighbors
        self.metric = metric
        self.weights = weights

    def fit(self, X, y):
        X = _check_X(X, self.metric)
        y = np.asarray(y)
        if len(y) != X.shape[0]:
            raise ValueError(f"X has {X.shape[0]} samples but y has {len(y)}")
        self.classes_, self._y_code = np.unique(y, return_inverse=True)
        index = _index_class(self.metric)()
        index.set(X)
        self._index = index
        self.n_samples_fit_ = X.shape[0]
        return self

    def predict_proba(self, X):
        """(n_queries, n_classes) class probabilities; columns follow classes_."""
        _check_fitted(self)
        X = _check_X(X, self.metric)
        dst, ind = _search(self._index, X, self.n_neighbors)
        w = _weights(dst, self.weights)
        proba = np.zeros((X.shape[0], len(self.classes_)))
        rows = np.repeat(np.arange(X.shape[0]), ind.shape[1])
        np.add.at(proba, (rows, self._y_code[ind].ravel()), w.ravel())
        sums = proba.sum(axis=1, keepdims=True)
        return proba / np.where(sums == 0, 1.0, sums)

    def predict(self, X):
        return self.classes_[np.argmax(self.predict_proba(X), axis=1)]


class PyNearKNeighborsRegressor(RegressorMixin, BaseEstimator):
    """k-NN regressor (``sklearn.neighbors.KNeighborsRegressor``)."""

    def __init__(self, n_neighbors: int = 5, metric: str = "euclidean", weights: str = "uniform"):
        self.n_neighbors = n_neighbors
        self.metric = metric
        self.weights = weights

    def fit(self, X, y):
        X = _check_X(X, self.metric)
        y = np.asarray(y, dtype=np.float64)
        if len(y) != X.shape[0]:
            raise ValueError(f"X has {X.shape[0]} samples but y has {len(y)}")
        index = _index_class(self.metric)()
        index.set(X)
        self._index, self._y = index, y
        self.n_samples_fit_ = X.shape[0]
        return self

    def predict(self, X):
        """Weighted mean of the neighbours' targets: (n_queries,) or (n_queries, n_outputs)."""
        _check_fitted(self)
        X = _check_X(X, self.metric)
        dst, ind = _search(self._index, X, self.n_neighbors)
        w = _weights(dst, self.weights)
        ny = self._y[ind]  # (nq, k) or (nq, k, n_outputs)
        wsum = w.sum(axis=1)
        if ny.ndim == 2:
            return (w * ny).sum(axis=1) / wsum
        return (w[:, :, None] * ny).sum(axis=1) / wsum[:, None]

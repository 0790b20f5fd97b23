"""scikit-learn style adapters over the GPU flat indexes, checked against
brute force (the cases of the reference's tests/test_sklearn_adapter.py), and
persistence of the indexes that carry extra state."""
import pickle

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _brute(X, Q, k, metric="l2"):
    diff = Q[:, None, :].astype(np.float64) - X[None, :, :]
    if metric == "l2":
        d = np.sqrt((diff ** 2).sum(-1))
    elif metric == "l1":
        d = np.abs(diff).sum(-1)
    else:
        d = np.abs(diff).max(-1)
    ind = np.argsort(d, axis=1, kind="stable")[:, :k]
    return np.take_along_axis(d, ind, 1), ind


@pytest.fixture
def data():
    rng = np.random.default_rng(3)
    X = rng.random((600, 12)).astype(np.float32)
    Q = rng.random((40, 12)).astype(np.float32)
    y = rng.integers(0, 4, 600)
    yr = rng.random(600)
    return X, Q, y, yr


def test_nearest_neighbors_matches_brute_force(gn, data):
    X, Q, _, _ = data
    nn = gn.PyNearNearestNeighbors(n_neighbors=6).fit(X)
    dst, ind = nn.kneighbors(Q)
    bd, bi = _brute(X, Q, 6)
    np.testing.assert_array_equal(ind, bi)
    np.testing.assert_allclose(dst, bd, rtol=1e-5)
    assert isinstance(nn.kneighbors(Q[:10], return_distance=False), np.ndarray)
    assert nn.kneighbors(Q[:5], n_neighbors=3)[1].shape == (5, 3)
    for metric, ref in (("manhattan", "l1"), ("chebyshev", "linf")):
        dst, ind = gn.PyNearNearestNeighbors(n_neighbors=4, metric=metric).fit(X).kneighbors(Q)
        bd, bi = _brute(X, Q, 4, ref)
        np.testing.assert_array_equal(ind, bi)
        np.testing.assert_allclose(dst, bd, rtol=1e-5)


def test_kneighbors_without_query_excludes_self(gn, data):
    X, _, _, _ = data
    nn = gn.PyNearNearestNeighbors(n_neighbors=4).fit(X)
    ind = nn.kneighbors(return_distance=False)
    assert ind.shape == (600, 4)
    assert not (ind == np.arange(600)[:, None]).any()
    G = nn.kneighbors_graph(n_neighbors=3)
    assert G.shape == (600, 600) and G.nnz == 600 * 3
    Gd = nn.kneighbors_graph(X[:10], n_neighbors=3, mode="distance")
    assert Gd.shape == (10, 600) and (Gd.data >= 0).all()


def test_hamming_metric_and_errors(gn):
    rng = np.random.default_rng(5)
    X = rng.integers(0, 256, (300, 16), dtype=np.uint8)
    nn = gn.PyNearNearestNeighbors(n_neighbors=3, metric="hamming").fit(X)
    dst, ind = nn.kneighbors(X[:7])
    np.testing.assert_array_equal(ind[:, 0], np.arange(7))
    assert (dst[:, 0] == 0).all()
    with pytest.raises(ValueError):
        gn.PyNearNearestNeighbors(metric="cosine").fit(X)
    with pytest.raises(Exception):
        gn.PyNearNearestNeighbors().kneighbors(X)


def test_classifier_matches_brute_force_vote(gn, data):
    X, Q, y, _ = data
    for weights in ("uniform", "distance"):
        clf = gn.PyNearKNeighborsClassifier(n_neighbors=5, weights=weights).fit(X, y)
        proba = clf.predict_proba(Q)
        np.testing.assert_allclose(proba.sum(1), 1.0, rtol=1e-6)
        bd, bi = _brute(X, Q, 5)
        w = np.ones_like(bd) if weights == "uniform" else 1.0 / bd
        expect = np.zeros((len(Q), 4))
        for q in range(len(Q)):
            np.add.at(expect[q], y[bi[q]], w[q])
        np.testing.assert_array_equal(clf.predict(Q), clf.classes_[np.argmax(expect, 1)])
    assert set(clf.classes_) == set(np.unique(y))
    assert clf.score(X, y) > 0.3
    with pytest.raises(ValueError):
        gn.PyNearKNeighborsClassifier(weights="bogus").fit(X, y).predict(Q)


def test_regressor_matches_brute_force_mean(gn, data):
    X, Q, _, yr = data
    bd, bi = _brute(X, Q, 5)
    reg = gn.PyNearKNeighborsRegressor(n_neighbors=5).fit(X, yr)
    np.testing.assert_allclose(reg.predict(Q), yr[bi].mean(1), rtol=1e-6)
    reg = gn.PyNearKNeighborsRegressor(n_neighbors=5, weights="distance").fit(X, yr)
    w = 1.0 / bd
    np.testing.assert_allclose(reg.predict(Q), (w * yr[bi]).sum(1) / w.sum(1), rtol=1e-5)
    Y = np.stack([yr, 2 * yr, yr ** 2], 1)
    assert gn.PyNearKNeighborsRegressor(n_neighbors=3).fit(X, Y).predict(Q[:10]).shape == (10, 3)
    assert gn.PyNearKNeighborsRegressor(n_neighbors=3).fit(X, yr).score(X, yr) > 0.0
    params = reg.get_params()
    assert params["weights"] == "distance" and reg.set_params(n_neighbors=2).n_neighbors == 2


def test_binary_ivf_pickle_roundtrip(gn):
    rng = np.random.default_rng(11)
    X = rng.integers(0, 256, (5000, 32), dtype=np.uint8)
    ix = gn.IVFFlatBinaryIndex(nlist=32, nprobe=4)
    ix.set(X)
    ix.set_nprobe(6)
    i0, d0, c0 = ix.search_knn_arrays(X[:50], 5)
    ix2 = pickle.loads(pickle.dumps(ix))
    assert ix2.nprobe() == 6 and ix2.nlist() == 32
    i1, d1, c1 = ix2.search_knn_arrays(X[:50], 5)
    np.testing.assert_array_equal(i0, i1)
    np.testing.assert_array_equal(d0, d1)
    empty = pickle.loads(pickle.dumps(gn.IVFFlatBinaryIndex(nlist=8)))
    assert empty.nlist() == 8


def test_ivf_pickle_keeps_attached_prober(gn):
    rng = np.random.default_rng(12)
    c = rng.standard_normal((200, 32), dtype=np.float32)
    X = (c[rng.integers(0, 200, 20000)] + np.float32(0.3) * rng.standard_normal((20000, 32), dtype=np.float32))
    Q = (c[rng.integers(0, 200, 100)] + np.float32(0.3) * rng.standard_normal((100, 32), dtype=np.float32))
    ix = gn.IVFFlatL2Index(n_clusters=80, n_probe=4, engine="tc")
    ix.set(X)
    pr = gn.LearnedProber(ix, seed=4)
    ix.set_prober(pr, 0.2)
    r0 = ix.search_knn_arrays(Q, 10)
    ix2 = pickle.loads(pickle.dumps(ix))
    r1 = ix2.search_knn_arrays(Q, 10)
    for a, b in zip(r0, r1):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(ix.last_lists_probed(len(Q)), ix2.last_lists_probed(len(Q)))

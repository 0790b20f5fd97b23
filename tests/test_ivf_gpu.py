"""Parity of the GPU k-means and IVF indexes with the reference and the oracle."""
import pickle

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def brute_knn_l2(data, queries, k):
    d = ((queries[:, None, :].astype(np.float64) - data[None, :, :]) ** 2).sum(-1)
    idx = np.argsort(d, axis=1, kind="stable")[:, :k]
    return idx, np.take_along_axis(d, idx, 1)


def recall(approx, exact):
    return float(np.mean([len(set(a) & set(e)) / max(len(e), 1) for a, e in zip(approx, exact)]))


def inertia(data, labels, cent):
    return float(((data.astype(np.float64) - cent[labels].astype(np.float64)) ** 2).sum())


# ── k-means ───────────────────────────────────────────────────────────────
def test_kmeans_matches_reference_fixture(gn):
    g = golden("kmeans.npz")
    for tag in ("a", "b"):
        data, ref_l, ref_c = g[f"{tag}_data"], g[f"{tag}_labels"], g[f"{tag}_cent"]
        labels, cent = gn.kmeans_l2(data, ref_c.shape[0], 100, 42)
        # same k-means++ seeds; the GEMM-form assignment and FP64 sums may
        # differ from the reference only at near ties
        assert np.mean(labels == ref_l) >= 0.99
        np.testing.assert_allclose(cent, ref_c, rtol=1e-4, atol=1e-5)
        assert inertia(data, labels, cent) <= inertia(data, ref_l, ref_c) * (1 + 1e-4)


def test_kmeans_seeds_equal_the_reference_rule(gn, oracle):
    """k-means++ seeding on the device (draws taken up front, weighted pick
    from parallel double running sums, the serial rule near a boundary)
    picks exactly the seeds of the reference's serial loop (KMeans.hpp:45-70),
    restated by the oracle: max_iter 0 returns the seeds."""
    rng = np.random.default_rng(8)
    cases = [(rng.random((1000, 8), dtype=np.float32), 37),
             (rng.standard_normal((300_001, 16)).astype(np.float32), 256),  # chunks longer than 256 rows
             (np.repeat(rng.random((50, 12), dtype=np.float32), 40, axis=0), 60)]  # duplicates: zero weights
    for data, k in cases:
        _, cent = gn.kmeans_l2(data, k, 0, 42)
        _, ocent, _ = oracle.kmeans_l2(data, k, 0, 42)
        assert np.array_equal(cent.view(np.uint32), ocent.view(np.uint32)), (data.shape, k)


def test_kmeans_converged_labels_are_nearest_centroid(gn):
    # well separated mixture: Lloyd converges (no label changes) well within
    # max_iter, so the returned labels name each point's nearest centroid
    rng = np.random.default_rng(21)
    centres = rng.normal(size=(64, 40)).astype(np.float32) * 4
    data = (centres[rng.integers(0, 64, 20000)] + 0.3 * rng.normal(size=(20000, 40))).astype(np.float32)
    labels, cent = gn.kmeans_l2(data, 64, 300, 7)
    d = ((data[:, None, :] - cent[None]) ** 2).sum(-1)
    best = d.min(1)
    assert np.all(d[np.arange(len(data)), labels] <= best + 1e-3 * (1 + best))
    assert len(np.unique(labels)) >= 60


# ── IVFFlatL2Index ────────────────────────────────────────────────────────
def test_ivfl2_reference_fixture_same_lists(gn, oracle):
    g = golden("ivf_l2.npz")
    for tag in ("a", "b"):
        nc, npb, k = (int(x) for x in g[f"{tag}_cfg"])
        ix = gn.IVFFlatL2Index(n_clusters=nc, n_probe=npb)
        ix.set_assigned(g[f"{tag}_db"], g[f"{tag}_cent"], g[f"{tag}_labels"])
        idx, dist, cnt = ix.search_knn_arrays(g[f"{tag}_q"], k)
        oi, od, oc = oracle.ivfl2_search(g[f"{tag}_db"], g[f"{tag}_cent"], g[f"{tag}_labels"], g[f"{tag}_q"], k, npb)
        assert np.array_equal(cnt, oc)
        np.testing.assert_allclose(dist, od, rtol=1e-4, atol=1e-4)
        np.testing.assert_allclose(dist, g[f"{tag}_dist"], rtol=1e-4, atol=1e-4)
        assert np.mean(idx == g[f"{tag}_idx"]) >= 0.99


def test_ivfl2_full_probe_is_exact(gn):
    rng = np.random.default_rng(0)
    data = rng.random((500, 32)).astype(np.float32)
    queries = rng.random((20, 32)).astype(np.float32)
    ix = gn.IVFFlatL2Index(n_clusters=20, n_probe=20)
    ix.set(data)
    approx_idx, _ = ix.searchKNN(queries, 5)
    exact_idx, _ = brute_knn_l2(data, queries, 5)
    assert recall(approx_idx, exact_idx) == pytest.approx(1.0)


def test_ivfl2_high_recall_reasonable_probe(gn):
    rng = np.random.default_rng(1)
    data = rng.random((2000, 8)).astype(np.float32)
    queries = rng.random((50, 8)).astype(np.float32)
    ix = gn.IVFFlatL2Index(n_clusters=20, n_probe=15)
    ix.set(data)
    approx_idx, _ = ix.searchKNN(queries, 10)
    exact_idx, _ = brute_knn_l2(data, queries, 10)
    assert recall(approx_idx, exact_idx) >= 0.90


def test_ivfl2_search1nn_matches_searchknn(gn):
    rng = np.random.default_rng(2)
    data = rng.random((500, 16)).astype(np.float32)
    queries = rng.random((10, 16)).astype(np.float32)
    ix = gn.IVFFlatL2Index(n_clusters=10, n_probe=10)
    ix.set(data)
    assert ix.search1NN(queries) == ix.searchKNN(queries, 1)


def test_ivfl2_single_query_and_small_clusters(gn):
    rng = np.random.default_rng(3)
    data = rng.random((200, 8)).astype(np.float32)
    ix = gn.IVFFlatL2Index(n_clusters=10, n_probe=5)
    ix.set(data)
    idx, dist = ix.searchKNN(rng.random(8).astype(np.float32), 3)
    assert len(idx) == 1 and len(idx[0]) == 3
    data = rng.random((50, 4)).astype(np.float32)
    ix = gn.IVFFlatL2Index(n_clusters=20, n_probe=20)
    ix.set(data)
    idx, _ = ix.searchKNN(rng.random((1, 4)).astype(np.float32), k=10)
    assert len(idx[0]) == 10
    ix = gn.IVFFlatL2Index(n_clusters=100, n_probe=100)
    ix.set(rng.random((10, 4)).astype(np.float32))
    assert ix.n_clusters <= 10


def test_ivfl2_fewer_results_than_k(gn):
    rng = np.random.default_rng(9)
    data = rng.random((60, 4)).astype(np.float32)
    ix = gn.IVFFlatL2Index(n_clusters=30, n_probe=1)
    ix.set(data)
    idx, dist, cnt = ix.search_knn_arrays(data[:5], 50)
    assert (cnt < 50).all() and (cnt >= 1).all()
    for i in range(5):
        assert (idx[i, cnt[i]:] == -1).all()
        assert list(dist[i, :cnt[i]]) == sorted(dist[i, :cnt[i]])


def test_ivfl2_high_dim_1024(gn):
    rng = np.random.default_rng(6)
    data = rng.random((2000, 1024)).astype(np.float32)
    queries = rng.random((5, 1024)).astype(np.float32)
    ix = gn.IVFFlatL2Index(n_clusters=40, n_probe=10)
    ix.set(data)
    idx, dist = ix.searchKNN(queries, k=5)
    assert len(idx) == 5 and all(len(r) == 5 for r in idx)


def test_ivfl2_pickle_roundtrip(gn):
    rng = np.random.default_rng(8)
    data = rng.random((500, 32)).astype(np.float32)
    queries = rng.random((10, 32)).astype(np.float32)
    ix = gn.IVFFlatL2Index(n_clusters=20, n_probe=20)
    ix.set(data)
    a = ix.searchKNN(queries, 5)
    ix2 = pickle.loads(pickle.dumps(ix))
    b = ix2.searchKNN(queries, 5)
    assert a[0] == b[0]
    np.testing.assert_allclose(a[1], b[1])


def test_ivfl2_vs_oracle_mixture(gn, oracle):
    """Uneven (Zipf) Gaussian mixture; same lists on both sides; many probes."""
    rng = np.random.default_rng(31)
    centres = rng.normal(size=(64, 48)).astype(np.float32)
    w = 1.0 / np.arange(1, 65) ** 1.1
    comp = rng.choice(64, size=30000, p=w / w.sum())
    data = (centres[comp] + 0.3 * rng.normal(size=(30000, 48))).astype(np.float32)
    q = (centres[rng.choice(64, 300, p=w / w.sum())] + 0.3 * rng.normal(size=(300, 48))).astype(np.float32)
    ix = gn.IVFFlatL2Index(n_clusters=32, n_probe=6)
    ix.set(data)
    cent, offs, ids = ix.export()
    labels = np.empty(len(data), np.int32)
    for c in range(len(offs) - 1):
        labels[ids[offs[c]:offs[c + 1]]] = c
    for k in (1, 10, 40, 100):
        idx, dist, cnt = ix.search_knn_arrays(q, k)
        oi, od, oc = oracle.ivfl2_search(data, cent, labels, q, k, 6)
        assert np.array_equal(cnt, oc)
        np.testing.assert_allclose(dist, od, rtol=2e-4, atol=2e-4)
        assert np.mean(idx == oi) >= 0.995


# ── IVFFlatBinaryIndex ────────────────────────────────────────────────────
def _make_db(n, nbytes, seed=0):
    return np.random.default_rng(seed).integers(0, 256, size=(n, nbytes), dtype=np.uint8)


def _near(db, ti, n_flips, seed=1):
    rng = np.random.default_rng(seed)
    out = []
    for i in ti:
        v = db[i].copy()
        for b in rng.choice(db.shape[1] * 8, size=n_flips, replace=False):
            v[b // 8] ^= np.uint8(1 << (b % 8))
        out.append(v)
    return np.array(out, np.uint8)


def test_ivfbin_build_is_bit_exact(gn, oracle):
    g = golden("ivf_binary.npz")
    for tag in ("a", "b", "c"):
        nlist, nprobe, k = (int(x) for x in g[f"{tag}_cfg"])
        db, q = g[f"{tag}_db"], g[f"{tag}_q"]
        ix = gn.IVFFlatBinaryIndex(nlist=nlist, nprobe=nprobe)
        ix.set(db)
        cent, labels = ix.export()
        oc, ol = oracle.ivfbin_build(db, nlist)
        assert np.array_equal(cent, oc) and np.array_equal(labels, ol)
        idx, dist, cnt = ix.search_knn_arrays(q, k)
        oi, od, ocnt = oracle.ivfbin_search(db, oc, ol, q, k, nprobe, tie_mode=1)
        assert np.array_equal(cnt, ocnt) and np.array_equal(idx, oi) and np.array_equal(dist, od)
        # against the reference's own output: same distances and counts
        assert np.array_equal(cnt, g[f"{tag}_cnt"])
        assert np.array_equal(dist, g[f"{tag}_dist"])


def test_ivfbin_reference_api(gn):
    db = _make_db(500, 64)
    ix = gn.IVFFlatBinaryIndex(nlist=16, nprobe=4)
    ix.set(db)
    ti = list(range(0, 50, 5))
    res_idx, res_dist = ix.searchKNN(_near(db, ti, 3), k=5)
    assert len(res_idx) == len(ti) and all(len(r) <= 5 for r in res_idx)
    assert all(d >= 0 for dv in res_dist for d in dv)
    db = _make_db(1000, 64)
    ti = list(range(0, 100, 10))
    ix = gn.IVFFlatBinaryIndex(nlist=32, nprobe=32)
    ix.set(db)
    res_idx, _ = ix.searchKNN(_near(db, ti, 4), k=10)
    assert all(t in r for t, r in zip(ti, res_idx))
    ix = gn.IVFFlatBinaryIndex(nlist=8, nprobe=2)
    ix.set(_make_db(200, 64))
    assert ix.nprobe() == 2
    ix.set_nprobe(4)
    assert ix.nprobe() == 4
    ix = gn.IVFFlatBinaryIndex(nlist=64)
    ix.set(_make_db(200, 64))
    assert ix.nlist() == 64
    for nb, k in ((32, 3), (16, 3)):
        db = _make_db(400, nb)
        ix = gn.IVFFlatBinaryIndex(nlist=16, nprobe=8)
        ix.set(db)
        ri, _ = ix.searchKNN(_near(db, [0, 10, 20], 2), k=k)
        assert len(ri) == 3
    db = _make_db(500, 64)
    ix = gn.IVFFlatBinaryIndex(nlist=16, nprobe=8)
    ix.set(db)
    _, dist = ix.searchKNN(_near(db, [0], 4), k=10)
    assert dist[0] == sorted(dist[0])
    db = _make_db(50, 64)
    ix = gn.IVFFlatBinaryIndex(nlist=10, nprobe=1)
    ix.set(db)
    ri, rd = ix.searchKNN(db[:3], k=100)
    assert len(ri) == 3 and all(len(r) <= 100 for r in ri)


def test_ivfbin_full_probe_equals_exact_scan(gn, oracle):
    rng = np.random.default_rng(77)
    db = rng.integers(0, 256, (20000, 64), dtype=np.uint8)
    q = _near(db, list(rng.integers(0, 20000, 40)), 24, seed=5)
    ix = gn.IVFFlatBinaryIndex(nlist=64, nprobe=64)
    ix.set(db)
    idx, dist, cnt = ix.search_knn_arrays(q, 10)
    oi, od = oracle.knn_hamming(db, q, 10)
    assert np.array_equal(idx, oi) and np.array_equal(dist, od)

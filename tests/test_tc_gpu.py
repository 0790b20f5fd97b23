"""Tensor-core shortlist (BF16 tcgen05 GEMM + top-S) followed by the exact FP32
re-rank: results must equal the exact flat scan (indices and the reference's
distance bits) and match an FP64 oracle within FP32 rounding."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def mixture(n, d, nc, nq, seed):
    rng = np.random.default_rng(seed)
    c = rng.standard_normal((nc, d), dtype=np.float32)
    db = (c[rng.integers(0, nc, n)] + np.float32(0.3) * rng.standard_normal((n, d), dtype=np.float32))
    q = (c[rng.integers(0, nc, nq)] + np.float32(0.3) * rng.standard_normal((nq, d), dtype=np.float32))
    return db.astype(np.float32), q.astype(np.float32)


@pytest.mark.parametrize("n,d,nq,k,S", [(4096, 128, 128, 10, 40), (50_000, 128, 300, 10, 40),
                                        (30_001, 64, 77, 5, 32), (20_000, 200, 129, 1, 16),
                                        (40_000, 96, 200, 10, 64), (10_000, 128, 130, 10, 48),
                                        # few rows per cluster: the zero-filled tail of the last
                                        # 256-row tile would outscore other clusters' rows
                                        (3000, 64, 77, 10, 40), (3000, 128, 200, 10, 16)])
def test_tc_shortlist_equals_exact(gn, oracle, n, d, nq, k, S):
    db, q = mixture(n, d, 256, nq, seed=n + d)
    tc = gn.FlatL2TCIndex(shortlist=S)
    tc.set(db)
    idx, dist = tc.search_knn_arrays(q, k)
    ex = gn.FlatL2Index()
    ex.set(db)
    ei, ed = ex.search_knn_arrays(q, k)
    assert np.array_equal(idx, ei)
    assert np.array_equal(dist.view(np.uint32), ed.view(np.uint32))
    oi, od = oracle.knn_l2sq_f64(db, q[:64], k)
    err = np.abs(dist[:64].astype(np.float64) - np.sqrt(od))
    assert err.max() <= 1e-5 * np.sqrt(od).max()


# FP8 E4M3 with per-row scales: the shortlist is approximate, the returned
# distances are still the exact FP32 distances of the returned rows.  Recall
# floors sit below the recall of a NumPy emulation of the same quantisation on
# these inputs (0.985, 0.998, 1.0, 0.99).
@pytest.mark.parametrize("n,d,nq,k,S,floor", [(50_000, 128, 300, 10, 40, 0.97), (20_000, 200, 129, 5, 32, 0.98),
                                              (3000, 64, 77, 10, 40, 0.99), (50_000, 128, 300, 10, 56, 0.98)])
def test_fp8_shortlist_recall_and_exact_distances(gn, oracle, n, d, nq, k, S, floor):
    db, q = mixture(n, d, 256, nq, seed=n + d)
    tc = gn.FlatL2TCIndex(shortlist=S, precision="fp8")
    tc.set(db)
    idx, dist = tc.search_knn_arrays(q, k)
    ex = gn.FlatL2Index()
    ex.set(db)
    ei, ed = ex.search_knn_arrays(q, k)
    recall = np.mean([len(set(idx[i]) & set(ei[i])) / k for i in range(nq)])
    assert recall >= floor, recall
    assert (idx >= 0).all() and all(len(set(r)) == k for r in idx)
    assert (np.diff(dist, axis=1) >= 0).all()
    ref = np.array([[oracle.dist("l2", q[i], db[j]) for j in idx[i]] for i in range(min(nq, 40))], np.float32)
    assert np.array_equal(dist[:len(ref)].view(np.uint32), ref.view(np.uint32))
    # rows found by both are reported with identical distances
    for i in range(nq):
        got = dict(zip(idx[i].tolist(), dist[i].view(np.uint32).tolist()))
        want = dict(zip(ei[i].tolist(), ed[i].view(np.uint32).tolist()))
        assert all(got[r] == want[r] for r in got.keys() & want.keys())


def test_precision_switch_after_set(gn):
    db, q = mixture(20_000, 128, 64, 100, seed=9)
    tc = gn.FlatL2TCIndex(shortlist=40)
    tc.set(db)
    i0, d0 = tc.search_knn_arrays(q, 10)
    gn._lib.call("gn_tcflat_set_precision", tc._h.h, 1)
    i1, _ = tc.search_knn_arrays(q, 10)
    assert np.mean([len(set(i1[i]) & set(i0[i])) / 10 for i in range(len(q))]) > 0.9
    gn._lib.call("gn_tcflat_set_precision", tc._h.h, 0)
    i2, d2 = tc.search_knn_arrays(q, 10)
    assert np.array_equal(i2, i0) and np.array_equal(d2.view(np.uint32), d0.view(np.uint32))
    with pytest.raises(RuntimeError):
        gn.FlatL2TCIndex(shortlist=64, precision="fp8")
    with pytest.raises(ValueError):
        gn.FlatL2TCIndex(precision="fp4")


def test_tc_small_batches_and_tiny_db(gn, oracle):
    db, q = mixture(300, 128, 8, 3, seed=5)
    tc = gn.FlatL2TCIndex(shortlist=40)
    tc.set(db)
    idx, dist = tc.search_knn_arrays(q, 10)
    oi, od = oracle.knn_float("l2", db, q, 10)
    assert np.array_equal(idx, oi)


def test_ivf_tc_engine_matches_exact_within_probed_lists(gn, oracle):
    """Tensor-core IVF: same lists and probes as the FP32 engine; its top-k are
    the exact top-k of the probed lists (FP64-checked distances)."""
    rng = np.random.default_rng(41)
    centres = rng.standard_normal((64, 256), dtype=np.float32)
    w = 1.0 / np.arange(1, 65) ** 1.1
    comp = rng.choice(64, size=40000, p=w / w.sum())
    data = (centres[comp] + np.float32(0.3) * rng.standard_normal((40000, 256), dtype=np.float32))
    q = (centres[rng.choice(64, 257, p=w / w.sum())] + np.float32(0.3) * rng.standard_normal((257, 256), dtype=np.float32))
    ix = gn.IVFFlatL2Index(n_clusters=48, n_probe=5, engine="tc")
    ix.set(data)
    cent, offs, ids = ix.export()
    labels = np.empty(len(data), np.int32)
    for c in range(len(offs) - 1):
        labels[ids[offs[c]:offs[c + 1]]] = c
    idx, dist, cnt = ix.search_knn_arrays(q, 10)
    oi, od, oc = oracle.ivfl2_search(data, cent, labels, q, 10, 5)
    assert np.array_equal(cnt, oc)
    assert np.mean(idx == oi) >= 0.995
    np.testing.assert_allclose(dist, od, rtol=1e-4, atol=1e-3)
    # exact distances: compare with an FP64 recomputation of the returned rows
    d64 = ((q[:, None, :].astype(np.float64) - data[idx].astype(np.float64)) ** 2).sum(-1)
    assert np.max(np.abs(dist - d64) / np.maximum(d64, 1e-6)) < 1e-6
    ix.set_engine("fp32")
    fi, fd, fc = ix.search_knn_arrays(q, 10)
    assert np.mean(fi == idx) >= 0.995


def test_ivf_tc_engine_same_results_for_every_batch_split(gn):
    """Small batches split each query's selection over several blocks; the
    results must equal those of a large batch (one block per query), with no
    repeated ids."""
    rng = np.random.default_rng(7)
    c = rng.standard_normal((300, 40), dtype=np.float32)
    db = (c[rng.integers(0, 300, 30000)] + np.float32(0.4) * rng.standard_normal((30000, 40), dtype=np.float32))
    q = (c[rng.integers(0, 300, 512)] + np.float32(0.4) * rng.standard_normal((512, 40), dtype=np.float32))
    for nprobe in (1, 5, 24):
        ix = gn.IVFFlatL2Index(n_clusters=64, n_probe=nprobe, engine="tc")
        ix.set(db)
        ref_i, ref_d, ref_c = ix.search_knn_arrays(q, 8)
        for row in ref_i:
            v = row[row >= 0]
            assert len(set(v.tolist())) == len(v)
        for n in (1, 3, 16, 33, 64, 128, 200):
            i, d, cnt = ix.search_knn_arrays(q[:n], 8)
            np.testing.assert_array_equal(i, ref_i[:n])
            np.testing.assert_array_equal(d, ref_d[:n])
            np.testing.assert_array_equal(cnt, ref_c[:n])


def test_tc_shortlist_full_size_1m_x128(gn, oracle):
    """The tensor-core shortlist configuration at full size: 1M x 128 mixture
    (1,024 centres, sigma 0.3), 10,000 queries, k 10, shortlist 40: the
    returned rows equal the exact scan's (indices and distance bits), and the
    distance error against FP64 on a subset stays within FP32 rounding."""
    from pynear_gb300 import workloads as W

    db, q, _, _ = W.gaussian_mixture(n=1_000_000, d=128, n_centres=1024, sigma=0.3, zipf_s=0, nq=10_000, seed=11)
    tc = gn.FlatL2TCIndex(shortlist=40)
    tc.set(db)
    idx, dist = tc.search_knn_arrays(q, 10)
    ex = gn.FlatL2Index()
    ex.set(db)
    ei, ed = ex.search_knn_arrays(q, 10)
    assert np.array_equal(idx, ei)
    assert np.array_equal(dist.view(np.uint32), ed.view(np.uint32))
    sub = 200
    d64 = np.sqrt(((q[:sub, None, :].astype(np.float64) - db[idx[:sub]].astype(np.float64)) ** 2).sum(-1))
    assert np.abs(dist[:sub] - d64).max() <= 1e-5 * d64.max()


def test_ivf_tc_score_bound_filters_and_stays_exact(gn, oracle):
    """Well separated clusters, one per list: the probe stage's score bound
    (the shortlist-th nearest row of a probed list lies within |q - c| + rho
    of the query) sits far below other clusters' rows, so the list scan stores
    only the score quarters of each query's own cluster.  The results must be
    the exact top-k of the probed lists all the same, for k up to the
    shortlist and with queries far from every cluster (a loose bound).  (The
    clusters' spread is kept large against the rows' norms: with small spread
    and large norms the BF16 scores' error reaches the spread and the BF16
    shortlist itself, bound or not, misses neighbours.)"""
    rng = np.random.default_rng(43)
    centres = rng.standard_normal((96, 128), dtype=np.float32)
    comp = np.repeat(np.arange(96), 400)
    data = (centres[comp] + np.float32(0.3) * rng.standard_normal((len(comp), 128), dtype=np.float32))
    q_near = centres[rng.integers(0, 96, 300)] + np.float32(0.3) * rng.standard_normal((300, 128), dtype=np.float32)
    q_far = np.float32(2.0) * rng.standard_normal((40, 128), dtype=np.float32)
    q = np.concatenate([q_near, q_far]).astype(np.float32)
    ix = gn.IVFFlatL2Index(n_clusters=96, n_probe=3, engine="tc")
    ix.set(data)
    cent, offs, ids = ix.export()
    labels = np.empty(len(data), np.int32)
    for c in range(len(offs) - 1):
        labels[ids[offs[c]:offs[c + 1]]] = c
    for k in (1, 10, 32):
        idx, dist, cnt = ix.search_knn_arrays(q, k)
        oi, od, oc = oracle.ivfl2_search(data, cent, labels, q, k, 3)
        assert np.array_equal(cnt, oc), k
        assert np.mean(idx == oi) >= 0.995, k
        np.testing.assert_allclose(dist, od, rtol=1e-4, atol=1e-3)
        d64 = ((q[:, None, :].astype(np.float64) - data[np.maximum(idx, 0)].astype(np.float64)) ** 2).sum(-1)
        ok = idx >= 0
        assert np.max(np.abs(dist[ok] - d64[ok]) / np.maximum(d64[ok], 1e-6)) < 1e-6

"""Pin the CPU oracle to the reference: committed golden fixtures (made by
tests/golden/make_golden.py from the reference's own build) and, where the
reference extension is built here (oracle/_ref), live cross-checks."""
import os
import sys

import numpy as np
import pytest

from conftest import REPO, golden

REF_DIR = os.path.join(REPO, "oracle", "_ref")


def _ref():
    if not any(f.startswith("_pynear") for f in os.listdir(REF_DIR)) if os.path.isdir(REF_DIR) else True:
        pytest.skip("reference extension not built here (oracle/_ref)")
    sys.path.insert(0, REF_DIR)
    import _pynear
    return _pynear


def test_float_distances_bitexact(oracle):
    g = golden("dist_float.npz")
    for d in g["dims"]:
        a, b = g[f"a{d}"], g[f"b{d}"]
        for m in ("l2", "l1", "linf"):
            got = np.array([oracle.dist(m, a[i], b[i]) for i in range(len(a))], np.float32)
            assert np.array_equal(got.view(np.uint32), g[f"{m}_{d}"].view(np.uint32)), (m, d)


def test_hamming_known_answers(oracle):
    g = golden("hamming_kat.npz")
    for a, b, w, dd in zip(g["a"], g["b"], g["width"], g["dist"]):
        assert oracle.hamming(a[:w], b[:w]) == dd
    # the reference C++ test's stated answers (tests/VPTreeTests.cpp:51-99)
    assert list(g["dist"][:6]) == [0, 2, 8, 9, 11, 256]


def test_hamming_reference_dispatch_wraps_odd_widths(oracle):
    # odd byte widths accumulate in int8 in the reference (wraps past 127);
    # the library (and oracle.hamming) return the true count
    a = np.zeros(17, np.uint8)
    b = np.full(17, 255, np.uint8)
    assert oracle.hamming(a, b) == 136
    assert oracle.hamming(a, b, ref_dispatch=True) == 136 - 256


@pytest.mark.parametrize("metric", ["l2", "l1", "linf"])
def test_exact_knn_matches_vptree(oracle, metric):
    g = golden("vptree_float.npz")
    for tag in ("a", "b", "c"):
        db, q = g[f"{tag}_db"], g[f"{tag}_q"]
        ref_idx, ref_dist = g[f"{metric}_{tag}_idx"], g[f"{metric}_{tag}_dist"]
        k = ref_idx.shape[1]
        idx, dist = oracle.knn_float(metric, db, q, k)
        assert np.array_equal(dist.view(np.uint32), ref_dist.view(np.uint32))
        # indices agree wherever the distance is not tied
        for i in range(len(q)):
            for j in range(k):
                if np.sum(dist[i] == dist[i, j]) == 1 and dist[i, j] < dist[i, -1]:
                    assert idx[i, j] == ref_idx[i, j]
        assert np.array_equal(idx[:, 0], g[f"{metric}_{tag}_idx1"])
        assert np.array_equal(dist[:, 0].view(np.uint32), g[f"{metric}_{tag}_dist1"].view(np.uint32))


def test_exact_hamming_matches_vptree(oracle):
    g = golden("vptree_binary.npz")
    for tag in ("a", "b", "c", "d"):
        db, q, ref_idx, ref_dist = g[f"{tag}_db"], g[f"{tag}_q"], g[f"{tag}_idx"], g[f"{tag}_dist"]
        idx, dist = oracle.knn_hamming(db, q, ref_idx.shape[1])
        assert np.array_equal(dist, ref_dist)
        for i in range(len(q)):  # untied positions name the same row
            for j in range(dist.shape[1]):
                if np.sum(dist[i] == dist[i, j]) == 1 and dist[i, j] < dist[i, -1]:
                    assert idx[i, j] == ref_idx[i, j]


def test_kmeans_bitexact(oracle):
    g = golden("kmeans.npz")
    for tag in ("a", "b"):
        data, cent = g[f"{tag}_data"], g[f"{tag}_cent"]
        labels, c, _ = oracle.kmeans_l2(data, cent.shape[0], 100, 42)
        assert np.array_equal(labels, g[f"{tag}_labels"])
        assert np.array_equal(c.view(np.uint32), cent.view(np.uint32))


def test_ivf_binary_bitexact(oracle):
    g = golden("ivf_binary.npz")
    for tag in ("a", "b", "c"):
        nlist, nprobe, k = g[f"{tag}_cfg"]
        cent, labels = oracle.ivfbin_build(g[f"{tag}_db"], int(nlist))
        idx, dist, cnt = oracle.ivfbin_search(g[f"{tag}_db"], cent, labels, g[f"{tag}_q"], int(k), int(nprobe),
                                              tie_mode=0)
        assert np.array_equal(cnt, g[f"{tag}_cnt"])
        assert np.array_equal(idx, g[f"{tag}_idx"])
        assert np.array_equal(dist, g[f"{tag}_dist"])


def test_ivf_l2_matches_forest(oracle):
    g = golden("ivf_l2.npz")
    for tag in ("a", "b"):
        nc, npb, k = (int(x) for x in g[f"{tag}_cfg"])
        idx, dist, cnt = oracle.ivfl2_search(g[f"{tag}_db"], g[f"{tag}_cent"], g[f"{tag}_labels"], g[f"{tag}_q"],
                                             k, npb)
        ref_idx, ref_dist = g[f"{tag}_idx"], g[f"{tag}_dist"]
        assert (cnt == k).all()
        # distances agree to float32 rounding of the BLAS dot products
        np.testing.assert_allclose(dist, ref_dist, rtol=1e-5, atol=1e-5)
        assert np.mean(idx == ref_idx) > 0.99


def test_live_against_reference(oracle):
    _pynear = _ref()
    rng = np.random.default_rng(7)
    db = rng.random((3000, 21), dtype=np.float32)
    q = rng.random((12, 21), dtype=np.float32)
    t = _pynear.VPTreeL2Index()
    t.set(db)
    ri, rd = t.searchKNN(q, 6)
    idx, dist = oracle.knn_float("l2", db, q, 6)
    assert np.array_equal(np.array(rd, np.float32)[:, ::-1].view(np.uint32), dist.view(np.uint32))
    data = rng.random((800, 5), dtype=np.float32)
    l1, c1 = _pynear.kmeans_l2(data, 9, 100, 42)
    l2, c2, _ = oracle.kmeans_l2(data, 9, 100, 42)
    assert np.array_equal(l1, l2) and np.array_equal(c1, c2)

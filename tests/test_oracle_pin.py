"""Pin the CPU oracle to the reference: committed golden fixtures (made by
tests/golden/make_golden.py from the reference's own build) and, where the
reference extension is built or installed here, live cross-checks."""
import os
import sys

import numpy as np
import pytest

from conftest import REPO, golden

# the reference extension: built from its sources by oracle/build_ref.sh, or
# installed with the reference package (pip) under baseline/_ref
REF_DIRS = [os.path.join(REPO, "oracle", "_ref"), os.path.join(REPO, "baseline", "_ref")]


def _ref():
    for d in REF_DIRS:
        if not os.path.isdir(d) or not any(f.startswith("_pynear") for f in os.listdir(d)):
            continue
        sys.path.insert(0, d)
        try:
            import _pynear
            return _pynear
        except ImportError:
            continue
        finally:
            sys.path.remove(d)
    pytest.skip("reference extension not built here (oracle/_ref, baseline/_ref)")


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


def _tie_free_agree(ids, dist, ref_ids, ref_dist, seeds, xs, ys):
    """Distances bit-exact; ids equal except where the reference's seed is at
    exactly the same distance (its tree returns either of two tied seeds)."""
    assert np.array_equal(dist.view(np.uint32), ref_dist.view(np.uint32))
    r, c = np.nonzero(ids != ref_ids)
    dx = xs[c] - seeds[ref_ids[r, c], 0]
    dy = ys[r] - seeds[ref_ids[r, c], 1]
    assert np.array_equal(np.sqrt(dx * dx + dy * dy), dist[r, c])
    return len(r)


def test_voronoi_raster_matches_reference_demo(oracle):
    g = golden("voronoi.npz")
    ties = {}
    for t in "abc":
        seeds = g[f"{t}_seeds"]
        w, h = g[f"{t}_wh"]
        xs = np.linspace(0, 1, w, dtype=np.float32)
        ys = np.linspace(0, 1, h, dtype=np.float32)
        ids, dist = oracle.voronoi_raster(seeds, xs, ys)
        ties[t] = _tie_free_agree(ids, dist, g[f"{t}_ids"], g[f"{t}_dist"], seeds, xs, ys)
    # distinct random seeds: no ties; case c repeats seeds 0-19 as 20-39
    assert ties["a"] == 0 and ties["b"] == 0 and ties["c"] > 0


def test_png_writer_and_palette(tmp_path):
    import zlib

    from pynear_gb300 import voronoi as vr

    pal = vr.make_palette(5)
    assert pal.shape == (5, 4) and (pal[:, 3] == 255).all() and len({tuple(p) for p in pal}) == 5
    img = np.random.default_rng(0).integers(0, 256, (7, 5, 4), dtype=np.uint8)
    path = str(tmp_path / "raster.png")
    vr.write_png(path, img)
    blob = open(path, "rb").read()
    assert blob[:8] == b"\x89PNG\r\n\x1a\n" and blob[12:16] == b"IHDR"
    w, h = int.from_bytes(blob[16:20], "big"), int.from_bytes(blob[20:24], "big")
    assert (w, h) == (5, 7)
    start = blob.index(b"IDAT") + 4
    n = int.from_bytes(blob[start - 8:start - 4], "big")
    raw = np.frombuffer(zlib.decompress(blob[start:start + n]), np.uint8).reshape(7, 1 + 5 * 4)
    assert (raw[:, 0] == 0).all() and np.array_equal(raw[:, 1:].reshape(7, 5, 4), img)


def _mih_agree(idx, dist, cnt, ref_idx, ref_dist, ref_cnt, db, q):
    """Same counts and distances; the same rows below each query's k-th
    distance; at the k-th distance the reference's rows (its hash-set order
    picks among ties) are at that distance."""
    assert np.array_equal(cnt, ref_cnt)
    assert np.array_equal(dist, ref_dist)
    pc = np.unpackbits(np.arange(256, dtype=np.uint8)[:, None], axis=1).sum(1)
    for i in range(len(q)):
        c = cnt[i]
        if c == 0:
            continue
        kth = dist[i, c - 1]
        below = dist[i, :c] < kth
        assert set(idx[i, :c][below].tolist()) == set(ref_idx[i, :c][below].tolist())
        tied = ref_idx[i, :c][~below]
        assert (pc[np.bitwise_xor(db[tied], q[i])].sum(1) == kth).all()


def test_mih_restatement_matches_reference(oracle):
    g = golden("mih.npz")
    for t in "abcd":
        m, k, radius = (int(v) for v in g[f"{t}_cfg"])
        db, q = g[f"{t}_db"], g[f"{t}_q"]
        oi, od, oc = oracle.mih_search(db, q, k, m, radius)
        _mih_agree(oi, od, oc, g[f"{t}_idx"], g[f"{t}_dist"], g[f"{t}_cnt"], db, q)

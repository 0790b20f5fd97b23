"""Parity of the GPU exact flat scans with the oracle and the reference fixtures.

Bar: bit-exact distances (the reference's float arithmetic order, exact Hamming
counts) and identical indices under the lexicographic (distance, index) order.
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

FLOAT_CLASSES = {"l2": "FlatL2Index", "l1": "FlatL1Index", "linf": "FlatChebyshevIndex"}
COMPAT_CLASSES = {"l2": "VPTreeL2Index", "l1": "VPTreeL1Index", "linf": "VPTreeChebyshevIndex"}


def _flat(gn, metric, db):
    ix = getattr(gn, FLOAT_CLASSES[metric])()
    ix.set(db)
    return ix


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("metric", ["l2", "l1", "linf"])
def test_golden_vptree_fixtures(gn, oracle, metric):
    g = golden("vptree_float.npz")
    for tag in ("a", "b", "c"):
        db, q = g[f"{tag}_db"], g[f"{tag}_q"]
        k = g[f"{metric}_{tag}_idx"].shape[1]
        ix = _flat(gn, metric, db)
        idx, dist = ix.search_knn_arrays(q, k)
        assert np.array_equal(_bits(dist), _bits(g[f"{metric}_{tag}_dist"]))
        oi, od = oracle.knn_float(metric, db, q, k)
        assert np.array_equal(idx, oi)
        i1, d1 = ix.search_1nn_arrays(q)
        assert np.array_equal(i1, g[f"{metric}_{tag}_idx1"])
        assert np.array_equal(_bits(d1), _bits(g[f"{metric}_{tag}_dist1"]))
        # the drop-in class returns the same rows farthest-first
        c = getattr(gn, COMPAT_CLASSES[metric])()
        c.set(db)
        ci, cd = c.searchKNN(q, k)
        assert np.array_equal(np.array(ci)[:, ::-1], oi)


def test_golden_pair_distances(gn):
    g = golden("dist_float.npz")
    for d in g["dims"]:
        a, b = g[f"a{d}"], g[f"b{d}"]
        for m in ("l2", "l1", "linf"):
            ix = _flat(gn, m, b)
            idx, dist = ix.search_knn_arrays(a, len(b))
            # recover the (i, i) pair distance from the full ranking
            diag = np.array([dist[i][idx[i] == i][0] for i in range(len(a))], np.float32)
            assert np.array_equal(_bits(diag), _bits(g[f"{m}_{d}"])), (m, d)


def test_golden_hamming(gn, oracle):
    g = golden("hamming_kat.npz")
    for a, b, w, dd in zip(g["a"], g["b"], g["width"], g["dist"]):
        assert gn.dist_hamming(a[:w], b[:w]) == dd
    g = golden("vptree_binary.npz")
    for tag in ("a", "b", "c", "d"):
        db, q, rd = g[f"{tag}_db"], g[f"{tag}_q"], g[f"{tag}_dist"]
        ix = gn.FlatHammingIndex()
        ix.set(db)
        idx, dist = ix.search_knn_arrays(q, rd.shape[1])
        assert np.array_equal(dist, rd)
        oi, od = oracle.knn_hamming(db, q, rd.shape[1])
        assert np.array_equal(idx, oi)


def test_exact_l2_uniform_100k_x32(gn, oracle):
    """Exact flat L2 workload (100,000 x 32 uniform, k=5 and 1-NN) on a query subset."""
    rng = np.random.default_rng(11)
    db = rng.random((100_000, 32), dtype=np.float32)
    q = rng.random((200, 32), dtype=np.float32)
    ix = gn.FlatL2Index()
    ix.set(db)
    idx, dist = ix.search_knn_arrays(q, 5)
    oi, od = oracle.knn_float("l2", db, q, 5)
    assert np.array_equal(idx, oi)
    assert np.array_equal(_bits(dist), _bits(od))
    i1, d1 = ix.search_1nn_arrays(q)
    assert np.array_equal(i1, oi[:, 0])


def _flip(db, src, nflip, rng):
    q = db[src].copy()
    for i in range(len(src)):
        bits = rng.choice(db.shape[1] * 8, size=nflip, replace=False)
        for b in bits:
            q[i, b // 8] ^= np.uint8(1 << (b % 8))
    return q


def test_exact_hamming_1m_x512(gn, oracle):
    """Full-size Hamming database (1,000,000 x 64 B), 24-bit flipped queries, k=10."""
    rng = np.random.default_rng(12)
    db = rng.integers(0, 256, (1_000_000, 64), dtype=np.uint8)
    src = rng.integers(0, len(db), 64)
    q = _flip(db, src, 24, rng)
    ix = gn.FlatHammingIndex()
    ix.set(db)
    idx, dist = ix.search_knn_arrays(q, 10)
    oi, od = oracle.knn_hamming(db, q, 10)
    assert np.array_equal(dist, od)
    assert np.array_equal(idx, oi)
    assert np.array_equal(idx[:, 0], src) and (dist[:, 0] == 24).all()


@pytest.mark.parametrize("k", [1, 2, 31, 32, 33, 64, 65, 128, 200, 256, 257, 600])
def test_k_sweep_and_large_k(gn, oracle, k):
    rng = np.random.default_rng(k)
    db = rng.random((3001, 13), dtype=np.float32)
    q = rng.random((37, 13), dtype=np.float32)
    ix = gn.FlatL2Index()
    ix.set(db)
    idx, dist = ix.search_knn_arrays(q, k)
    oi, od = oracle.knn_float("l2", db, q, k)
    assert np.array_equal(idx, oi)
    assert np.array_equal(_bits(dist), _bits(od))
    hb = rng.integers(0, 256, (2500, 24), dtype=np.uint8)  # 24-byte rows: padded to 32
    hq = rng.integers(0, 256, (19, 24), dtype=np.uint8)
    hx = gn.FlatHammingIndex()
    hx.set(hb)
    hi, hd = hx.search_knn_arrays(hq, k)
    oi, od = oracle.knn_hamming(hb, hq, k)
    assert np.array_equal(hi, oi) and np.array_equal(hd, od)


def test_k_equals_and_exceeds_n(gn, oracle):
    rng = np.random.default_rng(5)
    db = rng.random((2021, 8), dtype=np.float32)
    q = rng.random((8, 8), dtype=np.float32)
    for metric in ("l2", "l1", "linf"):
        ix = _flat(gn, metric, db)
        idx, dist = ix.search_knn_arrays(q, 2021)
        oi, od = oracle.knn_float(metric, db, q, 2021)
        assert np.array_equal(idx, oi) and np.array_equal(_bits(dist), _bits(od))
    small = rng.random((5, 8), dtype=np.float32)
    ix = gn.VPTreeL2Index()
    ix.set(small)
    ci, cd = ix.searchKNN(q[:2], 3)
    assert [len(r) for r in ci] == [3, 3]
    ci, cd = ix.searchKNN(q[:2], 9)  # k > n: all n rows come back
    assert [len(r) for r in ci] == [5, 5]


@pytest.mark.parametrize("d", [1, 2, 3, 5, 7, 9, 12, 17, 100, 513, 1024])
def test_odd_dimensions(gn, oracle, d):
    rng = np.random.default_rng(d)
    db = (rng.random((1500, d), dtype=np.float32) * 4 - 2)
    q = (rng.random((9, d), dtype=np.float32) * 4 - 2)
    for metric in ("l2", "l1", "linf"):
        ix = _flat(gn, metric, db)
        idx, dist = ix.search_knn_arrays(q, 7)
        oi, od = oracle.knn_float(metric, db, q, 7)
        assert np.array_equal(idx, oi), (metric, d)
        assert np.array_equal(_bits(dist), _bits(od)), (metric, d)


@pytest.mark.parametrize("nb", [1, 5, 8, 16, 17, 32, 64, 100, 128])
def test_hamming_widths(gn, oracle, nb):
    rng = np.random.default_rng(nb)
    db = rng.integers(0, 256, (3000, nb), dtype=np.uint8)
    q = rng.integers(0, 256, (11, nb), dtype=np.uint8)
    ix = gn.FlatHammingIndex()
    ix.set(db)
    idx, dist = ix.search_knn_arrays(q, 10)
    oi, od = oracle.knn_hamming(db, q, 10)
    assert np.array_equal(idx, oi) and np.array_equal(dist, od)


def test_duplicates_and_ties_go_to_lower_index(gn):
    db = np.zeros((50, 32), np.uint8)
    ix = gn.FlatHammingIndex()
    ix.set(db)
    idx, dist = ix.search_knn_arrays(db[:3], 10)
    assert (idx == np.arange(10)).all() and (dist == 0).all()
    f = np.ones((40, 4), np.float32)
    fx = gn.FlatL2Index()
    fx.set(f)
    idx, dist = fx.search_knn_arrays(f[:2], 5)
    assert (idx == np.arange(5)).all()
    # drop-in binary wrapper: duplicate rows, k = 2 (tests/test_vptree.py:183-195 shape)
    b = gn.VPTreeBinaryIndex()
    data = np.zeros((2, 32), np.uint8)
    b.set(data)
    indices, distances = b.searchKNN(data, 2)
    assert [sorted(i) for i in indices] == [[0, 1], [0, 1]]
    assert distances == [[0, 0], [0, 0]]


def test_single_row_and_no_queries(gn):
    ix = gn.FlatL1Index()
    ix.set(np.array([[1.0, 2.0]], np.float32))
    idx, dist = ix.search_knn_arrays(np.array([[1.0, 3.0]], np.float32), 4)
    assert idx.tolist() == [[0]] and dist.tolist() == [[1.0]]
    idx, dist = ix.search_knn_arrays(np.zeros((0, 2), np.float32), 3)
    assert idx.shape == (0, 1)


def test_empty_set_then_search_raises(gn):
    ix = gn.VPTreeL2Index()
    ix.set(np.array([]).reshape(-1, 2))
    with pytest.raises(RuntimeError):
        ix.search1NN(np.random.rand(1, 2).astype(np.float32))


def test_pickle_roundtrip(gn):
    import pickle
    rng = np.random.default_rng(3)
    db = rng.random((500, 16), dtype=np.float32)
    q = rng.random((5, 16), dtype=np.float32)
    ix = gn.VPTreeL2Index()
    ix.set(db)
    a = ix.searchKNN(q, 4)
    ix2 = pickle.loads(pickle.dumps(ix))
    assert ix2.searchKNN(q, 4) == a


@pytest.mark.parametrize("nq", [1, 2, 3, 4, 5, 8])
def test_small_batches(gn, oracle, nq):
    """Batches of at most 8 queries (the scan's one- and two-warp CTAs with
    one, two or four queries per warp, padding queries included): every
    width up to 129, odd ones included, k up to 32 and one k above it (two
    keys per lane)."""
    rng = np.random.default_rng(100 + nq)
    for d in (1, 5, 17, 32, 63, 64, 100, 128, 129):
        db = (rng.random((3000, d), dtype=np.float32) * 4 - 2)
        q = (rng.random((nq, d), dtype=np.float32) * 4 - 2)
        for metric in ("l2", "l1", "linf"):
            ix = _flat(gn, metric, db)
            for k in (1, 7, 32, 40):
                idx, dist = ix.search_knn_arrays(q, k)
                oi, od = oracle.knn_float(metric, db, q, k)
                assert np.array_equal(idx, oi), (metric, d, k)
                assert np.array_equal(_bits(dist), _bits(od)), (metric, d, k)


def test_exact_l2_1m_x128_8_queries(gn, oracle):
    """The HBM-bound case of the benchmark: 1,000,000 x 128 N(0,1) rows, 8
    queries, k 10 (about 2,000 row slices merged per query), bit-exact
    against the oracle."""
    rng = np.random.default_rng(17)
    db = rng.standard_normal((1_000_000, 128), dtype=np.float32)
    q = rng.standard_normal((8, 128), dtype=np.float32)
    ix = gn.FlatL2Index()
    ix.set(db)
    idx, dist = ix.search_knn_arrays(q, 10)
    oi, od = oracle.knn_float("l2", db, q, 10)
    assert np.array_equal(idx, oi)
    assert np.array_equal(_bits(dist), _bits(od))

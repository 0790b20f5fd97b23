"""MIHBinaryIndex: GPU candidate verification against the NumPy restatement
(exact results on the same candidate sets), the reference's argument checks,
and the empty index."""
import pickle

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(n, nbytes, nq, flips, seed):
    rng = np.random.default_rng(seed)
    db = rng.integers(0, 256, (n, nbytes), dtype=np.uint8)
    src = rng.integers(0, n, nq)
    q = db[src].copy()
    for i in range(nq):  # flip `flips` distinct bits of a database row
        bits = rng.choice(nbytes * 8, flips, replace=False)
        for b in bits:
            q[i, b // 8] ^= np.uint8(1 << (b % 8))
    return db, q, src


@pytest.mark.parametrize("nbytes,m,radius,k", [(64, 8, 8, 10), (64, 8, 16, 5), (32, 4, 4, 3), (16, 4, 0, 7)])
def test_mih_matches_numpy_restatement(gn, oracle, nbytes, m, radius, k):
    db, q, src = _data(3000, nbytes, 64, 6, nbytes + radius)
    ix = gn.MIHBinaryIndex(m=m)
    ix.set(db)
    assert (ix.m(), ix.n(), ix.nbytes()) == (m, 3000, nbytes)
    idx, dist, cnt = ix.search_knn_arrays(q, k, radius)
    oi, od, oc = oracle.mih_search(db, q, k, m, radius)
    np.testing.assert_array_equal(cnt, oc)
    np.testing.assert_array_equal(idx, oi)
    np.testing.assert_array_equal(dist, od)
    li, ld = ix.searchKNN(q, k, radius)
    assert li == [r[:c].tolist() for r, c in zip(oi, oc)]
    assert ld == [r[:c].tolist() for r, c in zip(od, oc)]


def test_mih_finds_planted_rows_and_pickles(gn):
    db, q, src = _data(20000, 64, 200, 4, 3)
    ix = gn.MIHBinaryIndex()
    ix.set(db)
    idx, dist, cnt = ix.search_knn_arrays(q, 3, radius=8)
    assert np.mean(idx[:, 0] == src) == 1.0  # 4 flipped bits <= radius: always a candidate
    assert (dist[:, 0] == 4).all()
    ix2 = pickle.loads(pickle.dumps(ix))
    for a, b in zip(ix2.search_knn_arrays(q, 3, radius=8), (idx, dist, cnt)):
        np.testing.assert_array_equal(a, b)


def test_mih_checks_and_empty_index(gn):
    rng = np.random.default_rng(1)
    with pytest.raises(ValueError):  # width not divisible by m
        gn.MIHBinaryIndex(m=3).set(rng.integers(0, 256, (10, 64), dtype=np.uint8))
    with pytest.raises(ValueError):  # sub-strings wider than 8 bytes
        gn.MIHBinaryIndex(m=4).set(rng.integers(0, 256, (10, 64), dtype=np.uint8))
    with pytest.raises(TypeError):
        gn.MIHBinaryIndex().set(np.zeros((4, 64), np.float32))
    empty = gn.MIHBinaryIndex()
    empty.set(np.zeros((0, 64), np.uint8))
    assert empty.searchKNN(rng.integers(0, 256, (3, 64), dtype=np.uint8), 5) == ([[], [], []], [[], [], []])


def test_mih_matches_reference_fixture(gn):
    """Against the reference's own MIHBinaryIndex output (tests/golden/mih.npz):
    same counts and distances, the same rows below each query's k-th distance,
    and rows at the k-th distance at that distance (the reference orders ties
    by its hash sets, the library by row)."""
    from conftest import golden
    from test_oracle_pin import _mih_agree

    g = golden("mih.npz")
    for t in "abcd":
        m, k, radius = (int(v) for v in g[f"{t}_cfg"])
        db, q = g[f"{t}_db"], g[f"{t}_q"]
        ix = gn.MIHBinaryIndex(m=m)
        ix.set(db)
        idx, dist, cnt = ix.search_knn_arrays(q, k, radius)
        _mih_agree(idx, dist, cnt, g[f"{t}_idx"], g[f"{t}_dist"], g[f"{t}_cnt"], db, q)

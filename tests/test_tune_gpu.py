"""Autotuner of the tensor-core IVF engine: it picks a launch configuration per
batch-size bucket, leaves results unchanged, and its table round-trips."""
import pickle

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _index(gn):
    rng = np.random.default_rng(21)
    c = rng.standard_normal((300, 48), dtype=np.float32)
    db = (c[rng.integers(0, 300, 40000)] + np.float32(0.4) * rng.standard_normal((40000, 48), dtype=np.float32))
    q = (c[rng.integers(0, 300, 600)] + np.float32(0.4) * rng.standard_normal((600, 48), dtype=np.float32))
    ix = gn.IVFFlatL2Index(n_clusters=96, n_probe=6, engine="tc")
    ix.set(db)
    return ix, q


def test_autotune_table_and_results_unchanged(gn):
    ix, q = _index(gn)
    ref = {n: ix.search_knn_arrays(q[:n], 10) for n in (1, 5, 40, 200, 600)}
    assert not ix.tuning.any()
    table = ix.autotune(q, 10, reps=2)
    assert table.shape == (7, 4)
    # the 600-query sample reaches the buckets up to [256, 1024)
    for b in range(5):
        rc, bmax, nt, qc = table[b]
        assert rc in (256, 1024, 4096) and bmax in (1, 4, 16) and nt in (32, 128, 256) and qc in (32, 64, 128)
    assert not table[5:].any()
    np.testing.assert_array_equal(ix.tuning, table)
    for n, r in ref.items():
        for a, b in zip(ix.search_knn_arrays(q[:n], 10), r):
            np.testing.assert_array_equal(a, b)
    ix2 = pickle.loads(pickle.dumps(ix))
    np.testing.assert_array_equal(ix2.tuning, table)


def test_tuning_table_is_checked(gn):
    ix, q = _index(gn)
    bad = np.zeros((7, 4), np.int32)
    bad[0] = (300, 1, 128, 0)  # not a multiple of 128
    with pytest.raises(ValueError):
        ix.tuning = bad
    bad[0] = (256, 1, 64, 0)  # no such selector width
    with pytest.raises(ValueError):
        ix.tuning = bad
    bad[0] = (256, 1, 128, 48)  # no such tile
    with pytest.raises(ValueError):
        ix.tuning = bad
    # a three-column table (saved before the tile column) still loads
    old = np.zeros((7, 3), np.int32)
    old[2] = (1024, 4, 256)
    ix.tuning = old
    np.testing.assert_array_equal(ix.tuning[2], (1024, 4, 256, 0))
    ix.set_engine("fp32")
    with pytest.raises(ValueError):
        ix.autotune(q, 10)


@pytest.mark.parametrize("shortlist", [16, 40, 64])
def test_selector_widths_give_identical_results(gn, shortlist):
    """The warp-per-query selector (tuning nt = 32) and the block selectors
    (128, 256 threads, split or not) return the same rows and distances, bit
    for bit, with fixed probing and with more probes than one warp's lanes."""
    rng = np.random.default_rng(50 + shortlist)
    c = rng.standard_normal((200, 96), dtype=np.float32)
    db = (c[rng.integers(0, 200, 50000)] + np.float32(0.35) * rng.standard_normal((50000, 96), dtype=np.float32))
    q = (c[rng.integers(0, 200, 700)] + np.float32(0.35) * rng.standard_normal((700, 96), dtype=np.float32))
    ix = gn.IVFFlatL2Index(n_clusters=128, n_probe=7, engine="tc", shortlist=shortlist)
    ix.set(db)
    k = min(10, shortlist)
    for nprobe in (7, 48):
        ix.n_probe = nprobe
        results = {}
        for nt in (32, 128, 256):
            t = np.zeros((7, 4), np.int32)
            t[:, 2] = nt
            ix.tuning = t
            results[nt] = [ix.search_knn_arrays(q[:n], k) for n in (1, 33, 700)]
        for nt in (128, 256):
            for got, ref in zip(results[nt], results[32]):
                for a, b in zip(got, ref):
                    np.testing.assert_array_equal(a, b)

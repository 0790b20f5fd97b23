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
        assert rc in (256, 1024, 4096) and bmax in (1, 4, 16) and nt in (128, 256) and qc in (32, 64, 128)
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
    bad[0] = (256, 1, 64, 0)
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

"""CUDA-graph replay of the IVF batch pipeline: a replayed batch returns
exactly what the uncaptured pipeline returns, across batch sizes, engines,
configuration changes and the device entry point."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(n, d, nq, seed):
    rng = np.random.default_rng(seed)
    c = rng.standard_normal((300, d), dtype=np.float32)
    db = c[rng.integers(0, 300, n)] + np.float32(0.4) * rng.standard_normal((n, d), dtype=np.float32)
    q = c[rng.integers(0, 300, nq)] + np.float32(0.4) * rng.standard_normal((nq, d), dtype=np.float32)
    return db.astype(np.float32), q.astype(np.float32)


def _same(a, b):
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("engine,d", [("fp32", 64), ("tc", 64), ("tc", 60), ("fp32", 36)])
def test_graph_replay_equals_uncaptured(gn, engine, d):
    db, q = _data(40_000, d, 700, 3)
    ix = gn.IVFFlatL2Index(n_clusters=128, n_probe=6, engine=engine)
    ix.set(db)
    sizes = [1, 7, 64, 300, 700, 7, 300, 1]
    ref = {n: ix.search_knn_arrays(q[:n], 10) for n in set(sizes)}
    ix.enable_graphs(700, 10)
    for rep in range(2):
        for n in sizes:
            _same(ix.search_knn_arrays(q[:n], 10), ref[n])
    info = ix.graph_info()
    assert info["capture_failures"] == 0
    assert info["graphs"] >= 1 and info["replays"] >= len(sizes)
    # another k bypasses the graphs and still searches
    i5, _, _ = ix.search_knn_arrays(q[:50], 5)
    np.testing.assert_array_equal(i5, ref[64][0][:50, :5])
    # configuration change: graphs of the old n_probe must not be replayed
    ix.n_probe = 11
    ix.enable_graphs(0, 0)
    ref11 = {n: ix.search_knn_arrays(q[:n], 10) for n in (7, 300)}
    ix.enable_graphs(700, 10)
    ix.n_probe = 6
    _same(ix.search_knn_arrays(q[:300], 10), ref[300])
    ix.n_probe = 11
    for n in (7, 300, 7):
        _same(ix.search_knn_arrays(q[:n], 10), ref11[n])
    assert ix.graph_info()["capture_failures"] == 0


def test_graph_replay_with_prober_and_rebuild(gn):
    db, q = _data(60_000, 64, 400, 5)
    ix = gn.IVFFlatL2Index(n_clusters=128, n_probe=4, engine="tc")
    ix.set(db)
    pr = gn.LearnedProber(ix, seed=3)
    ix.set_prober(pr, 0.3)
    ref = ix.search_knn_arrays(q, 10)
    nprobed = ix.last_lists_probed(len(q)).copy()
    ix.enable_graphs(512, 10)
    for _ in range(3):
        _same(ix.search_knn_arrays(q, 10), ref)
    np.testing.assert_array_equal(ix.last_lists_probed(len(q)), nprobed)
    # new weights are read by the replayed graph (same buffers, new values)
    p = pr.get_params()
    p2 = p + np.float32(0.05) * np.random.default_rng(1).standard_normal(p.shape, dtype=np.float32)
    pr.set_params(p2)
    ix.enable_graphs(0, 0)
    ref2 = ix.search_knn_arrays(q, 10)
    ix.enable_graphs(512, 10)
    pr.set_params(p)
    _same(ix.search_knn_arrays(q, 10), ref)
    pr.set_params(p2)
    _same(ix.search_knn_arrays(q, 10), ref2)
    # rebuilding the index on new rows drops every cached graph
    db2, _ = _data(30_000, 64, 1, 9)
    ix.set_prober(None)
    ix.set(db2)
    ix.enable_graphs(0, 0)
    ref3 = ix.search_knn_arrays(q[:100], 10)
    ix.enable_graphs(512, 10)
    ix.search_knn_arrays(q[:100], 10)
    ix.set(db)
    ix.set(db2)
    _same(ix.search_knn_arrays(q[:100], 10), ref3)
    assert ix.graph_info()["capture_failures"] == 0


@pytest.mark.parametrize("side_stream", [True, False])
def test_graph_device_entry_point(gn, side_stream):
    # the caller's stream may be a side stream or the legacy default stream
    # (which cannot be captured: the graphs run on the index's own stream)
    torch = pytest.importorskip("torch")
    from pynear_gb300 import _lib

    db, q = _data(30_000, 40, 256, 7)
    ix = gn.IVFFlatL2Index(n_clusters=64, n_probe=5, engine="tc")
    ix.set(db)
    ref = ix.search_knn_arrays(q, 8)
    ix.enable_graphs(256, 8)
    lib = _lib.load()
    dq = torch.from_numpy(q).cuda()
    s = torch.cuda.Stream() if side_stream else torch.cuda.default_stream()
    s.wait_stream(torch.cuda.current_stream())
    for n in (256, 33, 256, 33):
        di = torch.empty((n, 8), dtype=torch.int64, device="cuda")
        dd = torch.empty((n, 8), dtype=torch.float32, device="cuda")
        dc = torch.empty(n, dtype=torch.int64, device="cuda")
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            _lib.check(lib.gn_ivfl2_search_knn_device(ix._h.h, ctypes.c_void_p(dq.data_ptr()), n, 8,
                                                      ctypes.c_void_p(di.data_ptr()), ctypes.c_void_p(dd.data_ptr()),
                                                      ctypes.c_void_p(dc.data_ptr()), ctypes.c_void_p(s.cuda_stream)))
        s.synchronize()
        np.testing.assert_array_equal(di.cpu().numpy(), ref[0][:n])
        np.testing.assert_array_equal(dd.cpu().numpy(), ref[1][:n])
        np.testing.assert_array_equal(dc.cpu().numpy(), ref[2][:n])
    assert ix.graph_info()["replays"] >= 2

"""Forks of an IVF index: concurrent search contexts over one set of lists.

A fork shares the parent's device lists and owns its scratch, so batches on
the parent and on its forks run at the same time on different streams.  Every
search here is compared with the parent searched alone: indices, distances and
counts must be identical (same lists, same kernels, same launch choices)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(n, d, nq, seed):
    rng = np.random.default_rng(seed)
    c = rng.standard_normal((400, d), dtype=np.float32)
    db = c[rng.integers(0, 400, n)] + np.float32(0.35) * rng.standard_normal((n, d), dtype=np.float32)
    q = c[rng.integers(0, 400, nq)] + np.float32(0.35) * rng.standard_normal((nq, d), dtype=np.float32)
    return db.astype(np.float32), q.astype(np.float32)


def _same(a, b):
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("engine,graphs", [("tc", False), ("tc", True), ("fp32", False)])
def test_concurrent_forks_equal_the_parent(gn, engine, graphs):
    import torch

    db, q = _data(120_000, 128, 3100, 1)
    ix = gn.IVFFlatL2Index(n_clusters=256, n_probe=9, engine=engine)
    ix.set(db)
    sizes = [1, 37, 700, 5, 1200, 64, 3, 993]
    offs = np.concatenate([[0], np.cumsum(sizes)])
    ref = [ix.search_knn_arrays(q[o:o + n], 10) for o, n in zip(offs[:-1], sizes)]
    lanes = [ix, ix.fork(), ix.fork()]
    dev = torch.device("cuda", 0)
    if graphs:
        for x in lanes:
            x.enable_graphs(max(sizes), 10)
    dq = torch.from_numpy(q).to(dev)
    streams = [torch.cuda.Stream(dev) for _ in lanes]
    outs = [(torch.empty((n, 10), dtype=torch.int64, device=dev), torch.empty((n, 10), dtype=torch.float32, device=dev),
             torch.empty((n,), dtype=torch.int64, device=dev)) for n in sizes]
    start = torch.cuda.Event()
    start.record()
    for s in streams:
        s.wait_event(start)
    for rep in range(3):  # batches round-robin over the lanes, all in flight together
        for b, (o, n) in enumerate(zip(offs[:-1], sizes)):
            lane = (b + rep) % len(lanes)
            with torch.cuda.stream(streams[lane]):
                lanes[lane].search_knn_device(dq[o:o + n], 10, *outs[b], stream=streams[lane])
        torch.cuda.synchronize()
        for b in range(len(sizes)):
            _same([t.cpu().numpy() for t in outs[b]], ref[b])
    # host entry point on a fork
    _same(lanes[1].search_knn_arrays(q[:300], 10), ix.search_knn_arrays(q[:300], 10))


def test_fork_settings_are_its_own_and_lifetime(gn):
    import gc

    db, q = _data(60_000, 64, 400, 2)
    ix = gn.IVFFlatL2Index(n_clusters=128, n_probe=5, engine="tc")
    ix.set(db)
    base = ix.search_knn_arrays(q, 10)
    f = ix.fork()
    f.n_probe = 20
    wide = f.search_knn_arrays(q, 10)
    _same(ix.search_knn_arrays(q, 10), base)  # the parent keeps n_probe 5
    ix.n_probe = 20
    _same(ix.search_knn_arrays(q, 10), wide)
    ix.n_probe = 5
    f.set_engine("fp32")
    ix.set_engine("fp32")
    ix.n_probe = 20
    _same(f.search_knn_arrays(q, 10), ix.search_knn_arrays(q, 10))
    ix.n_probe = 5
    ix.set_engine("tc")
    # the lists cannot be rebuilt while a fork reads them, nor through a fork
    with pytest.raises(Exception):
        ix.set(db[:1000])
    with pytest.raises(Exception):
        f.set(db[:1000])
    with pytest.raises(Exception):
        f.fork()
    # dropping the parent first: the fork keeps the lists alive
    f.set_engine("tc")
    f.n_probe = 5
    del ix
    gc.collect()
    _same(f.search_knn_arrays(q, 10), base)
    # a fresh parent can be rebuilt once its forks are gone
    p = gn.IVFFlatL2Index(n_clusters=64, n_probe=4, engine="tc")
    p.set(db[:20_000])
    g = p.fork()
    r = g.search_knn_arrays(q[:50], 10)
    del g
    gc.collect()
    p.set(db[:20_000])
    _same(p.search_knn_arrays(q[:50], 10), r)


def test_fork_inherits_the_prober(gn):
    db, q = _data(80_000, 64, 300, 4)
    ix = gn.IVFFlatL2Index(n_clusters=128, n_probe=4, engine="tc")
    ix.set(db)
    pr = gn.LearnedProber(ix, seed=3)
    ix.set_prober(pr, 0.3)
    ref = ix.search_knn_arrays(q, 10)
    f = ix.fork()
    _same(f.search_knn_arrays(q, 10), ref)
    np.testing.assert_array_equal(f.last_lists_probed(len(q)), ix.last_lists_probed(len(q)))


@pytest.mark.parametrize("kind", ["flat", "ivf", "ivf_graphs", "tc"])
def test_threads_sharing_one_index(gn, kind):
    """Blocking host-buffer searches from several threads on ONE index: each
    call holds the index's lock for its whole length (its query, result and
    pinned staging buffers are the index's), so every thread gets exactly the
    results of the same search made alone.  Batch sizes mix small pageable
    copies (staged through pinned memory) and larger ones (copied directly)."""
    from concurrent.futures import ThreadPoolExecutor

    db, q = _data(60_000, 64, 3000, 3)
    if kind == "flat":
        ix = gn.FlatL2Index()
    elif kind == "tc":
        ix = gn.FlatL2TCIndex(shortlist=40)
    else:
        ix = gn.IVFFlatL2Index(n_clusters=128, n_probe=8, engine="tc")
    ix.set(db)
    if kind == "ivf_graphs":
        ix.enable_graphs(2048, 10)
    sizes = [1, 2, 9, 130, 2048, 1, 17, 600, 4, 1]
    offs = np.concatenate([[0], np.cumsum(sizes)])
    jobs = [(o, n) for o, n in zip(offs[:-1], sizes)] * 3
    ref = {(o, n): ix.search_knn_arrays(q[o:o + n], 10) for o, n in zip(offs[:-1], sizes)}
    with ThreadPoolExecutor(4) as pool:
        got = list(pool.map(lambda j: (j, ix.search_knn_arrays(q[j[0]:j[0] + j[1]], 10)), jobs))
    for j, r in got:
        _same(r, ref[j])

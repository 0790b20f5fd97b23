"""Failure path of the tensor-core pipeline's bounded waits, on the GPU
without a fault: the failure drill makes one list scan issue no tile copies
with its waits limited to 200,000 cycles, so the waits run out (nothing ever
completes the barriers they wait on).  The launch must end by itself with
the index's error word set and its tensor memory freed; the search reports
GN_ERR_TIMEOUT (a GpuNearError in Python, the analogue of the reference's
search exceptions, VPTree.hpp:145-147), and the next search on the same
index is correct again (oracle-equal), which also shows that the TMEM was
released and the error word cleared."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _index(gn):
    rng = np.random.default_rng(44)
    c = rng.standard_normal((120, 64), dtype=np.float32)
    db = (c[rng.integers(0, 120, 30000)] + np.float32(0.3) * rng.standard_normal((30000, 64), dtype=np.float32))
    q = (c[rng.integers(0, 120, 300)] + np.float32(0.3) * rng.standard_normal((300, 64), dtype=np.float32))
    ix = gn.IVFFlatL2Index(n_clusters=64, n_probe=6, engine="tc")
    ix.set(db)
    return ix, db, q


def _oracle_check(ix, db, q, oracle, got):
    cent, offs, ids = ix.export()
    labels = np.empty(len(db), np.int32)
    for c in range(len(offs) - 1):
        labels[ids[offs[c]:offs[c + 1]]] = c
    oi, od, oc = oracle.ivfl2_search(db, cent, labels, q, 10, 6)
    idx, dist, cnt = got
    assert np.array_equal(cnt, oc)
    same = idx == oi
    assert np.mean(same) >= 0.995
    np.testing.assert_allclose(dist[same], od[same], rtol=1e-4, atol=1e-3)


def test_expired_wait_is_reported_and_the_index_recovers(gn, oracle):
    from pynear_gb300 import _lib

    ix, db, q = _index(gn)
    ref = ix.search_knn_arrays(q, 10)
    _oracle_check(ix, db, q, oracle, ref)
    lib = _lib.load()
    # host entry point: the failed search raises, the next one is correct
    _lib.check(lib.gn_ivfl2_failure_drill(ix._h.h))
    with pytest.raises(_lib.GpuNearError, match="timed out"):
        ix.search_knn_arrays(q, 10)
    again = ix.search_knn_arrays(q, 10)
    for a, b in zip(again, ref):
        np.testing.assert_array_equal(a, b)


def test_expired_wait_on_the_device_entry_point(gn, oracle):
    import torch
    from pynear_gb300 import _lib

    ix, db, q = _index(gn)
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    d_q = torch.from_numpy(q).to(dev)
    nq = q.shape[0]
    d_i = torch.empty((nq, 10), dtype=torch.int64, device=dev)
    d_d = torch.empty((nq, 10), dtype=torch.float32, device=dev)
    d_c = torch.empty((nq,), dtype=torch.int64, device=dev)
    sp = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)

    def search():
        _lib.check(lib.gn_ivfl2_search_knn_device(ix._h.h, ctypes.c_void_p(d_q.data_ptr()), nq, 10,
                                                  ctypes.c_void_p(d_i.data_ptr()), ctypes.c_void_p(d_d.data_ptr()),
                                                  ctypes.c_void_p(d_c.data_ptr()), sp))
        torch.cuda.synchronize()

    err = ctypes.c_int32(-1)
    search()
    _lib.check(lib.gn_ivfl2_error(ix._h.h, ctypes.byref(err)))
    assert err.value == 0
    _lib.check(lib.gn_ivfl2_failure_drill(ix._h.h))
    search()  # returns without waiting; the caller reads the status
    _lib.check(lib.gn_ivfl2_error(ix._h.h, ctypes.byref(err)))
    assert err.value == 1
    _lib.check(lib.gn_ivfl2_error(ix._h.h, ctypes.byref(err)))
    assert err.value == 0  # read and cleared
    search()
    _lib.check(lib.gn_ivfl2_error(ix._h.h, ctypes.byref(err)))
    assert err.value == 0
    _oracle_check(ix, db, q, oracle, (d_i.cpu().numpy(), d_d.cpu().numpy(), d_c.cpu().numpy()))

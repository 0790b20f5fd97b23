"""The allocation-free Hamming entry point (gn_hamming_knn_noalloc).

It serves callers that cannot allocate device memory at search time; it keeps
its partial lists in a fixed array inside the library.  Checked here against
the allocating entry point (gn_flat_search_knn_device) on the same device
buffers, on two calls in a row (the second call finds the first call's
contents in the shared array) with the device's free memory unchanged
across each call, plus the size, overflow and alignment checks.  This file is collected
last so that a failure here does not hide the other tests' results.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_matches_allocating_entry_point(gn):
    import torch
    from pynear_gb300 import _lib, workloads as W

    lib = _lib.load()
    db, q, src = W.hamming_flips(n=200_000, nbytes=64, nq=3000, flips=24, seed=77)
    n, nbytes, nq, k = db.shape[0], db.shape[1], q.shape[0], 10
    dev = torch.device("cuda", 0)
    d_db = torch.from_numpy(db).to(dev)
    d_q = torch.from_numpy(q).to(dev)
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)

    ix = gn.FlatHammingIndex()
    ix.set(db)
    ref_i = torch.empty((nq, k), dtype=torch.int64, device=dev)
    ref_d = torch.empty((nq, k), dtype=torch.int64, device=dev)
    _lib.check(lib.gn_flat_search_knn_device(ix._h.h, _vp(d_q), nq, k, _vp(ref_i), _vp(ref_d), sp))
    torch.cuda.synchronize()
    assert (ref_i[:, 0].cpu().numpy() == src).all()

    # set-up call (no queries): loads the scan kernels and the fixed array
    _lib.check(lib.gn_hamming_knn_noalloc(_vp(d_db), n, nbytes, _vp(d_q), 0, k, _vp(ref_i), _vp(ref_d), sp))
    torch.cuda.synchronize()
    for call in range(2):
        out_i = torch.full((nq, k), -7, dtype=torch.int64, device=dev)
        out_d = torch.full((nq, k), -7, dtype=torch.int64, device=dev)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info(dev)[0]
        _lib.check(lib.gn_hamming_knn_noalloc(_vp(d_db), n, nbytes, _vp(d_q), nq, k, _vp(out_i), _vp(out_d), sp))
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info(dev)[0]
        assert torch.equal(out_i, ref_i)
        assert torch.equal(out_d, ref_d)
        # the point of the entry point: the device's free memory is untouched
        assert free_after == free_before, (call, free_before, free_after)


def test_noalloc_rejects_requests_beyond_its_scratch(gn):
    import torch
    from pynear_gb300 import _lib

    lib = _lib.load()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(5)
    db = torch.from_numpy(rng.integers(0, 256, (4096, 64), dtype=np.uint8)).to(dev)
    q = torch.from_numpy(rng.integers(0, 256, (10_000, 64), dtype=np.uint8)).to(dev)
    out_i = torch.empty((10_000, 256), dtype=torch.int64, device=dev)
    out_d = torch.empty((10_000, 256), dtype=torch.int64, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    # 10,000 queries x k = 256 = 2.56 Mi keys > the 2 Mi-key scratch
    rc = lib.gn_hamming_knn_noalloc(_vp(db), 4096, 64, _vp(q), 10_000, 256, _vp(out_i), _vp(out_d), stream)
    assert rc == _lib.GN_ERR_INVALID
    assert "scratch" in _lib.last_error()
    # a query count whose product with k wraps 64 bits is rejected, not divided by
    rc = lib.gn_hamming_knn_noalloc(_vp(db), 4096, 64, _vp(q), 1 << 56, 256, _vp(out_i), _vp(out_d), stream)
    assert rc == _lib.GN_ERR_INVALID
    # rows that are not a multiple of 16 bytes are rejected too
    rc = lib.gn_hamming_knn_noalloc(_vp(db), 4096, 60, _vp(q), 16, 10, _vp(out_i), _vp(out_d), stream)
    assert rc == _lib.GN_ERR_INVALID
    # so are buffers that do not start on a 16-byte boundary (rows are read as 16-byte vectors)
    odd = ctypes.c_void_p(db.data_ptr() + 8)
    rc = lib.gn_hamming_knn_noalloc(odd, 4095, 64, _vp(q), 16, 10, _vp(out_i), _vp(out_d), stream)
    assert rc == _lib.GN_ERR_INVALID
    assert "aligned" in _lib.last_error()

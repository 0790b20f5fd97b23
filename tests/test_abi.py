"""CPU-side checks of the C ABI library and the host-side API logic (no GPU)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import REPO


def _declared_symbols():
    text = open(os.path.join(REPO, "include", "gpunear.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gn_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_and_exports_every_declared_symbol(gn):
    from pynear_gb300 import _lib
    lib = ctypes.CDLL(_lib.LIB_PATH)
    names = _declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding declares a signature for every exported entry point
    assert set(names) <= set(_lib.SIGNATURES)


def test_version_and_error_string(gn):
    from pynear_gb300 import _lib
    lib = _lib.load()
    assert lib.gn_version() >= 100
    assert isinstance(_lib.last_error(), str)


def test_status_mapping():
    from pynear_gb300 import _lib
    with pytest.raises(ValueError):
        _lib.check(_lib.GN_ERR_INVALID, "x")
    with pytest.raises(RuntimeError):
        _lib.check(_lib.GN_ERR_EMPTY, "x")
    with pytest.raises(MemoryError):
        _lib.check(_lib.GN_ERR_OOM, "x")
    with pytest.raises(_lib.GpuNearError):
        _lib.check(_lib.GN_ERR_TIMEOUT, "x")
    _lib.check(_lib.GN_OK)


def test_create_rejects_bad_metric(gn):
    from pynear_gb300 import _lib
    h = ctypes.c_void_p()
    assert _lib.load().gn_flat_create(17, ctypes.byref(h)) == _lib.GN_ERR_INVALID
    assert "metric" in _lib.last_error()


def test_binary_wrapper_validation_matches_reference(gn):
    # pynear/__init__.py:99-104: 2-D check first (ValueError), then uint8 (TypeError)
    ix = gn.VPTreeBinaryIndex()
    with pytest.raises(ValueError):
        ix.set(np.zeros((4,), np.uint8))
    with pytest.raises(TypeError):
        ix.set(np.zeros((4, 8), np.float32))
    # searching an index that was never set returns empty lists
    assert ix.search1NN(np.zeros((1, 8), np.uint8)) == ([], [])


def test_float_wrapper_rejects_non_2d(gn):
    ix = gn.VPTreeL2Index()
    with pytest.raises(RuntimeError):
        ix.set(np.zeros((5,), np.float32))


def test_empty_flat_index_raises(gn):
    ix = gn.FlatL2Index()
    with pytest.raises(RuntimeError):
        ix.searchKNN(np.zeros((1, 4), np.float32), 1)


def test_ivf_empty_raises(gn):
    ix = gn.IVFFlatL2Index(n_clusters=4, n_probe=2)
    with pytest.raises(RuntimeError):
        ix.searchKNN(np.zeros((1, 4), np.float32), 1)
    assert ix.n_probe == 2
    assert ix.n_clusters == 0


def test_kmeans_argument_checks(gn):
    with pytest.raises(RuntimeError):
        gn.kmeans_l2(np.zeros((5, 2), np.float32), 6)
    with pytest.raises(RuntimeError):
        gn.kmeans_l2(np.zeros((5,), np.float32), 2)


def test_raster_and_precision_argument_checks_without_gpu(gn):
    """Argument checks of the raster and the shortlist precision run on the
    host before any CUDA call."""
    from pynear_gb300 import _lib
    lib = _lib.load()
    s = np.zeros((4, 2), np.float32)
    xs = np.zeros(3, np.float32)
    out = np.zeros(9, np.int32)
    P = _lib.ptr
    assert lib.gn_voronoi_raster(P(s), 0, P(xs), 3, P(xs), 3, P(out), None, None, 0, None) == _lib.GN_ERR_EMPTY
    assert lib.gn_voronoi_raster(P(s), 4, P(xs), 0, P(xs), 3, P(out), None, None, 0, None) == _lib.GN_ERR_INVALID
    assert lib.gn_voronoi_raster(P(s), 4, P(xs), 3, P(xs), 3, None, None, None, 0, None) == _lib.GN_ERR_INVALID
    rgba = np.zeros(36, np.uint8)
    assert lib.gn_voronoi_raster(P(s), 4, P(xs), 3, P(xs), 3, None, None, None, 0, P(rgba)) == _lib.GN_ERR_INVALID
    assert "palette" in _lib.last_error()
    h = ctypes.c_void_p()
    assert lib.gn_tcflat_create(56, ctypes.byref(h)) == _lib.GN_OK
    assert lib.gn_tcflat_set_precision(h, 2) == _lib.GN_ERR_INVALID
    assert lib.gn_tcflat_set_precision(h, 1) == _lib.GN_OK  # empty index: nothing to convert
    assert lib.gn_index_destroy(h) == _lib.GN_OK
    assert lib.gn_tcflat_create(64, ctypes.byref(h)) == _lib.GN_OK
    assert lib.gn_tcflat_set_precision(h, 1) == _lib.GN_ERR_UNSUPPORTED
    assert lib.gn_index_destroy(h) == _lib.GN_OK
    assert lib.gn_tcflat_create(24, ctypes.byref(h)) == _lib.GN_ERR_INVALID


def test_tc_flat_index_pickles_its_configuration(gn):
    import pickle
    ix = gn.FlatL2TCIndex(shortlist=56, precision="fp8")
    st = ix.__getstate__()
    assert st == {"shortlist": 56, "precision": "fp8", "data": None}
    ix2 = pickle.loads(pickle.dumps(ix))
    assert (ix2.shortlist, ix2.precision, ix2._n) == (56, "fp8", 0)

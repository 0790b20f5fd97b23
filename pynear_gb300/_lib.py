"""ctypes binding of libgpunear.so (the C ABI declared in include/gpunear.h).

The shared library is built in-tree (``python -m pynear_gb300.build``).  There
is no fallback: if the library is missing or no GPU is visible, index calls
raise instead of computing anything on the host.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgpunear.so")

GN_OK = 0
GN_ERR_INVALID = 1
GN_ERR_EMPTY = 2
GN_ERR_CUDA = 3
GN_ERR_OOM = 4
GN_ERR_TIMEOUT = 5
GN_ERR_UNSUPPORTED = 6

METRIC_L2 = 0
METRIC_L1 = 1
METRIC_LINF = 2
METRIC_HAMMING = 3

P = ctypes.c_void_p
I32 = ctypes.c_int32
I64 = ctypes.c_int64
U32 = ctypes.c_uint32
PP = ctypes.POINTER(ctypes.c_void_p)

# name -> argtypes; every function returns int (gn_status) unless listed in _RESTYPE
SIGNATURES = {
    "gn_version": [],
    "gn_last_error": [],
    "gn_device_info": [P, P, P],
    "gn_timing_enable": [ctypes.c_int],
    "gn_timing_last": [P, ctypes.c_char_p, ctypes.c_int],
    "gn_flat_create": [ctypes.c_int, PP],
    "gn_flat_set": [P, P, I64, I64],
    "gn_flat_search_knn": [P, P, I64, I64, P, P],
    "gn_flat_search_1nn": [P, P, I64, P, P],
    "gn_flat_search_knn_device": [P, P, I64, I64, P, P, P],
    "gn_index_size": [P, P, P],
    "gn_index_destroy": [P],
    "gn_dist": [I32, P, P, I64, P],
    "gn_hamming_knn_noalloc": [P, I64, I64, P, I64, I64, P, P, P],
    "gn_tcflat_create": [I32, PP],
    "gn_tcflat_set": [P, P, I64, I64],
    "gn_tcflat_search_knn": [P, P, I64, I64, P, P],
    "gn_tcflat_search_knn_device": [P, P, I64, I64, P, P, P],
    "gn_tcflat_set_precision": [P, I32],
    "gn_tc_error": [P, P],
    "gn_kmeans_l2": [P, I64, I64, I64, I64, U32, P, P, P],
    "gn_ivfl2_create": [I32, I32, PP],
    "gn_ivfl2_set": [P, P, I64, I64],
    "gn_ivfl2_set_assigned": [P, P, I64, I64, P, I32, P],
    "gn_ivfl2_fork": [P, PP],
    "gn_ivfl2_search_knn": [P, P, I64, I64, P, P, P],
    "gn_ivfl2_search_knn_device": [P, P, I64, I64, P, P, P, P],
    "gn_ivfl2_enable_graphs": [P, I64, I32],
    "gn_ivfl2_graph_info": [P, P],
    "gn_mih_create": [I32, PP],
    "gn_mih_set": [P, P, I64, I64],
    "gn_mih_search_knn": [P, P, I64, I64, I32, P, P, P],
    "gn_mih_info": [P, P, P, P],
    "gn_ivfl2_autotune": [P, P, I64, I64, I32, P],
    "gn_ivfl2_get_tuning": [P, P],
    "gn_ivfl2_set_tuning": [P, P],
    "gn_ivfl2_set_n_probe": [P, I32],
    "gn_ivfl2_set_mode": [P, I32, I32],
    "gn_ivfl2_error": [P, P],
    "gn_ivfl2_failure_drill": [P],
    "gn_ivfl2_last_work": [P, P],
    "gn_ivfl2_info": [P, P, P, P, P],
    "gn_ivfl2_export": [P, P, P, P],
    "gn_prober_create": [I32, U32, PP],
    "gn_prober_num_params": [P, P],
    "gn_prober_get_params": [P, P],
    "gn_prober_set_params": [P, P],
    "gn_prober_loss_grad": [P, I64, P, P, P, P, P],
    "gn_prober_train": [P, P, P, I64, P, I32, I32, I32, ctypes.c_float, P],
    "gn_ivfl2_set_prober": [P, P, ctypes.c_float],
    "gn_ivfl2_last_nprobed": [P, I64, P],
    "gn_ivfbin_create": [I32, I32, I32, U32, PP],
    "gn_ivfbin_set": [P, P, I64, I64],
    "gn_ivfbin_search_knn": [P, P, I64, I64, P, P, P],
    "gn_ivfbin_get_params": [P, P, P],
    "gn_ivfbin_set_nprobe": [P, I32],
    "gn_ivfbin_export": [P, P, P, P],
    "gn_voronoi_raster": [P, I64, P, I64, P, I64, P, P, P, I64, P],
    "gn_voronoi_raster_device": [P, I64, P, I64, P, I64, P, P, P, I64, P, P],
}
_RESTYPE = {"gn_last_error": ctypes.c_char_p}

_lib = None
_lock = threading.Lock()


class GpuNearError(RuntimeError):
    pass


def load():
    """Load libgpunear.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(
                    f"{LIB_PATH} is missing: build the CUDA library first (python -m pynear_gb300.build)")
            lib = ctypes.CDLL(LIB_PATH)
            for name, args in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.argtypes = args
                fn.restype = _RESTYPE.get(name, ctypes.c_int)
            _lib = lib
    return _lib


def last_error() -> str:
    msg = load().gn_last_error()
    return msg.decode("utf-8", "replace") if msg else ""


def check(status: int, what: str = "") -> None:
    if status == GN_OK:
        return
    msg = last_error() or what
    if status == GN_ERR_INVALID:
        raise ValueError(msg)
    if status == GN_ERR_OOM:
        raise MemoryError(msg)
    if status in (GN_ERR_EMPTY, GN_ERR_UNSUPPORTED):
        raise RuntimeError(msg)
    raise GpuNearError(f"{msg} (status {status})")


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)


class Handle:
    """Owns one gn_index*; destroyed with the Python object."""

    def __init__(self, creator: str, *args):
        h = ctypes.c_void_p()
        call(creator, *args, ctypes.byref(h))
        self.h = h

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value and _lib is not None:
            _lib.gn_index_destroy(h)
            self.h = None

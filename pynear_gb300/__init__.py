"""pynear_gb300 — GB300-native exact and IVF nearest-neighbour search.

The index classes keep PyNear's API (``set`` / ``searchKNN`` / ``search1NN``
returning ``(indices, distances)``) and run every search on the GPU through
libgpunear.so (C ABI in include/gpunear.h).
"""
from .flat import (FlatChebyshevIndex, FlatHammingIndex, FlatL1Index, FlatL2Index, FlatL2TCIndex, VPTreeBinaryIndex,
                   VPTreeChebyshevIndex, VPTreeL1Index, VPTreeL2Index, dist_chebyshev, dist_hamming, dist_l1,
                   dist_l2)
from .ivf import IVFFlatBinaryIndex, IVFFlatL2Index, kmeans_l2
from .mih import MIHBinaryIndex
from .prober import LearnedProber
from .sklearn_adapter import PyNearKNeighborsClassifier, PyNearKNeighborsRegressor, PyNearNearestNeighbors
from .voronoi import make_palette, voronoi_raster, voronoi_raster_device, write_png

__version__ = "0.1.0"

__all__ = [
    "FlatL2Index", "FlatL2TCIndex", "FlatL1Index", "FlatChebyshevIndex", "FlatHammingIndex",
    "VPTreeL2Index", "VPTreeL1Index", "VPTreeChebyshevIndex", "VPTreeBinaryIndex",
    "IVFFlatL2Index", "IVFFlatBinaryIndex", "MIHBinaryIndex", "kmeans_l2", "LearnedProber",
    "dist_l2", "dist_l1", "dist_chebyshev", "dist_hamming",
    "PyNearNearestNeighbors", "PyNearKNeighborsClassifier", "PyNearKNeighborsRegressor",
    "voronoi_raster", "voronoi_raster_device", "make_palette", "write_png",
]

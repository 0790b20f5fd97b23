"""Headless Voronoi raster: the nearest seed of every pixel of a grid.

Replaces the compute of the reference's Voronoi demo (demo/voronoi.py:84-110),
which builds the pixel grid on the host (pixel (r, c) = (xs[c], ys[r]) with
``xs = linspace(0, 1, w)``, ``ys = linspace(0, 1, h)``), runs one
``VPTreeL2Index.search1NN`` of all pixels against the seeds and colours the
result through a palette.  Here one GPU kernel reads the two axis vectors and
writes seed ids, distances and RGBA pixels straight into device (or host)
buffers; there is no window or graphics API, and an image is written to a PNG
file when one is wanted.  Distances follow the reference's L2 arithmetic bit
for bit; where two seeds are at exactly the same distance the lower seed index
is returned (the reference's tree picks either).
"""
from __future__ import annotations

import colorsys
import struct
import zlib
from typing import NamedTuple

import numpy as np

from . import _lib


class Raster(NamedTuple):
    ids: np.ndarray            # (h, w) int32 nearest seed
    dist: np.ndarray | None    # (h, w) float32 L2 distance, when asked for
    rgba: np.ndarray | None    # (h, w, 4) uint8 palette colour, when a palette is given


def make_palette(n: int) -> np.ndarray:
    """n distinct RGBA colours by golden-angle hue steps (the reference demo's
    palette rule, demo/voronoi.py:31-38): hue i*137.508 degrees, saturation
    0.5, value 0.88, opaque."""
    out = np.empty((int(n), 4), np.uint8)
    for i in range(int(n)):
        r, g, b = colorsys.hsv_to_rgb(((i * 137.508) % 360) / 360, 0.50, 0.88)
        out[i] = (int(r * 255), int(g * 255), int(b * 255), 255)
    return out


def grid_axes(width: int, height: int) -> tuple[np.ndarray, np.ndarray]:
    """The demo's pixel axes: xs = linspace(0, 1, width), ys = linspace(0, 1, height), float32."""
    return np.linspace(0, 1, int(width), dtype=np.float32), np.linspace(0, 1, int(height), dtype=np.float32)


def _seeds(seeds) -> np.ndarray:
    arr = np.ascontiguousarray(seeds, dtype=np.float32)
    if arr.ndim != 2 or arr.shape[1] != 2:
        raise ValueError("seeds must have shape (n, 2)")
    if arr.shape[0] == 0:
        raise RuntimeError("voronoi raster needs at least one seed")
    return arr


def _palette(palette) -> np.ndarray:
    pal = np.ascontiguousarray(palette, dtype=np.uint8)
    if pal.ndim != 2 or pal.shape[1] != 4 or pal.shape[0] == 0:
        raise ValueError("palette must have shape (n, 4) uint8 RGBA, n >= 1")
    return pal


def voronoi_raster(seeds, width: int | None = None, height: int | None = None, *, xs=None, ys=None,
                   palette=None, with_distance: bool = False) -> Raster:
    """Nearest seed of every pixel of a height x width grid.

    The grid is either the demo's unit square (``width``/``height``) or given
    by its axes ``xs`` (width floats) and ``ys`` (height floats).  With a
    ``palette`` ((n, 4) uint8) the raster is also coloured:
    ``rgba[r, c] = palette[ids[r, c] % n]``.
    """
    s = _seeds(seeds)
    if xs is None or ys is None:
        if width is None or height is None:
            raise ValueError("give width and height, or the grid axes xs and ys")
        gx, gy = grid_axes(width, height)
        xs = gx if xs is None else xs
        ys = gy if ys is None else ys
    xs = np.ascontiguousarray(xs, dtype=np.float32).ravel()
    ys = np.ascontiguousarray(ys, dtype=np.float32).ravel()
    w, h = len(xs), len(ys)
    if w == 0 or h == 0:
        raise ValueError("raster width and height must be positive")
    ids = np.empty((h, w), np.int32)
    dist = np.empty((h, w), np.float32) if with_distance else None
    pal = rgba = None
    if palette is not None:
        pal = _palette(palette)
        rgba = np.empty((h, w, 4), np.uint8)
    _lib.call("gn_voronoi_raster", _lib.ptr(s), s.shape[0], _lib.ptr(xs), w, _lib.ptr(ys), h, _lib.ptr(ids),
              _lib.ptr(dist), _lib.ptr(pal), 0 if pal is None else pal.shape[0], _lib.ptr(rgba))
    return Raster(ids, dist, rgba)


def voronoi_raster_device(seeds, xs, ys, palette=None, with_distance: bool = False, stream=None) -> Raster:
    """The same raster on CUDA torch tensors (seeds (n, 2) float32, xs, ys
    float32 vectors, palette (n, 4) uint8), launched on ``stream`` (default:
    torch's current stream) without a host synchronisation; the outputs are
    new device tensors."""
    import torch

    for name, t in (("seeds", seeds), ("xs", xs), ("ys", ys)):
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
            raise ValueError(f"{name} must be a contiguous float32 CUDA tensor")
    if seeds.dim() != 2 or seeds.shape[1] != 2:
        raise ValueError("seeds must have shape (n, 2)")
    w, h = xs.numel(), ys.numel()
    dev = seeds.device
    ids = torch.empty((h, w), dtype=torch.int32, device=dev)
    dist = torch.empty((h, w), dtype=torch.float32, device=dev) if with_distance else None
    rgba = None
    if palette is not None:
        if not (palette.is_cuda and palette.dtype == torch.uint8 and palette.dim() == 2 and palette.shape[1] == 4
                and palette.is_contiguous()):
            raise ValueError("palette must be a contiguous (n, 4) uint8 CUDA tensor")
        rgba = torch.empty((h, w, 4), dtype=torch.uint8, device=dev)
    st = stream if stream is not None else torch.cuda.current_stream(dev)
    _lib.call("gn_voronoi_raster_device", seeds.data_ptr(), seeds.shape[0], xs.data_ptr(), w, ys.data_ptr(), h,
              ids.data_ptr(), None if dist is None else dist.data_ptr(),
              None if palette is None else palette.data_ptr(), 0 if palette is None else palette.shape[0],
              None if rgba is None else rgba.data_ptr(), st.cuda_stream)
    return Raster(ids, dist, rgba)


def write_png(path: str, rgba: np.ndarray) -> None:
    """Write an (h, w, 4) uint8 image as an 8-bit RGBA PNG (no imaging library needed)."""
    img = np.ascontiguousarray(rgba, dtype=np.uint8)
    if img.ndim != 3 or img.shape[2] != 4:
        raise ValueError("image must have shape (h, w, 4)")
    h, w = img.shape[:2]
    raw = np.concatenate([np.zeros((h, 1), np.uint8), img.reshape(h, w * 4)], axis=1).tobytes()

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))

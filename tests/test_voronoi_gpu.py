"""Headless Voronoi raster on the GPU against the reference demo's own output
(tests/golden/voronoi.npz), the exact flat search1NN over the materialised
pixel grid, and the NumPy oracle."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _grid(xs, ys):
    gx, gy = np.meshgrid(xs, ys)
    return np.column_stack([gx.ravel(), gy.ravel()])


def test_matches_reference_demo_raster(gn, oracle):
    g = golden("voronoi.npz")
    for t in "abc":
        seeds = g[f"{t}_seeds"]
        w, h = (int(v) for v in g[f"{t}_wh"])
        r = gn.voronoi_raster(seeds, w, h, with_distance=True)
        assert r.ids.shape == (h, w) and r.ids.dtype == np.int32
        ref_ids, ref_dist = g[f"{t}_ids"], g[f"{t}_dist"]
        assert np.array_equal(r.dist.view(np.uint32), ref_dist.view(np.uint32)), t
        # the ids agree except where two seeds are at exactly the same distance
        xs, ys = gn.voronoi.grid_axes(w, h)
        rr, cc = np.nonzero(r.ids != ref_ids)
        dx = xs[cc] - seeds[ref_ids[rr, cc], 0]
        dy = ys[rr] - seeds[ref_ids[rr, cc], 1]
        assert np.array_equal(np.sqrt(dx * dx + dy * dy), r.dist[rr, cc]), t
        if t != "c":
            assert len(rr) == 0
        # against the oracle (ties to the lower index): identical
        o_ids, o_dist = oracle.voronoi_raster(seeds, xs, ys)
        assert np.array_equal(r.ids, o_ids)
        assert np.array_equal(r.dist.view(np.uint32), o_dist.view(np.uint32))


def test_matches_flat_search1nn_over_grid(gn):
    rng = np.random.default_rng(21)
    seeds = rng.random((64, 2), dtype=np.float32)
    xs, ys = gn.voronoi.grid_axes(333, 187)
    r = gn.voronoi_raster(seeds, xs=xs, ys=ys, with_distance=True)
    ix = gn.FlatL2Index()
    ix.set(seeds)
    idx, dist = ix.search_knn_arrays(_grid(xs, ys), 1)
    assert np.array_equal(r.ids.ravel(), idx.ravel())
    assert np.array_equal(r.dist.ravel().view(np.uint32), dist.ravel().view(np.uint32))


@pytest.mark.parametrize("ns,w,h", [(1, 17, 9), (2047, 130, 40), (2048, 64, 33), (5000, 300, 120), (6, 3, 70001)])
def test_tiles_strips_and_rows_against_oracle(gn, oracle, ns, w, h):
    # seed counts around the 2048-seed tile, widths around the 1024-pixel strip,
    # and more rows than one grid dimension holds (the kernel strides over rows)
    rng = np.random.default_rng(ns + w)
    seeds = (rng.random((ns, 2), dtype=np.float32) * 1.2 - 0.1).astype(np.float32)
    xs = np.sort(rng.random(w, dtype=np.float32))
    ys = np.linspace(-0.2, 1.3, h, dtype=np.float32)
    r = gn.voronoi_raster(seeds, xs=xs, ys=ys, with_distance=True)
    if h > 10000:  # the oracle on a row subset
        rows = np.r_[0:50, h // 2:h // 2 + 50, h - 50:h]
        o_ids, o_dist = oracle.voronoi_raster(seeds, xs, ys[rows])
        got_ids, got_dist = r.ids[rows], r.dist[rows]
    else:
        o_ids, o_dist = oracle.voronoi_raster(seeds, xs, ys)
        got_ids, got_dist = r.ids, r.dist
    assert np.array_equal(got_ids, o_ids)
    assert np.array_equal(got_dist.view(np.uint32), o_dist.view(np.uint32))


def test_duplicate_seeds_tie_to_lower_index(gn):
    seeds = np.array([[0.5, 0.5], [0.2, 0.8], [0.5, 0.5], [0.2, 0.8], [0.9, 0.1]], np.float32)
    r = gn.voronoi_raster(seeds, 50, 40)
    assert set(np.unique(r.ids)) <= {0, 1, 4}
    # two seeds mirrored about x = 0.5: the column at exactly x = 0.5 goes to the lower index
    seeds = np.array([[0.75, 0.5], [0.25, 0.5]], np.float32)
    xs = np.array([0.25, 0.5, 0.75], np.float32)
    r = gn.voronoi_raster(seeds, xs=xs, ys=np.array([0.1, 0.5], np.float32))
    assert r.ids.tolist() == [[1, 0, 0], [1, 0, 0]]


def test_palette_colours_and_device_path(gn):
    import torch

    rng = np.random.default_rng(5)
    seeds = rng.random((100, 2), dtype=np.float32)
    pal = gn.make_palette(64)
    r = gn.voronoi_raster(seeds, 256, 144, palette=pal, with_distance=True)
    assert np.array_equal(r.rgba, pal[r.ids % 64])
    xs, ys = gn.voronoi.grid_axes(256, 144)
    dev = torch.device("cuda:0")
    d = gn.voronoi_raster_device(torch.from_numpy(seeds).to(dev), torch.from_numpy(xs).to(dev),
                                 torch.from_numpy(ys).to(dev), palette=torch.from_numpy(pal).to(dev),
                                 with_distance=True)
    torch.cuda.synchronize()
    assert np.array_equal(d.ids.cpu().numpy(), r.ids)
    assert np.array_equal(d.dist.cpu().numpy().view(np.uint32), r.dist.view(np.uint32))
    assert np.array_equal(d.rgba.cpu().numpy(), r.rgba)
    only_rgba = gn.voronoi_raster(seeds, 256, 144, palette=pal)
    assert np.array_equal(only_rgba.rgba, r.rgba)


def test_errors(gn):
    with pytest.raises(RuntimeError):
        gn.voronoi_raster(np.zeros((0, 2), np.float32), 4, 4)
    with pytest.raises(ValueError):
        gn.voronoi_raster(np.zeros((3, 3), np.float32), 4, 4)
    with pytest.raises(ValueError):
        gn.voronoi_raster(np.zeros((3, 2), np.float32), 4, 4, palette=np.zeros((0, 4), np.uint8))
    with pytest.raises(ValueError):
        gn.voronoi_raster(np.zeros((3, 2), np.float32))


def test_lattice_seeds_many_ties_against_oracle(gn, oracle):
    """Seeds and pixels on lattices: many pixels are equally far from several
    seeds (and from seeds that repeat), so the kernel's four-seed groups often
    hold equal or nearly equal distances; ids (ties to the lower index) and
    distance bits equal the oracle's."""
    rng = np.random.default_rng(5)
    seeds = (rng.integers(0, 33, (3001, 2)) / np.float32(32.0)).astype(np.float32)
    xs = np.linspace(0, 1, 129, dtype=np.float32)
    ys = np.linspace(0, 1, 65, dtype=np.float32)
    r = gn.voronoi_raster(seeds, xs=xs, ys=ys, with_distance=True)
    o_ids, o_dist = oracle.voronoi_raster(seeds, xs, ys)
    assert np.array_equal(r.ids, o_ids)
    assert np.array_equal(r.dist.view(np.uint32), o_dist.view(np.uint32))

"""Generate the golden fixtures in this folder from the reference itself.

Run in a container that holds the PyNear 2.2.0 source tree, named by the
PYNEAR_REFERENCE environment variable, after ``bash oracle/build_ref.sh`` has
built its extension into oracle/_ref/:

    PYNEAR_REFERENCE=<source tree> python tests/golden/make_golden.py

Every fixture stores seeded inputs plus the reference's own outputs for them,
produced through its public Python API (the _pynear extension and the pynear
package's IVFFlatL2Index).  Machines without the reference tree (the GPU hosts)
read only these committed .npz files.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("PYNEAR_REFERENCE")
if not REF:
    sys.exit("make_golden: set PYNEAR_REFERENCE to the PyNear 2.2.0 source tree")
sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))
sys.path.insert(0, REF)

import _pynear  # noqa: E402  (reference extension built from its sources)
import pynear  # noqa: E402  (reference Python package)


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print("wrote", path, os.path.getsize(path), "bytes")


def float_distances():
    rng = np.random.default_rng(100)
    dims = np.array([1, 3, 4, 5, 7, 8, 9, 12, 13, 16, 17, 31, 32, 33, 64, 100, 128, 512], np.int64)
    per = 24
    out = {"dims": dims}
    for d in dims:
        a = rng.random((per, d), dtype=np.float32) * 4 - 2
        b = rng.random((per, d), dtype=np.float32) * 4 - 2
        out[f"a{d}"] = a
        out[f"b{d}"] = b
        out[f"l2_{d}"] = np.array([_pynear.dist_l2(a[i], b[i]) for i in range(per)], np.float32)
        out[f"l1_{d}"] = np.array([_pynear.dist_l1(a[i], b[i]) for i in range(per)], np.float32)
        out[f"linf_{d}"] = np.array([_pynear.dist_chebyshev(a[i], b[i]) for i in range(per)], np.float32)
    save("dist_float.npz", **out)


def hamming_kat():
    # Cases of the reference's C++ Hamming test (tests/VPTreeTests.cpp:51-99),
    # rebuilt here and evaluated by the reference's own dist_hamming_* bindings.
    full32 = [255] * 32
    cases = []
    cases.append(([255] * 8, [255] * 8))
    cases.append(([1] + full32[1:], [2] + full32[1:]))
    cases.append((full32, [0] + full32[1:]))
    x = list(full32); x[5] = 253
    cases.append((x, [0] + full32[1:]))
    y = list(x); y[7] = 9
    z = [0] + full32[1:]; z[7] = 0
    cases.append((y, z))
    cases.append((full32, [0] * 32))
    rng = np.random.default_rng(101)
    for nb in (8, 16, 32, 64):
        for _ in range(20):
            cases.append((list(rng.integers(0, 256, nb)), list(rng.integers(0, 256, nb))))
    fn = {8: _pynear.dist_hamming_64, 16: _pynear.dist_hamming_128, 32: _pynear.dist_hamming_256,
          64: _pynear.dist_hamming_512}
    A = np.zeros((len(cases), 64), np.uint8)
    B = np.zeros_like(A)
    W = np.zeros(len(cases), np.int64)
    D = np.zeros(len(cases), np.int64)
    for i, (a, b) in enumerate(cases):
        A[i, : len(a)] = a
        B[i, : len(b)] = b
        W[i] = len(a)
        D[i] = fn[len(a)](np.array(a, np.uint8), np.array(b, np.uint8))
    save("hamming_kat.npz", a=A, b=B, width=W, dist=D)


def vptree_float():
    rng = np.random.default_rng(102)
    out = {}
    sets = {}
    for tag, n, d, nq, k in (("a", 2021, 8, 16, 5), ("b", 2500, 32, 16, 10), ("c", 1501, 13, 8, 7)):
        sets[tag] = (rng.random((n, d), dtype=np.float32), rng.random((nq, d), dtype=np.float32), k)
        out[f"{tag}_db"], out[f"{tag}_q"] = sets[tag][0], sets[tag][1]
    for name, cls in (("l2", _pynear.VPTreeL2Index), ("l1", _pynear.VPTreeL1Index),
                      ("linf", _pynear.VPTreeChebyshevIndex)):
        for tag, (db, q, k) in sets.items():
            t = cls()
            t.set(db)
            ki, kd = t.searchKNN(q, k)
            i1, d1 = t.search1NN(q)
            # stored nearest-first (the reference returns farthest-first)
            out[f"{name}_{tag}_idx"] = np.array(ki, np.int64)[:, ::-1].copy()
            out[f"{name}_{tag}_dist"] = np.array(kd, np.float32)[:, ::-1].copy()
            out[f"{name}_{tag}_idx1"] = np.array(i1, np.int64)
            out[f"{name}_{tag}_dist1"] = np.array(d1, np.float32)
    save("vptree_float.npz", **out)


def flip_bits(vec, n_flips, rng):
    out = vec.copy()
    bits = rng.choice(len(out) * 8, size=n_flips, replace=False)
    for b in bits:
        out[b // 8] ^= np.uint8(1 << (b % 8))
    return out


def vptree_binary():
    rng = np.random.default_rng(103)
    out = {}
    for tag, n, nb, nq, k in (("a", 4000, 64, 16, 10), ("b", 3000, 32, 8, 5), ("c", 2000, 16, 8, 3),
                              ("d", 2000, 8, 8, 4)):
        db = rng.integers(0, 256, (n, nb), dtype=np.uint8)
        src = rng.integers(0, n, nq)
        q = np.array([flip_bits(db[i], min(24, nb * 8 // 4), rng) for i in src], np.uint8)
        t = pynear.VPTreeBinaryIndex()
        t.set(db)
        ki, kd = t.searchKNN(q, k)
        out[f"{tag}_db"] = db
        out[f"{tag}_q"] = q
        out[f"{tag}_idx"] = np.array(ki, np.int64)[:, ::-1].copy()
        out[f"{tag}_dist"] = np.array(kd, np.int64)[:, ::-1].copy()
    save("vptree_binary.npz", **out)


def kmeans():
    rng = np.random.default_rng(104)
    out = {}
    for tag, n, d, k in (("a", 3000, 16, 20), ("b", 1500, 7, 33)):
        data = rng.random((n, d), dtype=np.float32)
        labels, cent = _pynear.kmeans_l2(data, k, 100, 42)
        out[f"{tag}_data"] = data
        out[f"{tag}_labels"] = labels
        out[f"{tag}_cent"] = cent
    save("kmeans.npz", **out)


def ivf_binary():
    rng = np.random.default_rng(105)
    out = {}
    for tag, n, nb, nlist, nprobe, k in (("a", 3000, 64, 32, 4, 10), ("b", 1500, 32, 16, 16, 5),
                                         ("c", 50, 64, 10, 1, 100)):
        db = rng.integers(0, 256, (n, nb), dtype=np.uint8)
        src = rng.integers(0, n, 24)
        q = np.array([flip_bits(db[i], 6, rng) for i in src], np.uint8)
        ix = _pynear.IVFFlatBinaryIndex(nlist=nlist, nprobe=nprobe)
        ix.set(db)
        ri, rd = ix.searchKNN(q, k)
        cnt = np.array([len(r) for r in ri], np.int64)
        I = np.full((len(q), k), -1, np.int64)
        D = np.zeros((len(q), k), np.int64)
        for i in range(len(q)):
            I[i, : cnt[i]] = ri[i]
            D[i, : cnt[i]] = rd[i]
        out.update({f"{tag}_db": db, f"{tag}_q": q, f"{tag}_idx": I, f"{tag}_dist": D, f"{tag}_cnt": cnt,
                    f"{tag}_cfg": np.array([nlist, nprobe, k], np.int64)})
    save("ivf_binary.npz", **out)


def ivf_l2():
    rng = np.random.default_rng(106)
    out = {}
    for tag, n, d, nc, npb, k in (("a", 2000, 32, 20, 5, 10), ("b", 500, 16, 10, 10, 4)):
        data = rng.random((n, d), dtype=np.float32)
        q = rng.random((16, d), dtype=np.float32)
        ix = pynear.IVFFlatL2Index(n_clusters=nc, n_probe=npb)
        ix.set(data)
        ri, rd = ix.searchKNN(q, k)
        labels, cent = _pynear.kmeans_l2(data, nc, 100, 42)
        out.update({f"{tag}_db": data, f"{tag}_q": q, f"{tag}_idx": np.array(ri, np.int64),
                    f"{tag}_dist": np.array(rd, np.float32), f"{tag}_labels": labels, f"{tag}_cent": cent,
                    f"{tag}_cfg": np.array([nc, npb, k], np.int64)})
    save("ivf_l2.npz", **out)


def voronoi():
    # The reference demo's raster (demo/voronoi.py:93-110): pixel grid from
    # linspace(0, 1) axes, one VPTreeL2Index.search1NN of every pixel against
    # the seeds.  The last case repeats seeds, so some pixels tie.
    rng = np.random.default_rng(107)
    out = {}
    for tag, w, h, ns in (("a", 97, 61, 16), ("b", 160, 90, 64), ("c", 64, 48, 40)):
        seeds = rng.random((ns, 2), dtype=np.float32)
        if tag == "c":
            seeds[20:] = seeds[:20]
        xs = np.linspace(0, 1, w, dtype=np.float32)
        ys = np.linspace(0, 1, h, dtype=np.float32)
        gx, gy = np.meshgrid(xs, ys)
        grid = np.column_stack([gx.ravel(), gy.ravel()])
        t = _pynear.VPTreeL2Index()
        t.set(seeds)
        i1, d1 = t.search1NN(grid)
        out.update({f"{tag}_seeds": seeds, f"{tag}_wh": np.array([w, h], np.int64),
                    f"{tag}_ids": np.array(i1, np.int32).reshape(h, w),
                    f"{tag}_dist": np.array(d1, np.float32).reshape(h, w)})
    save("voronoi.npz", **out)


def mih():
    # MIHBinaryIndex (pynear/include/MIH.hpp:58-175) on the shapes of the
    # reference's tests/test_binary_approx.py:120-170 (random rows, queries a
    # few flipped bits away) and on clustered rows (bases with up to 6 flipped
    # bits), where many candidates and distance ties occur.
    def flip(vec, nf, rng):
        out = vec.copy()
        for b in rng.choice(len(out) * 8, size=nf, replace=False):
            out[b // 8] ^= np.uint8(1 << (b % 8))
        return out

    def clustered(nbase, per, nb, maxflip, rng):
        base = rng.integers(0, 256, (nbase, nb), dtype=np.uint8)
        rows = np.array([flip(base[i], int(rng.integers(0, maxflip + 1)), rng) for i in range(nbase)
                         for _ in range(per)])
        return rows[rng.permutation(len(rows))], base

    rng = np.random.default_rng(108)
    cases = []
    db = rng.integers(0, 256, (2000, 64), dtype=np.uint8)
    cases.append(("a", db, np.array([flip(db[i], 5, rng) for i in range(0, 200, 20)]), 8, 10, 8))
    db, base = clustered(50, 40, 64, 6, rng)
    cases.append(("b", db, np.array([flip(base[i % 50], 2, rng) for i in range(30)]), 8, 10, 16))
    db, base = clustered(40, 25, 32, 5, rng)
    cases.append(("c", db, np.array([flip(base[i % 40], 3, rng) for i in range(20)]), 4, 5, 8))
    db, base = clustered(30, 30, 16, 4, rng)
    cases.append(("d", db, np.array([flip(base[i % 30], 1, rng) for i in range(20)]), 4, 8, 12))
    out = {}
    for tag, db, q, m, k, radius in cases:
        ix = _pynear.MIHBinaryIndex(m)
        ix.set(db)
        ri, rd = ix.searchKNN(q, k, radius)
        idx = np.full((len(q), k), -1, np.int64)
        dist = np.zeros((len(q), k), np.int64)
        cnt = np.array([len(r) for r in ri], np.int64)
        for i, (r, d) in enumerate(zip(ri, rd)):
            idx[i, :len(r)] = r
            dist[i, :len(d)] = d
        out.update({f"{tag}_db": db, f"{tag}_q": q, f"{tag}_cfg": np.array([m, k, radius], np.int64),
                    f"{tag}_idx": idx, f"{tag}_dist": dist, f"{tag}_cnt": cnt})
    save("mih.npz", **out)


ALL = (float_distances, hamming_kat, vptree_float, vptree_binary, kmeans, ivf_binary, ivf_l2, voronoi, mih)

if __name__ == "__main__":
    # optional arguments name the fixtures to (re)generate; none = all
    want = set(sys.argv[1:])
    for fn in ALL:
        if not want or fn.__name__ in want:
            fn()

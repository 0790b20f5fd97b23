"""Seeded synthetic workloads with the shapes and distributions of the
benchmark configurations (no dataset files are read).

* uniform_l2:     database rng.random((100000, 32)), queries rng.random((1000, 32))
* hamming_flips:  database of uniform bytes, queries = random rows with exactly
                  `flips` distinct bits flipped
* gaussian_mixture: `n_centres` centres ~ N(0, I_d); component sizes uniform or
                  Zipf(s) over ranks 1..n_centres, normalised to n; points =
                  centre + N(0, sigma^2 I); queries drawn from the same mixture
"""
from __future__ import annotations

import numpy as np


def uniform_l2(n=100_000, d=32, nq=1000, seed=0):
    rng = np.random.default_rng(seed)
    return rng.random((n, d), dtype=np.float32), rng.random((nq, d), dtype=np.float32)


def hamming_flips(n=1_000_000, nbytes=64, nq=10_000, flips=24, seed=2024):
    rng = np.random.default_rng(seed)
    db = rng.integers(0, 256, (n, nbytes), dtype=np.uint8)
    src = rng.integers(0, n, nq)
    bits = np.argsort(rng.random((nq, nbytes * 8)), axis=1)[:, :flips]
    mask = np.zeros((nq, nbytes * 8), np.uint8)
    np.put_along_axis(mask, bits, 1, axis=1)
    q = db[src] ^ np.packbits(mask, axis=1, bitorder="little")
    return db, q, src


def zipf_sizes(n, n_centres, s):
    w = 1.0 / np.arange(1, n_centres + 1, dtype=np.float64) ** s
    sizes = np.floor(w / w.sum() * n).astype(np.int64)
    sizes[0] += n - sizes.sum()  # the remainder goes to the largest component
    return sizes


def gaussian_mixture(n=1_000_000, d=512, n_centres=2048, sigma=0.3, zipf_s=1.1, nq=10_000, seed=0,
                     query_seed=None):
    """Returns (database, queries, centres, component of each database row)."""
    rng = np.random.default_rng(seed)
    centres = rng.standard_normal((n_centres, d), dtype=np.float32)
    if zipf_s:
        sizes = zipf_sizes(n, n_centres, zipf_s)
    else:
        sizes = np.full(n_centres, n // n_centres, np.int64)
        sizes[: n - sizes.sum()] += 1
    comp = np.repeat(np.arange(n_centres), sizes)
    rng.shuffle(comp)
    db = np.empty((n, d), np.float32)
    step = 1 << 16
    for i in range(0, n, step):
        c = comp[i:i + step]
        db[i:i + step] = centres[c] + np.float32(sigma) * rng.standard_normal((len(c), d), dtype=np.float32)
    queries = mixture_queries(centres, sizes, nq, sigma, seed if query_seed is None else query_seed)
    return db, queries, centres, comp


def mixture_queries(centres, sizes, nq, sigma, seed):
    rng = np.random.default_rng(seed + 7919)
    p = sizes / sizes.sum()
    c = rng.choice(len(centres), size=nq, p=p)
    return (centres[c] + np.float32(sigma) * rng.standard_normal((nq, centres.shape[1]), dtype=np.float32)).astype(
        np.float32)


def log_uniform_batches(total, lo=1, hi=4096, seed=0):
    """Batch sizes round(exp(U(ln lo, ln hi))) until `total` queries are covered."""
    rng = np.random.default_rng(seed)
    out, s = [], 0
    while s < total:
        b = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        b = max(lo, min(hi, b, total - s))
        out.append(b)
        s += b
    return out


def gaussian_mixture_queries(n=1_000_000, d=512, n_centres=2048, sigma=0.3, zipf_s=1.1, nq=10_000, seed=0,
                             query_seed=1):
    """Queries from the same mixture as gaussian_mixture(n, ..., seed) without
    building the database (same centres, same component weights)."""
    rng = np.random.default_rng(seed)
    centres = rng.standard_normal((n_centres, d), dtype=np.float32)
    sizes = zipf_sizes(n, n_centres, zipf_s) if zipf_s else np.full(n_centres, max(1, n // n_centres), np.int64)
    return mixture_queries(centres, sizes, nq, sigma, query_seed)

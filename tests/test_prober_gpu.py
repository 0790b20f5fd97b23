"""Learned prober: CUDA forward/backward against the FP64 oracle, training on
exact-search labels, and what it gains over fixed n_probe at equal recall."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mixture(n, d, centres, nq, seed):
    rng = np.random.default_rng(seed)
    c = rng.standard_normal((centres, d), dtype=np.float32)
    w = 1.0 / np.arange(1, centres + 1) ** 1.1
    p = w / w.sum()
    db = c[rng.choice(centres, n, p=p)] + np.float32(0.3) * rng.standard_normal((n, d), dtype=np.float32)
    q = c[rng.choice(centres, nq, p=p)] + np.float32(0.3) * rng.standard_normal((nq, d), dtype=np.float32)
    return db.astype(np.float32), q.astype(np.float32)


def test_gradients_match_fp64_oracle(gn):
    from oracle import mlp
    rng = np.random.default_rng(3)
    db, _ = _mixture(20000, 32, 128, 10, 1)
    ix = gn.IVFFlatL2Index(n_clusters=96, n_probe=8)
    ix.set(db)
    pr = gn.LearnedProber(ix, seed=5)
    L = pr.n_lists
    B = 24
    cand = np.stack([rng.permutation(L)[:64] for _ in range(B)]).astype(np.int32)
    cand[3, 50:] = -1  # fewer candidates than 64
    feat = rng.random((B, 64), dtype=np.float32)
    lab = (rng.random((B, 64)) < 0.2).astype(np.float32)
    params = pr.get_params()
    loss, grads = pr.loss_and_grad(cand, feat, lab)
    ref_loss, ref = mlp.loss_grad(*pr.split(params.astype(np.float64)), cand, feat, lab)
    assert abs(loss - ref_loss) <= 1e-5 * max(1.0, abs(ref_loss))
    for g, r in zip(pr.split(grads), ref):
        scale = np.abs(r).max() + 1e-12
        assert np.abs(g - r).max() <= 2e-4 * scale, (np.abs(g - r).max(), scale)


def test_training_cuts_lists_scanned_at_fixed_recall(gn):
    db, q = _mixture(120_000, 64, 512, 9000, 2)
    train, held = q[:6000], q[6000:]
    ex = gn.FlatL2Index()
    ex.set(db)
    gt_train, _ = ex.search_knn_arrays(train, 10)
    gt_held, _ = ex.search_knn_arrays(held, 10)
    ix = gn.IVFFlatL2Index(n_clusters=256, n_probe=1, engine="tc")
    ix.set(db)

    def recall(idx, gt):
        return np.mean([len(set(a) & set(b)) / 10 for a, b in zip(idx, gt)])

    # fixed n_probe: smallest reaching 0.95
    fixed = None
    for p in range(1, 65):
        ix.n_probe = p
        idx, _, _ = ix.search_knn_arrays(held, 10)
        if recall(idx, gt_held) >= 0.95:
            fixed = p
            break
    assert fixed is not None
    pr = gn.LearnedProber(ix, seed=1)
    losses = pr.train(train, gt_train, epochs=6, batch=512, lr=2e-3)
    assert losses[-1] < losses[0]
    best = None
    for thr in (0.5, 0.3, 0.2, 0.1, 0.05, 0.02, 0.01, 0.005):
        ix.set_prober(pr, thr)
        idx, _, _ = ix.search_knn_arrays(held, 10)
        r = recall(idx, gt_held)
        mean_lists = float(ix.last_lists_probed(len(held)).mean())
        if r >= 0.95:
            best = (thr, r, mean_lists)
            break
    assert best is not None, "the prober never reached recall 0.95"
    assert best[2] < fixed, (best, fixed)
    # detaching the prober restores the fixed n_probe search
    ix.set_prober(None)
    ix.n_probe = fixed
    a, _, _ = ix.search_knn_arrays(held[:100], 10)
    ix.n_probe = fixed
    b, _, _ = ix.search_knn_arrays(held[:100], 10)
    assert np.array_equal(a, b)


def test_batched_mlp_matches_fused_mlp(gn):
    """Batches of 1,024 queries and more run the prober's layers 2 and 3 in a
    separate kernel over eight queries per block; smaller batches keep them
    fused in the probe kernel.  Both compute the same network (FP32 sums in a
    different order), so the probe counts and the results agree except where a
    logit sits at the threshold."""
    db, q = _mixture(60_000, 48, 256, 3000, 5)
    train = q[:1000]
    ex = gn.FlatL2Index()
    ex.set(db)
    gt_train, _ = ex.search_knn_arrays(train, 10)
    ix = gn.IVFFlatL2Index(n_clusters=192, n_probe=4, engine="tc")
    ix.set(db)
    pr = gn.LearnedProber(ix, seed=2)
    pr.train(train, gt_train, epochs=3, batch=512, lr=2e-3)
    ix.set_prober(pr, 0.2)
    held = q[1000:]
    big_i, big_d, big_c = ix.search_knn_arrays(held, 10)  # 2,000 queries: batched MLP
    big_lists = ix.last_lists_probed(len(held)).copy()
    sm_i, small_lists = [], []
    for s in range(0, len(held), 500):  # 500-query batches: fused MLP
        sm_i.append(ix.search_knn_arrays(held[s:s + 500], 10)[0])
        small_lists.append(ix.last_lists_probed(500).copy())
    sm_i, small_lists = np.concatenate(sm_i), np.concatenate(small_lists)
    assert np.mean(big_lists == small_lists) >= 0.99
    assert np.mean(np.all(big_i == sm_i, axis=1)) >= 0.99
    assert big_lists.min() >= 1

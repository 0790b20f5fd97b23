"""The batched IVF-flat L2 configuration at full size: 1,000,000 x 512 float32
drawn from a Gaussian mixture of 2,048 N(0, I) centres with Zipf(1.1)
component sizes and sigma 0.3, nlist 1,024 lists built by the GPU k-means,
k = 10 (the reference's IVFFlatL2Index, pynear/forest.py:63-111,189-194).

* Fixed n_probe 28, both engines (tensor-core shortlist + exact re-rank, and
  the FP32 scan), against the oracle's restatement of the reference search on
  the same lists, centroids and queries: equal result counts, >= 99.5 % of the
  indices equal (the oracle ranks centroids in the BLAS form, the GPU with an
  exact re-rank, so a near tie between two centroids can change one probe),
  distances of equal rows within FP32 rounding of the BLAS form, and every
  returned distance checked against an FP64 recomputation of its row
  (within 1e-6 relative for the tensor-core engine's exact re-rank).
* The learned prober (MLP trained on the GPU on exact-search labels, its
  probability threshold calibrated on separate queries): Recall@10 >= 0.95
  against the exact flat scan on held-out queries, fewer lists than the
  fixed n_probe that reaches the same recall, and every returned distance
  checked in FP64.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, D, CENTRES, NLIST, K = 1_000_000, 512, 2048, 1024, 10
N_CAL, N_EVAL = 1000, 1000


@pytest.fixture(scope="module")
def headline(gn):
    from pynear_gb300 import workloads as W

    db, q, _, _ = W.gaussian_mixture(n=N, d=D, n_centres=CENTRES, sigma=0.3, zipf_s=1.1, nq=N_CAL + N_EVAL,
                                     seed=0)
    ix = gn.IVFFlatL2Index(n_clusters=NLIST, n_probe=28, engine="tc")
    ix.set(db)
    cent, offs, ids = ix.export()
    labels = np.empty(len(db), np.int32)
    for c in range(len(offs) - 1):
        labels[ids[offs[c]:offs[c + 1]]] = c
    ex = gn.FlatL2Index()
    ex.set(db)
    gt, _ = ex.search_knn_arrays(q, K)
    del ex
    return {"db": db, "cal": q[:N_CAL], "ev": q[N_CAL:], "gt_cal": gt[:N_CAL], "gt_ev": gt[N_CAL:], "ix": ix,
            "cent": cent, "labels": labels}


def _recall(idx, gt):
    return float(np.mean([len(set(a[a >= 0].tolist()) & set(b.tolist())) / len(b) for a, b in zip(idx, gt)]))


def _fp64_sq(q, db, idx):
    return ((q[:, None, :].astype(np.float64) - db[idx].astype(np.float64)) ** 2).sum(-1)


@pytest.mark.parametrize("engine", ["tc", "fp32"])
def test_headline_fixed_nprobe_matches_oracle(headline, oracle, engine):
    h = headline
    ix = h["ix"]
    q = h["ev"][:200]
    ix.set_prober(None)
    ix.set_engine(engine)
    ix.n_probe = 28
    idx, dist, cnt = ix.search_knn_arrays(q, K)
    oi, od, oc = oracle.ivfl2_search(h["db"], h["cent"], h["labels"], q, K, 28)
    assert np.array_equal(cnt, oc)
    same = idx == oi
    assert np.mean(same) >= 0.995, np.mean(same)
    # the same rows: the same distance up to FP32 rounding of the BLAS form
    np.testing.assert_allclose(dist[same], od[same], rtol=1e-4, atol=1e-3)
    # every returned distance (including rows a changed probe brought in) is
    # its own row's squared distance: exact (compensated FP32) for the
    # tensor-core engine, the BLAS form's rounding for the FP32 engine
    d64 = _fp64_sq(q, h["db"], idx)
    rel = np.abs(dist - d64) / np.maximum(d64, 1e-6)
    assert rel.max() < (1e-6 if engine == "tc" else 1e-4), rel.max()
    ix.set_engine("tc")


def test_headline_learned_prober_reaches_recall(headline, gn):
    from pynear_gb300 import workloads as W

    h = headline
    ix = h["ix"]
    ix.set_engine("tc")
    # exact labels for the training queries (same mixture, other draws), by
    # the tensor-core flat scan with its exact re-rank
    train = W.gaussian_mixture_queries(n=N, d=D, n_centres=CENTRES, sigma=0.3, zipf_s=1.1, nq=100_000, seed=0,
                                       query_seed=4242)
    tcx = gn.FlatL2TCIndex(shortlist=40)
    tcx.set(h["db"])
    gt_train = np.concatenate([tcx.search_knn_arrays(train[i:i + 20000], K)[0] for i in range(0, len(train), 20000)])
    del tcx
    pr = gn.LearnedProber(ix, seed=1)
    losses = pr.train(train, gt_train, epochs=4, batch=1024, lr=2e-3)
    assert losses[-1] < losses[0]
    # largest threshold whose calibration recall reaches 0.955 (margin over 0.95)
    chosen = None
    for thr in (0.5, 0.4, 0.3, 0.25, 0.2, 0.15, 0.12, 0.1, 0.07, 0.05, 0.03, 0.02, 0.01):
        ix.set_prober(pr, thr)
        idx, _, _ = ix.search_knn_arrays(h["cal"], K)
        if _recall(idx, h["gt_cal"]) >= 0.955:
            chosen = thr
            break
    assert chosen is not None, "the prober never reached calibration recall 0.955"
    ix.set_prober(pr, chosen)
    idx, dist, cnt = ix.search_knn_arrays(h["ev"], K)
    lists = float(ix.last_lists_probed(len(h["ev"])).mean())
    rec = _recall(idx, h["gt_ev"])
    assert rec >= 0.95, (chosen, rec)
    assert (cnt == K).all()
    d64 = _fp64_sq(h["ev"], h["db"], idx)
    assert np.max(np.abs(dist - d64) / np.maximum(d64, 1e-6)) < 1e-6
    assert np.all(np.diff(dist, axis=1) >= 0)
    # the fixed n_probe that reaches the same held-out recall scans more lists
    ix.set_prober(None)
    ix.n_probe = int(np.ceil(lists))
    fi, _, _ = ix.search_knn_arrays(h["ev"], K)
    assert _recall(fi, h["gt_ev"]) < rec, (lists, rec)

"""Host logic of the multi-replica benchmark path (two gloo ranks on the CPU)
and the host-side checks of the scikit-learn style adapters."""
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    sys.path.insert(0, REPO)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench

    d = bench.Dist("gloo")
    assert (d.ws, d.rank) == (world, rank)
    d.barrier()
    # each replica times its own work; the job time is the slowest replica's
    out.put((rank, d.max(1.5 + rank), d.max(-float(rank))))
    d.barrier()
    d.close()


def test_two_gloo_ranks_barrier_and_max_over_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2.5, 0.0), (1, 2.5, 0.0)]


def test_reference_arm_runs_on_rank_zero_only():
    # under torchrun the other ranks of the reference arm exit at once, without work
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference"], env=env,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_sklearn_adapter_host_checks():
    sys.path.insert(0, REPO)
    from pynear_gb300 import sklearn_adapter as sk

    clf = sk.PyNearKNeighborsClassifier(n_neighbors=3, weights="distance")
    assert clf.get_params()["n_neighbors"] == 3
    assert clf.set_params(n_neighbors=7).n_neighbors == 7
    with pytest.raises(ValueError):
        sk.PyNearNearestNeighbors(metric="cosine").fit([[0.0, 1.0]])
    with pytest.raises(ValueError):
        sk.PyNearNearestNeighbors().fit([0.0, 1.0])  # not 2-D
    with pytest.raises(Exception):
        sk.PyNearNearestNeighbors().kneighbors([[0.0, 1.0]])  # not fitted
    import numpy as np
    w = sk._weights(np.array([[0.0, 2.0], [1.0, 4.0]]), "distance")
    np.testing.assert_allclose(w, [[1.0, 0.0], [1.0, 0.25]])
    with pytest.raises(ValueError):
        sk._weights(np.ones((1, 1)), "bogus")

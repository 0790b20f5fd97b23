"""The reference's own test files, run unmodified against this package.

The reference package (PyNear 2.2.0) installed from its source tree under
baseline/_ref (pip install --target; not part of this repository) carries its
tests in pynear/tests/.  Here the files that cover the rebuilt search path —
test_vptree.py (exact L2 / L1 / L-inf / Hamming k-NN and 1-NN against
exhaustive search, the distance functions), test_ivfflat.py (IVFFlatL2Index),
test_binary_approx.py (IVFFlatBinaryIndex, MIHBinaryIndex),
test_serialization.py (pickling) and, where scikit-learn is importable,
test_sklearn_adapter.py — are copied to a temporary directory at run time
and run by pytest in a child process whose `pynear` is a two-line shim
re-exporting pynear_gb300.  So every class they construct is this package's
GPU engine.  Skipped where the reference package is not installed.
"""
import os
import shutil
import subprocess
import sys

import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu

REF_TESTS = os.path.join(REPO, "baseline", "_ref", "pynear", "tests")
FILES = ["test_vptree.py", "test_ivfflat.py", "test_binary_approx.py", "test_serialization.py",
         "test_sklearn_adapter.py"]


def test_reference_test_files_pass_against_this_package(gn, tmp_path):
    if not os.path.isdir(REF_TESTS):
        pytest.skip("reference package not installed under baseline/_ref")
    files = [f for f in FILES if os.path.exists(os.path.join(REF_TESTS, f))]
    try:
        import sklearn  # noqa: F401
    except ImportError:
        files.remove("test_sklearn_adapter.py")  # it imports scikit-learn at module level
    shim = tmp_path / "shim" / "pynear"
    shim.mkdir(parents=True)
    (shim / "__init__.py").write_text("from pynear_gb300 import *  # noqa: F401,F403\n"
                                      "from pynear_gb300 import sklearn_adapter  # noqa: F401\n")
    (shim / "sklearn_adapter.py").write_text("from pynear_gb300.sklearn_adapter import *  # noqa: F401,F403\n")
    run = tmp_path / "suite"
    run.mkdir()
    for f in files:
        shutil.copy(os.path.join(REF_TESTS, f), run / f)
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join([str(tmp_path / "shim"), REPO])
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-p", "no:cacheprovider", "--durations=8",
                        "--rootdir", str(run), *files], cwd=run, env=env, capture_output=True, text=True,
                       timeout=1200)
    tail = (r.stdout + r.stderr)[-6000:]
    print(tail)
    assert r.returncode == 0, tail
    # the shim, not the reference package, served the tests
    probe = subprocess.run([sys.executable, "-c", "import pynear; print(pynear.VPTreeL2Index.__module__)"],
                           cwd=run, env=env, capture_output=True, text=True)
    assert probe.stdout.strip().startswith("pynear_gb300"), probe.stdout + probe.stderr

"""The bounds-checked build (libgpuai_checked.so, -DGPUAI_CHECKS) gives the
same results as the normal build on the parity tests of the playout kernel
and of the device searches, with no check failing (a failed check would
report GPUAI_ERR_LIMIT).  Runs those tests in a child process that loads the
checked library through GPUAI_LIB."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_parity_with_the_checked_build(lib_built):
    from gpu_ai_gb300.build import build
    so = build(checks=True)
    env = dict(os.environ, GPUAI_LIB=so)
    tests = ["test_gpu_playouts.py::test_replay_bit_exact", "test_gpu_playouts.py::test_empty_and_ragged",
             "test_gpu_search_oracle.py::test_plain_searches_node_for_node",
             "test_gpu_search_oracle.py::test_playouts_per_leaf_and_node_range_limits"]
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider", "-m", "gpu"] +
                       [os.path.join(HERE, t) for t in tests], env=env, capture_output=True, text=True,
                       timeout=1200)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert "passed" in r.stdout

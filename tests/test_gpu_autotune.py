"""The autotuner sweeps launch shapes and search-step sizes on the GPU and
caches the fastest per GPU name; a cached shape applies to a new Engine and
does not change results."""
import json
import subprocess
import sys

import numpy as np
import pytest

import oracle_lib as L
from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_autotune_quick_and_apply(lib_built, tmp_path):
    cache = tmp_path / "tune.json"
    r = subprocess.run([sys.executable, "-m", "gpu_ai_gb300.autotune", "--quick", "--cache", str(cache)],
                       capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    data = json.loads(cache.read_text())
    (gpu, entry), = data.items()
    assert entry["playouts"]["playouts_per_s"] > 0 and entry["searches"]["playouts_per_s"] > 0
    from gpu_ai_gb300 import Engine, autotune
    eng = Engine(0)
    assert autotune.apply(eng, str(cache))
    shape = eng.get_launch(0)
    assert shape["block_threads"] == entry["playouts"]["block_threads"]
    pos = L.random_positions(3, 8, 0, 20)
    reps = np.full(8, 50, np.uint32)
    exp, _ = L.replay_batch(pos, reps, seed=9)
    np.testing.assert_array_equal(eng.playouts(pos, reps, seed=9), exp)

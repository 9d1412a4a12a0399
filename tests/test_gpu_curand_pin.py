"""The project's Philox4x32-10 (the random streams of every playout) against
cuRAND's Philox4_32_10 generator, run on the GPU: 1 M seeded counters and keys
give the same four words (tests/curand_pin.cu)."""
import os
import re
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_philox_matches_curand():
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "curand_pin")
    subprocess.run(["nvcc", "-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I" + os.path.join(ROOT, "gpu_ai_gb300", "csrc"), os.path.join(HERE, "curand_pin.cu"),
                    "-o", exe], check=True)
    r = subprocess.run([exe, str(1 << 20)], capture_output=True, text=True, timeout=120)
    m = re.search(r"cases (\d+) mismatches (\d+)", r.stdout)
    assert m, r.stdout + r.stderr
    assert int(m.group(1)) == 1 << 20
    assert int(m.group(2)) == 0, r.stdout
    assert r.returncode == 0

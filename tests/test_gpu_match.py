"""GPU MCTS against the reference's mcts_host (tests/match.cpp) at equal time
per move: a short match must run to completion and the GPU player must not
score below one half."""
import json
import re
import subprocess

import pytest

from match_build import build_match

pytestmark = pytest.mark.gpu


def test_short_match_against_mcts_host(lib_built):
    exe = build_match()
    r = subprocess.run([exe, "-n", "2", "--ms-per-move", "60"], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr
    m = re.search(r"RESULT (\{.*\})", r.stdout)
    assert m, r.stdout
    res = json.loads(m.group(1))
    assert res["wins"] + res["draws"] + res["losses"] == 2
    assert res["score"] >= 0.5
    assert res["gpu_playouts"] > 0

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
    assert res["a_playouts"] > 0 and res["b_playouts"] > 0


def test_seeded_positions_in_parallel(lib_built):
    """Config-2 form: games from seeded mid-game positions, each played with
    both colours, two games at once, heuristic against plain GPU playouts."""
    exe = build_match()
    r = subprocess.run([exe, "-n", "4", "--ms-per-move", "40", "--positions", "2", "--min-plies", "10",
                        "--max-plies", "40", "-a", "mcts_device_eps_greedy", "-b", "mcts_device_multiple",
                        "--batch-min", "16384", "--batch-max", "65536", "--ppl", "2", "--parallel", "2",
                        "--max-game-plies", "30"], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr
    res = json.loads(re.search(r"RESULT (\{.*\})", r.stdout).group(1))
    assert res["wins"] + res["draws"] + res["losses"] == 4
    assert res["a_playouts"] > 0 and res["b_playouts"] > 0

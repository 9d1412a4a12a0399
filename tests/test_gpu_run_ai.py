"""run_ai, the C++ driver over the host layer (State / PlayoutDriver /
GameTree / players), in the reference's run modes (src/driver.cpp:266-394)."""
import os
import re
import subprocess

import pytest

pytestmark = pytest.mark.gpu

RUN_AI = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "gpu_ai_gb300", "lib", "run_ai")


def run(*args, timeout=600):
    r = subprocess.run([RUN_AI, *args], capture_output=True, text=True, timeout=timeout)
    return r.returncode, r.stdout + r.stderr


def counts(text):
    d = [int(x) for x in re.findall(r"Games drawn: (\d+)", text)]
    p1 = [int(x) for x in re.findall(r"Player 1 wins: (\d+)", text)]
    p2 = [int(x) for x in re.findall(r"Player 2 wins: (\d+)", text)]
    return list(zip(p1, d, p2))


def test_gen_moves_test_passes(lib_built):
    rc, out = run("-m", "gen_moves_test", "-n", "20000")
    assert rc == 0, out
    assert "Passed" in out


def test_playout_test_two_drivers(lib_built):
    rc, out = run("-m", "playout_test", "-n", "20000", "-1", "device_multiple", "-2", "device_heuristic")
    assert rc == 0, out
    c = counts(out)
    assert len(c) == 2 and all(sum(x) == 20000 for x in c)
    assert "Similar results" in out


def test_cpu_driver_names_are_rejected(lib_built):
    rc, out = run("-m", "playout_test", "-n", "10", "-1", "host", "-2", "device")
    assert rc == 2 and "CPU" in out


def test_mcts_beats_random(lib_built):
    rc, out = run("-m", "game_test", "-n", "2", "-1", "mcts", "-2", "random", "--ms-per-move", "150", timeout=900)
    assert rc == 0, out
    p1, d, p2 = counts(out)[-1]
    assert p1 + d + p2 == 2 and p2 == 0 and p1 >= 1


def test_mcts_bench_reports_leaf_batch_throughput(lib_built):
    """mcts_bench: host UCT searches with GPU leaf batches of 16K+ slots run for
    the requested time and account for every playout."""
    import json
    rc, out = run("-m", "mcts_bench", "-n", "3", "--ms-per-move", "60", "--playouts-per-leaf", "2",
                  "--threads", "2", "-1", "device", "-2", "device_eps_greedy")
    assert rc == 0, out
    lines = [json.loads(x[len("MCTS_BENCH "):]) for x in out.splitlines() if x.startswith("MCTS_BENCH ")]
    assert [x["driver"] for x in lines] == ["device", "device_eps_greedy"]
    for x in lines:
        assert x["positions"] == 3 and x["batches"] >= 3 and x["threads"] == 2
        assert x["mean_leaves_per_batch"] >= 16384
        assert x["playouts"] == 2 * x["leaves"]
        assert 0 < x["driver_seconds"] <= x["search_seconds"] <= 2 * x["seconds"]

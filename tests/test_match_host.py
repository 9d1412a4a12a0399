"""Host arithmetic behind the reported match results and the training split
(no GPU): the Wilson interval and the held-out split."""
import numpy as np
import pytest

from gpu_ai_gb300 import learn, match


@pytest.mark.parametrize("score,n,lo,hi", [
    ((367 + 0.5 * 32) / 400, 400, 0.933, 0.973),   # learned vs plain, 367-32-1
    ((182 + 0.5 * 8) / 200, 200, 0.886, 0.958),    # GPU MCTS vs mcts_host, 182-8-10
    (0.5, 100, 0.404, 0.596),
])
def test_wilson_interval_of_reported_results(score, n, lo, hi):
    a, b = match.wilson(score, n)
    assert (round(a, 3), round(b, 3)) == (lo, hi)


def test_wilson_edges():
    assert match.wilson(0.7, 0) == (0.0, 1.0)
    a, b = match.wilson(1.0, 50)
    assert 0.9 < a < 1.0 and b == pytest.approx(1.0)
    a, b = match.wilson(0.0, 50)
    assert a == pytest.approx(0.0, abs=1e-12) and 0.0 < b < 0.1


def test_split_holds_out_the_last_rows():
    m = 1000
    data = {"boards": np.arange(4 * m, dtype=np.uint32).reshape(m, 4), "value": np.arange(m, dtype=np.float32),
            "q": np.zeros((m, 32), np.float32), "nmoves": np.ones(m, np.uint8)}
    tr, te = learn.split(data, 150)
    assert tr["boards"].shape[0] == 850 and te["boards"].shape[0] == 150
    assert (te["value"] == np.arange(850, 1000)).all() and (tr["value"] == np.arange(850)).all()
    assert all(tr[k].shape[0] == 850 and te[k].shape[0] == 150 for k in ("boards", "value", "q", "nmoves"))

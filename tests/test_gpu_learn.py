"""The learned pipeline at small scale on the GPU: self-play positions,
playout labels, training, evaluation, and a short learned-vs-plain match."""
import numpy as np
import pytest

import oracle_lib as L

pytestmark = pytest.mark.gpu


def test_selfplay_positions_match_random_positions(engine):
    import torch
    from gpu_ai_gb300 import POLICY_EPS_GREEDY, POLICY_RANDOM
    n = 500
    d = torch.zeros((n, 4), dtype=torch.int32, device="cuda")
    engine.selfplay_positions(9, n, 0, 40, POLICY_RANDOM, d.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy().view(np.uint32), engine.random_positions(9, n, 0, 40))
    assert np.array_equal(d.cpu().numpy().view(np.uint32), L.random_positions(9, n, 0, 40))
    engine.selfplay_positions(9, n, 0, 40, POLICY_EPS_GREEDY, d.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    b = d.cpu().numpy().view(np.uint32)
    assert np.all((b[:, 0] & b[:, 1]) == 0) and not np.array_equal(b, L.random_positions(9, n, 0, 40))


def test_train_and_evaluate_small(engine):
    from gpu_ai_gb300 import Net
    from gpu_ai_gb300 import learn
    data = learn.make_dataset(engine, 40_000, playouts=256, seed=3, chunk=16384)
    m = data["boards"].shape[0]
    assert 20_000 < m <= 40_000  # finished games (about a quarter at up to 90 plies) are dropped
    assert float(data["value"].abs().max()) <= 1.0
    tr, te = learn.split(data, 4000)
    net = Net(0, max_batch=4096, seed=1)
    before = learn.evaluate(net, engine, te, baseline_playouts=16)
    res = learn.train(net, tr, epochs=3, batch=4096, lr=2e-3, log_every=10)
    after = learn.evaluate(net, engine, te, baseline_playouts=16)
    assert res["history"][-1][2] < res["history"][0][2]
    assert after["value_mae"] < 0.8 * before["value_mae"]
    assert after["policy_top1_vs_best_label"] > before["policy_top1_vs_best_label"]
    net.close()


def test_short_match_runs(engine):
    from gpu_ai_gb300 import Net
    from gpu_ai_gb300.match import play_match
    net = Net(0, max_batch=256, seed=2)
    r = play_match(net, engine, n_games=4, ms_per_move=5.0, leaves=16, node_capacity=20000, max_plies=40)
    assert r["games"] == 4
    assert r["learned_wins"] + r["draws"] + r["learned_losses"] == 4
    assert r["learned_playouts"] > 0 and r["plain_playouts"] > 0
    assert 0.0 <= r["ci95_wilson"][0] <= r["learned_score"] <= r["ci95_wilson"][1] <= 1.0
    net.close()

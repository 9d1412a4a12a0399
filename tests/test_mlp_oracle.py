"""Pins for the network oracle (oracle/mlp.py) on the CPU.

The network is the project's own component, so the oracle is pinned by its
own mathematics: analytic gradients against central finite differences in
float64, closed-form values, and the BF16 rounding rule.
"""
import numpy as np
import pytest

import oracle_lib as L
from oracle import mlp


def _batch(seed, n, min_plies=0, max_plies=40):
    boards = L.random_positions(seed, n * 3, min_plies, max_plies)
    out, counts = L.genmoves(boards)
    keep = (counts > 0) & (counts <= mlp.MAXM)
    boards, out, counts = boards[keep][:n], out[keep][:n], counts[keep][:n]
    assert len(boards) == n
    rng = np.random.default_rng(seed)
    z = rng.uniform(-1, 1, n)
    q = rng.uniform(-1, 1, (n, mlp.MAXM))
    return boards, out[:, :, 0], out[:, :, 1], counts, z, q


def _params(seed, scale=1.0):
    rng = np.random.default_rng(seed)
    d = {
        "W1": rng.normal(0, scale * 0.15, (mlp.H, mlp.IN_PAD)), "b1": rng.normal(0, 0.05, mlp.H),
        "W2": rng.normal(0, scale * 0.1, (mlp.H, mlp.H)), "b2": rng.normal(0, 0.05, mlp.H),
        "W3": rng.normal(0, scale * 0.1, (mlp.OUT, mlp.H)), "b3": rng.normal(0, 0.05, mlp.OUT),
        "wv": rng.normal(0, scale * 0.1, mlp.H), "bv": rng.normal(0, 0.05, 1),
    }
    d["W1"][:, mlp.IN:] = 0
    return mlp.pack(d)


def test_bf16_rounding_rule():
    x = np.array([1.0, 1.00390625, 1.01171875, -2.5, 65504.0, 1.0 + 2 ** -8 + 2 ** -20], np.float32)
    got = mlp.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: ties go to the even mantissa (1.0)
    want = np.array([1.0, 1.0, 1.015625, -2.5, 65536.0, 1.0078125], np.float32)
    assert np.array_equal(got, want)


def test_features_of_the_start_position():
    X = mlp.features(L.start_board())
    assert X.shape == (1, mlp.IN_PAD)
    assert X[0, 0:32].sum() == 12 and X[0, 0:12].all()       # PLAYER_1 men on squares 0..11
    assert X[0, 64:96].sum() == 12 and X[0, 84:96].all()     # opponent men on 20..31
    assert X[0, 32:64].sum() == 0 and X[0, 96:128].sum() == 0
    assert X[0, 128] == 0 and X[0, 129:].sum() == 0
    b = L.start_board().copy()
    b[0, 3] = 1  # PLAYER_2 to move: own/opponent planes swap
    X2 = mlp.features(b)
    assert X2[0, 128] == 1 and X2[0, 20:32].all() and X2[0, 64:76].all()


def test_zero_network_is_uniform():
    boards, fr, to, counts, z, q = _batch(5, 8)
    p = np.zeros(mlp.N_PARAMS)
    loss2, _, g = mlp.loss_grads(p, boards, z, q, fr, to, counts, emulate=False, dtype=np.float64)
    npairs = [len(set(int(a) * 32 + int(b) for a, b in zip(fr[i, :k], to[i, :k]))) for i, k in enumerate(counts)]
    assert loss2[0] == pytest.approx(np.mean(np.log(npairs)), rel=1e-12)
    assert loss2[1] == pytest.approx(np.mean(z ** 2), rel=1e-12)


@pytest.mark.parametrize("tau,value_coef", [(0.1, 1.0), (0.5, 0.25)])
def test_gradients_match_finite_differences(tau, value_coef):
    boards, fr, to, counts, z, q = _batch(11, 6)
    p = _params(3).astype(np.float64)
    _, total, g = mlp.loss_grads(p, boards, z, q, fr, to, counts, tau, value_coef, emulate=False, dtype=np.float64)
    rng = np.random.default_rng(7)
    idx = []
    for lo, hi in [(mlp.O_W1, mlp.O_B1), (mlp.O_B1, mlp.O_W2), (mlp.O_W2, mlp.O_B2), (mlp.O_B2, mlp.O_W3),
                   (mlp.O_W3, mlp.O_B3), (mlp.O_B3, mlp.O_WV), (mlp.O_WV, mlp.O_BV), (mlp.O_BV, mlp.N_PARAMS)]:
        # entries with a non-zero gradient where possible (most W3 rows are not legal moves)
        nz = lo + np.flatnonzero(np.abs(g[lo:hi]) > 1e-9)
        pool = nz if len(nz) else np.arange(lo, hi)
        idx += list(rng.choice(pool, size=min(6, len(pool)), replace=False))
    eps = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fp = mlp.loss_grads(pp, boards, z, q, fr, to, counts, tau, value_coef, emulate=False, dtype=np.float64)[1]
        fm = mlp.loss_grads(pm, boards, z, q, fr, to, counts, tau, value_coef, emulate=False, dtype=np.float64)[1]
        num = (fp - fm) / (2 * eps)
        assert num == pytest.approx(g[i], rel=1e-5, abs=1e-9), f"parameter {i}"


def test_padding_features_have_zero_gradient():
    boards, fr, to, counts, z, q = _batch(13, 5)
    p = _params(4)
    _, _, g = mlp.loss_grads(p, boards, z, q, fr, to, counts)
    W1g = g[mlp.O_W1:mlp.O_B1].reshape(mlp.H, mlp.IN_PAD)
    assert np.all(W1g[:, mlp.IN:] == 0)


def test_adam_first_step_moves_by_lr():
    p = np.ones(10)
    g = np.linspace(-1, 1, 10)
    g[5] = 0
    p2, m, v = mlp.adam(p, np.zeros(10), np.zeros(10), g, step=1, lr=0.01)
    # bias-corrected first step: -lr * sign(g) (eps aside), zero gradient stays put
    assert np.allclose(p2 - p, -0.01 * np.sign(g), atol=1e-6)

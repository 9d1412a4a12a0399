"""CPU restatement of the project's policy/value network -- TEST INFRASTRUCTURE ONLY.

Only tests/ import this module; the product computes in the CUDA kernels of
gpu_ai_gb300/csrc/net.cu.  The network has no counterpart in the reference
(krame505/gpu_ai evaluates positions only with its material heuristic,
src/heuristic.cu:20-49), so there is no reference code or golden vector to pin
against.  The oracle is pinned instead by (1) central finite differences of
its own loss in float64 (tests/test_mlp_oracle.py) and (2) closed-form cases
(zero weights give uniform move probabilities and value 0).  The GPU kernels are
then checked against it with the same BF16 rounding points
(tests/test_gpu_net.py).

Layout and dataflow (see include/gpuai.h):
  X  = 192 features (129 used): side to move's men, kings, opponent's men,
       kings (32 squares each), 1 if PLAYER_2 is to move, zero padding
  h1 = relu(X W1^T + b1)           (BF16-rounded when emulating the GPU)
  h2 = relu(h1 W2^T + b2)          (BF16-rounded)
  v  = tanh(h2 . wv + bv)          (value for the side to move)
  logits = h2 W3^T + b3            (1024 = from * 32 + to)
Loss per position: cross entropy between softmax(move_q / tau) over the legal
moves (moves sharing a (from, to) pair share one logit; their targets add) and
the softmax of the logits over the legal pairs, plus value_coef * (v - z)^2;
averaged over the batch.
"""
from __future__ import annotations

import numpy as np

IN, IN_PAD, H, OUT, MAXM = 129, 192, 256, 1024, 32
O_W1 = 0
O_B1 = O_W1 + H * IN_PAD
O_W2 = O_B1 + H
O_B2 = O_W2 + H * H
O_W3 = O_B2 + H
O_B3 = O_W3 + OUT * H
O_WV = O_B3 + OUT
O_BV = O_WV + H
N_PARAMS = O_BV + 1


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even), as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(p: np.ndarray) -> dict:
    return {
        "W1": p[O_W1:O_B1].reshape(H, IN_PAD), "b1": p[O_B1:O_W2],
        "W2": p[O_W2:O_B2].reshape(H, H), "b2": p[O_B2:O_W3],
        "W3": p[O_W3:O_B3].reshape(OUT, H), "b3": p[O_B3:O_WV],
        "wv": p[O_WV:O_BV], "bv": p[O_BV:O_BV + 1],
    }


def pack(d: dict) -> np.ndarray:
    return np.concatenate([d["W1"].ravel(), d["b1"], d["W2"].ravel(), d["b2"], d["W3"].ravel(), d["b3"],
                           d["wv"], d["bv"]])


def features(boards: np.ndarray) -> np.ndarray:
    """(n, 192) features of (n, 4) board records {p1, p2, kings, meta}."""
    b = np.asarray(boards, dtype=np.uint32).reshape(-1, 4)
    side = (b[:, 3] & 1).astype(bool)
    own = np.where(side, b[:, 1], b[:, 0])
    opp = np.where(side, b[:, 0], b[:, 1])
    k = b[:, 2]
    planes = [own & ~k, own & k, opp & ~k, opp & k]
    sq = np.arange(32, dtype=np.uint32)
    X = np.zeros((b.shape[0], IN_PAD), np.float32)
    for i, pl in enumerate(planes):
        X[:, 32 * i:32 * i + 32] = ((pl[:, None] >> sq[None, :]) & 1).astype(np.float32)
    X[:, 128] = side.astype(np.float32)
    return X


def forward(p: np.ndarray, boards, emulate: bool = True, dtype=np.float32) -> dict:
    """Forward pass.  emulate=True rounds weights and activations to BF16 where
    the GPU does; emulate=False is plain arithmetic in `dtype`."""
    d = unpack(np.asarray(p, dtype=np.float32 if emulate else dtype))
    X = features(boards).astype(dtype)
    r = bf16 if emulate else (lambda a: a)
    W1, W2, W3 = (r(d[k]).astype(dtype) for k in ("W1", "W2", "W3"))
    b1, b2, b3, wv, bv = (d[k].astype(dtype) for k in ("b1", "b2", "b3", "wv", "bv"))
    z1 = X @ W1.T + b1
    h1 = r(np.maximum(z1, 0)).astype(dtype)
    z2 = h1 @ W2.T + b2
    h2 = r(np.maximum(z2, 0)).astype(dtype)
    vraw = h2 @ wv + bv[0]
    logits = h2 @ W3.T + b3
    return {"X": X, "h1": h1, "h2": h2, "vraw": vraw, "value": np.tanh(vraw), "logits": logits,
            "W1": W1, "W2": W2, "W3": W3, "wv": wv}


def _pairs(frm: np.ndarray, to: np.ndarray, k: int):
    """Distinct (from, to) pairs in first-appearance order and each move's pair index."""
    pairs, of = [], []
    for m in range(k):
        pi = int(frm[m]) * 32 + int(to[m])
        if pi not in pairs:
            pairs.append(pi)
        of.append(pairs.index(pi))
    return pairs, of


def loss_grads(p: np.ndarray, boards, z, q, moves_from, moves_to, counts, tau: float = 0.1,
               value_coef: float = 1.0, emulate: bool = True, dtype=np.float32):
    """(loss2 = [policy, value] means, total loss, flat gradient) of the batch.

    moves_from / moves_to: (n, >= 32) move squares in the reference move-list
    order, counts: legal moves per position (positions with more than 32 moves
    train the value only)."""
    f = forward(p, boards, emulate, dtype)
    n = f["X"].shape[0]
    r = bf16 if emulate else (lambda a: a)
    z = np.asarray(z, dtype)
    q = np.asarray(q, dtype).reshape(n, MAXM)
    dZ3 = np.zeros((n, OUT), dtype)
    ce = np.zeros(n, dtype)
    for i in range(n):
        k = int(counts[i])
        if k < 1 or k > MAXM:
            continue
        pairs, of = _pairs(moves_from[i], moves_to[i], k)
        qi = q[i, :k]
        t = np.exp((qi - qi.max()) / dtype(tau))
        t = t / t.sum()
        tp = np.zeros(len(pairs), dtype)
        for m in range(k):
            tp[of[m]] += t[m]
        lg = f["logits"][i, pairs]
        logz = lg.max() + np.log(np.exp(lg - lg.max()).sum())
        lp = lg - logz
        ce[i] = -(tp * lp).sum()
        dZ3[i, pairs] = (np.exp(lp) - tp) / n
    dZ3 = r(dZ3).astype(dtype)
    th = f["value"]
    e = th - z
    loss_v = e * e
    dv = (value_coef * 2 * e * (1 - th * th) / n).astype(dtype)
    h1, h2, X = f["h1"], f["h2"], f["X"]
    dZ2 = r((dZ3 @ f["W3"] + dv[:, None] * f["wv"][None, :]) * (h2 > 0)).astype(dtype)
    dZ1 = r((dZ2 @ f["W2"]) * (h1 > 0)).astype(dtype)
    g = {
        "W3": dZ3.T @ h2, "b3": dZ3.sum(0),
        "W2": dZ2.T @ h1, "b2": dZ2.sum(0),
        "W1": dZ1.T @ X, "b1": dZ1.sum(0),
        "wv": h2.T @ dv, "bv": np.array([dv.sum()], dtype),
    }
    loss2 = np.array([ce.mean(), loss_v.mean()])
    total = ce.mean() + value_coef * loss_v.mean()
    return loss2, total, pack(g)


def adam(p, m, v, g, step: int, lr: float, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8):
    """One Adam update (bias-corrected); returns new (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v

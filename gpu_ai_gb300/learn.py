"""Training the policy/value network on GPU self-play positions.

The reference has no learned component (its playouts are uniformly random or
follow the material heuristic, src/heuristic.cu:20-49); this module is the
project's own.  Everything runs on one GPU:

  positions   self-play games of the random and the epsilon-greedy playout
              policies from the standard start, cut after U{0..max_plies}
              plies (gpuai_selfplay_positions)
  labels      per position, `playouts` GPU playouts split over its legal
              moves (gpuai_label_positions): the value z is their mean result
              for the side to move (the same estimate as that many random
              playouts from the position), move_q[m] the mean over the
              playouts after move m
  training    Adam on the library's tensor-core forward/backward kernels
              (gpuai_net_train_step), batches from a per-epoch shuffle, cosine
              learning-rate decay
  evaluation  value MAE against the labels of held-out positions; the MAE
              of a k-playout estimate against the same labels is reported
              beside it (plain random playouts judge the value error)

PyTorch only holds device buffers and shuffles indices.
"""
from __future__ import annotations

import argparse
import json
import math
import time
from typing import Dict, Optional

import numpy as np

from .engine import POLICY_EPS_GREEDY, POLICY_RANDOM, Engine, Net

BOARD_BYTES = 16


def _stream():
    import torch
    return torch.cuda.current_stream().cuda_stream


def make_dataset(eng: Engine, n: int, playouts: int = 4096, seed: int = 0, max_plies: int = 90,
                 policies=(POLICY_RANDOM, POLICY_EPS_GREEDY), chunk: int = 65536) -> Dict[str, "object"]:
    """n self-play positions (split evenly over `policies`) with labels, on the
    device; positions whose game is over (or with more than 32 moves) are
    dropped.  Returns torch tensors boards (m, 4) int32, value (m,), q (m, 32),
    nmoves (m,) and the labelling time."""
    import torch
    boards = torch.empty((n, 4), dtype=torch.int32, device="cuda")
    per = -(-n // len(policies))
    st = _stream()
    for i, pol in enumerate(policies):
        lo, hi = i * per, min(n, (i + 1) * per)
        if hi > lo:
            eng.selfplay_positions(seed * 16 + i, hi - lo, 0, max_plies, pol,
                                   boards.data_ptr() + lo * BOARD_BYTES, st)
    value = torch.empty(n, dtype=torch.float32, device="cuda")
    q = torch.empty((n, 32), dtype=torch.float32, device="cuda")
    k = torch.empty(n, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for c in range(0, n, chunk):
        m = min(chunk, n - c)
        eng.label_positions(boards.data_ptr() + c * BOARD_BYTES, m, playouts, seed, (seed << 44) + c * playouts,
                            POLICY_RANDOM, value.data_ptr() + 4 * c, q.data_ptr() + 128 * c, k.data_ptr() + c, st)
    torch.cuda.synchronize()
    label_s = time.perf_counter() - t0
    keep = k > 0
    return {"boards": boards[keep].contiguous(), "value": value[keep].contiguous(), "q": q[keep].contiguous(),
            "nmoves": k[keep].contiguous(), "label_seconds": label_s, "playouts": n * playouts}


def split(data: dict, holdout: int):
    """(train, held-out) views: the last `holdout` rows are held out."""
    m = data["boards"].shape[0]
    keys = ("boards", "value", "q", "nmoves")
    tr = {k: data[k][:m - holdout] for k in keys}
    te = {k: data[k][m - holdout:] for k in keys}
    return tr, te


def train(net: Net, data: dict, epochs: float = 2.0, batch: int = 8192, lr: float = 1e-3, lr_min: float = 2e-5,
          tau: float = 0.1, value_coef: float = 1.0, seed: int = 0, log_every: int = 0) -> dict:
    """Adam with cosine decay over `epochs` passes; returns the loss history and timing."""
    import torch
    n = data["boards"].shape[0]
    if n < batch:
        batch = max(128, n // 128 * 128)
    steps_per_epoch = n // batch
    total = max(1, int(round(epochs * steps_per_epoch)))
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    hist = []
    step = 0
    t_train = 0.0
    while step < total:
        perm = torch.randperm(n, generator=g, device="cuda")
        b = data["boards"][perm].contiguous()
        z = data["value"][perm].contiguous()
        q = data["q"][perm].contiguous()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for s in range(steps_per_epoch):
            if step >= total:
                break
            lr_t = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * step / total))
            want = (log_every and step % log_every == 0) or step == total - 1
            off = s * batch
            loss = net.train_step(b.data_ptr() + off * BOARD_BYTES, z.data_ptr() + 4 * off, q.data_ptr() + 128 * off,
                                  batch, lr_t, tau, value_coef, want_loss=bool(want))
            if loss is not None:
                hist.append((step, float(loss[0]), float(loss[1])))
            step += 1
        net.params()  # waits for the net's stream: the shuffled copies must outlive their steps
        t_train += time.perf_counter() - t0
    return {"steps": total, "batch": batch, "history": hist, "train_seconds": t_train,
            "positions_per_s": total * batch / max(t_train, 1e-9)}


def evaluate(net: Net, eng: Engine, data: dict, baseline_playouts: int = 64, seed: int = 99) -> dict:
    """Value MAE of the network and of a k-playout estimate against the labels,
    and how often the policy's top move is the labels' best move."""
    boards = data["boards"].cpu().numpy().view(np.uint32)
    z = data["value"].cpu().numpy()
    q = data["q"].cpu().numpy()
    k = data["nmoves"].cpu().numpy()
    v, logits = net.forward(boards)
    mae = float(np.abs(v - z).mean())
    out = eng.playouts(boards, np.full(len(boards), baseline_playouts, np.uint32), seed=seed,
                       stream_base=1 << 50).reshape(len(boards), baseline_playouts).astype(np.float64)
    sign = np.where(boards[:, 3] & 1, -1.0, 1.0)
    est = sign * out.mean(1)
    mae_playouts = float(np.abs(est - z).mean())
    moves, counts = eng.genmoves(boards, 64)
    top_ok = 0
    for i in range(len(boards)):
        kk = int(k[i])
        pair = moves[i, :kk, 0].astype(np.int64) * 32 + moves[i, :kk, 1]
        top_ok += int(np.argmax(logits[i, pair]) == np.argmax(q[i, :kk]))
    return {"positions": len(boards), "value_mae": mae, f"value_mae_{baseline_playouts}_playouts": mae_playouts,
            "policy_top1_vs_best_label": top_ok / max(1, len(boards))}


def main(argv: Optional[list] = None):
    ap = argparse.ArgumentParser(description="train the policy/value network on GPU self-play")
    ap.add_argument("--positions", type=int, default=10_000_000)
    ap.add_argument("--playouts", type=int, default=4096)
    ap.add_argument("--holdout", type=int, default=50_000)
    ap.add_argument("--epochs", type=float, default=2.0)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default="")
    a = ap.parse_args(argv)
    eng = Engine(0)
    t0 = time.perf_counter()
    data = make_dataset(eng, a.positions, a.playouts, a.seed)
    tr, te = split(data, min(a.holdout, data["boards"].shape[0] // 10))
    net = Net(0, max_batch=a.batch, seed=a.seed)
    res = train(net, tr, a.epochs, a.batch, a.lr, seed=a.seed, log_every=500)
    ev = evaluate(net, eng, te)
    if a.out:
        net.save(a.out)
    print(json.dumps({"positions": int(data["boards"].shape[0]), "label_seconds": data["label_seconds"],
                      "label_playouts_per_s": data["playouts"] / data["label_seconds"],
                      "train": {k: v for k, v in res.items() if k != "history"},
                      "loss_first_last": [res["history"][0], res["history"][-1]], "eval": ev,
                      "seconds": time.perf_counter() - t0}))


if __name__ == "__main__":
    main()

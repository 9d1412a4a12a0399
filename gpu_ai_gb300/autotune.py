"""Autotuner for the playout kernel and the batched-search step.

Sweeps, on the current GPU, (1) the playout kernel's layout (a thread per
playout, a warp per playout with one lane per square, or a thread per playout
with the block pool for deferred multi-jump plies) x launch shape
(threads per block 64-512 x resident blocks per SM) on a batch of random
playouts and
(2) the batched-search step's leaves per search and playouts per leaf, and
caches the fastest settings in a JSON file keyed by GPU name (default
``~/.cache/gpu_ai_gb300/autotune.json``).  ``apply(engine)`` sets a cached
layout and launch shape on an Engine.

    python -m gpu_ai_gb300.autotune [--quick] [--cache PATH]
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from .engine import LAYOUT_POOLED, LAYOUT_THREAD, LAYOUT_WARP, Engine, Searches

LAYOUT_NAMES = {LAYOUT_THREAD: "thread", LAYOUT_WARP: "warp", LAYOUT_POOLED: "pooled"}

DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "gpu_ai_gb300", "autotune.json")


def gpu_name() -> str:
    import torch
    return torch.cuda.get_device_name(0)


def _time_playouts(eng: Engine, pos, reps, repeats: int) -> float:
    eng.playouts(pos, reps, seed=1, stream_base=0)  # warm up
    best = float("inf")
    for k in range(repeats):
        t0 = time.perf_counter()
        eng.playouts(pos, reps, seed=2, stream_base=(k + 1) << 32)
        best = min(best, time.perf_counter() - t0)
    return best


def tune_playouts(eng: Engine, n_pos=64, reps_per_pos=4096, repeats=3, blocks=(64, 128, 256, 512),
                  layouts=(LAYOUT_THREAD, LAYOUT_WARP, LAYOUT_POOLED)):
    pos = eng.random_positions(2016, n_pos, 0, 30)
    reps = np.full(n_pos, reps_per_pos, np.uint32)
    total = n_pos * reps_per_pos
    results = []
    for layout in layouts:
        eng.set_layout(0, layout)
        for block in blocks:
            eng.set_launch(0, block, 0)
            mx = eng.get_launch(0)["max_blocks_per_sm"]
            for per_sm in sorted({max(1, mx // 2), max(1, (3 * mx) // 4), mx}):
                eng.set_launch(0, block, per_sm)
                t = _time_playouts(eng, pos, reps, repeats)
                results.append({"layout": LAYOUT_NAMES[layout], "block_threads": block,
                                "blocks_per_sm": per_sm, "seconds": t, "playouts_per_s": total / t})
    best = max(results, key=lambda r: r["playouts_per_s"])
    _set(eng, best)
    return best, results


def _set(eng: Engine, p: dict):
    by_name = {v: k for k, v in LAYOUT_NAMES.items()}
    eng.set_layout(0, by_name.get(p.get("layout"), LAYOUT_THREAD))
    eng.set_launch(0, p["block_threads"], p["blocks_per_sm"])


def tune_searches(n_games=512, leaves=(32, 64, 128, 256), ppls=(2, 4, 8), seed=7):
    eng = Engine(0)
    roots = eng.random_positions(seed, n_games, 0, 60)
    rng = np.random.default_rng(seed)
    budgets = np.clip(np.exp(rng.normal(np.log(8192), 1.0, n_games)), 1024, 65536).astype(np.int64)
    results = []
    for q in leaves:
        for ppl in ppls:
            b = (budgets + ppl - 1) // ppl * ppl
            caps = np.minimum(b, 65536) * 2
            s = Searches(n_games, int(caps.sum()) + 1024, q, playouts_per_leaf=ppl)
            for i in range(n_games):
                s.add(roots[i], int(b[i]), int(caps[i]), i << 40)
            t0 = time.perf_counter()
            while True:
                done, budget = s.poll()
                if (done >= budget).all():
                    break
                s.step(8, q, True)
            el = time.perf_counter() - t0
            results.append({"leaves_per_search": q, "playouts_per_leaf": ppl, "seconds": el,
                            "playouts_per_s": float(done.sum()) / el})
            s.close()
    best = max(results, key=lambda r: r["playouts_per_s"])
    return best, results


def load(cache: str = DEFAULT_CACHE):
    try:
        with open(cache) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def apply(eng: Engine, cache: str = DEFAULT_CACHE) -> bool:
    """Set the cached playout launch shape for this GPU on `eng`; False if none."""
    entry = load(cache).get(gpu_name())
    if not entry:
        return False
    _set(eng, entry["playouts"])
    return True


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cache", default=DEFAULT_CACHE)
    ap.add_argument("--quick", action="store_true", help="fewer settings (for tests)")
    args = ap.parse_args()
    eng = Engine(0)
    if args.quick:
        best_p, all_p = tune_playouts(eng, n_pos=16, reps_per_pos=1024, repeats=1, blocks=(128, 256))
        best_s, all_s = tune_searches(n_games=64, leaves=(32, 64), ppls=(4,))
    else:
        best_p, all_p = tune_playouts(eng)
        best_s, all_s = tune_searches()
    data = load(args.cache)
    data[gpu_name()] = {"playouts": best_p, "searches": best_s, "sweep": {"playouts": all_p, "searches": all_s}}
    os.makedirs(os.path.dirname(os.path.abspath(args.cache)), exist_ok=True)
    with open(args.cache, "w") as f:
        json.dump(data, f, indent=1)
    print(json.dumps({"gpu": gpu_name(), "playouts": best_p, "searches": best_s}))


if __name__ == "__main__":
    main()

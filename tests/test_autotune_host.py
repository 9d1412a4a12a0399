"""The autotuner's host logic on a fake engine (no GPU): which launch shapes
it sweeps, that it keeps the fastest and leaves it set, and the per-GPU
cache that apply() reads."""
import json

import numpy as np

from gpu_ai_gb300 import autotune
from gpu_ai_gb300.engine import LAYOUT_POOLED, LAYOUT_THREAD, LAYOUT_WARP


class FakeEngine:
    def __init__(self):
        self.layout, self.block, self.per_sm = LAYOUT_THREAD, 256, 0
        self.max_per_sm = {64: 16, 128: 8, 256: 4, 512: 2}

    def random_positions(self, seed, n, lo, hi):
        return np.zeros((n, 4), np.uint32)

    def set_layout(self, policy, layout):
        self.layout = layout

    def set_launch(self, policy, block, per_sm):
        self.block = block
        mx = self.max_per_sm[block]
        self.per_sm = mx if per_sm == 0 or per_sm > mx else per_sm

    def get_launch(self, policy):
        return {"block_threads": self.block, "blocks_per_sm": self.per_sm,
                "max_blocks_per_sm": self.max_per_sm[self.block]}


def _fake_time(eng, pos, reps, repeats):
    # fastest: thread layout, 512 threads, 2 blocks per SM
    t = 1.0 + abs(eng.block - 512) / 1024 + (eng.max_per_sm[eng.block] - eng.per_sm) / 16
    return t + (0.5 if eng.layout == LAYOUT_WARP else (0.25 if eng.layout == LAYOUT_POOLED else 0.0))


def test_sweep_keeps_and_sets_the_fastest(monkeypatch):
    monkeypatch.setattr(autotune, "_time_playouts", _fake_time)
    eng = FakeEngine()
    best, results = autotune.tune_playouts(eng, n_pos=4, reps_per_pos=8, repeats=1)
    shapes = {(r["layout"], r["block_threads"], r["blocks_per_sm"]) for r in results}
    # every layout x block size x {half, three quarters, all} of the resident blocks
    exp = {(l, b, p) for l in ("thread", "warp", "pooled") for b, mx in eng.max_per_sm.items()
           for p in {max(1, mx // 2), max(1, 3 * mx // 4), mx}}
    assert shapes == exp
    assert (best["layout"], best["block_threads"], best["blocks_per_sm"]) == ("thread", 512, 2)
    assert best["playouts_per_s"] == max(r["playouts_per_s"] for r in results)
    assert (eng.layout, eng.block, eng.per_sm) == (LAYOUT_THREAD, 512, 2)


def test_apply_reads_this_gpus_entry(monkeypatch, tmp_path):
    cache = tmp_path / "autotune.json"
    cache.write_text(json.dumps({
        "GPU A": {"playouts": {"layout": "warp", "block_threads": 128, "blocks_per_sm": 6}},
        "GPU B": {"playouts": {"layout": "thread", "block_threads": 64, "blocks_per_sm": 12}}}))
    eng = FakeEngine()
    monkeypatch.setattr(autotune, "gpu_name", lambda: "GPU A")
    assert autotune.apply(eng, str(cache))
    assert (eng.layout, eng.block, eng.per_sm) == (LAYOUT_WARP, 128, 6)
    monkeypatch.setattr(autotune, "gpu_name", lambda: "GPU C")
    assert not autotune.apply(eng, str(cache))  # no entry: settings untouched
    assert (eng.layout, eng.block, eng.per_sm) == (LAYOUT_WARP, 128, 6)


def test_unreadable_cache_is_empty(tmp_path):
    bad = tmp_path / "bad.json"
    bad.write_text("{not json")
    assert autotune.load(str(bad)) == {}
    assert autotune.load(str(tmp_path / "missing.json")) == {}

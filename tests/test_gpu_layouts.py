"""The warp-per-playout layout gives the thread-per-playout layout's outcomes
bit for bit (and the oracle replay's), for every launch shape."""
import numpy as np
import pytest

import oracle_lib as L

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("block", [64, 256, 512])
def test_warp_layout_equals_thread_layout(engine, block):
    from gpu_ai_gb300 import LAYOUT_THREAD, LAYOUT_WARP
    pos = L.random_positions(321, 96, 0, 80)
    reps = np.full(len(pos), 64, np.uint32)
    try:
        engine.set_layout(0, LAYOUT_THREAD)
        engine.set_launch(0, 256, 0)
        want = engine.playouts(pos, reps, seed=4, stream_base=77)
        _, plies_thread = engine.status()
        engine.set_layout(0, LAYOUT_WARP)
        engine.set_launch(0, block, 0)
        assert engine.get_layout(0) == LAYOUT_WARP
        got = engine.playouts(pos, reps, seed=4, stream_base=77)
        st, plies_warp = engine.status()
    finally:
        engine.set_layout(0, LAYOUT_THREAD)
        engine.set_launch(0, 256, 0)
    assert st == 0
    assert np.array_equal(got, want)
    assert plies_warp == plies_thread
    exp, _ = L.replay_batch(pos[:12], reps[:12], seed=4, stream_base=77)
    assert np.array_equal(got[:12 * 64], exp)


def test_warp_layout_only_for_the_random_policy(engine):
    from gpu_ai_gb300 import LAYOUT_WARP, GpuAIError
    with pytest.raises(GpuAIError):
        engine.set_layout(1, LAYOUT_WARP)
    with pytest.raises(GpuAIError):
        engine.set_layout(0, 7)


@pytest.mark.parametrize("policy", [0, 1, 2])
@pytest.mark.parametrize("block", [256, 512])
def test_pooled_layout_equals_thread_layout(engine, policy, block):
    """Deferred multi-jump plies gathered in the block pool and played by full
    warps: every game moves between lanes with its whole state, so outcomes
    and ply counts equal the thread layout's and the oracle replay's."""
    from gpu_ai_gb300 import LAYOUT_POOLED, LAYOUT_THREAD
    pos = L.random_positions(322 + policy, 128, 0, 60)
    reps = np.random.default_rng(policy).integers(0, 400, len(pos)).astype(np.uint32)
    try:
        engine.set_layout(policy, LAYOUT_THREAD)
        want = engine.playouts(pos, reps, seed=5, stream_base=99, policy=policy)
        _, plies_thread = engine.status()
        engine.set_layout(policy, LAYOUT_POOLED)
        engine.set_launch(policy, block, 0)
        got = engine.playouts(pos, reps, seed=5, stream_base=99, policy=policy)
        st, plies_pooled = engine.status()
    finally:
        engine.set_layout(policy, LAYOUT_THREAD)
        engine.set_launch(policy, 512 if policy == 0 else 256, 0)
    assert st == 0
    assert np.array_equal(got, want)
    assert plies_pooled == plies_thread
    exp, _ = L.replay_batch(pos[:16], reps[:16], seed=5, stream_base=99, policy=policy)
    assert np.array_equal(got[:int(reps[:16].sum())], exp)


def test_pooled_layout_full_benchmark_batch_bit_exact(engine):
    """All 262,144 playouts of the benchmark batch in the pooled layout replay
    bit-exact on the oracle."""
    from gpu_ai_gb300 import LAYOUT_POOLED, LAYOUT_THREAD
    pos = L.random_positions(2016, 64, 0, 30)
    reps = np.full(64, 4096, np.uint32)
    try:
        engine.set_layout(0, LAYOUT_POOLED)
        engine.set_launch(0, 512, 0)
        got = engine.playouts(pos, reps, seed=0x5EED, stream_base=3 << 20)
        st, plies = engine.status()
    finally:
        engine.set_layout(0, LAYOUT_THREAD)
        engine.set_launch(0, 512, 0)
    assert st == 0
    exp, pl = L.replay_batch(pos, reps, seed=0x5EED, stream_base=3 << 20, nthreads=0)
    assert np.array_equal(got, exp)
    assert plies == int(pl.sum())

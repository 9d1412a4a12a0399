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

"""Maximum sizes through the C ABI: one call of 2^31 - 1 playouts (the largest
total gpuai_playouts accepts), stream ids near the top of their 64-bit range,
and 2^20 positions in one call.  Playouts sampled at both ends of the index
range, where index, offset and stream arithmetic would overflow first, and
in between replay bit-exact on the oracle."""
import numpy as np
import pytest

import oracle_lib as L
from gpu_ai_gb300 import GpuAIError

pytestmark = pytest.mark.gpu

MAX_TOTAL = 2**31 - 1


def _replays(pos, offsets, out, seed, stream_base, idx):
    """Playout j (position p with offsets[p] <= j < offsets[p + 1]) of the
    call replayed alone on the oracle from stream stream_base + j."""
    for j in idx:
        p = int(np.searchsorted(offsets, j, side="right")) - 1
        o, _, _ = L.replay_one(pos[p], seed, stream_base + int(j))
        assert out[j] == o, (int(j), p)


def test_largest_total_in_one_call(engine):
    pos = L.random_positions(2016, 64, 0, 30)
    reps = np.full(64, MAX_TOTAL // 64, np.uint32)
    reps[-1] += np.uint32(MAX_TOTAL - int(reps.sum(dtype=np.uint64)))  # unequal: the offsets path
    assert int(reps.sum(dtype=np.uint64)) == MAX_TOTAL
    out = engine.playouts(pos, reps, seed=99, stream_base=5)
    assert out.shape == (MAX_TOTAL,)
    counts = np.bincount(out.view(np.uint8), minlength=256)
    assert int(counts[0]) + int(counts[1]) + int(counts[255]) == MAX_TOTAL  # every outcome is -1, 0 or 1
    status, plies = engine.status()
    assert status == 0 and 40 < plies / MAX_TOTAL < 70
    offsets = np.concatenate([[0], np.cumsum(reps.astype(np.int64))])
    rng = np.random.default_rng(1)
    idx = np.concatenate([np.arange(2000), np.arange(MAX_TOTAL - 2000, MAX_TOTAL), rng.integers(0, MAX_TOTAL, 2000)])
    _replays(pos, offsets, out, 99, 5, idx)
    more = reps.copy()
    more[0] += 1
    with pytest.raises(GpuAIError):  # one playout more is refused before any launch
        engine.playouts(pos, more, seed=99)


@pytest.mark.parametrize("base", [(1 << 63) + 12345, (1 << 64) - 3000])
def test_stream_ids_near_the_top_of_their_range(engine, base):
    pos = L.random_positions(7, 8, 0, 30)
    reps = np.full(8, 250, np.uint32)
    out = engine.playouts(pos, reps, seed=3, stream_base=base)
    exp, _ = L.replay_batch(pos, reps, seed=3, stream_base=base)
    np.testing.assert_array_equal(out, exp)


def test_a_million_positions_in_one_call(engine):
    n = 1 << 20
    pos = engine.random_positions(11, n, 0, 40)  # the GPU's generator (equal to the oracle's)
    out = engine.playouts(pos, None, seed=4, stream_base=0)
    assert out.shape == (n,)
    rng = np.random.default_rng(2)
    idx = np.concatenate([np.arange(500), np.arange(n - 500, n), rng.integers(0, n, 1000)])
    _replays(pos, np.arange(n + 1), out, 4, 0, idx)

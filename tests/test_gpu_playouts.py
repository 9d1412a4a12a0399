"""GPU playouts through the C ABI: every playout replays bit-exact on the CPU
oracle (same Philox streams, reference move-list order), and outcome
frequencies agree with the reference's own host playouts (99% chi-square)."""
import numpy as np
import pytest

import oracle_lib as L
from golden_boards import crafted_boards
from gpu_ai_gb300 import ERR_INVALID, GpuAIError
from stats import wdl_agreement

pytestmark = pytest.mark.gpu


def _mixed_positions():
    return np.concatenate([L.random_positions(5, 200, 0, 60), crafted_boards(),
                           L.random_positions(6, 100, 40, 120)])


@pytest.mark.parametrize("policy", [0, 1, 2])
def test_replay_bit_exact(engine, policy):
    pos = _mixed_positions()
    rng = np.random.default_rng(policy)
    reps = rng.integers(0, 40, len(pos)).astype(np.uint32)
    reps[:3] = 0
    got = engine.playouts(pos, reps, seed=0xC0FFEE + policy, stream_base=1000, policy=policy)
    exp, _ = L.replay_batch(pos, reps, seed=0xC0FFEE + policy, stream_base=1000, policy=policy)
    assert got.shape == exp.shape
    np.testing.assert_array_equal(got, exp)


def test_full_benchmark_batch_bit_exact(engine, golden_playout):
    """All 262,144 playouts of the benchmark batch replay bit-exact, and the
    kernel's ply counter equals the replayed plies."""
    pos = golden_playout["positions"]
    reps = np.full(len(pos), int(golden_playout["reps"]), dtype=np.uint32)
    got = engine.playouts(pos, reps, seed=2016, stream_base=0, policy=0)
    status, plies = engine.status()
    exp, exp_plies = L.replay_batch(pos, reps, seed=2016, stream_base=0, policy=0)
    np.testing.assert_array_equal(got, exp)
    assert status == 0
    assert plies == int(exp_plies.sum(dtype=np.uint64))



def test_reused_out_buffer(engine):
    """`out=` receives the same outcomes as a fresh array, is returned as is,
    and a buffer of the wrong type, size or layout is refused before launch."""
    pos = L.random_positions(9, 40, 0, 30)
    reps = np.full(len(pos), 17, dtype=np.uint32)
    exp = engine.playouts(pos, reps, seed=77, stream_base=5)
    buf = np.full(exp.size, 99, dtype=np.int8)
    got = engine.playouts(pos, reps, seed=77, stream_base=5, out=buf)
    assert got is buf
    np.testing.assert_array_equal(buf, exp)
    for bad in (np.empty(exp.size, np.int16), np.empty(exp.size + 1, np.int8),
                np.empty(2 * exp.size, np.int8)[::2]):
        with pytest.raises(ValueError):
            engine.playouts(pos, reps, seed=77, stream_base=5, out=bad)

def test_outcome_frequencies_match_reference_host(engine, golden_playout):
    pos = golden_playout["positions"]
    reps = np.full(len(pos), int(golden_playout["reps"]), dtype=np.uint32)
    got = engine.playouts(pos, reps, seed=77, policy=0).reshape(len(pos), -1)
    mine = np.stack([L.wdl(r) for r in got])
    ok, det = wdl_agreement(mine, golden_playout["wdl_host"])
    assert ok, det


def test_heuristic_frequencies_match_reference_host_heuristic(engine, golden_playout):
    pos = golden_playout["positions"]
    reps = np.full(len(pos), int(golden_playout["reps"]), dtype=np.uint32)
    got = engine.playouts(pos, reps, seed=78, policy=1).reshape(len(pos), -1)
    mine = np.stack([L.wdl(r) for r in got])
    ok, det = wdl_agreement(mine, golden_playout["wdl_host_heuristic"])
    assert ok, det


def test_split_calls_equal_one_call(engine):
    pos = L.random_positions(9, 50, 0, 30)
    reps = np.full(50, 64, dtype=np.uint32)
    whole = engine.playouts(pos, reps, seed=5, stream_base=0)
    a = engine.playouts(pos[:20], reps[:20], seed=5, stream_base=0)
    b = engine.playouts(pos[20:], reps[20:], seed=5, stream_base=20 * 64)
    np.testing.assert_array_equal(whole, np.concatenate([a, b]))
    np.testing.assert_array_equal(whole, engine.playouts(pos, reps, seed=5, stream_base=0))
    assert not np.array_equal(whole, engine.playouts(pos, reps, seed=6, stream_base=0))


def test_empty_and_ragged(engine):
    pos = L.random_positions(1, 4, 0, 10)
    assert engine.playouts(pos[:0]).shape == (0,)
    assert engine.playouts(pos, np.zeros(4, np.uint32)).shape == (0,)
    got = engine.playouts(pos, np.array([0, 3, 0, 2], np.uint32), seed=3)
    exp, _ = L.replay_batch(pos, np.array([0, 3, 0, 2], np.uint32), seed=3)
    np.testing.assert_array_equal(got, exp)
    one = engine.playouts(pos, None, seed=3)
    exp1, _ = L.replay_batch(pos, np.ones(4, np.uint32), seed=3)
    np.testing.assert_array_equal(one, exp1)


def test_terminal_positions(engine):
    b = crafted_boards()
    # PLAYER_1 to move without pieces loses; counter at 50 is a draw
    got = engine.playouts(b[[11, 12, 14]], np.array([3, 3, 3], np.uint32), seed=1)
    assert list(got) == [-1, -1, -1, -1, -1, -1, 0, 0, 0]


def test_invalid_inputs(engine):
    with pytest.raises(GpuAIError) as ei:
        engine.playouts(np.array([[0, 0, 1, 0]], np.uint32))  # king bit on an empty square
    assert ei.value.code == ERR_INVALID
    with pytest.raises(GpuAIError):
        engine.playouts(np.array([[1, 2, 0, 1 << 20]], np.uint32))  # reserved meta bits
    with pytest.raises(GpuAIError):
        engine.playouts(L.start_board(), policy=7)


def test_device_resident_path(engine, golden_playout):
    torch = pytest.importorskip("torch")
    pos = golden_playout["positions"]
    d_pos = torch.from_numpy(pos.view(np.int32).copy()).cuda()
    d_out = torch.empty(64 * 512, dtype=torch.int8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    engine.playouts_device(d_pos.data_ptr(), None, 64, 512, 64 * 512, 99, 7, 0, d_out.data_ptr(), stream)
    torch.cuda.synchronize()
    exp, _ = L.replay_batch(pos, np.full(64, 512, np.uint32), seed=99, stream_base=7)
    np.testing.assert_array_equal(d_out.cpu().numpy(), exp)
    offs = np.concatenate([[0], np.cumsum(np.full(64, 512))]).astype(np.uint32)
    d_off = torch.from_numpy(offs.view(np.int32).copy()).cuda()
    d_out.zero_()
    engine.playouts_device(d_pos.data_ptr(), d_off.data_ptr(), 64, 0, 64 * 512, 99, 7, 0, d_out.data_ptr(),
                           stream)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d_out.cpu().numpy(), exp)
    assert engine.status()[0] == 0


@pytest.mark.parametrize("block,per_sm", [(64, 0), (128, 3), (256, 1), (512, 0)])
def test_launch_shape_does_not_change_results(engine, block, per_sm):
    pos = L.random_positions(21, 64, 0, 30)
    reps = np.full(64, 300, dtype=np.uint32)
    exp, _ = L.replay_batch(pos, reps, seed=21, stream_base=5)
    old = engine.get_launch(0)
    try:
        engine.set_launch(0, block, per_sm)
        got = engine.playouts(pos, reps, seed=21, stream_base=5)
    finally:
        engine.set_launch(0, old["block_threads"], old["blocks_per_sm"])
    np.testing.assert_array_equal(got, exp)


def test_set_launch_rejects_bad_shapes(engine):
    with pytest.raises(GpuAIError):
        engine.set_launch(0, 96, 0)
    with pytest.raises(GpuAIError):
        engine.set_launch(5, 256, 0)


@pytest.mark.parametrize("seed", [78, 4079])
def test_heuristic_frequencies_32k_per_position(engine, seed):
    """The reference-heuristic policy against the reference's
    HostHeuristicPlayoutDriver with 32,768 playouts per position (8 times the
    benchmark count, so a smaller difference of distributions would show),
    for two seeds."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                             "playout_golden_heuristic_32k.npz"))
    pos = g["positions"]
    reps = np.full(len(pos), int(g["reps"]), dtype=np.uint32)
    got = engine.playouts(pos, reps, seed=seed, stream_base=1 << 36, policy=1).reshape(len(pos), -1)
    mine = np.stack([L.wdl(r) for r in got])
    ok, det = wdl_agreement(mine, g["wdl_host_heuristic"])
    assert ok, det

"""Pin the CPU oracle: Philox known answers, the reference's golden move
lists and outcome frequencies, and (where the reference sources are present)
the reference's own code run live."""
import numpy as np
import pytest

import oracle_lib as L
from golden_boards import crafted_boards, random_boards
from stats import wdl_agreement


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10 (Salmon et al., SC'11)
    assert L.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert L.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert L.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_stream_layout():
    # draw k of (seed, id, tag) is word k&3 of philox({k>>2, id_lo, id_hi, tag}, {seed_lo, seed_hi})
    seed, sid, tag = 0x0123456789ABCDEF, 0xFEDCBA9876543210, 1
    for k in range(9):
        blk = L.philox([k >> 2, sid & 0xFFFFFFFF, sid >> 32, tag], [seed & 0xFFFFFFFF, seed >> 32])
        assert L.stream_draw(seed, sid, tag, k) == blk[k & 3]


def test_oracle_matches_golden_reference_moves(golden_movegen):
    boards, moves, counts = golden_movegen
    got, gc = L.genmoves(boards, max_moves=moves.shape[1])
    np.testing.assert_array_equal(gc, counts)
    np.testing.assert_array_equal(got, moves)


def test_golden_covers_edge_cases(golden_movegen):
    boards, moves, counts = golden_movegen
    jumps = moves[:, :, 2]
    valid = np.arange(moves.shape[1])[None, :] < counts[:, None]
    assert (counts == 0).any(), "positions with no legal move"
    assert jumps[valid].max() >= 4, "long multi-jumps"
    assert ((moves[:, :, 3] == 1) & valid & (jumps > 0)).any(), "promoting captures"
    assert ((moves[:, :, 3] == 1) & valid & (jumps == 0)).any(), "promoting direct moves"
    kings_move = ((boards[:, 2] != 0) & (counts > 0)).sum()
    assert kings_move > 1000


def test_start_position_moves():
    m, c = L.genmoves(L.start_board())
    assert c[0] == 7  # PLAYER_1's seven opening moves
    assert all(m[0, k, 2] == 0 for k in range(7))


def test_seeded_positions_deterministic():
    a = L.random_positions(2016, 64, 0, 30)
    b = L.random_positions(2016, 64, 0, 30)
    np.testing.assert_array_equal(a, b)
    assert len({tuple(r) for r in a}) > 40
    c = L.random_positions(2017, 64, 0, 30)
    assert not np.array_equal(a, c)


def test_benchmark_positions_match_golden(golden_playout):
    pos = L.random_positions(int(golden_playout["seed"]), len(golden_playout["positions"]), 0,
                             int(golden_playout["max_plies"]))
    np.testing.assert_array_equal(pos, golden_playout["positions"])


def test_replay_distribution_matches_reference(golden_playout):
    """Uniform choice over the reference move list with the project's Philox
    streams reproduces the reference HostPlayoutDriver's outcome
    frequencies (99% chi-square, Bonferroni over the 64 positions)."""
    pos = golden_playout["positions"]
    reps = np.full(len(pos), 1024, dtype=np.uint32)
    out, plies = L.replay_batch(pos, reps, seed=11, policy=0)
    mine = np.stack([L.wdl(r) for r in out.reshape(len(pos), -1)])
    ok, det = wdl_agreement(mine, golden_playout["wdl_host"])
    assert ok, det


def test_host_port_distribution_matches_reference(golden_playout):
    """The restated HostPlayoutDriver (timed CPU baseline on machines where the
    reference cannot be built) has the reference's outcome frequencies."""
    pos = golden_playout["positions"]
    states = np.repeat(pos, 512, axis=0)
    out = L.host_playouts_port(states, nthreads=0, srand_seed=3)
    mine = np.stack([L.wdl(r) for r in out.reshape(len(pos), -1)])
    ok, det = wdl_agreement(mine, golden_playout["wdl_host"])
    assert ok, det


def test_terminal_positions():
    # no pieces to move: side to move loses; draw counter reached: draw
    b = crafted_boards()
    o, plies, draws = L.replay_one(b[11], 1, 0)
    assert (o, plies, draws) == (-1, 0, 0)
    o, plies, draws = L.replay_one(b[14], 1, 0)
    assert (o, plies) == (0, 0)


_ref_available = L.ref() is not None


@pytest.mark.skipif(not _ref_available, reason="reference sources not present")
def test_oracle_matches_reference_live():
    """The oracle's move lists equal the reference's own State::genMoves,
    byte for byte, on 10^6 positions of 0-150 random plies, 10^5 random dense
    boards (kings, forced captures, long multi-jumps) and the crafted cases."""
    pos = np.concatenate([L.random_positions(4242, 1_000_000, 0, 150),
                          random_boards(np.random.default_rng(99), 100_000),
                          crafted_boards()])
    a, ca = L.genmoves(pos, max_moves=64)
    b, cb = L.genmoves(pos, max_moves=64, lib=L.ref())
    np.testing.assert_array_equal(ca, cb)
    np.testing.assert_array_equal(a, b)


@pytest.mark.skipif(not _ref_available, reason="reference sources not present")
def test_apply_matches_reference_live():
    rng = np.random.default_rng(3)
    pos = L.random_positions(31, 3000, 0, 80)
    moves, counts = L.genmoves(pos)
    lib = L.ref()
    for i in range(len(pos)):
        if counts[i] == 0:
            continue
        k = int(rng.integers(counts[i]))
        a = pos[i].copy()
        assert L.oracle().or_apply_packed_b16(a.ctypes.data_as(L._u32p), moves[i, k].ctypes.data_as(L._u8p)) == 0
        b = pos[i].copy()
        assert lib.ref_apply_b16(b.ctypes.data_as(L._u32p), k) == 0
        np.testing.assert_array_equal(a, b)


def test_stronger_cpu_baseline_equals_the_replay():
    """The stronger CPU baseline (the kernel's bitboard ply on the host with the
    GPU's streams) gives every playout the outcome of the oracle's replay."""
    pos = L.random_positions(2016, 64, 0, 30)
    reps = np.full(64, 24, dtype=np.uint32)
    out, plies = L.cpu_playouts(pos, reps, 0x5EED, 77)
    exp, pl = L.replay_batch(pos, reps, 0x5EED, 77, 0)
    np.testing.assert_array_equal(out, exp)
    assert plies == int(pl.sum())

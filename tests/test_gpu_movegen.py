"""GPU move generation: bit-exact against the reference's genMoves (golden)
and the oracle, through the C ABI."""
import numpy as np
import pytest

import oracle_lib as L
from golden_boards import crafted_boards, random_boards
from gpu_ai_gb300 import ERR_INVALID, ERR_LIMIT, GpuAIError

pytestmark = pytest.mark.gpu


def test_genmoves_matches_reference_golden(engine, golden_movegen):
    boards, moves, counts = golden_movegen
    got, c = engine.genmoves(boards, max_moves=moves.shape[1])
    np.testing.assert_array_equal(c, counts)
    np.testing.assert_array_equal(got, moves)


def test_genmoves_matches_oracle_large(engine):
    pos = np.concatenate([L.random_positions(123, 200000, 0, 150),
                          random_boards(np.random.default_rng(11), 100000),
                          crafted_boards()])
    got, c = engine.genmoves(pos, max_moves=40)
    exp, ce = L.genmoves(pos, max_moves=40)
    np.testing.assert_array_equal(c, ce)
    np.testing.assert_array_equal(got, exp)


def test_genmoves_overflow_is_reported(engine):
    with pytest.raises(GpuAIError) as ei:
        engine.genmoves(L.start_board(), max_moves=3)
    assert ei.value.code == ERR_LIMIT


def test_genmoves_rejects_malformed_board(engine):
    bad = np.array([[1, 1, 0, 0]], dtype=np.uint32)  # square 0 held by both sides
    with pytest.raises(GpuAIError) as ei:
        engine.genmoves(bad)
    assert ei.value.code == ERR_INVALID


def test_random_positions_match_oracle(engine):
    for lo, hi in ((0, 30), (0, 120), (10, 40), (0, 0)):
        got = engine.random_positions(2016, 20000, lo, hi)
        np.testing.assert_array_equal(got, L.random_positions(2016, 20000, lo, hi))

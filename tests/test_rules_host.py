"""The device rules header compiled for the host agrees with the oracle.

gpu_ai_gb300/csrc/rules.cuh is the code the kernels run; a g++ build of it
(tests/rules_host.cpp) is checked here on the CPU: move lists, the per-ply
code of every policy, and the seeded position generator."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import oracle_lib as L
from golden_boards import crafted_boards, random_boards

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "_build", "librules_host.so")
SRC = os.path.join(HERE, "rules_host.cpp")
HDR = os.path.join(os.path.dirname(HERE), "gpu_ai_gb300", "csrc", "rules.cuh")

u32p = ctypes.POINTER(ctypes.c_uint32)
u8p = ctypes.POINTER(ctypes.c_uint8)


@pytest.fixture(scope="module")
def rh():
    if not os.path.exists(SO) or max(os.path.getmtime(SRC), os.path.getmtime(HDR)) > os.path.getmtime(SO):
        os.makedirs(os.path.dirname(SO), exist_ok=True)
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-Wno-unknown-pragmas", "-o", SO, SRC],
                       check=True)
    lib = ctypes.CDLL(SO)
    lib.rh_genmoves_b16.argtypes = [u32p, ctypes.c_uint32, u8p, ctypes.c_uint32, u8p]
    lib.rh_playout.argtypes = [u32p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, u32p, u32p]
    lib.rh_playout_ring.argtypes = [u32p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int, u32p, u32p]
    lib.rh_random_positions.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, u32p]
    return lib


def rh_genmoves(lib, pos, max_moves=64):
    pos = np.ascontiguousarray(pos, dtype=np.uint32)
    out = np.zeros((len(pos), max_moves, 32), np.uint8)
    c = np.zeros(len(pos), np.uint8)
    rc = lib.rh_genmoves_b16(pos.ctypes.data_as(u32p), len(pos), out.ctypes.data_as(u8p), max_moves,
                             c.ctypes.data_as(u8p))
    assert rc == 0
    return out, c


def test_moves_match_golden(rh, golden_movegen):
    boards, moves, counts = golden_movegen
    got, c = rh_genmoves(rh, boards, moves.shape[1])
    np.testing.assert_array_equal(c, counts)
    np.testing.assert_array_equal(got, moves)


def test_moves_match_oracle(rh):
    pos = np.concatenate([L.random_positions(5, 60000, 0, 150), random_boards(np.random.default_rng(1), 40000),
                          crafted_boards()])
    a, ca = L.genmoves(pos, 64)
    b, cb = rh_genmoves(rh, pos, 64)
    np.testing.assert_array_equal(ca, cb)
    np.testing.assert_array_equal(a, b)


def test_random_positions_match_oracle(rh):
    out = np.zeros((5000, 4), np.uint32)
    rh.rh_random_positions(2016, 5000, 0, 60, out.ctypes.data_as(u32p))
    np.testing.assert_array_equal(out, L.random_positions(2016, 5000, 0, 60))


@pytest.mark.parametrize("policy", [0, 1, 2])
def test_playouts_replay_on_oracle(rh, policy):
    pos = np.concatenate([L.random_positions(8, 300, 0, 60), crafted_boards()])
    for i in range(1200):
        p = np.ascontiguousarray(pos[i % len(pos)])
        pl = np.zeros(1, np.uint32)
        dr = np.zeros(1, np.uint32)
        o = rh.rh_playout(p.ctypes.data_as(u32p), 77, 1000 + i, policy, pl.ctypes.data_as(u32p),
                          dr.ctypes.data_as(u32p))
        assert (o, int(pl[0]), int(dr[0])) == L.replay_one(p, 77, 1000 + i, policy), (policy, i)


@pytest.mark.parametrize("policy", [0, 1, 2])
def test_buffered_draw_schedule_replays_on_oracle(rh, policy):
    """The warp-synchronous Philox schedule of the playout kernel for every
    policy (branch-free plies, the reference heuristic's per-move loop,
    deferred capture searches) consumes exactly the stream the oracle
    replays."""
    pos = np.concatenate([L.random_positions(12, 500, 0, 80), crafted_boards()])
    for i in range(3000):
        p = np.ascontiguousarray(pos[i % len(pos)])
        pl = np.zeros(1, np.uint32)
        dr = np.zeros(1, np.uint32)
        sparse_from = (0, 37, 1 << 30)[i % 3]  # defers nothing from the start / from iteration 37 / never
        o = rh.rh_playout_ring(p.ctypes.data_as(u32p), 4242, i * 7, sparse_from, policy, pl.ctypes.data_as(u32p),
                               dr.ctypes.data_as(u32p))
        assert (o, int(pl[0]), int(dr[0])) == L.replay_one(p, 4242, i * 7, policy), (policy, i)


def test_uniform_random_fast_ply_equals_depth_first_search(rh):
    """The uniform random ply the kernels play (branch-free common plies, the
    men's tree, forced men's multi-jumps and forced king captures followed as
    a chain) plays the same move with the same draws as the depth-first
    play_ply on 1 M random boards, among them boards of both forced kinds."""
    rh.rh_random_fast_matches_dfs.restype = ctypes.c_long
    rh.rh_random_fast_matches_dfs.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64),
                                              ctypes.POINTER(ctypes.c_uint64)]
    forced, forced_king = ctypes.c_uint64(), ctypes.c_uint64()
    assert rh.rh_random_fast_matches_dfs(1_000_000, 23, ctypes.byref(forced), ctypes.byref(forced_king)) == 0
    assert forced.value > 1000 and forced_king.value > 1000


def _sq(row, col):
    """Dark square (row, col) -> bit index row*4 + col/2."""
    assert (row + col) % 2 == 1
    return row * 4 + col // 2


def _bits(*cells):
    return sum(1 << _sq(r, c) for r, c in cells)


@pytest.mark.parametrize("name,board,n,after", [
    # PLAYER_1 man (3,2) jumps (4,3) then (6,5), landing on the far row: forced, promotes
    ("man_double_jump_promotes", (_bits((3, 2)), _bits((4, 3), (6, 5)), 0, 0), 1,
     (_bits((7, 6)), 0, _bits((7, 6)), 1)),
    # PLAYER_2 man (5,4) jumps (4,3) then (2,1): forced, no promotion on row 1
    ("player2_man_double_jump", (_bits((4, 3), (2, 1)), _bits((5, 4)), 0, 1), 1,
     (0, _bits((1, 0)), 0, 0)),
    # PLAYER_1 king (2,1) jumps (3,2) then (5,4); it may not land on its start square again
    ("king_double_jump", (_bits((2, 1)), _bits((3, 2), (5, 4)), _bits((2, 1)), 0), 1,
     (_bits((6, 5)), 0, _bits((6, 5)), 1)),
    # the man's chain forks after the first jump: two moves, not forced
    ("man_chain_forks", (_bits((3, 2)), _bits((4, 3), (6, 5), (6, 3)), 0, 0), 2, None),
])
def test_capture_chains_on_crafted_boards(rh, name, board, n, after):
    """Forced capture chains (one legal move) are played at once and equal the
    depth-first search's move; a forking chain is left to the search."""
    u32p, ip = ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_int)
    rh.rh_ply_fast_and_dfs.restype = None
    rh.rh_ply_fast_and_dfs.argtypes = [u32p, ctypes.c_uint64, u32p, u32p, ip, ip]
    b = np.array(board, dtype=np.uint32)
    fast, dfs = np.zeros(4, np.uint32), np.zeros(4, np.uint32)
    nf, nd = ctypes.c_int(), ctypes.c_int()
    rh.rh_ply_fast_and_dfs(b.ctypes.data_as(u32p), 5, fast.ctypes.data_as(u32p), dfs.ctypes.data_as(u32p),
                           ctypes.byref(nf), ctypes.byref(nd))
    assert nf.value == nd.value == n, name
    assert (fast == dfs).all(), name
    if after is not None:
        assert tuple(int(x) for x in fast) == after, name


def test_branch_free_eps_greedy_equals_enumeration(rh):
    """The eps-greedy ply the kernels play without enumerating moves (best-move
    masks, bit-sliced jump gains) picks the same move with the same draws as
    the enumerating policy, on 300 K random boards with kings."""
    rh.rh_eps_fast_matches_enum.restype = ctypes.c_long
    rh.rh_eps_fast_matches_enum.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
    assert rh.rh_eps_fast_matches_enum(300_000, 17) == 0


def test_one_step_per_move_reference_heuristic_equals_enumeration(rh):
    """The reference-heuristic ply the kernels play with one loop step per move
    picks the same move with the same draws as the enumerating policy, on
    300 K random boards with kings."""
    rh.rh_heur_fast_matches_enum.restype = ctypes.c_long
    rh.rh_heur_fast_matches_enum.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
    assert rh.rh_heur_fast_matches_enum(300_000, 23) == 0


def test_simple_move_masks_list_the_moves_in_order(rh):
    """The per-lane move list of the network kernels (simple_move_masks +
    nth_move, for positions where no capture can continue) gives move i of
    the reference list order on 1 M random boards, single jumps included."""
    rh.rh_simple_moves_match_enum.restype = ctypes.c_long
    rh.rh_simple_moves_match_enum.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64),
                                              ctypes.POINTER(ctypes.c_uint64)]
    simple, captures = ctypes.c_uint64(), ctypes.c_uint64()
    assert rh.rh_simple_moves_match_enum(1_000_000, 29, ctypes.byref(simple), ctypes.byref(captures)) == 0
    assert simple.value > 500_000 and captures.value > 50_000

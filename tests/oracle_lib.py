"""ctypes access to the CPU oracle (test infrastructure only).

Loads ``oracle/_build/liboracle.so`` (the plain-C restatement, built by
``oracle/Makefile``) and, where it was built, ``oracle/_ref/libref.so`` (the
reference's own host code compiled from its sources).  Board records are
``(n, 4) uint32`` arrays ``[p1, p2, kings, meta]``; packed moves are 32-byte
records ``[from, to, jumps, promoted, path[12], removed[12], pad[4]]``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "_build", "liboracle.so")
REF_SO = os.path.join(ORACLE_DIR, "_ref", "libref.so")
CPU_SO = os.path.join(ORACLE_DIR, "_build", "libcpu_playouts.so")
# the reference's sources, where present (GPUAI_REFERENCE_SRC overrides)
REF_SRC = os.environ.get("GPUAI_REFERENCE_SRC", "/root/reference/src")

_u32p = ctypes.POINTER(ctypes.c_uint32)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_i8p = ctypes.POINTER(ctypes.c_int8)

_oracle = None
_ref = None


def build_oracle() -> None:
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def build_ref() -> bool:
    """Compile the reference's host code from its sources, where present."""
    if not os.path.isdir(REF_SRC):
        return False
    subprocess.run(["make", "-s", "-j8", "-C", ORACLE_DIR, "ref", "REF_SRC=" + REF_SRC], check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return os.path.exists(REF_SO)


def _ptr(a, t):
    return a.ctypes.data_as(t)


def oracle():
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_SO) or (
                os.path.getmtime(ORACLE_SO) < os.path.getmtime(os.path.join(ORACLE_DIR, "oracle.c"))):
            build_oracle()
        lib = ctypes.CDLL(ORACLE_SO)
        lib.or_genmoves_b16.argtypes = [_u32p, ctypes.c_uint32, _u8p, ctypes.c_uint32, _u8p]
        lib.or_genmoves_b16.restype = ctypes.c_int
        lib.or_apply_packed_b16.argtypes = [_u32p, _u8p]
        lib.or_apply_packed_b16.restype = ctypes.c_int
        lib.or_philox4x32_10.argtypes = [_u32p, _u32p, _u32p]
        lib.or_stream_draw.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32]
        lib.or_stream_draw.restype = ctypes.c_uint32
        lib.or_replay_playout.argtypes = [_u32p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, _u32p, _u32p]
        lib.or_replay_playout.restype = ctypes.c_int
        lib.or_replay_batch.argtypes = [_u32p, _u32p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64,
                                        ctypes.c_int, _i8p, _u32p, ctypes.c_int]
        lib.or_random_positions.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                                            ctypes.c_uint32, _u32p]
        lib.or_host_playouts.argtypes = [_u32p, ctypes.c_uint32, _i8p, ctypes.c_int, ctypes.c_uint]
        lib.or_host_heuristic_playouts.argtypes = [_u32p, ctypes.c_uint32, _i8p, ctypes.c_uint64]
        _oracle = lib
    return _oracle


def ref():
    """The reference's own host code, or None where it cannot be built."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO) and not build_ref():
            return None
        lib = ctypes.CDLL(REF_SO)
        lib.ref_genmoves_b16.argtypes = [_u32p, ctypes.c_uint32, _u8p, ctypes.c_uint32, _u8p]
        lib.ref_genmoves_b16.restype = ctypes.c_int
        lib.ref_apply_b16.argtypes = [_u32p, ctypes.c_int]
        lib.ref_apply_b16.restype = ctypes.c_int
        lib.ref_host_playouts.argtypes = [_u32p, ctypes.c_uint32, _i8p, ctypes.c_uint]
        lib.ref_host_heuristic_playouts.argtypes = [_u32p, ctypes.c_uint32, _i8p]
        _ref = lib
    return _ref


# ---------------------------------------------------------------- helpers

def start_board() -> np.ndarray:
    p1 = 0x00000FFF
    p2 = 0xFFF00000
    return np.array([[p1, p2, 0, 0]], dtype=np.uint32)


def genmoves(pos: np.ndarray, max_moves: int = 128, lib=None):
    """Move lists of the reference (lib=ref()) or of the restatement."""
    lib = lib or oracle()
    pos = np.ascontiguousarray(pos, dtype=np.uint32).reshape(-1, 4)
    n = pos.shape[0]
    out = np.zeros((n, max_moves, 32), dtype=np.uint8)
    counts = np.zeros(n, dtype=np.uint8)
    fn = lib.or_genmoves_b16 if hasattr(lib, "or_genmoves_b16") else lib.ref_genmoves_b16
    rc = fn(_ptr(pos, _u32p), n, _ptr(out, _u8p), max_moves, _ptr(counts, _u8p))
    if rc != 0:
        raise RuntimeError("move list overflow")
    return out, counts


_children_cache: dict = {}


def children(board):
    """(child boards (k, 4), packed moves (k, 32)) of one board in move-list
    order, by the restatement's genMoves and State::move (memoised)."""
    key = tuple(int(v) for v in board)
    hit = _children_cache.get(key)
    if hit is not None:
        return hit
    pos = np.array([key], dtype=np.uint32)
    mv, cnt = genmoves(pos, max_moves=128)
    k = int(cnt[0])
    moves = np.ascontiguousarray(mv[0, :k])
    boards = np.repeat(pos, k, axis=0)
    lib = oracle()
    for i in range(k):
        row = np.ascontiguousarray(boards[i])
        if lib.or_apply_packed_b16(_ptr(row, _u32p), _ptr(np.ascontiguousarray(moves[i]), _u8p)) != 0:
            raise RuntimeError("apply failed")
        boards[i] = row
    if len(_children_cache) > 1_000_000:
        _children_cache.clear()
    _children_cache[key] = (boards, moves)
    return boards, moves


def fake_outcome(board, salt: int) -> int:
    """The deterministic stand-in for a playout of tests/host_tree.cpp and
    oracle/ref_shim.cpp: +1 (PLAYER_1), -1 (PLAYER_2) or 0 from a hash of the board."""
    m = (1 << 64) - 1
    b = [int(v) for v in board]
    x = ((b[0] | (b[1] << 32)) ^ ((b[2] * 0x9E3779B97F4A7C15) & m) ^ ((b[3] * 0xC2B2AE3D27D4EB4F) & m) ^ salt) & m
    x ^= x >> 31
    x = (x * 0x7FB5D329728EA185) & m
    x ^= x >> 27
    x = (x * 0x81DADEF4BC2DD44D) & m
    x ^= x >> 33
    r = x % 7
    return 1 if r < 3 else (-1 if r < 6 else 0)


def canonical_moves(out: np.ndarray, counts: np.ndarray):
    """Per-position tuple of move byte strings (unused slots cleared)."""
    res = []
    for i in range(out.shape[0]):
        res.append(tuple(out[i, j].tobytes() for j in range(int(counts[i]))))
    return res


def philox(ctr, key):
    lib = oracle()
    c = np.array(ctr, dtype=np.uint32)
    k = np.array(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    lib.or_philox4x32_10(_ptr(c, _u32p), _ptr(k, _u32p), _ptr(o, _u32p))
    return [int(x) for x in o]


def stream_draw(seed: int, sid: int, tag: int, k: int) -> int:
    return int(oracle().or_stream_draw(seed, sid, tag, k))


def random_positions(seed: int, n: int, min_plies: int, max_plies: int) -> np.ndarray:
    out = np.zeros((n, 4), dtype=np.uint32)
    oracle().or_random_positions(seed, n, min_plies, max_plies, _ptr(out, _u32p))
    return out


def replay_batch(pos, reps, seed, stream_base=0, policy=0, nthreads=0):
    pos = np.ascontiguousarray(pos, dtype=np.uint32).reshape(-1, 4)
    reps = np.ascontiguousarray(reps, dtype=np.uint32)
    total = int(reps.sum())
    out = np.zeros(total, dtype=np.int8)
    plies = np.zeros(total, dtype=np.uint32)
    oracle().or_replay_batch(_ptr(pos, _u32p), _ptr(reps, _u32p), pos.shape[0], seed, stream_base,
                             policy, _ptr(out, _i8p), _ptr(plies, _u32p), nthreads)
    return out, plies


def replay_one(pos_row, seed, sid, policy=0):
    p = np.ascontiguousarray(pos_row, dtype=np.uint32).reshape(4)
    plies = np.zeros(1, dtype=np.uint32)
    draws = np.zeros(1, dtype=np.uint32)
    o = oracle().or_replay_playout(_ptr(p, _u32p), seed, sid, policy, _ptr(plies, _u32p),
                                   _ptr(draws, _u32p))
    return o, int(plies[0]), int(draws[0])


_cpu = None


def cpu_playouts(pos, reps, seed, stream_base=0, nthreads=0):
    """The stronger CPU baseline (oracle/cpu_playouts.cpp): the project's
    bitboard ply with the GPU's random streams on every host core.  Returns
    (outcomes, plies)."""
    global _cpu
    if _cpu is None:
        src = os.path.join(ORACLE_DIR, "cpu_playouts.cpp")
        if not os.path.exists(CPU_SO) or os.path.getmtime(CPU_SO) < os.path.getmtime(src):
            build_oracle()
        lib = ctypes.CDLL(CPU_SO)
        lib.cp_playouts.argtypes = [_u32p, _u32p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64, _i8p,
                                    ctypes.c_int]
        lib.cp_playouts.restype = ctypes.c_uint64
        _cpu = lib
    pos = np.ascontiguousarray(pos, dtype=np.uint32).reshape(-1, 4)
    reps = np.ascontiguousarray(reps, dtype=np.uint32)
    out = np.zeros(int(reps.sum()), dtype=np.int8)
    plies = _cpu.cp_playouts(_ptr(pos, _u32p), _ptr(reps, _u32p), pos.shape[0], seed, stream_base,
                             _ptr(out, _i8p), nthreads)
    return out, int(plies)


def host_playouts_port(states, nthreads=0, srand_seed=1):
    states = np.ascontiguousarray(states, dtype=np.uint32).reshape(-1, 4)
    out = np.zeros(states.shape[0], dtype=np.int8)
    oracle().or_host_playouts(_ptr(states, _u32p), states.shape[0], _ptr(out, _i8p), nthreads, srand_seed)
    return out


def host_playouts_ref(states, srand_seed=1):
    lib = ref()
    states = np.ascontiguousarray(states, dtype=np.uint32).reshape(-1, 4)
    out = np.zeros(states.shape[0], dtype=np.int8)
    lib.ref_host_playouts(_ptr(states, _u32p), states.shape[0], _ptr(out, _i8p), srand_seed)
    return out


def host_heuristic_ref(states):
    lib = ref()
    states = np.ascontiguousarray(states, dtype=np.uint32).reshape(-1, 4)
    out = np.zeros(states.shape[0], dtype=np.int8)
    lib.ref_host_heuristic_playouts(_ptr(states, _u32p), states.shape[0], _ptr(out, _i8p))
    return out


def wdl(outcomes: np.ndarray) -> np.ndarray:
    """[P1 wins, draws, P2 wins] counts."""
    o = np.asarray(outcomes)
    return np.array([(o == 1).sum(), (o == 0).sum(), (o == -1).sum()], dtype=np.int64)

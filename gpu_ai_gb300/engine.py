"""Python binding of libgpuai (include/gpuai.h) over ctypes.

This is the reference-facing entry for Python callers and the test/bench
harness: a batch of positions in, one int8 outcome per playout out
(+1 PLAYER_1 won, -1 PLAYER_2 won, 0 drawn), mirroring
``PlayoutDriver::runPlayouts`` (src/playout.hpp:27-33).  All computation runs
in the CUDA kernels of libgpuai.so; there is no CPU path, and a missing or
unbuilt library raises instead of falling back.
"""
from __future__ import annotations

import ctypes
import os
import re
from typing import Optional, Tuple

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
# GPUAI_LIB selects another build of the library, e.g. lib/libgpuai_checked.so
# (the kernels' bounds checks compiled in)
LIB_PATH = os.environ.get("GPUAI_LIB") or os.path.join(PKG, "lib", "libgpuai.so")
HEADER = os.path.join(ROOT, "include", "gpuai.h")

POLICY_RANDOM = 0
POLICY_REF_HEURISTIC = 1
POLICY_EPS_GREEDY = 2

LAYOUT_THREAD = 0
LAYOUT_WARP = 1
LAYOUT_POOLED = 2

OK = 0
ERR_INVALID = -1
ERR_CUDA = -2
ERR_OOM = -3
ERR_LIMIT = -4
ERR_NO_DEVICE = -5

START_BOARD = np.array([0x00000FFF, 0xFFF00000, 0, 0], dtype=np.uint32)

_u32p = ctypes.POINTER(ctypes.c_uint32)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_i8p = ctypes.POINTER(ctypes.c_int8)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u64p = ctypes.POINTER(ctypes.c_uint64)

_lib = None


class GpuAIError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gpuai error {code}: {msg}")
        self.code = code


def header_symbols() -> list:
    """Function names declared in include/gpuai.h."""
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gpuai_[a-z_]+)\s*\(", src)))


def load_library(path: str = LIB_PATH):
    """Load libgpuai.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with gpu_ai_gb300.build.build()")
    lib = ctypes.CDLL(path)
    lib.gpuai_last_error.restype = ctypes.c_char_p
    lib.gpuai_create.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    lib.gpuai_destroy.argtypes = [ctypes.c_void_p]
    lib.gpuai_destroy.restype = None
    # raw addresses (ndarray.ctypes.data) for the array arguments: cheaper per call than data_as
    lib.gpuai_playouts.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                   ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int32, ctypes.c_void_p]
    lib.gpuai_playouts_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                          ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64,
                                          ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    lib.gpuai_status.argtypes = [ctypes.c_void_p, _u32p, _u64p]
    lib.gpuai_genmoves.argtypes = [ctypes.c_void_p, _u32p, ctypes.c_uint32, _u8p, ctypes.c_uint32, _u8p]
    lib.gpuai_random_positions.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                                           ctypes.c_uint32, _u32p]
    lib.gpuai_device_info.argtypes = [ctypes.c_void_p, _i32p, _i32p, _i32p]
    lib.gpuai_set_launch.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]
    lib.gpuai_get_launch.argtypes = [ctypes.c_void_p, ctypes.c_int32, _i32p, _i32p, _i32p]
    lib.gpuai_searches_create.argtypes = [ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                          ctypes.c_uint32, ctypes.c_int32, ctypes.c_uint64,
                                          ctypes.POINTER(ctypes.c_void_p)]
    lib.gpuai_searches_destroy.argtypes = [ctypes.c_void_p]
    lib.gpuai_searches_destroy.restype = None
    lib.gpuai_searches_add.argtypes = [ctypes.c_void_p, _u32p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64,
                                       _i32p]
    lib.gpuai_searches_remove.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    lib.gpuai_searches_step.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int32]
    lib.gpuai_searches_poll.argtypes = [ctypes.c_void_p, _u64p, _u64p, ctypes.c_uint32, _u32p]
    lib.gpuai_searches_children.argtypes = [ctypes.c_void_p, ctypes.c_int32, _u8p, _u32p, _u32p, ctypes.c_uint32,
                                            _u32p, _u32p]
    _f32p = ctypes.POINTER(ctypes.c_float)
    vp = ctypes.c_void_p
    lib.gpuai_net_create.argtypes = [ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64, ctypes.POINTER(vp)]
    lib.gpuai_net_destroy.argtypes = [vp]
    lib.gpuai_net_destroy.restype = None
    lib.gpuai_net_get_params.argtypes = [vp, _f32p]
    lib.gpuai_net_set_params.argtypes = [vp, _f32p]
    lib.gpuai_net_save.argtypes = [vp, ctypes.c_char_p]
    lib.gpuai_net_load.argtypes = [vp, ctypes.c_char_p]
    lib.gpuai_net_forward.argtypes = [vp, _u32p, ctypes.c_uint32, _f32p, _f32p]
    lib.gpuai_net_gradients.argtypes = [vp, _u32p, _f32p, _f32p, ctypes.c_uint32, ctypes.c_float, ctypes.c_float,
                                        _f32p, _f32p]
    lib.gpuai_net_train_step.argtypes = [vp, vp, vp, vp, ctypes.c_uint32, ctypes.c_float, ctypes.c_float,
                                         ctypes.c_float, _f32p]
    lib.gpuai_label_positions.argtypes = [vp, vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64,
                                          ctypes.c_int32, vp, vp, vp, vp]
    lib.gpuai_selfplay_positions.argtypes = [vp, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                             ctypes.c_int32, vp, vp]
    lib.gpuai_apply_move.argtypes = [_u32p, _u8p, _u32p]
    lib.gpuai_set_layout.argtypes = [vp, ctypes.c_int32, ctypes.c_int32]
    lib.gpuai_get_layout.argtypes = [vp, ctypes.c_int32, _i32p]
    lib.gpuai_searches_set_net.argtypes = [vp, vp, ctypes.c_float, ctypes.c_float]
    lib.gpuai_playouts_learned.argtypes = [vp, vp, vp, vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                           ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_float, vp, vp,
                                           vp, vp]
    lib.gpuai_net_wait_selftest.argtypes = [vp, ctypes.c_uint32, _u32p]
    lib.gpuai_searches_set_proposal.argtypes = [vp, ctypes.c_uint32, ctypes.c_float]
    lib.gpuai_searches_nodes.argtypes = [vp, ctypes.c_int32, ctypes.c_uint32, vp, vp, vp, vp, _u32p]
    lib.gpuai_searches_leaves.argtypes = [vp, ctypes.c_uint32, _u32p, vp, vp, vp, vp, vp, vp, vp]
    for name in header_symbols():
        if name not in ("gpuai_last_error", "gpuai_destroy", "gpuai_searches_destroy", "gpuai_net_destroy"):
            getattr(lib, name).restype = ctypes.c_int
    _lib = lib
    return lib


def _check(rc: int):
    if rc != OK:
        raise GpuAIError(rc, load_library().gpuai_last_error().decode())


def apply_move(board, move) -> np.ndarray:
    """Board after `move` (a 32-byte record of the board's move list)."""
    b = np.ascontiguousarray(board, dtype=np.uint32).reshape(4)
    m = np.ascontiguousarray(move, dtype=np.uint8).reshape(32)
    out = np.zeros(4, np.uint32)
    lib = load_library()
    _check(lib.gpuai_apply_move(b.ctypes.data_as(_u32p), m.ctypes.data_as(_u8p), out.ctypes.data_as(_u32p)))
    return out


def _boards(pos) -> np.ndarray:
    a = np.ascontiguousarray(pos, dtype=np.uint32)
    if a.ndim == 1:
        a = a.reshape(-1, 4)
    if a.ndim != 2 or a.shape[1] != 4:
        raise ValueError("boards must have shape (n, 4): p1, p2, kings, meta")
    return a


class Engine:
    """One libgpuai context (one CUDA stream) on `device`."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        ctx = ctypes.c_void_p()
        _check(self.lib.gpuai_create(device, ctypes.byref(ctx)))
        self.ctx = ctx

    def close(self):
        if self.ctx:
            self.lib.gpuai_destroy(self.ctx)
            self.ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def playouts(self, pos, reps=None, seed: int = 0, stream_base: int = 0,
                 policy: int = POLICY_RANDOM, out: Optional[np.ndarray] = None) -> np.ndarray:
        """reps[p] playouts from pos[p] (one each if reps is None); int8 outcomes in order.

        `out`, if given, is a C-contiguous int8 array of exactly the number of
        playouts that receives the outcomes (a caller running many batches can
        reuse one buffer) and is returned."""
        b = _boards(pos)
        n = b.shape[0]
        if reps is None:
            total = n
            rp = None
        else:
            r = np.ascontiguousarray(reps, dtype=np.uint32)
            if r.shape != (n,):
                raise ValueError("reps must have one entry per board")
            total = int(r.sum(dtype=np.uint64))
            rp = r.ctypes.data
        if out is None:
            out = np.empty(total, dtype=np.int8)
        elif out.dtype != np.int8 or out.shape != (total,) or not out.flags.c_contiguous or not out.flags.writeable:
            raise ValueError(f"out must be a writeable C-contiguous int8 array of {total} outcomes")
        _check(self.lib.gpuai_playouts(self.ctx, b.ctypes.data, rp, n, seed, stream_base, policy, out.ctypes.data))
        return out

    def playouts_device(self, d_pos: int, d_offsets: Optional[int], npos: int, uniform_reps: int, total: int,
                        seed: int, stream_base: int, policy: int, d_out: int, stream: Optional[int] = None):
        """Enqueue playouts on device pointers (no synchronisation)."""
        _check(self.lib.gpuai_playouts_device(self.ctx, d_pos, d_offsets, npos, uniform_reps, total, seed,
                                              stream_base, policy, d_out, stream))

    def playouts_learned(self, net: "Net", d_pos: int, d_offsets: Optional[int], npos: int, uniform_reps: int,
                         total: int, seed: int, stream_base: int, guided_plies: int, temperature: float, d_out: int,
                         stream: Optional[int] = None, d_trace_boards: Optional[int] = None,
                         d_trace_logits: Optional[int] = None):
        """Enqueue learned-proposal playouts on device pointers (gpuai_playouts_learned):
        the first `guided_plies` plies drawn from the network's policy, the rest random."""
        _check(self.lib.gpuai_playouts_learned(self.ctx, net.h, d_pos, d_offsets, npos, uniform_reps, total, seed,
                                               stream_base, guided_plies, temperature, d_out, stream,
                                               d_trace_boards, d_trace_logits))

    def status(self) -> Tuple[int, int]:
        st = ctypes.c_uint32()
        pl = ctypes.c_uint64()
        _check(self.lib.gpuai_status(self.ctx, ctypes.byref(st), ctypes.byref(pl)))
        return int(st.value), int(pl.value)

    def genmoves(self, pos, max_moves: int = 64):
        b = _boards(pos)
        n = b.shape[0]
        out = np.zeros((n, max_moves, 32), dtype=np.uint8)
        counts = np.zeros(n, dtype=np.uint8)
        _check(self.lib.gpuai_genmoves(self.ctx, b.ctypes.data_as(_u32p), n, out.ctypes.data_as(_u8p),
                                       max_moves, counts.ctypes.data_as(_u8p)))
        return out, counts

    def random_positions(self, seed: int, n: int, min_plies: int, max_plies: int) -> np.ndarray:
        out = np.zeros((n, 4), dtype=np.uint32)
        _check(self.lib.gpuai_random_positions(self.ctx, seed, n, min_plies, max_plies, out.ctypes.data_as(_u32p)))
        return out

    def selfplay_positions(self, seed: int, n: int, min_plies: int, max_plies: int, policy: int, d_out: int,
                           stream: Optional[int] = None):
        """Enqueue n self-play positions of `policy` into device buffer d_out (n x 16 bytes)."""
        _check(self.lib.gpuai_selfplay_positions(self.ctx, seed, n, min_plies, max_plies, policy, d_out, stream))

    def label_positions(self, d_pos: int, n: int, playouts_per_position: int, seed: int, stream_base: int,
                        policy: int, d_value: int, d_move_q: int, d_nmoves: int, stream: Optional[int] = None):
        """Enqueue GPU-playout training labels for n device boards (gpuai_label_positions)."""
        _check(self.lib.gpuai_label_positions(self.ctx, d_pos, n, playouts_per_position, seed, stream_base, policy,
                                              d_value, d_move_q, d_nmoves, stream))

    def set_launch(self, policy: int, block_threads: int, blocks_per_sm: int = 0):
        _check(self.lib.gpuai_set_launch(self.ctx, policy, block_threads, blocks_per_sm))

    def set_layout(self, policy: int, layout: int):
        """LAYOUT_THREAD (thread per playout) or LAYOUT_WARP (warp per playout, random policy)."""
        _check(self.lib.gpuai_set_layout(self.ctx, policy, layout))

    def get_layout(self, policy: int = POLICY_RANDOM) -> int:
        v = ctypes.c_int32()
        _check(self.lib.gpuai_get_layout(self.ctx, policy, ctypes.byref(v)))
        return v.value

    def get_launch(self, policy: int = POLICY_RANDOM):
        a, b, c = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _check(self.lib.gpuai_get_launch(self.ctx, policy, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"block_threads": a.value, "blocks_per_sm": b.value, "max_blocks_per_sm": c.value}

    def device_info(self):
        a, b, c = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _check(self.lib.gpuai_device_info(self.ctx, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"sms": a.value, "blocks_per_sm": b.value, "block_threads": c.value}


class Searches:
    """Many MCTS searches with device-resident trees (gpuai_searches_*)."""

    def __init__(self, max_searches: int, pool_nodes: int, max_leaves_per_step: int = 64,
                 playouts_per_leaf: int = 1, policy: int = POLICY_RANDOM, seed: int = 0, device: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        _check(self.lib.gpuai_searches_create(device, max_searches, pool_nodes, max_leaves_per_step,
                                              playouts_per_leaf, policy, seed, ctypes.byref(h)))
        self.h = h
        self.max_searches = max_searches
        self.ppl = playouts_per_leaf

    def close(self):
        if self.h:
            self.lib.gpuai_searches_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, root, budget: int, node_capacity: int, stream_base: int) -> int:
        b = np.ascontiguousarray(root, dtype=np.uint32).reshape(4)
        slot = ctypes.c_int32()
        _check(self.lib.gpuai_searches_add(self.h, b.ctypes.data_as(_u32p), budget, node_capacity, stream_base,
                                           ctypes.byref(slot)))
        return slot.value

    def try_add(self, root, budget: int, node_capacity: int, stream_base: int):
        """Slot, or None when admission is refused (no slot / node range free)."""
        try:
            return self.add(root, budget, node_capacity, stream_base)
        except GpuAIError as e:
            if e.code == ERR_OOM:
                return None
            raise

    def remove(self, slot: int):
        _check(self.lib.gpuai_searches_remove(self.h, slot))

    def step(self, steps: int, leaves_per_search: int, use_graph: bool = True):
        _check(self.lib.gpuai_searches_step(self.h, steps, leaves_per_search, 1 if use_graph else 0))

    def poll(self):
        done = np.zeros(self.max_searches, np.uint64)
        budget = np.zeros(self.max_searches, np.uint64)
        st = ctypes.c_uint32()
        _check(self.lib.gpuai_searches_poll(self.h, done.ctypes.data_as(_u64p), budget.ctypes.data_as(_u64p),
                                            self.max_searches, ctypes.byref(st)))
        return done, budget

    def children(self, slot: int, max_children: int = 64):
        moves = np.zeros((max_children, 32), np.uint8)
        visits = np.zeros(max_children, np.uint32)
        score2 = np.zeros(max_children, np.uint32)
        n = ctypes.c_uint32()
        used = ctypes.c_uint32()
        _check(self.lib.gpuai_searches_children(self.h, slot, moves.ctypes.data_as(_u8p), visits.ctypes.data_as(_u32p),
                                                score2.ctypes.data_as(_u32p), max_children, ctypes.byref(n),
                                                ctypes.byref(used)))
        k = min(n.value, max_children)
        return {"moves": moves[:k], "visits": visits[:k], "score2": score2[:k], "nodes": used.value}

    def set_net(self, net: Optional["Net"], value_weight: float = 1.0, c_puct: float = 1.5):
        """Evaluate leaves with `net` (None: plain playout searches)."""
        _check(self.lib.gpuai_searches_set_net(self.h, net.h if net is not None else None, value_weight, c_puct))
        self.net = net  # keep the network alive while the searches use it

    def set_proposal(self, guided_plies: int, temperature: float = 1.0):
        """Learned-proposal playouts: the first guided_plies plies of every
        playout drawn from the attached network's policy (0: off)."""
        _check(self.lib.gpuai_searches_set_proposal(self.h, guided_plies, temperature))

    def nodes(self, slot: int, priors: bool = False):
        """The search's tree, nodes numbered from its root: info (n, 4) = {first
        child (0xFFFFFFFF before expansion), children | state << 16, visits,
        score2}, boards (n, 4), parent (n,), and priors (n, 32) FP16 when asked."""
        n = ctypes.c_uint32()
        _check(self.lib.gpuai_searches_nodes(self.h, slot, 0, None, None, None, None, ctypes.byref(n)))
        k = n.value
        info = np.zeros((k, 4), np.uint32)
        boards = np.zeros((k, 4), np.uint32)
        parent = np.zeros(k, np.int32)
        pri = np.zeros((k, 32), np.uint16) if priors else None
        _check(self.lib.gpuai_searches_nodes(self.h, slot, k, info.ctypes.data, boards.ctypes.data,
                                             parent.ctypes.data, pri.ctypes.data if priors else None,
                                             ctypes.byref(n)))
        out = {"info": info, "boards": boards, "parent": parent}
        if priors:
            out["priors"] = pri.view(np.float16)
        return out

    def leaves(self, net: bool = False):
        """The last step's leaf slots: search, node (from the search's root),
        boards, first stream id, outcomes (n, playouts_per_leaf) and, with
        net, the raw value output and the (n, 1024) logits as float32
        (playouts_per_leaf outcomes per slot)."""
        n = ctypes.c_uint32()
        _check(self.lib.gpuai_searches_leaves(self.h, 0, ctypes.byref(n), None, None, None, None, None, None, None))
        k = n.value
        search = np.zeros(k, np.int32)
        node = np.zeros(k, np.int32)
        boards = np.zeros((k, 4), np.uint32)
        streams = np.zeros(k, np.uint64)
        outcomes = np.zeros((k, self.ppl), np.int8)
        value = np.zeros(k, np.float32) if net else None
        logits = np.zeros((k, NET_LOGITS), np.uint16) if net else None
        _check(self.lib.gpuai_searches_leaves(self.h, k, ctypes.byref(n), search.ctypes.data, node.ctypes.data,
                                              boards.ctypes.data, streams.ctypes.data, outcomes.ctypes.data,
                                              value.ctypes.data if net else None,
                                              logits.ctypes.data if net else None))
        out = {"search": search, "node": node, "boards": boards, "streams": streams, "outcomes": outcomes}
        if net:
            out["net_value"] = value
            out["net_logits"] = (logits.astype(np.uint32) << 16).view(np.float32)
        return out

    def best(self, slot: int):
        """Most visited root move (None for a finished game) and the child statistics."""
        c = self.children(slot)
        if len(c["visits"]) == 0:
            return None, c
        i = int(np.argmax(c["visits"]))
        return c["moves"][i], c


NET_FEATURES = 129
NET_HIDDEN = 256
NET_LOGITS = 1024
NET_MAX_MOVES = 32
NET_PARAMS = 378625


class Net:
    """Policy/value network (gpuai_net_*): BF16 tensor-core forward, backward and Adam."""

    def __init__(self, device: int = 0, max_batch: int = 8192, seed: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        _check(self.lib.gpuai_net_create(device, max_batch, seed, ctypes.byref(h)))
        self.h = h
        self.max_batch = max_batch

    def close(self):
        if self.h:
            self.lib.gpuai_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        p = np.zeros(NET_PARAMS, np.float32)
        _check(self.lib.gpuai_net_get_params(self.h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return p

    def set_params(self, p):
        a = np.ascontiguousarray(p, dtype=np.float32)
        if a.shape != (NET_PARAMS,):
            raise ValueError(f"expected {NET_PARAMS} parameters")
        _check(self.lib.gpuai_net_set_params(self.h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))

    def save(self, path: str):
        _check(self.lib.gpuai_net_save(self.h, os.fsencode(path)))

    def load(self, path: str):
        _check(self.lib.gpuai_net_load(self.h, os.fsencode(path)))

    def forward(self, boards, want_logits: bool = True):
        """(value for the side to move, n x 1024 logits or None)."""
        b = _boards(boards)
        n = b.shape[0]
        fp = ctypes.POINTER(ctypes.c_float)
        value = np.zeros(n, np.float32)
        logits = np.zeros((n, NET_LOGITS), np.float32) if want_logits else None
        _check(self.lib.gpuai_net_forward(self.h, b.ctypes.data_as(_u32p), n, value.ctypes.data_as(fp),
                                          logits.ctypes.data_as(fp) if logits is not None else None))
        return value, logits

    def gradients(self, boards, value_target, move_q, tau: float = 0.1, value_coef: float = 1.0):
        """(gradient in parameter order, [policy loss, value loss]) without updating."""
        b = _boards(boards)
        n = b.shape[0]
        fp = ctypes.POINTER(ctypes.c_float)
        z = np.ascontiguousarray(value_target, np.float32)
        q = np.ascontiguousarray(move_q, np.float32).reshape(n, NET_MAX_MOVES)
        g = np.zeros(NET_PARAMS, np.float32)
        loss = np.zeros(2, np.float32)
        _check(self.lib.gpuai_net_gradients(self.h, b.ctypes.data_as(_u32p), z.ctypes.data_as(fp),
                                            q.ctypes.data_as(fp), n, tau, value_coef, g.ctypes.data_as(fp),
                                            loss.ctypes.data_as(fp)))
        return g, loss

    def wait_selftest(self, wait_limit_us: int = 2000) -> int:
        """Status word of a GEMM launched with no loads and a short wait limit
        (gpuai_net_wait_selftest): bit 16 set when its bounded wait ran out."""
        st = ctypes.c_uint32()
        _check(self.lib.gpuai_net_wait_selftest(self.h, wait_limit_us, ctypes.byref(st)))
        return int(st.value)

    def train_step(self, d_boards: int, d_value: int, d_move_q: int, n: int, lr: float, tau: float = 0.1,
                   value_coef: float = 1.0, want_loss: bool = False):
        """One Adam step on device rows; returns [policy, value] loss when want_loss (waits)."""
        loss = np.zeros(2, np.float32) if want_loss else None
        _check(self.lib.gpuai_net_train_step(self.h, d_boards, d_value, d_move_q, n, lr, tau, value_coef,
                                             loss.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
                                             if loss is not None else None))
        return loss

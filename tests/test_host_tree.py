"""The host UCT tree (the caller of the playout path) against the reference's
own GameTree: the same select/update schedule with a deterministic stand-in
for playout outcomes must give identical root statistics (src/mcts.cpp:63-191),
and the project's default perspective keeps the same invariants."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import oracle_lib as L

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SO = os.path.join(HERE, "_build", "libhost_tree.so")
HOST = os.path.join(ROOT, "gpu_ai_gb300", "csrc", "host")
SRCS = [os.path.join(HERE, "host_tree.cpp"), os.path.join(HOST, "state.cpp"), os.path.join(HOST, "mcts.cpp")]
u32p = ctypes.POINTER(ctypes.c_uint32)


@pytest.fixture(scope="module")
def ht():
    deps = SRCS + [os.path.join(HOST, f) for f in ("state.hpp", "mcts.hpp")] + \
        [os.path.join(ROOT, "gpu_ai_gb300", "csrc", "rules.cuh")]
    if not os.path.exists(SO) or max(os.path.getmtime(d) for d in deps) > os.path.getmtime(SO):
        os.makedirs(os.path.dirname(SO), exist_ok=True)
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + os.path.join(ROOT, "include"),
                        "-I" + os.path.join(ROOT, "gpu_ai_gb300", "csrc"), "-o", SO] + SRCS, check=True)
    lib = ctypes.CDLL(SO)
    lib.ht_tree_run.argtypes = [u32p, u32p, ctypes.c_int, ctypes.c_uint64, u32p, ctypes.c_int, ctypes.c_int, u32p]
    lib.ht_tree_reroot.argtypes = [u32p, ctypes.c_uint, ctypes.c_int, ctypes.c_uint64, u32p, u32p]
    lib.ht_zero_weights.argtypes = [u32p]
    return lib


def _run(lib, fn, root, trials, salt, *extra):
    root = np.ascontiguousarray(root, dtype=np.uint32)
    tr = np.ascontiguousarray(trials, dtype=np.uint32)
    out = np.zeros(3 * 64, np.uint32)
    n = getattr(lib, fn)(root.ctypes.data_as(u32p), tr.ctypes.data_as(u32p), len(tr), salt,
                         out.ctypes.data_as(u32p), 64, *extra)
    assert n >= 0
    return out[:3 * n].reshape(-1, 3)


SCHEDULES = [[50, 50, 50, 50], [2, 3, 100, 7, 500, 1, 1000], [64] * 30, [4096, 4096]]


@pytest.mark.skipif(L.ref() is None, reason="reference sources not present")
@pytest.mark.parametrize("sched", SCHEDULES)
def test_tree_statistics_match_reference_tree(ht, sched):
    roots = [L.start_board()[0]] + list(L.random_positions(31, 6, 4, 30))
    for i, root in enumerate(roots):
        mine = _run(ht, "ht_tree_run", root, sched, 1234 + i, 1, None)
        ref = _run(L.ref(), "ref_tree_run", root, sched, 1234 + i)
        np.testing.assert_array_equal(mine, ref)


def test_tree_invariants_default_perspective(ht):
    for i, root in enumerate(L.random_positions(8, 5, 0, 40)):
        seen = ctypes.c_uint32()
        stats = _run(ht, "ht_tree_run", root, [1000] * 12, 77 + i, 0, ctypes.byref(seen))
        assert seen.value == 12000
        assert stats[:, 0].sum() == 12000       # every playout passes through one root child
        assert (stats[:, 1] + stats[:, 2] <= stats[:, 0]).all()


def test_reroot_keeps_subtree(ht):
    root = np.ascontiguousarray(L.start_board()[0], dtype=np.uint32)
    before, after = ctypes.c_uint32(), ctypes.c_uint32()
    assert ht.ht_tree_reroot(root.ctypes.data_as(u32p), 500, 10, 9, ctypes.byref(before), ctypes.byref(after)) == 0
    assert before.value == after.value > 0


def test_all_zero_ucb_weights(ht):
    from golden_boards import crafted_boards
    b = crafted_boards()
    forced = [r for r in b if L.genmoves(r)[1][0] == 1]
    assert forced
    root = np.ascontiguousarray(forced[0], dtype=np.uint32)
    assert ht.ht_zero_weights(root.ctypes.data_as(u32p)) == 0

"""The device-search oracle (oracle/search.py) on the CPU.

In reference mode it must reproduce the reference's own GameTree
(src/mcts.cpp:63-191, built from its sources by oracle/Makefile) root
statistics exactly under the deterministic stand-in for playouts: that pins
the level-synchronous split and the update to the reference.  Its float32
elementary functions must stay within a few units in the last place of the
exact functions, and its trees must keep the invariants the kernels keep."""
import math

import numpy as np
import pytest

import oracle_lib as L
from oracle import search as S

SCHEDULES = [[50, 50, 50, 50], [2, 3, 100, 7, 500, 1, 1000], [64] * 30, [4096, 4096]]


def _fake_slots(o, slot, leaves, salt):
    s = o.slots[slot]
    return [[slot, n, s.nodes[n].board, 0, np.array([L.fake_outcome(s.nodes[n].board, salt)], np.int8)]
            for n in leaves]


@pytest.mark.skipif(L.ref() is None, reason="reference sources not present")
@pytest.mark.parametrize("sched", SCHEDULES)
def test_reference_mode_matches_reference_tree(sched):
    roots = [L.start_board()[0]] + list(L.random_positions(31, 6, 4, 30))
    for i, root in enumerate(roots):
        o = S.SearchesOracle(1, 1, 0, 0, children=L.children, mode="reference")
        slot = o.add(root, 1 << 40, 1 << 30, 0)
        for t in sched:
            leaves = o.select(o.slots[slot], t)
            assert len(leaves) == t
            o._backprop(_fake_slots(o, slot, leaves, 1234 + i))
        out = np.zeros(3 * 64, np.uint32)
        r = np.ascontiguousarray(root, dtype=np.uint32)
        tr = np.ascontiguousarray(sched, dtype=np.uint32)
        n = L.ref().ref_tree_run(r.ctypes.data_as(L._u32p), tr.ctypes.data_as(L._u32p), len(tr), 1234 + i,
                                 out.ctypes.data_as(L._u32p), 64)
        np.testing.assert_array_equal(o.root_stats(slot), out[:3 * n].reshape(-1, 3))


def test_elementary_functions_close_to_exact():
    xs = np.concatenate([np.arange(1, 5000), np.unique(np.logspace(0, 9, 3000).astype(np.int64))])
    for x in xs:
        got = float(S.det_log(np.float32(x)))
        want = math.log(float(np.float32(x)))
        assert abs(got - want) <= 4 * np.spacing(np.float32(want)) + 1e-12, x
    for x in np.linspace(-87.0, 0.0, 4001, dtype=np.float32):
        got = float(S.det_exp(x))
        want = math.exp(float(x))
        assert abs(got - want) <= 4 * float(np.spacing(np.float32(want))) + 1e-44, x
    for x in np.linspace(-12.0, 12.0, 2401, dtype=np.float32):
        assert abs(float(S.det_tanh(x)) - math.tanh(float(x))) < 2e-7, x


def test_device_mode_invariants():
    """Playouts are conserved through the tree, node ranges are respected and
    every child is its parent's move, on random playout outcomes."""
    roots = L.random_positions(44, 3, 0, 30)
    o = S.SearchesOracle(3, 2, 0, 5, children=L.children,
                         playouts=lambda b, r, seed, base, pol: L.replay_batch(b, r, seed, base, pol)[0])
    caps = [200, 3000, 3000]
    slots = [o.add(r, 4000, caps[i], i << 32) for i, r in enumerate(roots)]
    while any(s.done < s.budget for s in o.slots):
        o.step(32)
    for k, slot in enumerate(slots):
        t = o.tree(slot)
        info, parent = t["info"], t["parent"]
        assert len(info) <= caps[k]
        assert info[0, 2] == 4000
        root_kids = info[0, 1] & 0xFFFF
        first = info[0, 0]
        assert info[first:first + root_kids, 2].sum() == 4000
        for n in range(1, len(info)):
            assert parent[n] < n
            boards, _ = L.children(t["boards"][parent[n]])
            fc = info[parent[n], 0]
            np.testing.assert_array_equal(t["boards"][n], boards[n - fc])

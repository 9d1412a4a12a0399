"""Many searches with device-resident trees (gpuai_searches_*): a search's
result is the same alone and among others, graph replay equals eager launches,
playouts are conserved through the tree, admission is by free node range."""
import numpy as np
import pytest

import oracle_lib as L
from golden_boards import board, sq
from gpu_ai_gb300 import ERR_OOM, GpuAIError, Searches

pytestmark = pytest.mark.gpu


def run_to_end(s, q=32, graph=True, max_rounds=10000):
    for _ in range(max_rounds):
        done, budget = s.poll()
        if (done >= budget).all():
            return done, budget
        s.step(4, q, graph)
    raise AssertionError("searches did not finish")


def stats(s, slot):
    c = s.children(slot)
    return c["visits"].copy(), c["score2"].copy(), c["moves"].copy()


def test_result_alone_equals_result_in_mix(lib_built):
    root = L.random_positions(3, 1, 6, 6)[0]
    a = Searches(64, 400000, 32)
    slot = a.add(root, 20000, 60000, 1 << 40)
    run_to_end(a)
    alone = stats(a, slot)
    b = Searches(64, 400000, 32)
    others = L.random_positions(9, 20, 0, 40)
    for i, r in enumerate(others[:10]):
        b.add(r, 5000 + 1700 * i, 15000, i << 32)
    slot_b = b.add(root, 20000, 60000, 1 << 40)
    for i, r in enumerate(others[10:]):
        b.add(r, 3000 + 2900 * i, 15000, (i + 10) << 32)
    run_to_end(b)
    mixed = stats(b, slot_b)
    for x, y in zip(alone, mixed):
        np.testing.assert_array_equal(x, y)


def test_graph_replay_equals_eager(lib_built):
    roots = L.random_positions(5, 8, 0, 30)
    res = []
    for graph in (True, False):
        s = Searches(8, 200000, 16, playouts_per_leaf=2)
        slots = [s.add(r, 8000, 20000, i << 36) for i, r in enumerate(roots)]
        run_to_end(s, q=16, graph=graph)
        res.append([stats(s, k) for k in slots])
    for x, y in zip(*res):
        for u, v in zip(x, y):
            np.testing.assert_array_equal(u, v)


def test_playouts_conserved_and_moves_legal(lib_built):
    roots = L.random_positions(6, 6, 0, 30)
    s = Searches(16, 300000, 32, playouts_per_leaf=4)
    slots = [s.add(r, 12000, 40000, i << 36) for i, r in enumerate(roots)]
    done, budget = run_to_end(s)
    for k, r in zip(slots, roots):
        assert done[k] == budget[k] == 12000
        c = s.children(k)
        assert c["visits"].sum() == 12000
        assert 1 < c["nodes"] <= 40000
        legal, cnt = L.genmoves(r)
        assert len(c["moves"]) == cnt[0]
        np.testing.assert_array_equal(c["moves"], legal[0, :cnt[0]])


def test_material_advantage_scores_high(lib_built):
    # PLAYER_1 to move with five kings against one man
    kings = [sq(0, 1), sq(2, 3), sq(4, 5), sq(6, 1), sq(3, 6)]
    root = np.array(board(p1=kings, p2=[sq(7, 4)], kings=kings), np.uint32)
    s = Searches(4, 100000, 32)
    slot = s.add(root, 20000, 100000, 7)
    run_to_end(s)
    best, c = s.best(slot)
    i = int(np.argmax(c["visits"]))
    assert c["score2"][i] / (2.0 * c["visits"][i]) > 0.9


def test_admission_by_free_node_range(lib_built):
    root = L.start_board()[0]
    s = Searches(4, 1000, 8)
    a = s.add(root, 100, 800, 0)
    assert s.try_add(root, 100, 800, 1) is None
    with pytest.raises(GpuAIError) as ei:
        s.add(root, 100, 800, 1)
    assert ei.value.code == ERR_OOM
    s.remove(a)
    b = s.add(root, 100, 800, 2)
    run_to_end(s, q=8)
    assert s.children(b)["visits"].sum() == 100


def test_wide_steps_of_512_leaves_per_search(lib_built):
    """Steps of 512 leaf slots per search (the widest frontier the select step
    holds): every playout is accounted for, the result is the same alone and
    in a mix, and the tree keeps the root's legal moves."""
    root = L.random_positions(12, 1, 20, 20)[0]
    a = Searches(8, 600000, 512, playouts_per_leaf=2)
    slot = a.add(root, 60000, 150000, 1 << 40)
    done, budget = run_to_end(a, q=512)
    assert done[slot] == budget[slot] == 60000
    alone = stats(a, slot)
    assert alone[0].sum() == 60000
    legal, cnt = L.genmoves(root)
    np.testing.assert_array_equal(alone[2], legal[0, :cnt[0]])
    b = Searches(8, 600000, 512, playouts_per_leaf=2)
    for i, r in enumerate(L.random_positions(13, 5, 0, 40)):
        b.add(r, 9000 + 7000 * i, 40000, i << 32)
    slot_b = b.add(root, 60000, 150000, 1 << 40)
    run_to_end(b, q=512)
    for x, y in zip(alone, stats(b, slot_b)):
        np.testing.assert_array_equal(x, y)

"""Device-resident searches against their CPU restatement (oracle/search.py),
node for node.

Each step the GPU searches (gpuai_searches_step, through the C ABI) and the
oracle advance the same searches; the oracle selects its own leaves, expands
with the oracle's move generation and replays the playouts on the oracle's
Philox streams, then both trees are compared: leaf slots (search, node,
board, stream id, outcomes) and every node's {first child, children | state,
visits, score2}, board and parent.  Learned searches take the network's
outputs for the leaf slots from the GPU (checked separately against the
network oracle within the forward tolerance) and compare priors too.
Reference: GameTree::select / update (src/mcts.cpp:63-180)."""
import numpy as np
import pytest

import oracle_lib as L
from golden_boards import board, sq
from oracle import mlp
from oracle import search as S

pytestmark = pytest.mark.gpu


def _replay(boards, reps, seed, base, policy):
    return L.replay_batch(boards, reps, seed, base, policy)[0]


def _compare_step(gpu, o, step, net=False):
    lv = gpu.leaves(net=net)
    want = o.last_leaves
    assert len(lv["search"]) == len(want), f"step {step}: leaf count"
    if want:
        np.testing.assert_array_equal(lv["search"], [w[0] for w in want], err_msg=f"step {step}: search")
        np.testing.assert_array_equal(lv["node"], [w[1] for w in want], err_msg=f"step {step}: node")
        np.testing.assert_array_equal(lv["boards"], np.array([w[2] for w in want], np.uint32),
                                      err_msg=f"step {step}: boards")
        np.testing.assert_array_equal(lv["streams"], [w[3] for w in want], err_msg=f"step {step}: streams")
        np.testing.assert_array_equal(lv["outcomes"], np.array([w[4] for w in want]),
                                      err_msg=f"step {step}: outcomes")
    return lv


def _compare_trees(gpu, o, slots, step, priors=False):
    for slot in slots:
        if o.slots[slot] is None:
            continue
        g = gpu.nodes(slot, priors=priors)
        w = o.tree(slot)
        assert len(g["info"]) == len(w["info"]), f"step {step} search {slot}: node count"
        for key in ("info", "boards", "parent"):
            np.testing.assert_array_equal(g[key], w[key], err_msg=f"step {step} search {slot}: {key}")
        if priors:
            np.testing.assert_array_equal(g["priors"].view(np.uint16), o.priors(slot).view(np.uint16),
                                          err_msg=f"step {step} search {slot}: priors")


def _terminal_root():
    # PLAYER_2 to move without pieces: the game is over at the root
    return np.array(board(p1=[sq(2, 1), sq(3, 4)], p2=[], kings=[], turn=1), np.uint32)


def _run(policy, ppl, q, budgets, caps, roots, graph, steps, seed=11):
    from gpu_ai_gb300 import Searches
    gpu = Searches(len(roots) + 1, 200000, q, playouts_per_leaf=ppl, policy=policy, seed=seed)
    o = S.SearchesOracle(len(roots) + 1, ppl, policy, seed, children=L.children, playouts=_replay)
    slots = []
    for i, (r, b, c) in enumerate(zip(roots, budgets, caps)):
        a = gpu.add(r, b, c, (i + 1) << 36)
        assert o.add(r, b, c, (i + 1) << 36) == a
        slots.append(a)
    for step in range(steps):
        gpu.step(1, q, graph)
        done, _ = gpu.poll()
        o.step(q)
        _compare_step(gpu, o, step)
        _compare_trees(gpu, o, slots, step)
        np.testing.assert_array_equal(done[:len(slots)], [o.slots[k].done for k in slots])
        if all(o.slots[k].done >= o.slots[k].budget for k in slots):
            break
    return gpu, o, slots


def test_plain_searches_node_for_node():
    roots = list(L.random_positions(21, 3, 0, 30))
    _run(policy=0, ppl=1, q=32, budgets=[600, 900, 300], caps=[5000, 5000, 5000], roots=roots, graph=True,
         steps=40)


def test_playouts_per_leaf_and_node_range_limits():
    """Four playouts per leaf, a search whose node range runs out (expansions
    then play out instead), a finished game at the root and a budget that
    ends in the middle of a step."""
    roots = list(L.random_positions(22, 2, 5, 40)) + [_terminal_root()]
    _run(policy=0, ppl=4, q=64, budgets=[4000, 2500, 400], caps=[40, 6000, 10], roots=roots, graph=False,
         steps=30)


def test_wide_steps_block_per_search():
    """Steps of 128, 256 and 512 leaves per search, where a whole block of as
    many threads selects for one search (that many frontier entries per
    round), with a node range that runs out in the middle of a round."""
    roots = list(L.random_positions(26, 3, 0, 30))
    _run(policy=0, ppl=2, q=128, budgets=[6000, 4000, 2000], caps=[150, 12000, 12000], roots=roots, graph=True,
         steps=30)
    _run(policy=0, ppl=1, q=512, budgets=[8000, 5000, 3000], caps=[700, 20000, 20000], roots=roots, graph=False,
         steps=30)
    _run(policy=2, ppl=2, q=256, budgets=[7000, 3000, 5000], caps=[20000, 400, 20000], roots=roots, graph=True,
         steps=30)


@pytest.mark.parametrize("policy", [1, 2])
def test_other_playout_policies(policy):
    roots = list(L.random_positions(23 + policy, 3, 10, 40))
    _run(policy=policy, ppl=2, q=48, budgets=[1500, 1000, 700], caps=[8000, 8000, 8000], roots=roots,
         graph=True, steps=25)


def _peaky_params(seed):
    rng = np.random.default_rng(seed)
    d = {
        "W1": rng.normal(0, 0.15, (mlp.H, mlp.IN_PAD)), "b1": rng.normal(0, 0.05, mlp.H),
        "W2": rng.normal(0, 0.08, (mlp.H, mlp.H)), "b2": rng.normal(0, 0.05, mlp.H),
        "W3": rng.normal(0, 0.4, (mlp.OUT, mlp.H)), "b3": rng.normal(0, 0.5, mlp.OUT),
        "wv": rng.normal(0, 0.15, mlp.H), "bv": rng.normal(0, 0.05, 1),
    }
    d["W1"][:, mlp.IN:] = 0
    return mlp.pack(d).astype(np.float32)


@pytest.mark.parametrize("ppl,graph,guided,q", [(2, True, 0, 32), (1, False, 0, 32), (2, True, 3, 32),
                                                (1, True, 0, 128)])
def test_learned_searches_node_for_node(ppl, graph, guided, q):
    """PUCT split with the network's priors, expansion once evaluated, and the
    blended leaf value, with a fixed network; with guided plies the playouts
    are learned-proposal playouts (their outcomes are taken from the GPU: the
    proposal playouts are replayed on their own in test_gpu_proposal.py)."""
    from gpu_ai_gb300 import Net, Searches
    params = _peaky_params(5)
    net = Net(0, max_batch=256, seed=1)
    net.set_params(params)
    roots = list(L.random_positions(25, 3, 0, 30))
    gpu = Searches(4, 200000, q, playouts_per_leaf=ppl, policy=0, seed=3)
    gpu.set_net(net, value_weight=0.5, c_puct=1.5)
    if guided:
        gpu.set_proposal(guided, 1.0)
    learned = {"value_weight": 0.5, "c_puct": 1.5}
    o = S.SearchesOracle(4, ppl, 0, 3, children=L.children, playouts=_replay, learned=learned)
    budgets = [300, 500, 200]
    slots = []
    for i, r in enumerate(roots):
        a = gpu.add(r, budgets[i], 6000, (i + 7) << 36)
        assert o.add(r, budgets[i], 6000, (i + 7) << 36) == a
        slots.append(a)
    for step in range(40):
        gpu.step(1, q, graph)
        gpu.poll()
        lv = gpu.leaves(net=True)
        if len(lv["search"]):
            # the network's outputs for the leaf boards, against the network oracle
            ref = mlp.forward(params, lv["boards"], emulate=True)
            scale = float(np.abs(ref["logits"]).max())
            assert np.abs(lv["net_logits"] - ref["logits"]).max() <= 2e-2 * scale
            assert np.abs(lv["net_value"] - ref["vraw"]).max() <= 2e-2 * max(1.0, float(np.abs(ref["vraw"]).max()))
        o.step(q, net_value=lv["net_value"], net_logits=lv["net_logits"],
               outcomes=lv["outcomes"] if guided else None)
        _compare_step(gpu, o, step, net=True)
        _compare_trees(gpu, o, slots, step, priors=True)
        if all(o.slots[k].done >= o.slots[k].budget for k in slots):
            break
    assert all(o.slots[k].done >= o.slots[k].budget for k in slots)
    gpu.close()
    net.close()

"""The CPU restatement of the guided proposal ply (oracle/proposal.py): its
integer weights are the softmax of the legal pairs' logits, split equally
among moves that share a pair, and its draws follow them."""
import numpy as np

import oracle_lib as L
from golden_boards import board, sq
from oracle import proposal as P


def _moves(b):
    return L.children(np.array(b, np.uint32))


def test_equal_logits_give_equal_weights():
    boards, moves = L.children(L.start_board()[0])
    w = P.weights(moves, np.zeros(1024, np.float32), np.float32(1))
    assert w == [1 << 24] * len(moves)


def test_weights_are_the_softmax():
    rng = np.random.default_rng(0)
    for b in L.random_positions(3, 50, 0, 40):
        boards, moves = L.children(b)
        if len(moves) < 2:
            continue
        logits = rng.normal(0, 2, 1024).astype(np.float32)
        for t in (1.0, 0.5, 2.0):
            w = np.array(P.weights(moves, logits, np.float32(1) / np.float32(t)), np.float64)
            pairs = [int(m[0]) * 32 + int(m[1]) for m in moves]
            mult = np.array([pairs.count(p) for p in pairs])
            l = logits[pairs].astype(np.float64) / t
            ref = np.exp(l - l.max()) / mult
            ref = ref / ref.sum()
            np.testing.assert_allclose(w / w.sum(), ref, atol=1e-6)


def test_shared_pairs_split_their_share():
    # a king with two capture routes to the same square: same (from, to) pair
    k = sq(4, 3)
    b = board(p1=[k], p2=[sq(5, 2), sq(5, 4), sq(3, 2), sq(3, 4)], kings=[k])
    boards, moves = _moves(b)
    pairs = [int(m[0]) * 32 + int(m[1]) for m in moves]
    w = P.weights(moves, np.zeros(1024, np.float32), np.float32(1))
    for i, p in enumerate(pairs):
        assert w[i] == (1 << 24) // pairs.count(p)


def test_pick_frequencies_follow_the_weights():
    boards, moves = L.children(L.start_board()[0])
    rng = np.random.default_rng(1)
    logits = rng.normal(0, 1, 1024).astype(np.float32)
    w = np.array(P.weights(moves, logits, np.float32(1)), np.float64)
    draws = rng.integers(0, 1 << 32, 40000, dtype=np.uint64)
    counts = np.bincount([P.pick(moves, logits, np.float32(1), int(d)) for d in draws], minlength=len(moves))
    np.testing.assert_allclose(counts / counts.sum(), w / w.sum(), atol=0.01)

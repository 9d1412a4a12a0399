"""CPU restatement of one guided ply of the learned-proposal playouts
(proposal_ply_kernel in gpu_ai_gb300/csrc/kernels.cu) -- test infrastructure
only.

The reference's move-scoring playout (heuristicPlayoutKernel,
src/heuristicPlayout.cu:54-88) scores every legal move and picks one; here the
score is the network's policy: each legal move's (from, to) logit l, weight
w = max(1, floor(2^24 e^((l - lmax) / T)) // multiplicity) where the
multiplicity is the number of legal moves sharing that (from, to) pair, and
the move taken is the first whose running weight sum exceeds
mulhi(draw, sum w).  e^x is detmath.cuh's det_exp (restated in
oracle/search.py), so given the same logits and draw the pick is the GPU's.
"""
from __future__ import annotations

import numpy as np

from .search import F, det_exp

MAX_MOVES = 64
DRAW_PLIES = 50
TAG_PROPOSAL = 2


def weights(moves: np.ndarray, logits_row: np.ndarray, inv_temperature) -> list:
    """Integer weights of a move list (packed 32-byte records, reference order)."""
    pairs = [int(m[0]) * 32 + int(m[1]) for m in moves]
    lg = [F(logits_row[p]) for p in pairs]
    lmax = max(lg)
    out = []
    for i, p in enumerate(pairs):
        mult = pairs.count(p)
        e = det_exp((lg[i] - lmax) * F(inv_temperature))
        v = int(e * F(16777216.0)) // mult
        out.append(v if v > 0 else 1)
    return out


def pick(moves: np.ndarray, logits_row: np.ndarray, inv_temperature, draw: int) -> int:
    n = len(moves)
    if n > MAX_MOVES:
        return (draw * n) >> 32
    if n < 2:
        return 0
    w = weights(moves, logits_row, inv_temperature)
    r = (draw * sum(w)) >> 32
    acc = 0
    for m, x in enumerate(w):
        acc += x
        if acc > r:
            return m
    raise AssertionError("unreachable: r < sum of the weights")


def guided_ply(board, logits_row, inv_temperature, draw, children):
    """(board after the guided ply, index of the move taken or -1 when the game is over)."""
    if (int(board[3]) >> 8) & 0xFF >= DRAW_PLIES:
        return np.asarray(board, np.uint32), -1
    boards, moves = children(board)
    if len(moves) == 0:
        return np.asarray(board, np.uint32), -1
    m = pick(moves, logits_row, inv_temperature, draw)
    return boards[m], m

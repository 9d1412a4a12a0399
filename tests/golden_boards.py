"""Seeded and hand-placed boards for the move-generation tests.

Boards are ``[p1, p2, kings, meta]`` uint32 rows; square s = row*4 + col//2.
"""
from __future__ import annotations

import numpy as np


def sq(row: int, col: int) -> int:
    assert (row + col) % 2 == 1, "dark squares only"
    return row * 4 + col // 2


def bits(*squares) -> int:
    v = 0
    for s in squares:
        v |= 1 << s
    return v


def board(p1=(), p2=(), kings=(), turn=0, msc=0):
    return [bits(*p1), bits(*p2), bits(*kings), turn | (msc << 8)]


def random_boards(rng: np.random.Generator, n: int) -> np.ndarray:
    """Random piece placements of varying density and king share."""
    out = []
    per = n // 4
    for pfill, pking in ((0.5, 0.5), (0.3, 0.9), (0.7, 0.7), (0.4, 0.2)):
        occ = rng.random((per, 32)) < pfill
        own = rng.random((per, 32)) < 0.5
        king = rng.random((per, 32)) < pking
        w = 1 << np.arange(32, dtype=np.uint64)
        p1 = ((occ & ~own) * w).sum(1).astype(np.uint32)
        p2 = ((occ & own) * w).sum(1).astype(np.uint32)
        kings = ((occ & king) * w).sum(1).astype(np.uint32)
        kings |= (p1 & np.uint32(0xF0000000)) | (p2 & np.uint32(0x0000000F))  # men on the far row are kings
        turn = rng.integers(0, 2, per).astype(np.uint32)
        msc = rng.integers(0, 60, per).astype(np.uint32)
        out.append(np.stack([p1, p2, kings, turn | (msc << 8)], 1))
    return np.concatenate(out).astype(np.uint32)


def crafted_boards() -> np.ndarray:
    """Hand-placed cases: cycle check, origin quirk, promotions, no moves, draw counter."""
    b = []
    # PLAYER_1 king enters a ring of four PLAYER_2 men; the landing-square
    # cycle check (src/state.cu:134-139) ends both 4-jump sequences one jump
    # short of closing the ring.
    ring = [sq(6, 5), sq(4, 3), sq(4, 5), sq(2, 3), sq(2, 5)]
    b.append(board(p1=[sq(7, 6)], p2=ring, kings=[sq(7, 6)]))
    # king starting on the ring: its own origin stays occupied during the search
    b.append(board(p1=[sq(3, 2)], p2=[sq(2, 3), sq(2, 5), sq(4, 5), sq(4, 3)], kings=[sq(3, 2)]))
    # same rings for PLAYER_2
    b.append(board(p2=[sq(7, 6)], p1=ring, kings=[sq(7, 6)], turn=1))
    b.append(board(p2=[sq(3, 2)], p1=[sq(2, 3), sq(2, 5), sq(4, 5), sq(4, 3)], kings=[sq(3, 2)], turn=1))
    # man capture that promotes; two-jump capture that promotes
    b.append(board(p1=[sq(5, 2)], p2=[sq(6, 3), sq(0, 1)]))
    b.append(board(p1=[sq(3, 0)], p2=[sq(4, 1), sq(6, 3), sq(0, 7)]))
    # PLAYER_2 man capture onto row 0
    b.append(board(p2=[sq(2, 5)], p1=[sq(1, 4), sq(7, 0)], turn=1))
    # direct promotions for both sides
    b.append(board(p1=[sq(6, 1)], p2=[sq(0, 7)]))
    b.append(board(p2=[sq(1, 2)], p1=[sq(7, 6)], turn=1))
    # man branching capture: left then right
    b.append(board(p1=[sq(2, 3)], p2=[sq(3, 2), sq(3, 4), sq(5, 2), sq(5, 6)]))
    # forced capture beside direct moves
    b.append(board(p1=[sq(2, 1), sq(2, 5), sq(1, 0)], p2=[sq(3, 2), sq(7, 0)]))
    # side to move has no pieces / is blocked
    b.append(board(p2=[sq(4, 3)], turn=0))
    b.append(board(p1=[sq(0, 1)], p2=[sq(1, 0), sq(1, 2), sq(2, 3)], turn=0))
    # draw counter at and below the limit
    b.append(board(p1=[sq(0, 1), sq(2, 3)], p2=[sq(7, 0), sq(5, 4)], kings=[sq(0, 1), sq(7, 0)], msc=49))
    b.append(board(p1=[sq(0, 1), sq(2, 3)], p2=[sq(7, 0), sq(5, 4)], kings=[sq(0, 1), sq(7, 0)], msc=50))
    # the standard start, both sides to move
    b.append([0x00000FFF, 0xFFF00000, 0, 0])
    b.append([0x00000FFF, 0xFFF00000, 0, 1])
    # many kings: long branching king captures
    b.append(board(p1=[sq(0, 1), sq(7, 6)],
                   p2=[sq(1, 2), sq(3, 2), sq(3, 4), sq(5, 4), sq(5, 2), sq(1, 4), sq(6, 5)],
                   kings=[sq(0, 1), sq(7, 6), sq(3, 4)]))
    return np.array(b, dtype=np.uint32)

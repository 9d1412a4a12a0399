"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run in a checkout where the reference sources are present: it builds the
reference's own host code (oracle/Makefile target `ref`, compiled from the
unmodified sources) and records its outputs:

  movegen_golden.npz  boards + the reference State::genMoves move lists
                      (src/state.cu:239-245), packed 32-byte records
  playout_golden.npz  the 64 benchmark positions (seed 2016, 0-30 random
                      plies from the start) and the reference's
                      HostPlayoutDriver (src/playout.cpp:17-32) and
                      HostHeuristicPlayoutDriver (src/heuristicPlayout.cpp:12-48)
                      win/draw/loss counts, 4096 playouts per position

  playout_golden_heuristic_32k.npz  (--heuristic-32k) the reference's
                      HostHeuristicPlayoutDriver counts on the same 64
                      positions with 32,768 playouts each: the larger-count
                      check of the heuristic policy's distribution

The reference host drivers are run with OMP_NUM_THREADS=1 so the counts are
reproducible (their rand()/engine state is shared across OpenMP threads).

    OMP_NUM_THREADS=1 python tests/golden/make_golden.py [--heuristic-32k]
"""
from __future__ import annotations

import os
import sys

os.environ.setdefault("OMP_NUM_THREADS", "1")

import numpy as np  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import oracle_lib as L  # noqa: E402
from golden_boards import crafted_boards, random_boards  # noqa: E402

CONFIG_SEED = 2016
CONFIG_POSITIONS = 64
CONFIG_MAX_PLIES = 30
CONFIG_REPS = 4096


def main():
    ref = L.ref()
    if ref is None:
        raise SystemExit("reference sources not available: cannot generate golden fixtures")

    # ---- move generation
    boards = np.concatenate([
        L.random_positions(77, 4000, 0, 120),
        random_boards(np.random.default_rng(5), 3000),
        crafted_boards(),
    ])
    moves, counts = L.genmoves(boards, max_moves=32, lib=ref)
    np.savez_compressed(os.path.join(HERE, "movegen_golden.npz"), boards=boards, moves=moves, counts=counts)

    # ---- playout outcome frequencies on the benchmark positions
    pos = L.random_positions(CONFIG_SEED, CONFIG_POSITIONS, 0, CONFIG_MAX_PLIES)
    states = np.repeat(pos, CONFIG_REPS, axis=0)
    host = L.host_playouts_ref(states, srand_seed=12345).reshape(CONFIG_POSITIONS, CONFIG_REPS)
    heur = L.host_heuristic_ref(states).reshape(CONFIG_POSITIONS, CONFIG_REPS)
    wdl_host = np.stack([L.wdl(r) for r in host])
    wdl_heur = np.stack([L.wdl(r) for r in heur])
    np.savez_compressed(os.path.join(HERE, "playout_golden.npz"), positions=pos, reps=CONFIG_REPS,
                        seed=CONFIG_SEED, max_plies=CONFIG_MAX_PLIES, wdl_host=wdl_host,
                        wdl_host_heuristic=wdl_heur)
    print("boards", boards.shape, "max moves", counts.max())
    print("host W/D/L", wdl_host.sum(0), "heuristic W/D/L", wdl_heur.sum(0))


def heuristic_32k():
    ref = L.ref()
    if ref is None:
        raise SystemExit("reference sources not available: cannot generate golden fixtures")
    reps = 32768
    pos = L.random_positions(CONFIG_SEED, CONFIG_POSITIONS, 0, CONFIG_MAX_PLIES)
    wdl = np.zeros((CONFIG_POSITIONS, 3), np.int64)
    for i in range(CONFIG_POSITIONS):  # one position at a time: bounded memory, same engine stream
        wdl[i] = L.wdl(L.host_heuristic_ref(np.repeat(pos[i:i + 1], reps, axis=0)))
    np.savez_compressed(os.path.join(HERE, "playout_golden_heuristic_32k.npz"), positions=pos, reps=reps,
                        seed=CONFIG_SEED, max_plies=CONFIG_MAX_PLIES, wdl_host_heuristic=wdl)
    print("heuristic 32k W/D/L", wdl.sum(0))


if __name__ == "__main__":
    if "--heuristic-32k" in sys.argv:
        heuristic_32k()
    else:
        main()

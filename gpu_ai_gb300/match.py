"""Learned-proposal MCTS against plain GPU MCTS at equal milliseconds per move.

Both players are device-resident batched searches (gpuai_searches_*) on the
same GPU: the plain player's leaves are valued by uniformly random playouts and
its slots split by UCB1 (the reference's GameTree::select rule,
src/mcts.cpp:63-157); the learned player's leaves are valued by the policy/value
network (blended with its own playouts), its slots split by PUCT on the
network's move priors, and with guided plies its playouts are learned-proposal
playouts (their first plies drawn from the network's policy).  play_configs
plays any two such players against each other, e.g. the learned player with
and without the proposal.

All games run at once.  A round has two phases, one per player: the player
starts a fresh search in every game where it is to move and runs them all
together for exactly `ms_per_move` of wall-clock time, then plays each
search's most visited root move.  Each player thus gets the same time per move
and the same share of the GPU per search.  Openings are short random-play
lines, each played twice with colours swapped.
"""
from __future__ import annotations

import argparse
import json
import math
import time
from typing import Optional

import numpy as np

from .engine import POLICY_RANDOM, Engine, Net, Searches, apply_move

DRAW_PLIES = 50


def wilson(score: float, n: int, z: float = 1.96):
    """95 % Wilson interval of a proportion."""
    if n == 0:
        return (0.0, 1.0)
    d = 1 + z * z / n
    c = (score + z * z / (2 * n)) / d
    h = z * math.sqrt(score * (1 - score) / n + z * z / (4 * n * n)) / d
    return (c - h, c + h)


def openings(eng: Engine, n: int, seed: int, min_plies: int = 2, max_plies: int = 8) -> np.ndarray:
    """n distinct live positions after a few random plies from the start."""
    got, seen = [], set()
    s = seed
    while len(got) < n:
        cand = eng.random_positions(s, 4 * n, min_plies, max_plies)
        _, counts = eng.genmoves(cand)
        for b, c in zip(cand, counts):
            key = tuple(int(x) for x in b)
            if c > 0 and key not in seen:
                seen.add(key)
                got.append(b)
                if len(got) == n:
                    break
        s += 1
    return np.array(got, np.uint32)


def _searches(cfg: dict, n_games: int, leaves: int, node_capacity: int, seed: int) -> Searches:
    """The device searches of one player.  cfg: ppl (playouts per leaf), policy,
    and for a learned player net, value_weight, c_puct and guided plies /
    temperature of its learned-proposal playouts."""
    s = Searches(n_games, n_games * node_capacity, leaves, cfg.get("ppl", 8), cfg.get("policy", POLICY_RANDOM),
                 seed=seed)
    if cfg.get("net") is not None:
        s.set_net(cfg["net"], cfg.get("value_weight", 0.5), cfg.get("c_puct", 1.5))
        if cfg.get("guided", 0):
            s.set_proposal(cfg["guided"], cfg.get("temperature", 1.0))
    return s


def describe(cfg: dict) -> dict:
    d = {k: v for k, v in cfg.items() if k != "net"}
    d["network"] = cfg.get("net") is not None
    return d


def play_configs(eng: Engine, cfg_a: dict, cfg_b: dict, n_games: int = 400, ms_per_move: float = 100.0,
                 seed: int = 0, leaves: int = 64, node_capacity: int = 131072, max_plies: int = 300,
                 verbose: bool = False) -> dict:
    """Player A against player B, every opening played twice with colours
    swapped; A's score (win 1, draw 0.5) with 95 % intervals."""
    n_games -= n_games % 2
    opens = openings(eng, n_games // 2, seed)
    boards = np.repeat(opens, 2, axis=0)
    a_p1 = np.tile([True, False], n_games // 2)  # A plays PLAYER_1 in even games
    plies = np.zeros(n_games, np.int64)
    result = np.full(n_games, -2, np.int64)  # +1 P1 won, -1 P2 won, 0 draw, -2 running
    sides = {"a": _searches(cfg_a, n_games, leaves, node_capacity, seed * 2 + 2),
             "b": _searches(cfg_b, n_games, leaves, node_capacity, seed * 2 + 1)}
    stats = {"a_playouts": 0, "b_playouts": 0, "a_steps": 0, "b_steps": 0, "phases": 0}
    t_start = time.perf_counter()

    def finish_checks():
        live = np.flatnonzero(result == -2)
        if len(live) == 0:
            return
        _, counts = eng.genmoves(boards[live], 64)
        for g, c in zip(live, counts):
            if c == 0:
                result[g] = -1 if (boards[g, 3] & 1) == 0 else 1  # the side to move has lost
            elif ((boards[g, 3] >> 8) & 0xFF) >= DRAW_PLIES or plies[g] >= max_plies:
                result[g] = 0

    finish_checks()
    while np.any(result == -2):
        for key in ("a", "b"):
            live = np.flatnonzero(result == -2)
            p1_to_move = (boards[live, 3] & 1) == 0
            mine = live[np.where(key == "a", p1_to_move == a_p1[live], p1_to_move != a_p1[live])]
            if len(mine) == 0:
                continue
            S = sides[key]
            slots = {}
            for g in mine:
                slots[g] = S.add(boards[g], 1 << 40, node_capacity, (int(g) << 40) | (int(plies[g]) << 28))
            t0 = time.perf_counter()
            steps = 0
            while (time.perf_counter() - t0) * 1e3 < ms_per_move:
                S.step(2, leaves)
                S.poll()
                steps += 2
            done, _ = S.poll()
            stats[f"{key}_playouts"] += int(sum(int(done[slots[g]]) for g in mine))
            stats[f"{key}_steps"] += steps
            stats["phases"] += 1
            for g in mine:
                move, _ = S.best(slots[g])
                S.remove(slots[g])
                boards[g] = apply_move(boards[g], move)
                plies[g] += 1
            finish_checks()
        if verbose:
            print(f"round: {int(np.sum(result != -2))}/{n_games} finished", flush=True)
    for S in sides.values():
        S.close()
    aw = int(np.sum((result == 1) & a_p1) + np.sum((result == -1) & ~a_p1))
    al = int(np.sum((result == -1) & a_p1) + np.sum((result == 1) & ~a_p1))
    dr = int(np.sum(result == 0))
    score = (aw + 0.5 * dr) / n_games
    # per-game score variance for the normal interval (draws count half)
    per_game = np.where(result == 0, 0.5, np.where((result == 1) == a_p1, 1.0, 0.0))
    se = float(per_game.std(ddof=1) / math.sqrt(n_games)) if n_games > 1 else 1.0
    return {"games": n_games, "ms_per_move": ms_per_move, "a_wins": aw, "draws": dr, "a_losses": al,
            "a_score": score, "ci95_normal": [score - 1.96 * se, score + 1.96 * se],
            "ci95_wilson": list(wilson(score, n_games)), "mean_plies": float(plies.mean()),
            "seconds": time.perf_counter() - t_start, "leaves_per_search_per_step": leaves,
            "a": describe(cfg_a), "b": describe(cfg_b), **stats}


def play_match(net: Net, eng: Engine, n_games: int = 400, ms_per_move: float = 100.0, seed: int = 0,
               leaves: int = 64, plain_ppl: int = 8, learned_ppl: int = 2, value_weight: float = 0.5,
               c_puct: float = 1.5, node_capacity: int = 131072, max_plies: int = 300, verbose: bool = False,
               guided: int = 0, temperature: float = 1.0) -> dict:
    """The learned player (network priors and leaf values, and with guided > 0
    learned-proposal playouts) against plain GPU MCTS."""
    learned = {"net": net, "ppl": learned_ppl, "value_weight": value_weight, "c_puct": c_puct, "guided": guided,
               "temperature": temperature}
    plain = {"ppl": plain_ppl}
    m = play_configs(eng, learned, plain, n_games, ms_per_move, seed, leaves, node_capacity, max_plies, verbose)
    m.update({"learned_wins": m["a_wins"], "learned_losses": m["a_losses"], "learned_score": m["a_score"],
              "learned_playouts": m["a_playouts"], "plain_playouts": m["b_playouts"],
              "learned_steps": m["a_steps"], "plain_steps": m["b_steps"],
              "config": {"leaves_per_search_per_step": leaves, "plain_playouts_per_leaf": plain_ppl,
                         "learned_playouts_per_leaf": learned_ppl, "value_weight": value_weight,
                         "c_puct": c_puct, "guided_plies": guided, "temperature": temperature}})
    return m


def main(argv: Optional[list] = None):
    ap = argparse.ArgumentParser(description="learned-proposal MCTS vs plain GPU MCTS")
    ap.add_argument("--net", required=True, help="network file (gpuai_net_save)")
    ap.add_argument("--games", type=int, default=400)
    ap.add_argument("--ms", type=float, default=100.0)
    ap.add_argument("--leaves", type=int, default=64)
    ap.add_argument("--plain-ppl", type=int, default=8)
    ap.add_argument("--learned-ppl", type=int, default=2)
    ap.add_argument("--value-weight", type=float, default=0.5)
    ap.add_argument("--c-puct", type=float, default=1.5)
    ap.add_argument("--guided", type=int, default=0, help="learned-proposal plies per playout")
    ap.add_argument("--temperature", type=float, default=1.0)
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args(argv)
    net = Net(0, max_batch=256)
    net.load(a.net)
    eng = Engine(0)
    print(json.dumps(play_match(net, eng, a.games, a.ms, a.seed, a.leaves, a.plain_ppl, a.learned_ppl,
                                a.value_weight, a.c_puct, verbose=True, guided=a.guided,
                                temperature=a.temperature)))


if __name__ == "__main__":
    main()

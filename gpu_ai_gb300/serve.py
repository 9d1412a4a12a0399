"""Search-request serving loop with continuous batching on one GPU.

Requests (a position and a budget) arrive over time.  A request is admitted
as soon as the device-resident search pool (``Searches``) has a free search
slot and a free node range of the size it reserves; otherwise it waits in a
FIFO queue.  Every step advances all admitted searches together (one batched
leaf selection, one playout launch, one backpropagation, replayed as a CUDA
graph), so requests that arrive while others run join the next step.  A
request finishes when its playout budget is spent or its time budget has
elapsed; its result is the most visited root move.

Because each search is advanced by its own warp in a fixed order and uses its
own random-stream range, a request with a playout budget gets the same tree,
and the same result, whether it runs alone or among other requests.

With a policy/value network attached, the same loop serves learned searches
(network leaf values and move priors; the network's forward pass runs once per
step on the leaves of all admitted requests together).

``simulate()`` drives the loop with Poisson arrivals and reports latency
percentiles, playouts/s and peak device memory.
"""
from __future__ import annotations

import collections
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from .engine import POLICY_RANDOM, Searches

NODE_BYTES = 52  # device bytes per tree node (record, board, parent, move)
LEARNED_NODE_BYTES = 64  # learned searches: 32 FP16 move priors per node


@dataclass
class Request:
    rid: int
    board: np.ndarray
    arrival: float                    # seconds, on the server's clock
    budget_ms: Optional[float] = None  # time budget from admission
    budget_playouts: int = 1 << 40     # playout budget
    node_capacity: int = 65536
    # filled in by the server
    admitted: float = 0.0
    finished: float = 0.0
    slot: int = -1
    playouts: int = 0
    best_move: Optional[np.ndarray] = None
    visits: Optional[np.ndarray] = None
    score2: Optional[np.ndarray] = None

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


class SearchServer:
    def __init__(self, max_searches: int = 4096, pool_nodes: Optional[int] = None, pool_fraction: float = 0.25,
                 leaves_per_search: int = 64, playouts_per_leaf: int = 8, policy: int = POLICY_RANDOM,
                 seed: int = 0, use_graph: bool = True, steps_per_poll: int = 2, net=None,
                 value_weight: float = 0.5, c_puct: float = 1.5, searches=None, guided: int = 0,
                 temperature: float = 1.0):
        """`searches`: an already created search pool with the `Searches`
        interface (try_add / step / poll / best / remove / close) to serve
        from instead of creating one; pool_nodes must then be given."""
        node_bytes = NODE_BYTES + (LEARNED_NODE_BYTES if net is not None else 0)
        if pool_nodes is None:  # admission by free device memory
            if searches is not None:
                raise ValueError("pool_nodes is required with an existing search pool")
            import torch
            free, _ = torch.cuda.mem_get_info()
            pool_nodes = int(free * pool_fraction) // node_bytes
        self.pool_nodes = pool_nodes
        self.node_bytes = node_bytes
        self.s = searches if searches is not None else Searches(max_searches, pool_nodes, leaves_per_search,
                                                                playouts_per_leaf, policy, seed)
        if net is not None:  # learned searches: network leaf values and move priors
            self.s.set_net(net, value_weight, c_puct)
            if guided:  # and learned-proposal playouts
                self.s.set_proposal(guided, temperature)
        self.q = leaves_per_search
        self.ppl = playouts_per_leaf
        self.use_graph = use_graph
        self.steps_per_poll = steps_per_poll
        self.queue: collections.deque = collections.deque()
        self.active: Dict[int, Request] = {}
        self.done: List[Request] = []
        self.t0 = time.perf_counter()
        self.nodes_reserved = 0
        self.peak_nodes_reserved = 0
        self.steps = 0

    def now(self) -> float:
        return time.perf_counter() - self.t0

    def submit(self, req: Request):
        self.queue.append(req)

    def _admit(self):
        while self.queue:
            r = self.queue[0]
            budget = -(-r.budget_playouts // self.ppl) * self.ppl
            slot = self.s.try_add(r.board, budget, r.node_capacity, r.rid << 40)
            if slot is None:
                return  # refused: wait for a running request to release its nodes
            self.queue.popleft()
            r.slot, r.admitted = slot, self.now()
            self.active[slot] = r
            self.nodes_reserved += r.node_capacity
            self.peak_nodes_reserved = max(self.peak_nodes_reserved, self.nodes_reserved)

    def _finish(self, slot: int, playouts: int):
        r = self.active.pop(slot)
        best, c = self.s.best(slot)
        r.best_move, r.visits, r.score2 = best, c["visits"], c["score2"]
        r.playouts = playouts
        r.finished = self.now()
        self.s.remove(slot)
        self.nodes_reserved -= r.node_capacity
        self.done.append(r)

    def pump(self):
        """Admit, run a few steps, collect finished requests."""
        self._admit()
        if not self.active:
            return
        self.s.step(self.steps_per_poll, self.q, self.use_graph)
        self.steps += self.steps_per_poll
        done, budget = self.s.poll()
        t = self.now()
        for slot, r in list(self.active.items()):
            timed_out = r.budget_ms is not None and (t - r.admitted) * 1e3 >= r.budget_ms
            if done[slot] >= budget[slot] or timed_out:
                self._finish(slot, int(done[slot]))

    def drain(self):
        while self.queue or self.active:
            self.pump()

    def close(self):
        self.s.close()


def simulate(rate: float = 1000.0, n_requests: int = 2000, n_games: int = 10000, budget_ms=(10.0, 200.0),
             policy: int = POLICY_RANDOM, seed: int = 1, leaves_per_search: int = 64, playouts_per_leaf: int = 8,
             node_capacity: int = 65536, server: Optional[SearchServer] = None, net=None,
             value_weight: float = 0.5, c_puct: float = 1.5, guided: int = 0, temperature: float = 1.0,
             device_memory=None) -> dict:
    """Poisson arrivals at `rate` req/s of requests on positions drawn from
    `n_games` seeded games (0-60 random plies), time budgets U(budget_ms).
    device_memory: a function returning (free, total) bytes of the device
    (cudaMemGetInfo); when given, the peak device memory in use during the
    run is reported."""
    from .engine import Engine
    rng = np.random.default_rng(seed)
    games = Engine(0).random_positions(seed, n_games, 0, 60)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    budgets = rng.uniform(budget_ms[0], budget_ms[1], n_requests)
    picks = rng.integers(0, n_games, n_requests)
    srv = server or SearchServer(leaves_per_search=leaves_per_search, playouts_per_leaf=playouts_per_leaf,
                                 policy=policy, seed=seed, net=net, value_weight=value_weight, c_puct=c_puct,
                                 guided=guided, temperature=temperature)
    srv.t0 = time.perf_counter()
    peak_used = 0
    if device_memory is not None:
        free, total = device_memory()
        peak_used = total - free
    i = 0
    pumps = 0
    while i < n_requests or srv.queue or srv.active:
        t = srv.now()
        while i < n_requests and arrivals[i] <= t:
            srv.submit(Request(rid=i, board=games[picks[i]], arrival=float(arrivals[i]),
                               budget_ms=float(budgets[i]), node_capacity=node_capacity))
            i += 1
        if not srv.queue and not srv.active:
            time.sleep(max(0.0, min(0.002, arrivals[i] - t)) if i < n_requests else 0.0)
            continue
        srv.pump()
        pumps += 1
        if device_memory is not None and pumps % 16 == 0:
            free, total = device_memory()
            peak_used = max(peak_used, total - free)
    elapsed = srv.now()
    lat = np.array([r.latency for r in srv.done]) * 1e3
    playouts = sum(r.playouts for r in srv.done)
    out = {
        "requests": len(srv.done), "rate_req_s": rate, "policy": policy, "elapsed_s": elapsed,
        "latency_ms_p50": float(np.percentile(lat, 50)), "latency_ms_p99": float(np.percentile(lat, 99)),
        "latency_ms_max": float(lat.max()), "playouts_per_s": playouts / elapsed,
        "mean_playouts_per_request": playouts / max(1, len(srv.done)),
        "peak_tree_bytes": srv.peak_nodes_reserved * srv.node_bytes, "pool_bytes": srv.pool_nodes * srv.node_bytes,
        "steps": srv.steps,
    }
    if device_memory is not None:
        out["peak_device_bytes_in_use"] = peak_used
    if server is None:
        srv.close()
    return out

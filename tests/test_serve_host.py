"""The serving loop's host logic on a fake search pool (no GPU): FIFO
admission by free slot and node range, playout and time budgets, node
accounting, and results handed back per request."""
import numpy as np
import pytest

from gpu_ai_gb300.serve import Request, SearchServer


class FakeSearches:
    """The `Searches` interface over host counters: each step adds
    leaves x playouts-per-leaf playouts to every admitted search; node ranges
    are allocated first-fit from a pool of `pool_nodes`."""

    def __init__(self, max_searches, pool_nodes, ppl):
        self.max_searches, self.pool_nodes, self.ppl = max_searches, pool_nodes, ppl
        self.ranges = {}  # slot -> (start, size)
        self.done = np.zeros(max_searches, np.uint64)
        self.budget = np.zeros(max_searches, np.uint64)
        self.added = []
        self.closed = False

    def _fit(self, size):
        at = 0
        for start, n in sorted(self.ranges.values()):
            if start - at >= size:
                return at
            at = start + n
        return at if self.pool_nodes - at >= size else None

    def try_add(self, board, budget, node_capacity, stream_base):
        free = [i for i in range(self.max_searches) if i not in self.ranges]
        at = self._fit(node_capacity)
        if not free or at is None:
            return None
        slot = free[0]
        self.ranges[slot] = (at, node_capacity)
        self.done[slot], self.budget[slot] = 0, budget
        self.added.append((slot, int(budget), stream_base))
        return slot

    def step(self, steps, leaves, use_graph=True):
        for slot in self.ranges:
            self.done[slot] = min(int(self.budget[slot]), int(self.done[slot]) + steps * leaves * self.ppl)

    def poll(self):
        return self.done.copy(), self.budget.copy()

    def best(self, slot):
        v = np.array([3, 9, 1], np.uint32) + slot
        return np.full(32, slot, np.uint8), {"visits": v, "score2": 2 * v}

    def remove(self, slot):
        del self.ranges[slot]

    def close(self):
        self.closed = True


def _server(max_searches=4, pool_nodes=1000, leaves=4, ppl=2, steps_per_poll=1):
    fake = FakeSearches(max_searches, pool_nodes, ppl)
    srv = SearchServer(max_searches=max_searches, pool_nodes=pool_nodes, leaves_per_search=leaves,
                       playouts_per_leaf=ppl, steps_per_poll=steps_per_poll, searches=fake)
    return srv, fake


def _req(rid, playouts=1 << 40, ms=None, nodes=100):
    return Request(rid=rid, board=np.zeros(4, np.uint32), arrival=0.0, budget_ms=ms, budget_playouts=playouts,
                   node_capacity=nodes)


def test_playout_budgets_finish_and_release_nodes():
    srv, fake = _server()
    for i, b in enumerate([8, 20, 7]):
        srv.submit(_req(i, playouts=b))
    srv.drain()
    assert sorted(r.rid for r in srv.done) == [0, 1, 2]
    got = {r.rid: r.playouts for r in srv.done}
    # budgets are rounded up to whole leaves of 2 playouts: 8, 20, 8
    assert got == {0: 8, 1: 20, 2: 8}
    assert [b for _, b, _ in fake.added] == [8, 20, 8]
    assert [s for _, _, s in fake.added] == [0, 1 << 40, 2 << 40]  # disjoint random-stream ranges
    assert srv.nodes_reserved == 0 and srv.peak_nodes_reserved == 300 and not fake.ranges
    for r in srv.done:  # each request gets its own search's result
        assert (r.best_move == r.slot).all() and list(r.visits) == [3 + r.slot, 9 + r.slot, 1 + r.slot]


def test_fifo_admission_waits_for_nodes():
    srv, fake = _server(max_searches=8, pool_nodes=1000)
    srv.submit(_req(0, playouts=80, nodes=600))
    srv.submit(_req(1, playouts=8, nodes=600))   # does not fit until request 0 leaves
    srv.submit(_req(2, playouts=8, nodes=100))   # fits, but waits behind request 1 (FIFO)
    srv.pump()
    assert set(r.rid for r in srv.active.values()) == {0}
    assert [r.rid for r in srv.queue] == [1, 2]
    srv.drain()
    order = [r.rid for r in srv.done]
    assert order[0] == 0 and sorted(order) == [0, 1, 2]
    assert srv.peak_nodes_reserved == 700 and srv.nodes_reserved == 0


def test_slots_bound_admission():
    srv, fake = _server(max_searches=2, pool_nodes=10_000)
    for i in range(5):
        srv.submit(_req(i, playouts=16))
    srv.pump()
    assert len(srv.active) == 2 and len(srv.queue) == 3
    srv.drain()
    assert sorted(r.rid for r in srv.done) == list(range(5))


def test_time_budget_ends_a_search():
    srv, fake = _server()
    clock = [0.0]
    srv.now = lambda: clock[0]
    srv.submit(_req(0, ms=50.0))              # unlimited playouts, 50 ms
    srv.submit(_req(1, playouts=16, ms=1e9))  # ends by its playout budget
    srv.pump()
    clock[0] = 0.049
    srv.pump()
    assert [r.rid for r in srv.done] == [1] and 0 in [r.rid for r in srv.active.values()]
    clock[0] = 0.050
    srv.pump()
    r0 = [r for r in srv.done if r.rid == 0][0]
    assert r0.finished == pytest.approx(0.050) and r0.latency == pytest.approx(0.050)
    assert r0.playouts == 3 * 4 * 2  # three steps of 4 leaves x 2 playouts


def test_existing_pool_needs_pool_nodes():
    with pytest.raises(ValueError):
        SearchServer(searches=FakeSearches(1, 10, 1))


def test_close_closes_the_pool():
    srv, fake = _server()
    srv.close()
    assert fake.closed

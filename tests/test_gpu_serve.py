"""Serving loop (gpu_ai_gb300.serve): continuous batching of search requests,
admission by free tree memory, and the same result for a request alone and
in the mix."""
import numpy as np
import pytest

import oracle_lib as L
from gpu_ai_gb300.serve import Request, SearchServer, simulate

pytestmark = pytest.mark.gpu


def _req(rid, board, playouts, cap=40000):
    return Request(rid=rid, board=board, arrival=0.0, budget_playouts=playouts, node_capacity=cap)


def _live(boards):
    """Boards whose game is not over."""
    _, counts = L.genmoves(boards)
    return boards[(counts > 0) & (((boards[:, 3] >> 8) & 0xff) < 50)]


def test_request_same_alone_and_in_mix(lib_built):
    boards = _live(L.random_positions(17, 60, 0, 60))[:40]
    assert len(boards) == 40
    srv = SearchServer(max_searches=64, pool_nodes=4_000_000, leaves_per_search=32, playouts_per_leaf=4)
    srv.submit(_req(7, boards[7], 24000))
    srv.drain()
    alone = srv.done[0]
    srv.close()
    mix = SearchServer(max_searches=64, pool_nodes=4_000_000, leaves_per_search=32, playouts_per_leaf=4)
    for i in range(0, 20):  # requests that arrive before, with and after request 7
        if i != 7:
            mix.submit(_req(i, boards[i], 4000 + 1000 * i))
    mix.pump()
    mix.pump()
    mix.submit(_req(7, boards[7], 24000))
    for i in range(20, 40):
        mix.pump()
        mix.submit(_req(i, boards[i], 3000 + 500 * i))
    mix.drain()
    got = {r.rid: r for r in mix.done}
    mix.close()
    assert len(got) == 40
    r = got[7]
    assert r.playouts == alone.playouts == 24000
    np.testing.assert_array_equal(r.visits, alone.visits)
    np.testing.assert_array_equal(r.score2, alone.score2)
    np.testing.assert_array_equal(r.best_move, alone.best_move)


def test_admission_waits_for_free_nodes(lib_built):
    boards = _live(L.random_positions(3, 12, 0, 30))[:6]
    srv = SearchServer(max_searches=16, pool_nodes=25000, leaves_per_search=16, playouts_per_leaf=2)
    for i in range(6):
        srv.submit(_req(i, boards[i], 2000, cap=10000))
    srv.pump()
    assert len(srv.active) == 2 and len(srv.queue) == 4  # only two 10K-node ranges fit
    srv.drain()
    assert len(srv.done) == 6 and srv.peak_nodes_reserved <= 25000
    assert all(r.playouts == 2000 for r in srv.done)
    srv.close()


def test_simulated_poisson_load(lib_built):
    out = simulate(rate=400.0, n_requests=120, n_games=1000, budget_ms=(10.0, 30.0), leaves_per_search=32,
                   playouts_per_leaf=4, node_capacity=20000)
    assert out["requests"] == 120
    assert 10.0 <= out["latency_ms_p50"] <= out["latency_ms_p99"] < 2000.0
    assert out["playouts_per_s"] > 0 and out["peak_tree_bytes"] <= out["pool_bytes"]

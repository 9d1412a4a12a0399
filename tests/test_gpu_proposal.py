"""Learned-proposal playouts (gpuai_playouts_learned) against the CPU replay.

Every playout's guided plies are replayed on the CPU (oracle/proposal.py) from
the logits the kernel used (traced) and the same Philox draws, and its random
continuation by the oracle's playout replay: board after every guided ply and
the outcome must equal the GPU's bit for bit.  The traced logits themselves
are the network's forward pass on the traced boards, within the forward
tolerance of the network oracle (oracle/mlp.py).  Reference shape: the
move-scoring playout of src/heuristicPlayout.cu:54-88."""
import numpy as np
import pytest

import oracle_lib as L
from oracle import mlp
from oracle import proposal as P

pytestmark = pytest.mark.gpu


def _params(seed, scale=0.4):
    rng = np.random.default_rng(seed)
    d = {
        "W1": rng.normal(0, 0.15, (mlp.H, mlp.IN_PAD)), "b1": rng.normal(0, 0.05, mlp.H),
        "W2": rng.normal(0, 0.08, (mlp.H, mlp.H)), "b2": rng.normal(0, 0.05, mlp.H),
        "W3": rng.normal(0, scale, (mlp.OUT, mlp.H)), "b3": rng.normal(0, 0.5, mlp.OUT),
        "wv": rng.normal(0, 0.08, mlp.H), "bv": rng.normal(0, 0.05, 1),
    }
    d["W1"][:, mlp.IN:] = 0
    return mlp.pack(d).astype(np.float32)


@pytest.fixture(scope="module")
def net(lib_built):
    from gpu_ai_gb300 import Net
    n = Net(0, max_batch=256, seed=1)
    p = _params(8)
    n.set_params(p)
    n.p = p
    yield n
    n.close()


def _run(engine, net, pos, reps, seed, base, guided, temperature, trace=True):
    torch = pytest.importorskip("torch")
    reps = np.asarray(reps, np.uint32)
    total = int(reps.sum())
    offs = np.concatenate([[0], np.cumsum(reps)]).astype(np.uint32)
    d_pos = torch.from_numpy(np.ascontiguousarray(pos, np.uint32).view(np.int32)).cuda()
    d_off = torch.from_numpy(offs.view(np.int32)).cuda()
    d_out = torch.full((total,), 7, dtype=torch.int8, device="cuda")
    tb = torch.zeros((max(guided, 1) * total, 4), dtype=torch.int32, device="cuda")
    tl = torch.zeros((max(guided, 1) * total, 1024), dtype=torch.int16, device="cuda")
    torch.cuda.synchronize()
    engine.playouts_learned(net, d_pos.data_ptr(), d_off.data_ptr(), len(pos), 0, total, seed, base, guided,
                            temperature, d_out.data_ptr(), None,
                            tb.data_ptr() if trace else None, tl.data_ptr() if trace else None)
    torch.cuda.synchronize()
    st, _ = engine.status()
    assert st == 0
    out = d_out.cpu().numpy()
    tb = tb.cpu().numpy().view(np.uint32).reshape(max(guided, 1), total, 4)
    tl = tl.cpu().numpy().view(np.uint16).reshape(max(guided, 1), total, 1024)
    return out, tb, tl, offs


@pytest.mark.parametrize("guided,temperature", [(1, 1.0), (3, 1.0), (4, 0.5)])
def test_guided_plies_replay_bit_exact(engine, net, guided, temperature):
    pos = L.random_positions(61, 40, 0, 50)
    reps = np.random.default_rng(guided).integers(0, 40, len(pos))
    reps[3] = 0
    seed, base = 123 + guided, 1 << 33
    out, tb, tl, offs = _run(engine, net, pos, reps, seed, base, guided, temperature)
    total = len(out)
    inv_t = np.float32(1.0) / np.float32(temperature)
    pidx = np.searchsorted(offs, np.arange(total), side="right") - 1
    finals = np.zeros((total, 4), np.uint32)
    for j in range(total):
        b = pos[pidx[j]]
        for g in range(guided):
            np.testing.assert_array_equal(tb[g, j], b, err_msg=f"playout {j} guided ply {g}")
            logits = (tl[g, j].astype(np.uint32) << 16).view(np.float32)
            draw = L.stream_draw(seed, base + j, P.TAG_PROPOSAL, g)
            b, _ = P.guided_ply(b, logits, inv_t, draw, L.children)
        finals[j] = b
    # the random continuations, on the oracle's streams (tag 0, stream_base + j)
    exp, _ = L.replay_batch(finals, np.ones(total, np.uint32), seed, base, 0)
    np.testing.assert_array_equal(out, exp)
    # the traced logits are the network's on the traced boards
    for g in range(guided):
        rows = np.arange(0, total, 7)
        ref = mlp.forward(net.p, tb[g, rows], emulate=True)["logits"]
        got = (tl[g, rows].astype(np.uint32) << 16).view(np.float32)
        assert np.abs(got - ref).max() <= 2e-2 * float(np.abs(ref).max())


def test_zero_guided_plies_are_random_playouts(engine, net):
    pos = L.random_positions(62, 16, 0, 30)
    reps = np.full(len(pos), 32)
    out, _, _, _ = _run(engine, net, pos, reps, 9, 0, 0, 1.0, trace=False)
    np.testing.assert_array_equal(out, engine.playouts(pos, reps.astype(np.uint32), seed=9, stream_base=0))


def test_split_batches_equal_one_call(engine, net):
    pos = L.random_positions(63, 24, 0, 40)
    reps = np.full(len(pos), 20)
    whole, _, _, _ = _run(engine, net, pos, reps, 4, 1000, 2, 1.0, trace=False)
    a, _, _, _ = _run(engine, net, pos[:10], reps[:10], 4, 1000, 2, 1.0, trace=False)
    b, _, _, _ = _run(engine, net, pos[10:], reps[10:], 4, 1000 + 200, 2, 1.0, trace=False)
    np.testing.assert_array_equal(whole, np.concatenate([a, b]))


def test_low_temperature_follows_the_policy(engine, net):
    """At a low temperature the first guided move is a legal move of the pair
    with the largest logit in nearly every playout."""
    pos = L.random_positions(64, 32, 0, 30)
    reps = np.full(len(pos), 16)
    out, tb, tl, offs = _run(engine, net, pos, reps, 5, 0, 2, 0.01)
    hits = 0
    for j in range(len(out)):
        boards, moves = L.children(tb[0, j])
        if len(moves) < 2:
            hits += 1
            continue
        logits = (tl[0, j].astype(np.uint32) << 16).view(np.float32)
        pl = np.array([logits[int(m[0]) * 32 + int(m[1])] for m in moves])
        taken = [m for m in range(len(moves)) if np.array_equal(boards[m], tb[1, j])]
        assert taken, f"playout {j}: the board after the guided ply is not a child"
        hits += pl[taken[0]] == pl.max()
    assert hits >= 0.97 * len(out)

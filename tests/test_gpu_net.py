"""GPU parity of the policy/value network kernels (net.cu) against the CPU
oracle (oracle/mlp.py), training-label parity against plain GPU playouts, and
learned searches."""
import os

import numpy as np
import pytest

import oracle_lib as L
from golden_boards import random_boards
from gpu_ai_gb300 import GpuAIError
from oracle import mlp

pytestmark = pytest.mark.gpu


def _positions(seed, n, max_plies=60):
    boards = L.random_positions(seed, n * 3, 0, max_plies)
    out, counts = L.genmoves(boards)
    keep = (counts > 0) & (counts <= mlp.MAXM) & (((boards[:, 3] >> 8) & 0xFF) < 50)
    boards, out, counts = boards[keep][:n], out[keep][:n], counts[keep][:n]
    assert len(boards) == n
    return boards, out[:, :, 0], out[:, :, 1], counts


def _params(seed):
    rng = np.random.default_rng(seed)
    d = {
        "W1": rng.normal(0, 0.15, (mlp.H, mlp.IN_PAD)), "b1": rng.normal(0, 0.05, mlp.H),
        "W2": rng.normal(0, 0.08, (mlp.H, mlp.H)), "b2": rng.normal(0, 0.05, mlp.H),
        "W3": rng.normal(0, 0.08, (mlp.OUT, mlp.H)), "b3": rng.normal(0, 0.05, mlp.OUT),
        "wv": rng.normal(0, 0.08, mlp.H), "bv": rng.normal(0, 0.05, 1),
    }
    d["W1"][:, mlp.IN:] = 0
    return mlp.pack(d).astype(np.float32)


def _segments():
    return {"W1": (mlp.O_W1, mlp.O_B1), "b1": (mlp.O_B1, mlp.O_W2), "W2": (mlp.O_W2, mlp.O_B2),
            "b2": (mlp.O_B2, mlp.O_W3), "W3": (mlp.O_W3, mlp.O_B3), "b3": (mlp.O_B3, mlp.O_WV),
            "wv": (mlp.O_WV, mlp.O_BV), "bv": (mlp.O_BV, mlp.N_PARAMS)}


@pytest.fixture(scope="module")
def Net(lib_built):
    from gpu_ai_gb300 import Net
    return Net


def test_forward_matches_oracle(Net):
    net = Net(0, max_batch=512, seed=1)
    p = _params(2)
    net.set_params(p)
    boards, _, _, _ = _positions(3, 300)
    value, logits = net.forward(boards)
    ref = mlp.forward(p, boards, emulate=True)
    scale = np.abs(ref["logits"]).max()
    assert np.abs(logits - ref["logits"]).max() <= 1e-2 * scale
    assert np.abs(logits - ref["logits"]).mean() <= 1e-3 * scale
    assert np.abs(value - ref["value"]).max() <= 1e-2
    # chunked forward (more boards than the batch capacity) gives the same rows
    big = np.concatenate([boards, boards, boards])
    v3, l3 = net.forward(big)
    assert np.array_equal(v3[:300], value) and np.array_equal(l3[600:], logits)
    net.close()


def test_default_initialisation(Net):
    net = Net(0, max_batch=128, seed=5)
    p = net.params()
    d = mlp.unpack(p)
    assert np.all(d["W1"][:, mlp.IN:] == 0)
    for k, fan in (("W2", 512), ("W3", 1280)):
        bound = np.sqrt(6.0 / fan)
        assert np.abs(d[k]).max() <= bound and np.abs(d[k]).max() > 0.95 * bound
    assert np.all(d["b1"] == 0) and np.all(d["b3"] == 0)
    assert not np.array_equal(Net(0, max_batch=128, seed=6).params(), p)
    net.close()


@pytest.mark.parametrize("n,tau,vc", [(300, 0.1, 1.0), (128, 0.3, 0.5), (517, 0.1, 2.0)])
def test_gradients_match_oracle(Net, n, tau, vc):
    net = Net(0, max_batch=640, seed=1)
    p = _params(n)
    net.set_params(p)
    boards, fr, to, counts = _positions(n + 7, n)
    rng = np.random.default_rng(n)
    z = rng.uniform(-1, 1, n).astype(np.float32)
    q = rng.uniform(-1, 1, (n, mlp.MAXM)).astype(np.float32)
    g, loss = net.gradients(boards, z, q, tau, vc)
    loss_ref, _, g_ref = mlp.loss_grads(p, boards, z, q, fr, to, counts, tau, vc, emulate=True)
    assert loss == pytest.approx(loss_ref, rel=2e-3)
    for name, (lo, hi) in _segments().items():
        a, b = g[lo:hi], g_ref[lo:hi].astype(np.float32)
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
        assert err < 2e-2, f"{name}: relative error {err:.3g}"
    assert np.all(g[mlp.O_W1:mlp.O_B1].reshape(mlp.H, mlp.IN_PAD)[:, mlp.IN:] == 0)
    net.close()


def test_gradients_with_two_rows_per_loss_warp(Net):
    """Batches larger than one wave of loss warps put two rows in a warp (one
    per half, each lane's move from the move masks).  1024 positions repeated
    16 times (16384 rows: two per warp) give the gradient of the 1024 alone
    (one per warp): the mean over rows is the same and 16 is a power of two,
    so every row's BF16 gradient scales exactly; what remains is the order of
    the FP32 sums.  A row whose moves were mapped wrongly would be off by
    about 1/1024 of the affected entries."""
    net = Net(0, max_batch=16384, seed=1)
    net.set_params(_params(7))
    boards, _, _, counts = _positions(61, 768)
    # random placements with kings: longer move lists and continuing captures
    extra = random_boards(np.random.default_rng(8), 4000)
    extra[:, 3] &= np.uint32(1)  # no draw counter
    _, c = L.genmoves(extra)
    extra = extra[(c > 0) & (c <= mlp.MAXM)][:256]
    boards = np.concatenate([boards, extra])
    _, counts = L.genmoves(boards)

    def continues(x):  # some legal move takes two or more pieces
        side = int(x[3]) & 1
        opp = int(x[1 - side])
        return any(bin(opp & ~int(c[1 - side])).count("1") >= 2 for c in L.children(x)[0])

    whole = np.array([continues(x) for x in boards]) | (counts > 16)  # rows a warp takes on all 32 lanes
    assert len(boards) == 1024 and 50 < whole.sum() < 512
    rng = np.random.default_rng(7)
    z = rng.uniform(-1, 1, 1024).astype(np.float32)
    q = rng.uniform(-1, 1, (1024, mlp.MAXM)).astype(np.float32)
    g1, l1 = net.gradients(boards, z, q)
    g16, l16 = net.gradients(np.tile(boards, (16, 1)), np.tile(z, 16), np.tile(q, (16, 1)))
    for name, (lo, hi) in _segments().items():
        a, b = g1[lo:hi], g16[lo:hi]
        assert np.abs(a - b).max() <= 1e-4 * max(np.abs(a).max(), 1e-12), name
    assert np.allclose(l1, l16, rtol=1e-5)
    net.close()


def test_forward_is_the_same_for_both_tile_widths_of_the_second_layer(Net):
    """A batch whose row blocks fill the SMs runs the second layer in
    256-column tiles, a smaller one in 128-column tiles; values (whose
    dot product is summed per 64 columns either way) and logits of the same
    boards are bit-identical."""
    net = Net(0, max_batch=20480, seed=1)
    net.set_params(_params(5))
    boards = L.random_positions(17, 20000, 0, 60)
    v_big, l_big = net.forward(boards)
    v_small, l_small = net.forward(boards[:300])
    assert np.array_equal(v_big[:300], v_small) and np.array_equal(l_big[:300], l_small)
    net.close()


def _device_rows(boards, z, q):
    import torch
    b = torch.from_numpy(np.ascontiguousarray(boards, np.uint32).view(np.int32)).cuda()
    zt = torch.from_numpy(np.ascontiguousarray(z, np.float32)).cuda()
    qt = torch.from_numpy(np.ascontiguousarray(q, np.float32)).cuda()
    return b, zt, qt


def test_train_step_is_adam_on_the_gradient(Net):
    net = Net(0, max_batch=256, seed=1)
    p = _params(9)
    net.set_params(p)
    boards, _, _, _ = _positions(21, 200)
    rng = np.random.default_rng(1)
    z = rng.uniform(-1, 1, 200).astype(np.float32)
    q = rng.uniform(-1, 1, (200, mlp.MAXM)).astype(np.float32)
    g, _ = net.gradients(boards, z, q)
    b, zt, qt = _device_rows(boards, z, q)
    loss = net.train_step(b.data_ptr(), zt.data_ptr(), qt.data_ptr(), 200, lr=1e-3, want_loss=True)
    assert loss is not None and np.all(np.isfinite(loss))
    want, _, _ = mlp.adam(p.astype(np.float64), 0.0, 0.0, g.astype(np.float64), step=1, lr=1e-3)
    assert np.abs(net.params() - want).max() < 1e-6
    net.close()


def test_graph_replays_take_each_steps_rows_and_learning_rate(Net):
    """The training step is one CUDA graph replayed step after step; a replay
    on other rows (other device addresses) with another learning rate is Adam
    step 2 on those rows' gradient at that rate, from step 1's parameters and
    moments."""
    net, grad = Net(0, max_batch=256, seed=1), Net(0, max_batch=256, seed=2)
    p0 = _params(12)
    net.set_params(p0)
    rng = np.random.default_rng(4)
    rows = []
    for seed in (51, 52):
        boards, _, _, _ = _positions(seed, 192)
        rows.append((boards, rng.uniform(-1, 1, 192).astype(np.float32),
                     rng.uniform(-1, 1, (192, mlp.MAXM)).astype(np.float32)))
    dev = [_device_rows(*r) for r in rows]
    assert dev[0][0].data_ptr() != dev[1][0].data_ptr()
    g1, _ = net.gradients(*rows[0])
    net.train_step(*(t.data_ptr() for t in dev[0]), 192, lr=1e-3)
    p1 = net.params()
    want1, m1, v1 = mlp.adam(p0.astype(np.float64), 0.0, 0.0, g1.astype(np.float64), step=1, lr=1e-3)
    assert np.abs(p1 - want1).max() < 1e-6
    grad.set_params(p1)
    g2, _ = grad.gradients(*rows[1])
    net.train_step(*(t.data_ptr() for t in dev[1]), 192, lr=3e-4)
    want2, _, _ = mlp.adam(p1.astype(np.float64), m1, v1, g2.astype(np.float64), step=2, lr=3e-4)
    assert np.abs(net.params() - want2).max() < 1e-6
    with pytest.raises(GpuAIError):  # rows not 16-byte aligned
        net.train_step(dev[0][0].data_ptr() + 4, dev[0][1].data_ptr(), dev[0][2].data_ptr(), 100, lr=1e-3)
    net.close()
    grad.close()


def test_training_is_reproducible_and_resumable(Net, tmp_path):
    boards, _, _, _ = _positions(31, 384)
    rng = np.random.default_rng(2)
    z = rng.uniform(-1, 1, 384).astype(np.float32)
    q = rng.uniform(-1, 1, (384, mlp.MAXM)).astype(np.float32)
    b, zt, qt = _device_rows(boards, z, q)
    a, c = Net(0, max_batch=384, seed=11), Net(0, max_batch=384, seed=11)
    for _ in range(3):
        a.train_step(b.data_ptr(), zt.data_ptr(), qt.data_ptr(), 384, lr=1e-3)
        c.train_step(b.data_ptr(), zt.data_ptr(), qt.data_ptr(), 384, lr=1e-3)
    assert np.array_equal(a.params(), c.params())
    path = os.path.join(tmp_path, "net.bin")
    a.save(path)
    d = Net(0, max_batch=384, seed=99)
    d.load(path)
    assert np.array_equal(d.params(), a.params())
    a.train_step(b.data_ptr(), zt.data_ptr(), qt.data_ptr(), 384, lr=1e-3)
    d.train_step(b.data_ptr(), zt.data_ptr(), qt.data_ptr(), 384, lr=1e-3)
    assert np.array_equal(d.params(), a.params())  # Adam state and step count travel with the file
    for x in (a, c, d):
        x.close()


def test_training_fits_a_batch(Net):
    net = Net(0, max_batch=512, seed=3)
    boards, _, _, counts = _positions(41, 512)
    rng = np.random.default_rng(3)
    z = np.tanh(rng.normal(0, 1, 512)).astype(np.float32)
    q = rng.uniform(-1, 1, (512, mlp.MAXM)).astype(np.float32)
    b, zt, qt = _device_rows(boards, z, q)
    first = net.train_step(b.data_ptr(), zt.data_ptr(), qt.data_ptr(), 512, lr=2e-3, want_loss=True)
    for _ in range(300):
        net.train_step(b.data_ptr(), zt.data_ptr(), qt.data_ptr(), 512, lr=2e-3)
    last = net.train_step(b.data_ptr(), zt.data_ptr(), qt.data_ptr(), 512, lr=2e-3, want_loss=True)
    assert last[1] < 0.25 * first[1]   # value loss
    assert last[0] < 0.8 * first[0]    # policy cross entropy
    net.close()


def test_labels_are_child_playouts(engine):
    import torch
    n, P, seed, base = 40, 96, 5, 1000
    boards = L.random_positions(8, n, 0, 60)
    boards[0] = [0x1, 0x0, 0x0, 0x1]  # PLAYER_2 to move with no pieces: game over
    d = torch.from_numpy(boards.view(np.int32)).cuda()
    v = torch.zeros(n, dtype=torch.float32, device="cuda")
    qd = torch.zeros(n * 32, dtype=torch.float32, device="cuda")
    k = torch.zeros(n, dtype=torch.uint8, device="cuda")
    engine.label_positions(d.data_ptr(), n, P, seed, base, 0, v.data_ptr(), qd.data_ptr(), k.data_ptr(),
                           torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    v, qd, k = v.cpu().numpy(), qd.cpu().numpy().reshape(n, 32), k.cpu().numpy()
    moves, counts = engine.genmoves(boards)
    assert k[0] == 0 and v[0] == 0 and np.all(qd[0] == 0)
    for i in range(1, n):
        kk = int(counts[i])
        live = 0 < kk <= 32 and ((boards[i, 3] >> 8) & 0xFF) < 50
        assert k[i] == (kk if live else 0)
        if k[i] == 0:
            continue
        children = []
        for m in range(kk):
            b = boards[i:i + 1].copy()
            assert L.oracle().or_apply_packed_b16(L._ptr(b, L._u32p),
                                                  L._ptr(np.ascontiguousarray(moves[i, m]), L._u8p)) == 0
            children.append(b[0])
        reps = np.array([P // kk + (1 if m < P % kk else 0) for m in range(kk)], np.uint32)
        out = engine.playouts(np.array(children), reps, seed=seed, stream_base=base + i * P)
        sign = -1.0 if boards[i, 3] & 1 else 1.0
        off = np.concatenate([[0], np.cumsum(reps)]).astype(np.int64)
        for m in range(kk):
            s = int(out[off[m]:off[m + 1]].astype(np.int64).sum())
            assert qd[i, m] == np.float32(sign * s) / np.float32(reps[m])
        assert v[i] == np.float32(sign * int(out.astype(np.int64).sum())) / np.float32(P)
        assert np.all(qd[i, kk:] == 0)


def _learned_searches(Net, boards, bases, budget, seed=4):
    from gpu_ai_gb300 import Searches
    net = Net(0, max_batch=256, seed=seed)
    cap = 30_000
    s = Searches(len(boards), cap * len(boards), max_leaves_per_step=32, playouts_per_leaf=2, seed=7)
    s.set_net(net, value_weight=0.5, c_puct=1.5)
    slots = [s.add(b, budget, cap, base) for b, base in zip(boards, bases)]
    while True:
        s.step(4, 32)
        done, bud = s.poll()
        if all(done[sl] >= bud[sl] for sl in slots):
            break
    res = [s.children(sl) for sl in slots]
    s.close()
    net.close()
    return res


def test_learned_search_same_alone_and_in_mix(Net):
    boards, _, _, _ = _positions(51, 6, max_plies=30)
    bases = [1_000_000 * i for i in range(6)]
    mix = _learned_searches(Net, boards, bases, 4096)
    alone = _learned_searches(Net, boards[2:3], bases[2:3], 4096)
    for key in ("visits", "score2", "moves"):
        assert np.array_equal(alone[0][key], mix[2][key])
    for r, b in zip(mix, boards):
        assert r["visits"].sum() > 0
        _, counts = L.genmoves(b[None])
        assert len(r["visits"]) == counts[0]


def test_set_net_rejected_while_searches_run(Net):
    from gpu_ai_gb300 import GpuAIError, Searches
    net = Net(0, max_batch=128, seed=1)
    s = Searches(4, 10_000, 16, 1)
    s.add(L.start_board()[0], 100, 1000, 0)
    with pytest.raises(GpuAIError):
        s.set_net(net)
    s.close()
    net.close()


def test_bounded_wait_runs_out_cleanly(Net):
    """A GEMM launched with no TMA load and a 2 ms wait limit: its MMA warp's
    barrier wait runs out, the kernel reports it in the status word, frees its
    tensor memory and returns; the network keeps working afterwards (a kernel
    that kept its TMEM would leave later allocations waiting)."""
    net = Net(0, max_batch=256, seed=1)
    p = _params(4)
    net.set_params(p)
    for _ in range(2):
        st = net.wait_selftest(2000)
        assert st & 16
    boards, _, _, _ = _positions(7, 200)
    value, logits = net.forward(boards)
    ref = mlp.forward(p, boards, emulate=True)
    assert np.abs(logits - ref["logits"]).max() <= 1e-2 * np.abs(ref["logits"]).max()
    assert net.wait_selftest(1000) & 16
    net.close()

"""The N>1 path of bench.py on CPU: two gloo ranks (replicas, no collective on
the data path): barrier, max-over-ranks timing, disjoint random-stream
ranges, and the reference arm printing one line from rank 0 only."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), BENCH_GLOO="1")
    sys.path.insert(0, ROOT)
    import bench
    r, w, _ = bench.dist_setup(world)
    bench.barrier(w)
    m = bench.max_over_ranks(float(r) + 1.5, w)
    q.put((r, w, m, bench.rank_stream_base(r)))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks_barrier_and_max():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, *_ in res] == [0, 1]
    assert all(w == 2 and m == 2.5 for _, w, m, _ in res)
    bases = [b for *_, b in res]
    steps_playouts = 100_000 * 64 * 4096  # far more than any bench run (2,003 steps by default)
    assert bases[1] - bases[0] > steps_playouts


def test_reference_arm_under_torchrun_prints_once():
    env = dict(os.environ, BENCH_GLOO="1", OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0

#!/usr/bin/env python
"""Checkers Monte Carlo playout throughput on GB300.

Workload (one step): 64 seeded positions (seed 2016; each plays U{0..30}
uniformly random legal plies from the start) x 4,096 uniformly random
playouts = 262,144 playouts, int8 outcomes.  Each step uses fresh random
streams (stream_base advances), so no step repeats work.

  value  playouts/s of the playout kernel on device-resident inputs, summed
         CUDA-event time of the K timed launches (L2 flushed between steps)
  e2e    the same metric through the public C ABI call gpuai_playouts() on
         host buffers: H2D of boards + offsets and D2H of outcomes every step
  roofline  integer-issue roofline of the playout kernel: plies/s x OPS_PER_PLY
         lane operations against SMs x 128 lanes x the maximum SM clock
  clocks nvidia-smi samples (every 50 ms) that arrived during the timed
         loop of `value`: median SM clock and active throttle reasons
  cpu_baseline  the reference's HostPlayoutDriver (built from its sources
         where present, else the oracle's restatement of it) on the host's
         cores, on a bounded sample of the same positions

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "checkers playouts/sec on 1 GB300 vs host CPU; win rate vs plain at equal ms/move"
UNIT = "playouts/s"
N_POS, REPS, POS_SEED, MAX_PLIES = 64, 4096, 2016, 30
TOTAL = N_POS * REPS
REPS_BENCH = REPS
WORKLOAD = {
    "workload": "uniform random playouts: 64 seeded positions (0-30 random plies, seed 2016) x 4096",
    "positions": N_POS,
    "playouts_per_position": REPS,
    "playouts_per_step": TOTAL,
    "policy": "random",
    "l2": "flushed between steps (256 MiB write, outside the timed events)",
}
# Lane-instructions per ply of the playout kernel, frozen from the first
# correct kernel's ncu capture (smsp__thread_inst_executed.sum / plies);
# the algorithmic work unit of the integer-issue roofline.
OPS_PER_PLY = 260.0
# Lane instructions per ply of the other two policies' kernels (playout_kernel<1,
# 256>, playout_kernel<2, 256>), frozen from one ncu capture of the benchmark
# batch (smsp__thread_inst_executed_pred_on.sum / plies): 12.25e9 / 12.65e6 and
# 6.66e9 / 15.72e6.
OPS_PER_PLY_POLICY = {"ref_heuristic": 969.0, "eps_greedy": 424.0}
# DRAM bytes per launch of the playout kernel from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum).
TRAFFIC_BYTES = 47104  # one ncu capture of the benchmark launch: 46.3 KB read, 0.8 KB written


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"sm_max_mhz": 2070.0, "hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms; stop(t0, t1)
    keeps the samples that arrived inside the timed window [t0, t1]
    (perf_counter seconds)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, bus_id=None):
        self.rows = []
        self.proc = None
        cmd = ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits", "-lms", "50"]
        if bus_id:
            cmd += ["-i", bus_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append((time.perf_counter(), parts))

    def wait_first(self, timeout=5.0):
        """Block until nvidia-smi has printed its first sample (or timeout)."""
        end = time.perf_counter() + timeout
        while self.proc and not self.rows and time.perf_counter() < end:
            time.sleep(0.01)

    def stop(self, t0=None, t1=None):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        return summarize_clocks(self.rows, t0, t1)


def summarize_clocks(rows, t0=None, t1=None):
    """(arrival time, nvidia-smi fields) rows -> the `clocks` object: median SM
    clock, maximum SM clock and throttle reasons of the rows inside [t0, t1]."""
    rows = [r for t, r in rows if t0 is None or t0 <= t <= t1]
    sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
    mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
    reasons = set()
    for r in rows:
        for name, v in zip(ClockSampler.NAMES, r[5:9]):
            if v.lower() == "active":
                reasons.add(name)
    return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
            "reasons": sorted(reasons), "samples": len(rows), "window_s": (t1 - t0) if t0 is not None else None}


def cpu_reference_runner():
    """The reference's host playout path on this machine's cores.

    Returns (run(states) -> outcomes, kind, threads).  kind "reference" is the
    reference's own HostPlayoutDriver compiled from its sources (only where
    those sources were present at build time and the objects match this
    machine); otherwise "port", the oracle's line-by-line restatement of it.
    """
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as L  # the CPU baseline is the one product-external use of the oracle

    threads = os.cpu_count() or 1
    try:
        if os.path.exists(L.REF_SO):
            lib = L.ref()
            if lib is not None:
                return (lambda st: L.host_playouts_ref(st, srand_seed=1)), "reference", threads
    except OSError:
        pass
    L.oracle()
    return (lambda st: L.host_playouts_port(st, nthreads=threads, srand_seed=1)), "port", threads


def time_cpu_baseline(positions, min_seconds=10.0, max_seconds=30.0):
    run, kind, threads = cpu_reference_runner()
    chunk = np.repeat(positions, 64, axis=0)  # 64 playouts per position per chunk
    done, t0 = 0, time.perf_counter()
    while True:
        run(chunk)
        done += len(chunk)
        el = time.perf_counter() - t0
        if el >= min_seconds or el >= max_seconds:
            break
    return {"value": done / el, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": f"{done} playouts ({done // len(positions)} per position) of the same 64 positions, "
                      f"{el:.1f} s, HostPlayoutDriver (src/playout.cpp:17-32)"}


def time_cpu_strong(positions, min_seconds=5.0):
    """The stronger CPU figure: the project's bitboard ply with per-playout
    Philox streams (oracle/cpu_playouts.cpp) on every host core, on the same
    positions; its outcomes equal the GPU kernel's."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as L
    threads = os.cpu_count() or 1
    reps = np.full(len(positions), 256, dtype=np.uint32)
    done, plies, t0, k = 0, 0, time.perf_counter(), 0
    while True:
        _, pl = L.cpu_playouts(positions, reps, 0xC0DE, k * int(reps.sum()), threads)
        done += int(reps.sum())
        plies += pl
        k += 1
        el = time.perf_counter() - t0
        if el >= min_seconds:
            break
    return {"value": done / el, "unit": UNIT, "cores": threads, "kind": "project bitboard restatement",
            "plies_per_s": plies / el,
            "sample": f"{done} playouts of the same 64 positions, {el:.1f} s, the GPU kernel's bitboard ply and "
                      "Philox streams on the host (oracle/cpu_playouts.cpp)"}


def time_cpu_heuristic(positions, min_seconds=5.0):
    """The reference's HostHeuristicPlayoutDriver (src/heuristicPlayout.cpp:12-48,
    OpenMP over the states) on all of this machine's cores: built from the
    reference's sources where they were present at build time, else the
    oracle's restatement of it."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as L
    threads = os.cpu_count() or 1
    run, kind = None, "port"
    try:
        if os.path.exists(L.REF_SO) and L.ref() is not None:
            run, kind = L.host_heuristic_ref, "reference"
    except OSError:
        run = None
    if run is None:
        lib = L.oracle()
        seed = [0]

        def run(st):
            st = np.ascontiguousarray(st, dtype=np.uint32)
            out = np.zeros(st.shape[0], dtype=np.int8)
            seed[0] += 1
            lib.or_host_heuristic_playouts(L._ptr(st, L._u32p), st.shape[0], L._ptr(out, L._i8p), seed[0])
            return out
    chunk = np.repeat(positions, 16, axis=0)
    done, t0 = 0, time.perf_counter()
    while True:
        run(chunk)
        done += len(chunk)
        el = time.perf_counter() - t0
        if el >= min_seconds:
            break
    return {"value": done / el, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": f"{done} playouts of the same 64 positions, {el:.1f} s, HostHeuristicPlayoutDriver "
                      "(src/heuristicPlayout.cpp:12-48)"}


def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if os.environ.get("BENCH_GLOO") is None else "gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_stream_base(rank):
    """First random-stream id of a rank: replicas use disjoint id ranges
    (2^40 playouts per rank) so no two ranks replay the same playouts."""
    return rank << 40


def run_reference(args):
    rank, world, _ = dist_setup(args.gpus)
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as L
    positions = L.random_positions(POS_SEED, N_POS, 0, MAX_PLIES)
    run, kind, threads = cpu_reference_runner()
    per_pos = 256
    states = np.repeat(positions, per_pos, axis=0)
    for _ in range(args.warmup):
        run(states)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        run(states)
    el = time.perf_counter() - t0
    value = args.steps * len(states) / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": dict(WORKLOAD, sample_per_step=f"{len(states)} playouts ({per_pos} per position)"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": f"{per_pos} playouts per position per step, HostPlayoutDriver "
                                   "(src/playout.cpp:17-32)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(line), flush=True)


def workload(reps):
    """The playouts workload with `reps` playouts per position (4,096 is the
    benchmark batch)."""
    w = dict(WORKLOAD, playouts_per_position=reps, playouts_per_step=N_POS * reps)
    if reps != REPS:
        w["workload"] = (f"uniform random playouts: 64 seeded positions (0-30 random plies, seed 2016) x {reps}")
    return w


def run_ours(args):
    REPS, TOTAL = args.playouts_per_position, N_POS * args.playouts_per_position  # noqa: N806
    rank, world, local = dist_setup(args.gpus)
    import torch
    from gpu_ai_gb300 import Engine

    torch.cuda.set_device(local)
    eng = Engine(local)
    layouts = {"thread": 0, "warp": 1, "pooled": 2}
    if args.layout:
        eng.set_layout(0, layouts[args.layout])
    if args.block:
        eng.set_launch(0, args.block, args.blocks_per_sm)
    info = eng.device_info()
    positions = eng.random_positions(POS_SEED, N_POS, 0, MAX_PLIES)
    reps = np.full(N_POS, REPS, dtype=np.uint32)
    d_pos = torch.from_numpy(positions.view(np.int32).copy()).cuda()
    d_out = torch.empty(TOTAL, dtype=torch.int8, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sid = stream.cuda_stream
    base = rank_stream_base(rank)

    def step(k):
        eng.playouts_device(d_pos.data_ptr(), None, N_POS, REPS, TOTAL, 0x5EED, base + k * TOTAL, 0,
                            d_out.data_ptr(), sid)

    bus = None
    try:
        bus = torch.cuda.get_device_properties(local).pci_bus_id if hasattr(
            torch.cuda.get_device_properties(local), "pci_bus_id") else None
    except Exception:
        bus = None
    # clocks are sampled from the warm-up on, through the timed loop, the
    # end-to-end loop and the other policies' legs
    sampler = ClockSampler(bus)
    sampler.wait_first()
    for k in range(args.warmup):
        flush.zero_()
        step(k)
    torch.cuda.synchronize()
    st, _ = eng.status()
    if st:
        raise RuntimeError(f"kernel status {st}")

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    plies = 0
    barrier(world)
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        step(args.warmup + k)
        ev[k][1].record(stream)
        st, pl = eng.status()  # synchronises; outside the event pair
        if st:
            raise RuntimeError(f"kernel status {st}")
        plies += pl
    torch.cuda.synchronize()
    wall1 = time.perf_counter()
    wall = wall1 - wall0
    barrier(world)
    kern_s = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    kern_s_max = max_over_ranks(kern_s, world)
    value = world * args.steps * TOTAL / kern_s_max

    # ---- end to end through the public host-buffer call
    # gpuai_playouts copies [boards | control block] up, the outcomes and the
    # control block down (equal repetitions need no offsets)
    h2d = N_POS * 16 + 16
    d2h = 16 + TOTAL
    out = np.empty(TOTAL, dtype=np.int8)  # the caller's outcome buffer, reused every step
    for k in range(2):
        eng.playouts(positions, reps, seed=0xE2E, stream_base=base + k * TOTAL, out=out)
    barrier(world)
    t0 = time.perf_counter()
    for k in range(args.steps):
        eng.playouts(positions, reps, seed=0xE2E, stream_base=base + (k + 2) * TOTAL, out=out)
    e2e_s = time.perf_counter() - t0
    if rank != 0:
        sampler.stop()
    e2e_s = max_over_ranks(e2e_s, world)
    assert out.shape == (TOTAL,)
    e2e = {"value": world * args.steps * TOTAL / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h}

    if rank != 0:
        return
    peaks, src = measured_peaks()
    sm_mhz = float(peaks.get("sm_max_mhz", 2070.0))
    peak_ops = info["sms"] * 128 * sm_mhz * 1e6  # lanes issued per second: SMs x 4 schedulers x 32 lanes
    clocks = summarize_clocks(sampler.rows, wall0, wall1)  # the timed loop
    plies_s = plies / kern_s
    roof = {"bound": "int_issue", "unit": "Tlane-op/s",
            "peak": peak_ops / 1e12, "peak_source": f"{info['sms']} SMs x 128 lanes x {sm_mhz:.0f} MHz ({src})",
            "ops_per_ply": OPS_PER_PLY, "plies_per_s": plies_s,
            "traffic": TRAFFIC_BYTES if REPS == REPS_BENCH else None}
    if OPS_PER_PLY:
        roof["achieved"] = plies_s * OPS_PER_PLY / 1e12
        roof["frac"] = roof["achieved"] / roof["peak"]
    else:
        roof["achieved"] = None
        roof["frac"] = None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": kern_s / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded positions)",
        "config": dict(workload(REPS), parallelism=f"replicas{world}" if world > 1 else "single"),
        "plies_per_playout": plies / (args.steps * TOTAL),
        "wall_ms_per_step": wall / args.steps * 1e3,
        "gpu_launches": args.steps,
        "e2e": e2e,
        "roofline": roof,
        "clocks": clocks,
        "device": info,
    }
    # the other playout policies on the same batch: device-resident, CUDA events
    pols = {}
    for pol, name in ((1, "ref_heuristic"), (2, "eps_greedy")):
        ts, pl_sum = [], 0
        for k in range(5):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            eng.playouts_device(d_pos.data_ptr(), None, N_POS, REPS, TOTAL, 0x5EED, base + (1000 + k) * TOTAL, pol,
                                d_out.data_ptr(), sid)
            b.record(stream)
            st, pl = eng.status()
            if st:
                raise RuntimeError(f"kernel status {st}")
            if k >= 2:
                ts.append(a.elapsed_time(b) / 1e3)
                pl_sum += pl
        pols[name] = {"playouts_per_s": len(ts) * TOTAL / sum(ts), "ms_per_step": sum(ts) / len(ts) * 1e3,
                      "plies_per_playout": pl_sum / (len(ts) * TOTAL)}
        pl_s = pl_sum / sum(ts)
        ach = pl_s * OPS_PER_PLY_POLICY[name] / 1e12
        pols[name]["roofline"] = {"bound": "int_issue", "unit": "Tlane-op/s", "ops_per_ply": OPS_PER_PLY_POLICY[name],
                                  "plies_per_s": pl_s, "achieved": ach, "peak": peak_ops / 1e12,
                                  "frac": ach / (peak_ops / 1e12)}
    line["policies"] = pols
    # a short timed loop (20 steps are 8 ms) can fall between two 50 ms
    # samples: then the same launches run on, untimed, for 0.3 s after the
    # policy legs, and the clocks of that stretch are reported
    if (clocks.get("samples") or 0) < 3:
        soak0 = time.perf_counter()
        k = 0
        while time.perf_counter() - soak0 < 0.3:
            for _ in range(50):
                step(args.warmup + args.steps + 4000 + k)
                k += 1
            torch.cuda.synchronize()
        soak1 = time.perf_counter()
        clocks = dict(sampler.stop(soak0, soak1),
                      window=f"the benchmark launch repeated {k} times for {soak1 - soak0:.2f} s after the timed "
                             "loop (the timed loop spans fewer than 3 samples)")
    else:
        sampler.stop()
        clocks["window"] = "timed loop"
    line["clocks"] = clocks
    if roof.get("frac") and clocks.get("sm_mhz"):
        roof["frac_at_sampled_clock"] = roof["frac"] * sm_mhz / clocks["sm_mhz"]
    if world == 1 and not args.no_cpu:
        line["cpu_baseline"] = time_cpu_baseline(positions)
        line["cpu_baseline_strong"] = time_cpu_strong(positions)
        pols["ref_heuristic"]["cpu_baseline"] = time_cpu_heuristic(positions)
    print(json.dumps(line), flush=True)


def run_searches(args):
    """Batched searches with device-resident trees: 2,048 games at U{0..60}
    random plies, playout budgets lognormal clipped to [1K, 256K], all advanced
    together; total playouts/s with graph-replayed steps and with eager
    launches.  Leaves per search start at --leaves and double (up to
    --leaves-max) whenever the searches still running would put fewer
    playouts into a step than the first step had: as the small budgets finish,
    the large searches take more leaves per step instead of running
    latency-bound steps of a few thousand playouts."""
    import torch
    from gpu_ai_gb300 import Engine, Searches

    n_games, q, ppl, qmax = args.games, args.leaves, args.playouts_per_leaf, max(args.leaves, args.leaves_max)
    eng = Engine(0)
    roots = eng.random_positions(4242, n_games, 0, 60)
    rng = np.random.default_rng(4242)
    budgets = np.clip(np.exp(rng.normal(np.log(16384), 1.2, n_games)), 1024, 262144).astype(np.int64)
    budgets = (budgets + ppl - 1) // ppl * ppl
    caps = np.minimum(budgets, 131072).astype(np.int64) * 2
    target = n_games * q * ppl  # playouts of the first step
    result = {}
    for mode in ("graph", "eager"):
        s = Searches(n_games, int(caps.sum()) + 1024, qmax, playouts_per_leaf=ppl)
        for i in range(n_games):
            s.add(roots[i], int(budgets[i]), int(caps[i]), i << 40)
        torch.cuda.synchronize()
        steps, schedule = 0, {}
        t0 = time.perf_counter()
        while True:
            done, budget = s.poll()
            active = int((done < budget).sum())
            if active == 0:
                break
            qq = q
            while qq < qmax and active * qq * ppl < target:
                qq *= 2
            schedule[qq] = schedule.get(qq, 0) + 8
            s.step(8, qq, mode == "graph")
            steps += 8
        el = time.perf_counter() - t0
        total = int(done.sum())
        result[mode] = {"seconds": el, "steps": steps, "playouts": total, "playouts_per_s": total / el,
                        "steps_by_leaves_per_search": {str(k): v for k, v in sorted(schedule.items())}}
        s.close()
    g, e = result["graph"], result["eager"]
    line = {
        "metric": "checkers playouts/sec, batched searches with device-resident trees", "value": g["playouts_per_s"],
        "unit": UNIT, "n_gpus": 1, "higher_is_better": True, "dtype": "u32", "data": "synthetic (seeded positions)",
        "config": {"workload": f"{n_games} games at 0-60 random plies, budgets lognormal in [1K, 256K]",
                   "leaves_per_search_per_step": f"{q}, doubling up to {qmax} as searches finish",
                   "playouts_per_leaf": ppl,
                   "total_budget": int(budgets.sum())},
        "graph": g, "eager": e,
        "launch_overhead_us_per_step": (e["seconds"] - g["seconds"]) / max(1, g["steps"]) * 1e6,
    }
    print(json.dumps(line), flush=True)


def run_mcts(args):
    """Host UCT searches with GPU leaf batches (the reference's MCTSPlayer
    worker loop, src/player.cpp:134-150): 32 seeded positions at 10-40 random
    plies, --ms-per-position of search each, leaf batches of 16K-64K slots x
    --playouts-per-leaf playouts; plain random playouts against the
    eps-greedy and the reference-heuristic playout policies.  Up to 16
    searches run at once, one host thread, playout driver and CUDA stream
    each.  Runs gpu_ai_gb300/lib/run_ai -m mcts_bench (the host tree is C++)."""
    exe = os.path.join(ROOT, "gpu_ai_gb300", "lib", "run_ai")
    if not os.path.exists(exe):
        raise RuntimeError(f"{exe} is missing: build it with gpu_ai_gb300.build.build()")
    cmd = [exe, "-m", "mcts_bench", "-n", "32", "--seed", "2016", "--ms-per-move", str(args.ms_per_position),
           "--leaves-min", "16384", "--leaves-max", "65536", "--playouts-per-leaf", str(args.playouts_per_leaf)]
    res = {}
    for name, drv in (("plain", "device"), ("eps_greedy", "device_eps_greedy"), ("ref_heuristic", "device_heuristic")):
        r = subprocess.run(cmd + ["-1", drv], capture_output=True, text=True, check=True)
        line = [x for x in r.stdout.splitlines() if x.startswith("MCTS_BENCH ")][-1]
        res[name] = json.loads(line[len("MCTS_BENCH "):])
    p = res["plain"]
    print(json.dumps({
        "metric": "checkers playouts/sec, host UCT searches with GPU leaf batches", "value": p["playouts_per_s"],
        "unit": UNIT, "higher_is_better": True, "n_gpus": 1, "dtype": "u32", "data": "synthetic (seeded positions)",
        "config": {"workload": f"32 positions (10-40 random plies, seed 2016), {args.ms_per_position} ms of host UCT "
                               f"search each, leaf batches of 16K-64K slots x {args.playouts_per_leaf} playouts, "
                               f"up to 16 searches at once",
                   "tree": "host C++ GameTree, UCB1 c=sqrt(2)"},
        "threads": p["threads"], "driver_share_of_search_time": p["driver_share"],
        "plain": p, "eps_greedy": res["eps_greedy"], "ref_heuristic": res["ref_heuristic"],
    }), flush=True)


def quick_net(args):
    """The network file given with --net, or one trained here on 1M self-play
    positions with 1,024-playout labels (a few seconds)."""
    from gpu_ai_gb300 import Engine, Net
    from gpu_ai_gb300 import learn
    net = Net(0, max_batch=8192, seed=1)
    if args.net:
        net.load(args.net)
        return net
    data = learn.make_dataset(Engine(0), 1_000_000, 1024, seed=1)
    learn.train(net, data, epochs=3, batch=8192, lr=1e-3)
    return net


def run_serve(args):
    """Serving loop: Poisson arrivals of search requests on 10K seeded games
    (0-60 random plies), time budgets U(10, 200) ms, continuous batching;
    random playouts, reference-heuristic playouts and learned searches
    (network leaf values and priors, 2 random playouts per leaf) side by side."""
    import torch
    from gpu_ai_gb300.serve import simulate
    from gpu_ai_gb300 import POLICY_RANDOM, POLICY_REF_HEURISTIC
    mem = torch.cuda.mem_get_info  # (free, total) of the whole device: this process's peak in use
    res = {}
    q = args.serve_leaves
    for name, pol in (("random", POLICY_RANDOM), ("ref_heuristic", POLICY_REF_HEURISTIC)):
        res[name] = simulate(rate=args.rate, n_requests=args.requests, n_games=10000, budget_ms=(10.0, 200.0),
                             policy=pol, leaves_per_search=q, playouts_per_leaf=args.playouts_per_leaf,
                             device_memory=mem)
    net = quick_net(args)
    res["learned"] = simulate(rate=args.rate, n_requests=args.requests, n_games=10000, budget_ms=(10.0, 200.0),
                              policy=POLICY_RANDOM, leaves_per_search=q, playouts_per_leaf=2, net=net,
                              device_memory=mem)
    res["learned"]["network"] = args.net or "trained here: 1M positions x 1024 playouts, 3 epochs"
    res["learned_proposal"] = simulate(rate=args.rate, n_requests=args.requests, n_games=10000,
                                       budget_ms=(10.0, 200.0), policy=POLICY_RANDOM, leaves_per_search=q,
                                       playouts_per_leaf=2, net=net, guided=args.guided,
                                       temperature=args.temperature, device_memory=mem)
    res["learned_proposal"]["guided_plies"] = args.guided
    line = {"metric": "serving: search requests with continuous batching", "unit": "ms",
            "value": res["random"]["latency_ms_p99"], "higher_is_better": False, "n_gpus": 1,
            "data": "synthetic (seeded games, Poisson arrivals)",
            "config": {"workload": f"{args.requests} requests at {args.rate} req/s, budgets U(10,200) ms",
                       "leaves_per_search_per_step": q, "playouts_per_leaf": args.playouts_per_leaf},
            "random": res["random"], "ref_heuristic": res["ref_heuristic"], "learned": res["learned"],
            "learned_proposal": res["learned_proposal"]}
    print(json.dumps(line), flush=True)


# FLOPs per position of one training step (forward + backward GEMMs, padded
# shapes): forward 2*(192*256 + 256*256 + 256*1024), backward dH2, dH1 and the
# three weight gradients.
TRAIN_FLOPS_PER_POSITION = 2 * (192 * 256 + 256 * 256 + 256 * 1024) + 2 * (1024 * 256 + 256 * 256) + \
    2 * (1024 * 256 + 256 * 256 + 256 * 192)


def _train_rows(n, seed=3):
    """n seeded positions (0-60 random plies, 1-32 legal moves) with random
    value and move-value targets, as device tensors."""
    import torch
    from gpu_ai_gb300 import Engine
    eng = Engine(0)
    pos = eng.random_positions(seed, 3 * n, 0, 60)
    _, counts = eng.genmoves(pos)
    pos = pos[(counts > 0) & (counts <= 32)][:n]
    rng = np.random.default_rng(seed)
    b = torch.from_numpy(np.ascontiguousarray(pos).view(np.int32)).cuda()
    z = torch.from_numpy(rng.uniform(-1, 1, n).astype(np.float32)).cuda()
    q = torch.from_numpy(rng.uniform(-1, 1, (n, 32)).astype(np.float32)).cuda()
    return b, z, q


def run_train(args):
    """Network training steps at batch 8192 (features, 8 tcgen05 GEMMs, loss,
    bias sums, Adam): positions/s and tensor TFLOP/s against the measured BF16
    peak.  Host-timed over K steps on the network's stream (synchronised on
    both sides); inputs stay resident."""
    from gpu_ai_gb300 import Net
    peaks, peak_kind = measured_peaks()
    n = args.train_batch
    b, z, q = _train_rows(n)
    net = Net(0, max_batch=n, seed=1)
    for _ in range(args.warmup):
        net.train_step(b.data_ptr(), z.data_ptr(), q.data_ptr(), n, 1e-4)
    net.params()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        net.train_step(b.data_ptr(), z.data_ptr(), q.data_ptr(), n, 1e-4)
    net.params()
    el = time.perf_counter() - t0
    step_s = el / max(1, args.steps)
    tflops = TRAIN_FLOPS_PER_POSITION * n / step_s / 1e12
    print(json.dumps({
        "metric": "policy/value network training throughput", "value": n / step_s, "unit": "positions/s",
        "higher_is_better": True, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": step_s * 1e3, "dtype": "bf16 (fp32 accumulation)",
        "data": "synthetic (seeded positions, random targets)",
        "config": {"workload": f"Adam steps on {n} positions, 129-256-256-(1024+1)", "batch": n},
        "roofline": {"bound": "tensor", "achieved": tflops, "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                     "frac": tflops / peaks["bf16_tflops"], "peak_kind": peak_kind,
                     "flop_per_position": TRAIN_FLOPS_PER_POSITION},
    }), flush=True)


def run_learned_search(args):
    """Learned device searches: 400 searches x 64 leaves per step, 2 playouts
    per leaf, network forward on every leaf; K eager steps timed, without and
    with learned-proposal playouts (--guided plies drawn from the network)."""
    from gpu_ai_gb300 import Engine, Net, Searches
    eng = Engine(0)
    net = Net(0, max_batch=256, seed=1)
    roots = eng.random_positions(5, 400, 0, 60)
    res = {}
    for guided in (0, args.guided):
        s = Searches(400, 400 * 20000, 64, 2, seed=1)
        s.set_net(net, 0.5, 1.5)
        if guided:
            s.set_proposal(guided, args.temperature)
        for i, r in enumerate(roots):
            s.add(r, 1 << 40, 20000, i << 40)
        for _ in range(args.warmup):
            s.step(1, 64, False)
        s.poll()
        t0 = time.perf_counter()
        s.step(args.steps, 64, False)
        s.poll()
        el = time.perf_counter() - t0
        s.close()
        res[guided] = {"ms_per_step": el / max(1, args.steps) * 1e3,
                       "leaf_evaluations_per_s": 400 * 64 * args.steps / el,
                       "playouts_per_s": 400 * 64 * 2 * args.steps / el}
    base = res[0]
    print(json.dumps({
        "metric": "learned search steps", "value": base["leaf_evaluations_per_s"], "unit": "leaf evaluations/s",
        "higher_is_better": True, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": base["ms_per_step"], "dtype": "bf16 network, u32 playouts",
        "data": "synthetic (seeded positions)",
        "config": {"workload": "400 searches x 64 leaves/step, 2 playouts/leaf, lambda 0.5"},
        "with_proposal": dict(res[args.guided], guided_plies=args.guided, temperature=args.temperature)}),
        flush=True)


def run_learned(args):
    """Learned part end to end: self-play positions labelled with GPU playouts,
    training with the library's forward/backward/Adam kernels, value MAE on
    held-out positions, and a learned-vs-plain MCTS match at equal ms/move."""
    from gpu_ai_gb300 import Engine, Net
    from gpu_ai_gb300 import learn
    from gpu_ai_gb300.match import play_configs, play_match
    peaks, peak_kind = measured_peaks()
    eng = Engine(0)
    t0 = time.perf_counter()
    data = learn.make_dataset(eng, args.positions, args.label_playouts, seed=1)
    tr, te = learn.split(data, 50_000)
    net = Net(0, max_batch=8192, seed=1)
    res = learn.train(net, tr, epochs=args.epochs, batch=8192, lr=1e-3, log_every=500)
    # steady-state training step time (tensor-core GEMMs plus the loss / row-sum / Adam kernels)
    import torch
    b, z, qv = tr["boards"][:8192].contiguous(), tr["value"][:8192].contiguous(), tr["q"][:8192].contiguous()
    for _ in range(5):
        net.train_step(b.data_ptr(), z.data_ptr(), qv.data_ptr(), 8192, 0.0)
    net.params()
    k = 50
    ts = time.perf_counter()
    for _ in range(k):
        net.train_step(b.data_ptr(), z.data_ptr(), qv.data_ptr(), 8192, 0.0)
    net.params()
    step_s = (time.perf_counter() - ts) / k
    tflops = TRAIN_FLOPS_PER_POSITION * 8192 / step_s / 1e12
    ev = learn.evaluate(net, eng, te)
    if args.save_net:
        net.save(args.save_net)
    # the learned player with learned-proposal playouts against plain MCTS, the
    # same player without the proposal (priors and leaf values only) against
    # plain MCTS, and the two learned players against each other: the
    # proposal's own gain
    mp = play_match(net, eng, n_games=args.match_games, ms_per_move=args.ms, seed=5, leaves=64, plain_ppl=8,
                    learned_ppl=2, value_weight=0.5, c_puct=1.5, guided=args.guided, temperature=args.temperature)
    m = play_match(net, eng, n_games=args.match_games, ms_per_move=args.ms, seed=5, leaves=64, plain_ppl=8,
                   learned_ppl=2, value_weight=0.5, c_puct=1.5)
    with_p = {"net": net, "ppl": 2, "value_weight": 0.5, "c_puct": 1.5, "guided": args.guided,
              "temperature": args.temperature}
    without_p = {"net": net, "ppl": 2, "value_weight": 0.5, "c_puct": 1.5}
    head = play_configs(eng, with_p, without_p, n_games=args.match_games, ms_per_move=args.ms, seed=6, leaves=64)
    line = {
        "metric": "learned-proposal MCTS score vs plain GPU MCTS at equal ms/move",
        "value": mp["learned_score"], "unit": "score (win 1, draw 0.5)", "higher_is_better": True, "n_gpus": 1,
        "dtype": "bf16 (fp32 accumulation)", "data": "synthetic (GPU self-play positions, GPU playout labels)",
        "config": {"workload": f"{args.positions} self-play positions x {args.label_playouts} playouts, "
                               f"{args.epochs} epochs, {args.match_games} games at {args.ms} ms/move, "
                               f"{args.guided} guided plies at temperature {args.temperature}",
                   "network": "129-256-256-(1024 logits + tanh value)"},
        "ci95_wilson": mp["ci95_wilson"], "ci95_normal": mp["ci95_normal"], "match": mp,
        "priors_and_value_only_vs_plain": m,
        "proposal_vs_no_proposal": head,
        "labels": {"positions_kept": int(data["boards"].shape[0]), "seconds": data["label_seconds"],
                   "playouts_per_s": data["playouts"] / data["label_seconds"]},
        "training": {"steps": res["steps"], "batch": res["batch"], "seconds": res["train_seconds"],
                     "positions_per_s": res["positions_per_s"], "loss_first": res["history"][0],
                     "loss_last": res["history"][-1], "step_ms": step_s * 1e3,
                     "tensor_tflops": tflops, "tensor_frac_of_bf16_peak": tflops / peaks["bf16_tflops"],
                     "peak": f"{peaks['bf16_tflops']} TFLOP/s bf16 ({peak_kind})"},
        "eval": ev, "seconds": time.perf_counter() - t0,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 2000 for the playouts workload, so that the timed region spans "
                         "about a second of clock samples; 20 for the reference arm and the other workloads)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--playouts-per-position", type=int, default=REPS,
                    help="playouts workload: playouts per position (4,096 is the benchmark batch)")
    ap.add_argument("--block", type=int, default=0, help="threads per block of the playout kernel (0: default)")
    ap.add_argument("--blocks-per-sm", type=int, default=0, help="resident blocks per SM (0: as many as fit)")
    ap.add_argument("--layout", choices=["", "thread", "warp", "pooled"], default="",
                    help="playout kernel layout of the uniform random policy (default: the library's)")
    ap.add_argument("--workload", choices=["playouts", "mcts", "searches", "serve", "learned", "train",
                                           "learned-search"],
                    default="playouts")
    ap.add_argument("--net", default="", help="serve workload: network file for the learned leg")
    ap.add_argument("--positions", type=int, default=10_000_000, help="learned workload: self-play positions")
    ap.add_argument("--label-playouts", type=int, default=4096, help="learned workload: playouts per label")
    ap.add_argument("--epochs", type=float, default=3.0, help="learned workload: training epochs")
    ap.add_argument("--match-games", type=int, default=400, help="learned workload: match games")
    ap.add_argument("--ms", type=float, default=100.0, help="learned workload: milliseconds per move")
    ap.add_argument("--guided", type=int, default=2,
                    help="learned workload: plies of every playout drawn from the network's policy")
    ap.add_argument("--temperature", type=float, default=1.0, help="learned workload: proposal temperature")
    ap.add_argument("--save-net", default="", help="learned workload: save the trained network to this file")
    ap.add_argument("--train-batch", type=int, default=8192, help="train workload: positions per Adam step")
    ap.add_argument("--rate", type=float, default=1000.0, help="serve workload: requests per second")
    ap.add_argument("--serve-leaves", type=int, default=512,
                    help="serve workload: leaves per search per step (1..512; every request gets the same)")
    ap.add_argument("--requests", type=int, default=2000, help="serve workload: number of requests")
    ap.add_argument("--games", type=int, default=2048, help="searches workload: number of games")
    ap.add_argument("--leaves", type=int, default=128, help="searches workload: leaves per search per step")
    ap.add_argument("--leaves-max", type=int, default=512,
                    help="searches workload: leaves per search per step once most searches have finished (<= 512)")
    ap.add_argument("--playouts-per-leaf", type=int, default=8, help="searches / mcts workloads: playouts per leaf")
    ap.add_argument("--ms-per-position", type=int, default=1000, help="mcts workload: search time per position")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 2000 if args.impl == "ours" and args.workload == "playouts" else 20
    if args.steps < 1:
        ap.error("--steps must be >= 1")
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "searches":
        run_searches(args)
    elif args.workload == "mcts":
        run_mcts(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "learned":
        run_learned(args)
    elif args.workload == "train":
        run_train(args)
    elif args.workload == "learned-search":
        run_learned_search(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

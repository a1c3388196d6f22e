"""Benchmark: validated edges/s of DiscreteMotionValidator::checkMotion on the planar 10-link
kinematic-chain workload (32 world segments, segment fraction 0.005 of the extent, edges between
valid states of a seeded 1M-state set), on one GB300.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one batch of 100,000 edges checked by the batched form (persistent work-queue kernel,
FP32 bulk with FP64 re-check, autotuned schedule). Twelve distinct batches (192 MB of endpoints,
more than the 129 MB L2) rotate across steps, so no step re-reads L2-resident inputs. `e2e` is the
same metric through the host-memory C-ABI call (gbo_check_motion_host: H2D of both endpoint
arrays, kernel, D2H of results and lastValid fractions inside the timed region). Also reported:
the plain one-launch-per-batch FP64 form on the same batches, state validity of the 1M states,
and nearestK (k=16) over the 1M states.

Under torchrun each rank runs an independent replica on its own GPU ("replicas only": the path
has no exchange step); value = all ranks' edges / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_STATES = 1_000_000
N_EDGES = 100_000
N_BATCHES = 12
KNN_QUERIES = 20_000
METRIC = "validated edges/s (DiscreteMotionValidator, 10-link kinematic chain)"
# algorithmic work of one checked state of the chain predicate: 20 sincos + 50 FMA-chain flops +
# (55 + 352) segment tests x 21 flops, credited per checked state (states the reference's ordered
# DiscreteMotionValidator evaluates)
FLOP_PER_STATE = 50 + (55 + 352) * 21


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="chain", choices=["chain", "arm", "prm", "serve"],
                   help="chain: the headline 10-link chain workload; arm: 7-DoF DH arm, 256k edges of 2..2000 "
                        "steps; prm: PRM roadmap of the DH arm among 16,384 spheres from 2M samples")
    p.add_argument("--profile", default=None, choices=["validity", "motion", "motion_plain", "knn", "peaks", "arm"],
                   help="launch one kernel kind twice on the chain workload (for ncu) and exit")
    return p.parse_args()


def workload(seed=1):
    from ompl_gb300 import workloads as W
    return W.config1(seed=seed, n_states=N_STATES, n_edges=10, n_queries=10)


def make_batches(valid_states, n_batches, seed=7):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_batches):
        i = rng.integers(0, len(valid_states), N_EDGES)
        j = rng.integers(0, len(valid_states), N_EDGES)
        out.append((valid_states[i], valid_states[j]))
    return out


class Clocks:
    """Samples nvidia-smi every 200 ms from before the warm-up to after the timed region; summary()
    keeps the samples taken within 0.25 s of the timed region (the nearest one if the region is
    shorter than the sampling period)."""

    def __init__(self, index=0):
        self.samples = []
        self.proc = None
        self.index = index

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 8:
                self.samples.append((time.perf_counter(), p))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, t0, t1):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        win = [p for t, p in self.samples if t0 - 0.25 <= t <= t1 + 0.25]
        if not win:
            win = [min(self.samples, key=lambda tp: min(abs(tp[0] - t0), abs(tp[0] - t1)))[1]]
        sm = [float(s[1]) for s in win if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in win if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in win for k in range(4) if s[4 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(win)}


def cpu_edges_per_s(port, sd, cd, s1, s2, threads):
    port.set_threads(threads)
    t = time.perf_counter()
    port.check_motion(sd, cd, s1, s2, want_state=False, want_bisect=False)
    return len(s1) / (time.perf_counter() - t)


def bench_config():
    """The workload both arms report (the reference arm times a bounded sample of each step)."""
    return {"workload": "kinematic_chain10: 10 links x 0.1, 32 segments, 1M states, 100k edges/step between "
                        "valid states, segment fraction 0.005, FP32 bulk + FP64 re-check, autotuned persistent "
                        "schedule", "edges_per_step": N_EDGES, "batches_rotated": N_BATCHES,
            "l2": "inputs larger than L2 (12 x 16 MB batches rotate)", "parallelism": "replicas"}


def reference_arm(args, rank, world):
    if rank != 0:
        return
    from oracle.oracle import CheckerDesc, Oracle, SpaceDesc
    port = Oracle.port()
    threads = os.cpu_count() or 1
    port.set_threads(threads)
    w = workload()
    sd = SpaceDesc(w.space_kind, w.dim, link_length=w.link_length, lvs_fraction=w.lvs_fraction)
    cd = CheckerDesc(w.checker_kind, w.obstacles)
    valid = port.is_valid(sd, cd, w.states).astype(bool)
    batches = make_batches(w.states[valid], N_BATCHES)
    sample = 20_000
    for i in range(args.warmup):
        s1, s2 = batches[i % N_BATCHES]
        port.check_motion(sd, cd, s1[:sample], s2[:sample], want_state=False, want_bisect=False)
    t = time.perf_counter()
    for i in range(args.steps):
        s1, s2 = batches[i % N_BATCHES]
        port.check_motion(sd, cd, s1[:sample], s2[:sample], want_state=True, want_bisect=False)
    dt = time.perf_counter() - t
    v = sample * args.steps / dt
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "edges/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {**bench_config(), "reference_sample_edges_per_step": sample},
        "cpu_baseline": {"value": v, "unit": "edges/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} edges per step of each 100k-edge batch, all host threads"},
        "e2e": {"value": v, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def replica_totals(edges_per_step, steps, dev_s, wall_s, world, device):
    """Whole-job figures of `world` replicas (one per GPU, no exchange: every rank checks its own
    batches): the job processed world * edges_per_step * steps edges in the slowest rank's time (max
    over ranks of the device time and of the wall time). Returns (edges/s, device s, wall s)."""
    import torch
    t = torch.tensor([dev_s, wall_s], device=device, dtype=torch.float64)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    dev_s, wall_s = t.tolist()
    return world * edges_per_step * steps / dev_s, dev_s, wall_s


def ours(args, rank, world, local_rank):
    import torch

    from ompl_gb300 import base as B
    from ompl_gb300 import capi
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    w = workload()
    space = B.KinematicChainSpace(w.dim, w.link_length)
    space.setLongestValidSegmentFraction(w.lvs_fraction)
    checker = B.KinematicChainValidityChecker(space, w.obstacles)
    checker.setPrecision("fp32_guarded")
    mv = B.DiscreteMotionValidator(checker)
    stream = torch.cuda.current_stream()

    states_soa = torch.as_tensor(w.states.T.copy(), device=dev)
    # validity of the 1M states (also yields the valid pool the edges are drawn from)
    valid = checker.isValid(states_soa, soa=True)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(5):
        valid = checker.isValid(states_soa, soa=True)
    ev1.record()
    torch.cuda.synchronize()
    states_per_s = 5 * N_STATES / (ev0.elapsed_time(ev1) * 1e-3)
    vmask = valid.cpu().numpy().astype(bool)
    host_batches = make_batches(w.states[vmask], N_BATCHES)
    dev_batches = [(torch.as_tensor(a.T.copy(), device=dev), torch.as_tensor(b.T.copy(), device=dev))
                   for a, b in host_batches]

    def run(i, schedule):
        s1, s2 = dev_batches[i % N_BATCHES]
        return mv.checkMotions(s1, s2, schedule=schedule, soa=True)

    clk = Clocks(local_rank).start()
    for i in range(max(3, args.warmup)):
        run(i, capi.SCHEDULE_AUTO)
    torch.cuda.synchronize()
    # checked states per batch (the reference's ordered DiscreteMotionValidator evaluates first_j
    # states of an invalid motion and max(nd, 1) of a valid one)
    checked = []
    for i in range(N_BATCHES):
        r = run(i, capi.SCHEDULE_AUTO)
        fj, nd = r["first_j"].long(), r["nd"].long()
        checked.append(int(torch.where(fj >= 0, fj, torch.clamp(nd, min=1)).sum().item()))
    torch.cuda.synchronize()

    if world > 1:
        torch.distributed.barrier()
    launches0 = B.launch_count()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(args.steps):
        evs[i][0].record(stream)
        run(i, capi.SCHEDULE_AUTO)
        evs[i][1].record(stream)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    wall = t1 - t0
    time.sleep(0.3)
    clk.stop()
    launches = B.launch_count() - launches0
    step_ms = [a.elapsed_time(b) for a, b in evs]
    stats = checker.stats()  # states evaluated / re-checked in FP64 by the last timed step
    value, dev_s, wall = replica_totals(N_EDGES, args.steps, sum(step_ms) * 1e-3, wall, world, dev)
    mean_ms = statistics.mean(step_ms)
    mean_checked = statistics.mean(checked[i % N_BATCHES] for i in range(args.steps))

    # each persistent schedule on its own (the autotuner picks between them)
    sched_eps = {}
    for name, sch in (("tile", capi.SCHEDULE_TILE), ("warp", capi.SCHEDULE_WARP)):
        run(0, sch)
        torch.cuda.synchronize()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record()
        for i in range(N_BATCHES):
            run(i, sch)
        a1.record()
        torch.cuda.synchronize()
        sched_eps[name] = N_BATCHES * N_EDGES / (a0.elapsed_time(a1) * 1e-3)

    # the same steps replayed from CUDA graphs (one graph per batch, captured after the autotuner ran):
    # the persistent launch and its counter reset are stream work and capture as they are
    graphs = []
    for i in range(N_BATCHES):
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            run(i, capi.SCHEDULE_AUTO)
        graphs.append(g)
    for g in graphs:
        g.replay()
    torch.cuda.synchronize()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record()
    for i in range(args.steps):
        graphs[i % N_BATCHES].replay()
    g1.record()
    torch.cuda.synchronize()
    graph_eps = N_EDGES * args.steps / (g0.elapsed_time(g1) * 1e-3)
    del graphs

    # plain one-launch-per-batch FP64 form on the same batches
    checker.setPrecision("fp64")
    run(0, capi.SCHEDULE_PLAIN)
    torch.cuda.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record()
    for i in range(N_BATCHES):
        run(i, capi.SCHEDULE_PLAIN)
    p1.record()
    torch.cuda.synchronize()
    plain_eps = N_BATCHES * N_EDGES / (p0.elapsed_time(p1) * 1e-3)
    checker.setPrecision("fp32_guarded")

    # end to end through the host-memory C-ABI call (gbo_check_motion_host): endpoints in pinned host
    # memory (OMPL's per-state row layout), results (ok + lastValid fractions) read back to pinned memory
    import ctypes as C
    pin_in = [(torch.as_tensor(a).pin_memory(), torch.as_tensor(b).pin_memory()) for a, b in host_batches]
    ok_h = torch.empty(N_EDGES, dtype=torch.uint8).pin_memory()
    lt_h = torch.empty(N_EDGES, dtype=torch.float64).pin_memory()

    def e2e_step(i):
        a, b = pin_in[i % N_BATCHES]
        capi.check(capi.lib().gbo_check_motion_host(checker._h, C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()),
                                                    N_EDGES, C.c_void_p(ok_h.data_ptr()),
                                                    C.c_void_p(lt_h.data_ptr()), None))

    e2e_step(0)
    t = time.perf_counter()
    for i in range(args.steps):
        e2e_step(i)
    e2e_s = time.perf_counter() - t
    e2e = N_EDGES * args.steps / e2e_s

    # nearestK k=16 over the 1M states
    nn = B.NearestNeighborsGPU(space, capacity=N_STATES)
    nn.add(states_soa, soa=True)
    qi = np.random.default_rng(11).integers(0, N_STATES, KNN_QUERIES)
    q = torch.as_tensor(w.states[qi].T.copy(), device=dev)
    nn.nearestK(q[:, :256], 16, soa=True)
    torch.cuda.synchronize()
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k0.record()
    nn.nearestK(q, 16, soa=True, want_dist=False)
    k1.record()
    torch.cuda.synchronize()
    knn_qps = KNN_QUERIES / (k0.elapsed_time(k1) * 1e-3)
    knn_stats = nn.stats()

    # sampling on one sampler's stream: 1M uniform states, then 1M Gaussian states around them
    smp = B.StateSampler(space, 5)
    smp.sampleUniform(1000, host=False)
    smp.sampleGaussian(torch.zeros((1000, w.dim), dtype=torch.float64, device=dev), 0.1)
    torch.cuda.synchronize()
    s0, s1e, s2e = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    s0.record()
    means = smp.sampleUniform(N_STATES, host=False)
    s1e.record()
    smp.sampleGaussian(means, 0.1)
    s2e.record()
    torch.cuda.synchronize()
    sampling = {"states": N_STATES, "dim": w.dim,
                "uniform_states_per_s": N_STATES / (s0.elapsed_time(s1e) * 1e-3),
                "gaussian_states_per_s": N_STATES / (s1e.elapsed_time(s2e) * 1e-3)}
    del means

    if rank != 0:
        return
    peak_fp32 = B.measure_fp32_peak()
    achieved = mean_checked * FLOP_PER_STATE / (mean_ms * 1e-3)
    # DRAM read + write bytes of one launch of the timed kernel, from the committed ncu summary
    # (same 100k-edge batch as one step)
    traffic = issue = None
    prof = os.path.join(ROOT, "profiles", "chain_motion_warp_kernel_chain10.md")
    if os.path.exists(prof):
        for line in open(prof):
            if line.startswith("traffic_bytes_per_launch:"):
                traffic = int(line.split(":")[1])
            elif line.startswith("issue_active_frac:"):
                issue = float(line.split(":")[1])
    # CPU baseline: the oracle port on all host threads, bounded sample of batch 0
    from oracle.oracle import CheckerDesc, Oracle, SpaceDesc
    port = Oracle.port()
    sd = SpaceDesc(w.space_kind, w.dim, link_length=w.link_length, lvs_fraction=w.lvs_fraction)
    cd = CheckerDesc(w.checker_kind, w.obstacles)
    threads = os.cpu_count() or 1
    sample = 20_000
    cpu_v = cpu_edges_per_s(port, sd, cd, host_batches[0][0][:sample], host_batches[0][1][:sample], threads)
    clocks = clk.summary(t0, t1)
    out = {
        "metric": METRIC, "value": value, "unit": "edges/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mean_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32+f64", "data": "synthetic (seeded)",
        "config": bench_config(),
        "e2e": {"value": e2e, "unit": "edges/s", "h2d_bytes_per_step": 2 * N_EDGES * 10 * 8,
                "d2h_bytes_per_step": N_EDGES * (1 + 8)},
        "gpu_launches": launches,
        "wall_s": wall,
        "roofline": {"bound": "fp32", "achieved": achieved / 1e12, "peak": peak_fp32 / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / peak_fp32, "traffic": traffic,
                     "issue_active_frac": issue,
                     "note": "the limiter is instruction issue (guard-band compares, shuffles), not FP32 FMA: "
                             "issue_active_frac is ncu's smsp__issue_active of the same launch",
                     "peak_source": "FP32 FMA throughput measured in this run (gbo_measure_fp32_peak)",
                     "work": f"{FLOP_PER_STATE} flop x checked states ({mean_checked:.0f} per step)"},
        "cpu_baseline": {"value": cpu_v, "unit": "edges/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} edges of batch 0, oracle restatement, all host threads"},
        "plain_fp64_edges_per_s": plain_eps,
        "batched_vs_plain": value / world / plain_eps,
        "schedule_edges_per_s": sched_eps,
        "graph_replay_edges_per_s": graph_eps,
        "recheck_rate": stats["rechecked"] / max(stats["evaluated"], 1),
        "states_per_s": states_per_s,
        "knn_queries_per_s": knn_qps,
        "knn": {"k": 16, "points": N_STATES, "queries": KNN_QUERIES, **knn_stats},
        "sampling": sampling,
        "recheck": stats,
        "clocks": clocks,
    }
    print(json.dumps(out))


def profile(kind):
    """Two launches of one kernel kind on the 10-link chain workload (first = warm-up), for ncu."""
    import torch

    from ompl_gb300 import base as B
    from ompl_gb300 import capi
    if kind == "arm":
        # DH arm (4,096 spheres): the 256k edges of the arm workload, tile schedule, two launches
        from ompl_gb300 import workloads as W
        wa = W.config2()
        space = B.RealVectorStateSpace(7, wa.low, wa.high)
        space.setLongestValidSegmentFraction(wa.lvs_fraction)
        checker = B.DHSphereArmValidityChecker(space, wa.dh, wa.obstacles, 8, 0.05)
        checker.setPrecision("fp32_guarded")
        mv = B.DiscreteMotionValidator(checker)
        a = torch.as_tensor(wa.s1.T.copy(), device="cuda")
        b = torch.as_tensor(wa.s2.T.copy(), device="cuda")
        for _ in range(2):
            mv.checkMotions(a, b, schedule=capi.SCHEDULE_TILE, soa=True)
        torch.cuda.synchronize()
        print(json.dumps({"profile": kind, "ok": True}))
        return
    w = workload()
    space = B.KinematicChainSpace(w.dim, w.link_length)
    space.setLongestValidSegmentFraction(w.lvs_fraction)
    checker = B.KinematicChainValidityChecker(space, w.obstacles)
    checker.setPrecision("fp64" if kind == "motion_plain" else "fp32_guarded")
    if kind == "peaks":
        print(json.dumps({"fp32_flops": B.measure_fp32_peak(), "fp64_flops": B.measure_fp64_peak()}))
        return
    states = torch.as_tensor(w.states.T.copy(), device="cuda")
    if kind == "validity":
        for _ in range(2):
            checker.isValid(states, soa=True)
    elif kind in ("motion", "motion_plain"):
        valid = checker.isValid(states, soa=True).cpu().numpy().astype(bool)
        (a, b), = make_batches(w.states[valid], 1)
        s1, s2 = torch.as_tensor(a.T.copy(), device="cuda"), torch.as_tensor(b.T.copy(), device="cuda")
        mv = B.DiscreteMotionValidator(checker)
        sch = capi.SCHEDULE_PLAIN if kind == "motion_plain" else capi.SCHEDULE_WARP
        n = 20_000 if kind == "motion_plain" else N_EDGES
        for _ in range(2):
            mv.checkMotions(s1[:, :n].contiguous(), s2[:, :n].contiguous(), schedule=sch, soa=True)
    elif kind == "knn":
        nn = B.NearestNeighborsGPU(space, capacity=N_STATES)
        nn.add(states, soa=True)
        # the bench's kNN leg: KNN_QUERIES queries drawn from the states, k = 16
        qi = torch.as_tensor(np.random.default_rng(11).integers(0, N_STATES, KNN_QUERIES), device=states.device)
        q = states[:, qi].contiguous()
        for _ in range(2):
            nn.nearestK(q, 16, soa=True, want_dist=False)
    torch.cuda.synchronize()
    print(json.dumps({"profile": kind, "ok": True}))


def arm_bench(args):
    """7-DoF DH arm among 4,096 spheres: 256k edges with 2..2000 interpolation steps, one launch."""
    import torch

    from ompl_gb300 import base as B
    from ompl_gb300 import capi
    from ompl_gb300 import workloads as W
    w = W.config2()
    space = B.RealVectorStateSpace(7, w.low, w.high)
    space.setLongestValidSegmentFraction(w.lvs_fraction)
    checker = B.DHSphereArmValidityChecker(space, w.dh, w.obstacles, 8, 0.05)
    mv = B.DiscreteMotionValidator(checker)
    s1 = torch.as_tensor(w.s1.T.copy(), device="cuda")
    s2 = torch.as_tensor(w.s2.T.copy(), device="cuda")
    n = s1.shape[1]
    res = {}
    for prec, sch, name in (("fp32_guarded", capi.SCHEDULE_TILE, "tile"), ("fp32_guarded", capi.SCHEDULE_WARP, "warp"),
                            ("fp64", capi.SCHEDULE_PLAIN, "plain_fp64")):
        checker.setPrecision(prec)
        m = n if name != "plain_fp64" else 16_384
        a, b = s1[:, :m].contiguous(), s2[:, :m].contiguous()
        r = mv.checkMotions(a, b, schedule=sch, soa=True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        reps = 3 if name != "plain_fp64" else 1
        for _ in range(reps):
            r = mv.checkMotions(a, b, schedule=sch, soa=True)
        e1.record()
        torch.cuda.synchronize()
        res[name] = reps * m / (e0.elapsed_time(e1) * 1e-3)
        if name == "tile":
            fj, nd = r["first_j"].long(), r["nd"].long()
            checked = int(torch.where(fj >= 0, fj, torch.clamp(nd, min=1)).sum().item())
            valid = float(r["ok"].float().mean().item())
            st = checker.stats()
    print(json.dumps({"metric": "validated edges/s (DH arm, 4096 spheres)", "edges": n,
                      "edges_per_s": res, "checked_states_per_edge": checked / n, "valid_fraction": valid,
                      "recheck": st}))


def prm_bench(args):
    """Full PRM roadmap construction (2M uniform samples, validity filter, prefix nearestK k=10 in
    the wrap-L2 joint space, n->m edges at 0.01 rad) for the DH arm among 16,384 spheres.
    PRM_STAR=1: PRM* connection counts (KStarStrategy, k(m) = ceil((e + e/7) log(m + 1)))."""
    import torch

    from ompl_gb300 import base as B
    from ompl_gb300 import prm
    from ompl_gb300 import workloads as W
    w = W.config4()
    n = int(os.environ.get("PRM_SAMPLES", w.extra["n_samples"]))
    star = os.environ.get("PRM_STAR", "0") == "1"
    space = B.WrapL2StateSpace(7)
    space.setLongestValidSegmentFraction(w.lvs_fraction)
    checker = B.DHSphereArmValidityChecker(space, w.dh, w.obstacles, 8, 0.05)
    checker.setPrecision("fp32_guarded")
    prm.construct_roadmap(space, checker, w.extra["sampler_seed"], 20_000, star=star)  # warm-up (autotune, allocs)
    torch.cuda.synchronize()
    t = time.perf_counter()
    rm = prm.construct_roadmap(space, checker, w.extra["sampler_seed"], n, star=star)
    total = time.perf_counter() - t
    nm = rm.milestones.shape[1]
    # the motion phase under each persistent schedule (the autotuner picks one per checker)
    from ompl_gb300 import capi
    mv = B.DiscreteMotionValidator(checker)
    s1 = rm.milestones[:, rm.edge_src[:200_000]].contiguous()
    s2 = rm.milestones[:, rm.edge_dst[:200_000]].contiguous()
    sched = {}
    for name, sch in (("tile", capi.SCHEDULE_TILE), ("warp", capi.SCHEDULE_WARP)):
        mv.checkMotions(s1, s2, schedule=sch, soa=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mv.checkMotions(s1, s2, schedule=sch, soa=True)
        torch.cuda.synchronize()
        sched[name] = s1.shape[1] / (time.perf_counter() - t0)
    comps = prm.connected_components(nm, rm.edge_src.cpu().numpy(), rm.edge_dst.cpu().numpy())
    print(json.dumps({"metric": "PRM%s roadmap construction (DH arm, 16384 spheres)" % ("*" if star else ""),
                      "samples": n,
                      "milestones": nm, "candidate_edges": rm.candidate_edges, "edges": int(rm.edge_src.numel()),
                      "components": comps, "total_s": total, "timings_ms": rm.timings_ms,
                      "edges_per_s": rm.candidate_edges / (rm.timings_ms["motion"] * 1e-3),
                      "knn_queries_per_s": nm / (rm.timings_ms["nn add+prefix kNN"] * 1e-3),
                      "checked_states": rm.checked_states, "valid_edge_schedules_edges_per_s": sched}))


def serve_bench(args):
    """Serving: 512 clients, each with its own world (1,024..8,192 spheres, the 7-DoF DH arm) and roadmap
    (10k..200k joint states, nearestK k=10); Poisson arrivals of motion requests (16..65,536 edges) and
    nearestK requests (1..4,096 queries). Reports saturation throughput and, at 70% of it, p50/p99."""
    import threading as th

    import torch

    from ompl_gb300 import base as B
    from ompl_gb300 import capi
    from ompl_gb300 import serve
    from ompl_gb300 import workloads as W
    n_clients = int(os.environ.get("SERVE_CLIENTS", 512))
    n_req = int(os.environ.get("SERVE_REQUESTS", 3000))
    rng = np.random.default_rng(3)
    dh = W.dh_arm(np.random.default_rng(2))
    lvs_fraction = 1.0 / 2500.0
    clients = []
    t_setup = time.perf_counter()
    for c in range(n_clients):
        crng = np.random.default_rng(3 + 1000 * (c + 1))
        world = W.sphere_world(crng, int(crng.integers(1024, 8193)))
        space = B.RealVectorStateSpace(7, -math.pi, math.pi)
        space.setLongestValidSegmentFraction(lvs_fraction)
        ck = B.DHSphereArmValidityChecker(space, dh, world, 8, 0.05)
        ck.setPrecision("fp32_guarded")
        nroad = int(np.exp(crng.uniform(np.log(10_000), np.log(200_000))))
        wspace = B.WrapL2StateSpace(7)
        nn = B.NearestNeighborsGPU(wspace, capacity=nroad)
        nn.add(torch.as_tensor(crng.uniform(-math.pi, math.pi, size=(7, nroad)), device="cuda"), soa=True)
        clients.append((ck, nn, nroad))
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t_setup
    lo, hi = np.full(7, -math.pi), np.full(7, math.pi)
    e1, e2 = W.arm_edges(rng, 262_144, 2 * math.pi * math.sqrt(7) * lvs_fraction, lo, hi)
    qpool = rng.uniform(-math.pi, math.pi, size=(262_144, 7))
    reqs = []
    for i in range(n_req):
        c = int(rng.integers(0, n_clients))
        if rng.random() < 0.5:
            n = int(np.exp(rng.uniform(np.log(16), np.log(65_536))))
            o = int(rng.integers(0, len(e1) - n))
            reqs.append(("motion", c, e1[o:o + n], e2[o:o + n]))
        else:
            n = int(np.exp(rng.uniform(np.log(1), np.log(4096))))
            o = int(rng.integers(0, len(qpool) - n))
            reqs.append(("knn", c, qpool[o:o + n], None))
    srv = serve.Server(n_streams=32, arena_bytes=8 << 30)

    def submit(r):
        kind, c, a, b = r
        ck, nn, _ = clients[c]
        if kind == "motion":
            return srv.submit_motion(ck, a, b, schedule=capi.SCHEDULE_TILE)
        return srv.submit_knn(nn, a, 10, want_dist=False)

    for r in reqs[:64]:  # warm-up: allocations of every code path
        srv.wait(submit(r))

    def run(rate):
        lat = [None] * len(reqs)
        tickets = [None] * len(reqs)
        done = th.Event()

        def waiter():
            for i in range(len(reqs)):
                while tickets[i] is None:
                    time.sleep(0.0002)
                lat[i] = srv.wait(tickets[i])[1]
            done.set()

        w = th.Thread(target=waiter)
        w.start()
        t0 = time.perf_counter()
        gaps = np.random.default_rng(9).exponential(1.0 / rate, len(reqs)) if rate else np.zeros(len(reqs))
        t_next = t0
        for i, r in enumerate(reqs):
            t_next += gaps[i]
            d = t_next - time.perf_counter()
            if d > 0:
                time.sleep(d)
            tickets[i] = submit(r)
        done.wait()
        wall = time.perf_counter() - t0
        w.join()
        return wall, lat

    wall_sat, _ = run(None)
    edges = sum(len(r[2]) for r in reqs if r[0] == "motion")
    queries = sum(len(r[2]) for r in reqs if r[0] == "knn")
    rate = 0.7 * len(reqs) / wall_sat
    wall, lat = run(rate)

    def pct(kind, q):
        xs = [l for r, l in zip(reqs, lat) if kind in (None, r[0])]
        return float(np.percentile(xs, q) * 1e3)

    # plain form: the same requests one at a time, FP64 plain motion schedule and FP64 exact nearestK
    sample = reqs[:200]
    t = time.perf_counter()
    pe = pq = 0
    for kind, c, a, b in sample:
        ck, nn, _ = clients[c]
        if kind == "motion":
            ck.setPrecision("fp64")
            B.DiscreteMotionValidator(ck).checkMotions(a, b, schedule=capi.SCHEDULE_PLAIN)
            ck.setPrecision("fp32_guarded")
            pe += len(a)
        else:
            nn.setPrecision("fp64")
            nn.nearestK(a, 10, want_dist=False)
            nn.setPrecision("fp32_guarded")
            pq += len(a)
    plain_s = time.perf_counter() - t
    st = srv.stats()
    srv.close()
    print(json.dumps({
        "metric": "serving: validated edges/s and kNN queries/s, p50/p99 latency", "clients": n_clients,
        "requests": n_req, "setup_s": setup_s,
        "saturation": {"wall_s": wall_sat, "edges_per_s": edges / wall_sat, "queries_per_s": queries / wall_sat,
                       "requests_per_s": n_req / wall_sat},
        "offered_load_requests_per_s": rate,
        "at_offered_load": {"wall_s": wall, "edges_per_s": edges / wall, "queries_per_s": queries / wall,
                            "p50_ms": pct(None, 50), "p99_ms": pct(None, 99),
                            "motion_p50_ms": pct("motion", 50), "motion_p99_ms": pct("motion", 99),
                            "knn_p50_ms": pct("knn", 50), "knn_p99_ms": pct("knn", 99)},
        "plain_sequential_sample": {"requests": len(sample), "wall_s": plain_s,
                                    "edges_per_s": pe / plain_s if plain_s else None,
                                    "work_units_per_s": (pe + pq) / plain_s},
        "served_vs_plain_edges": (edges / wall_sat) / (pe / plain_s) if pe else None,
        "server": st}))


def main():
    args = parse()
    if args.workload == "serve" and not args.profile and args.impl == "ours":
        serve_bench(args)
        return
    if args.workload == "arm" and not args.profile and args.impl == "ours":
        arm_bench(args)
        return
    if args.workload == "prm" and not args.profile and args.impl == "ours":
        prm_bench(args)
        return
    if args.profile:
        profile(args.profile)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    ours(args, rank, world, local_rank)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

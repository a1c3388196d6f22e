"""Benchmark: validated edges/s of DiscreteMotionValidator::checkMotion on the planar 10-link
kinematic-chain workload (32 world segments, segment fraction 0.005 of the extent, edges between
valid states of a seeded 1M-state set), on one GB300, plus the other workloads of the path.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--only-headline]

One step = one batch of 100,000 edges checked by the batched form (persistent work-queue kernel,
FP32 bulk with FP64 re-check, autotuned schedule). Twelve distinct batches (192 MB of endpoints,
more than the 129 MB L2) rotate across steps, so no step re-reads L2-resident inputs. `e2e` is the
same metric through the host-memory C-ABI call (gbo_check_motion_host: H2D of both endpoint
arrays, kernel, D2H of results and lastValid fractions inside the timed region). `parity` compares
the timed results with the oracle (20,000 edges of a timed batch; 500 of the kNN queries).

The same JSON line carries one object per further workload ("workloads"): circles in RealVector(2)
at full size, the 7-DoF DH arm among 4,096 spheres (256k edges of 2..2000 steps), the serving loop
(512 clients, Poisson arrivals, p50/p99) and the PRM roadmap (2M samples, 16,384 spheres); each with
the plain one-launch-per-call GPU form, the batched/served form, its roofline, parity against the
oracle and the oracle's CPU time on one thread and on all host threads.

Under torchrun each rank runs an independent replica on its own GPU ("replicas only": the path
has no exchange step); value = all ranks' edges / max-over-ranks time; only rank 0 runs the
further workloads.
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
# measured peaks of this GPU pool (copy bandwidth, bf16 GEMM), when the file is present
PEAKS = {}
if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")):
    with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as _f:
        PEAKS = json.load(_f)
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
    p.add_argument("--workload", default="chain", choices=["chain", "arm", "prm", "serve", "rrt"],
                   help="chain: the headline 10-link chain workload; arm: 7-DoF DH arm, 256k edges of 2..2000 "
                        "steps; prm: PRM roadmap of the DH arm among 16,384 spheres from 2M samples")
    p.add_argument("--profile", default=None,
                   choices=["validity", "motion", "motion_plain", "knn", "peaks", "arm", "sample", "gauss"],
                   help="launch one kernel kind twice on the chain workload (for ncu) and exit")
    p.add_argument("--only-headline", action="store_true",
                   help="the chain workload alone (no circles / arm / serving / PRM objects)")
    return p.parse_args()


def cpu_info():
    """Host CPU model and thread count (lscpu's model name; /proc/cpuinfo as a fallback)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if model is None:
        try:
            for line in open("/proc/cpuinfo"):
                if line.lower().startswith(("model name", "cpu part")):
                    model = line.split(":", 1)[1].strip()
                    break
        except Exception:
            pass
    return {"cpu_model": model, "threads": os.cpu_count() or 1}


def timed(fn):
    t = time.perf_counter()
    r = fn()
    return r, time.perf_counter() - t


def cpu_rates(n_all, n_one, run):
    """Oracle CPU rate on all host threads (n_all units) and on one thread (n_one units): run(n, threads)
    performs n units. Returns dict(all_core, single_thread, cores)."""
    threads = os.cpu_count() or 1
    _, t_all = timed(lambda: run(n_all, threads))
    _, t_one = timed(lambda: run(n_one, 1))
    return {"all_core": n_all / t_all, "single_thread": n_one / t_one, "cores": threads,
            "sample_all_core": n_all, "sample_single_thread": n_one}


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
    for i in range(args.warmup):
        s1, s2 = batches[i % N_BATCHES]
        port.check_motion(sd, cd, s1, s2, want_state=False, want_bisect=False)
    t = time.perf_counter()
    for i in range(args.steps):
        s1, s2 = batches[i % N_BATCHES]
        port.check_motion(sd, cd, s1, s2, want_state=True, want_bisect=False)
    dt = time.perf_counter() - t
    v = N_EDGES * args.steps / dt
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "edges/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": bench_config(),
        "cpu_baseline": {"value": v, "unit": "edges/s", "cores": threads, "kind": "port", **cpu_info(),
                         "sample": "every step: the whole 100k-edge batch (ordered DiscreteMotionValidator with "
                                   "lastValid), all host threads"},
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
    stats = checker.stats()  # states evaluated / re-checked in FP64 / one-ulp hazards of the last timed step
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

    # precision statistics of the FP32 form over the 1M states (flip rate before re-check, FP32 error)
    precision = checker.precisionStats(states_soa, soa=True)

    # nearestK k=16 over the 1M states
    nn = B.NearestNeighborsGPU(space, capacity=N_STATES)
    nn.add(states_soa, soa=True)
    qi = np.random.default_rng(11).integers(0, N_STATES, KNN_QUERIES)
    q = torch.as_tensor(w.states[qi].T.copy(), device=dev)
    nn.nearestK(q[:, :256], 16, soa=True)
    torch.cuda.synchronize()
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k0.record()
    knn_idx, _ = nn.nearestK(q, 16, soa=True, want_dist=False)
    k1.record()
    torch.cuda.synchronize()
    knn_ms = k0.elapsed_time(k1)
    knn_qps = KNN_QUERIES / (knn_ms * 1e-3)
    knn_stats = nn.stats()
    # roofline of the chain cell search: the element-feature and box bytes it read (counted on the
    # device), over the call's time, against the measured copy bandwidth; DRAM traffic of one launch from
    # the committed ncu summary (the 80 MB of features stay in L2)
    knn_dram = None
    kprof = os.path.join(ROOT, "profiles", "knn_ccell_warp_kernel_chain10.md")
    if os.path.exists(kprof):
        for line in open(kprof):
            if line.startswith("traffic_bytes_per_launch:"):
                knn_dram = int(line.split(":")[1])
    knn_gbs = knn_stats["search_bytes"] / (knn_ms * 1e-3) / 1e9
    knn_roofline = {"bound": "l2 latency (the 80 MB of features stay in L2)", "achieved": knn_gbs,
                    "peak": PEAKS.get("hbm_gbs"), "unit": "GB/s",
                    "frac": knn_gbs / PEAKS["hbm_gbs"] if PEAKS.get("hbm_gbs") else None,
                    "work": f"{knn_stats['search_bytes']} bytes: 48 per visited element (links 4..9; the inner "
                            "links' 32 bytes, read for candidates only, are not counted) and 80 per cell or "
                            "chunk box tested",
                    "note": "peak = measured HBM copy bandwidth, but these bytes are served from L2, so the "
                            "fraction can exceed 1; traffic = DRAM bytes of one launch from ncu",
                    "traffic": knn_dram, "feature_array_bytes": N_STATES * 80}
    knn_idx = knn_idx.cpu().numpy()
    pq = np.random.default_rng(12).choice(KNN_QUERIES, 500, replace=False)
    _, knn_dist500 = nn.nearestK(q[:, pq].contiguous(), 16, soa=True)
    knn_dist500 = knn_dist500.cpu().numpy()
    # results of the timed batches, for the parity check against the oracle
    r0 = run(0, capi.SCHEDULE_AUTO)
    timed0 = {k: r0[k].cpu().numpy() for k in ("ok", "first_j", "nd")}

    # sampling on one sampler's stream: 1M uniform states, then 1M Gaussian states around them; calls
    # of the same sizes come first (the jump polynomials of a call size are prepared once per process
    # on the host, and the sampler's scratch grows once)
    smp = B.StateSampler(space, 5)
    for _ in range(2):
        warm_means = smp.sampleUniform(N_STATES, host=False)
    smp.sampleGaussian(warm_means, 0.1)
    del warm_means
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
    u_ms = s0.elapsed_time(s1e)
    sampling_bytes = N_STATES * w.dim * 8
    sampling = {"states": N_STATES, "dim": w.dim,
                "uniform_states_per_s": N_STATES / (u_ms * 1e-3),
                "gaussian_states_per_s": N_STATES / (s1e.elapsed_time(s2e) * 1e-3),
                "uniform_ms": u_ms,
                "roofline": {"bound": "hbm", "achieved": sampling_bytes / (u_ms * 1e-3) / 1e9,
                             "peak": PEAKS.get("hbm_gbs"), "unit": "GB/s",
                             "frac": sampling_bytes / (u_ms * 1e-3) / 1e9 / PEAKS["hbm_gbs"]
                             if PEAKS.get("hbm_gbs") else None,
                             "work": f"{sampling_bytes} bytes of coordinates written per call (8 per value)",
                             "peak_source": "measured copy bandwidth (MEASURED_PEAKS.json)"}}
    sampled_host = means.cpu().numpy()
    del means

    if rank != 0:
        return
    peak_fp32 = _fp32_peak()
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
    # CPU baseline: the oracle port on all host threads and on one thread, bounded samples of batch 0;
    # the all-core answers double as the parity check of the timed batch
    from oracle.oracle import CheckerDesc, Oracle, SpaceDesc
    port = Oracle.port()
    sd = SpaceDesc(w.space_kind, w.dim, link_length=w.link_length, lvs_fraction=w.lvs_fraction)
    cd = CheckerDesc(w.checker_kind, w.obstacles)
    threads = os.cpu_count() or 1
    sample = 20_000
    a0, b0 = host_batches[0][0][:sample], host_batches[0][1][:sample]
    port.set_threads(threads)
    ref0, dt_all = timed(lambda: port.check_motion(sd, cd, a0, b0, want_state=False, want_bisect=False))
    port.set_threads(1)
    _, dt_one = timed(lambda: port.check_motion(sd, cd, a0[:2000], b0[:2000], want_state=False, want_bisect=False))
    port.set_threads(threads)
    cpu_v = sample / dt_all
    agree = (ref0["ok"] == timed0["ok"][:sample]) & (ref0["first_j"] == timed0["first_j"][:sample]) & \
        (ref0["nd"] == timed0["nd"][:sample])
    ref_idx, ref_dist = port.knn(sd, w.states, w.states[qi[pq]], 16)
    knn_agree = (ref_idx == knn_idx[pq]).all(axis=1) & \
        np.all(np.abs(ref_dist - knn_dist500) <= 1e-12 * np.maximum(np.abs(ref_dist), np.abs(knn_dist500)), axis=1)
    # the timed uniform call, every value, against the oracle's sequential stream (same calls before it;
    # the Gaussian calls' stream consumption does not depend on their means)
    ref_s = port.sample_script(sd, 5, [("uniform", N_STATES), ("uniform", N_STATES), ("gaussian", N_STATES),
                                       ("uniform", 1000), ("gaussian", 1000), ("uniform", N_STATES)],
                               mean=np.zeros((N_STATES + 1000, w.dim)), stddev=0.1)[-N_STATES:]
    sampling["parity"] = {"values_checked": int(ref_s.size),
                          "values_agree": int((ref_s.view(np.uint64) == sampled_host.view(np.uint64)).sum()),
                          "compared": "every coordinate of the timed sampleUniform call, bitwise, against the "
                                      "oracle's sequential mt19937 stream after the same earlier calls"}
    parity = {"edges_checked": sample, "edges_agree": int(agree.sum()), "knn_checked": len(pq),
              "knn_agree": int(knn_agree.sum()),
              "compared": "ok, first invalid index and segment count of 20,000 edges of timed batch 0; "
                          "index lists (exact) and distances (relative 1e-12, FP64 sin/cos) of 500 of the "
                          "20,000 kNN queries, against the oracle"}
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
        "cpu_baseline": {"value": cpu_v, "unit": "edges/s", "cores": threads, "kind": "port", **cpu_info(),
                         "single_thread": 2000 / dt_one,
                         "sample": f"{sample} edges of batch 0 on all host threads, 2,000 on one thread "
                                   "(oracle restatement, FP64)"},
        "parity": parity,
        "plain_fp64_edges_per_s": plain_eps,
        "batched_vs_plain": value / world / plain_eps,
        "schedule_edges_per_s": sched_eps,
        "graph_replay_edges_per_s": graph_eps,
        "recheck_rate": stats["rechecked"] / max(stats["evaluated"], 1),
        "flip_rate": precision["flip_rate"],
        "precision": {**precision, "over": "the 1M states of the workload, all 397 segment tests each",
                      "hazards_last_step": stats["hazards"],
                      "note": "flip = FP32 verdict taken at face value differs from the FP64 verdict; the "
                              "guarded form re-checks every ambiguous state in FP64, so its answers equal "
                              "the FP64 ones; hazards = FP64 decisions a one-ulp change of a C-library "
                              "sin/cos could reverse"},
        "states_per_s": states_per_s,
        "knn_queries_per_s": knn_qps,
        "knn": {**knn_stats, "k": 16, "points": N_STATES, "queries": KNN_QUERIES, "roofline": knn_roofline},
        "sampling": sampling,
        "recheck": stats,
        "clocks": clocks,
    }
    if not args.only_headline and world == 1:
        del dev_batches, pin_in, states_soa, nn
        torch.cuda.empty_cache()
        out["workloads"] = other_workloads(port)
    bad = parity_shortfalls(out)
    if bad:
        print("bench: parity shortfall in " + ", ".join(bad), file=sys.stderr)
    print(json.dumps(out))


def parity_shortfalls(obj, path=""):
    """Paths of the parity objects in the bench line whose agreement count is below their checked count."""
    bad = []
    if isinstance(obj, dict):
        for key, val in obj.items():
            sub = f"{path}/{key}"
            if isinstance(val, dict) and key in ("parity", "alone_equals_mix"):
                for ck, cv in val.items():
                    if ck.endswith("_checked"):
                        agree = val.get(ck[: -len("_checked")] + "_agree", val.get(ck[: -len("_checked")] + "_same"))
                        if agree is not None and agree < cv:
                            bad.append(f"{sub}/{ck}")
                if val.get("digest_match") is False:
                    bad.append(f"{sub}/digest_match")
            bad += parity_shortfalls(val, sub)
    return bad


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
    if kind == "sample":
        # sampleUniform of 1M states of the 10-D chain space, three calls on one stream
        smp = B.StateSampler(space, 5)
        for _ in range(3):
            smp.sampleUniform(N_STATES, soa=True, host=False)
        torch.cuda.synchronize()
        print(json.dumps({"profile": kind, "ok": True}))
        return
    if kind == "gauss":
        # sampleGaussian of 1M states of the 10-D chain space around uniform means, three calls
        smp = B.StateSampler(space, 5)
        means = smp.sampleUniform(N_STATES, host=False)
        for _ in range(3):
            smp.sampleGaussian(means, 0.1)
        torch.cuda.synchronize()
        print(json.dumps({"profile": kind, "ok": True}))
        return
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


ARM_FLOP_PER_STATE = 504 + 1008 + 672  # FK (7 x (sincos + 36 FMA)), 56 sphere transforms, 56 cell lookups
NARROW_FLOP_PER_PAIR = 10


def _events(n=2):
    import torch
    return [torch.cuda.Event(enable_timing=True) for _ in range(n)]


def _checked_states(r):
    """States the reference's ordered DiscreteMotionValidator evaluates: first_j of an invalid motion,
    max(nd, 1) of a valid one."""
    import torch
    fj, nd = r["first_j"].long(), r["nd"].long()
    return int(torch.where(fj >= 0, fj, torch.clamp(nd, min=1)).sum().item())


def _fp32_peak():
    from ompl_gb300 import base as B
    if not hasattr(_fp32_peak, "v"):
        _fp32_peak.v = B.measure_fp32_peak()
    return _fp32_peak.v


def circles_workload(port):
    """Point robot in RealVector(2) among 100 circles at full size: 10,000 states, 10,000 edges at
    segment fraction 0.01, nearestK k = 10 for 1,000 queries; FP64 throughout (the circles checker has no
    FP32 form). Every output compared with the oracle."""
    import torch

    from ompl_gb300 import base as B
    from ompl_gb300 import capi
    from ompl_gb300 import workloads as W
    from oracle.oracle import CheckerDesc, SpaceDesc
    w = W.config0()
    space = B.RealVectorStateSpace(2, w.low, w.high)
    space.setLongestValidSegmentFraction(w.lvs_fraction)
    ck = B.CirclesValidityChecker(space, w.obstacles)
    mv = B.DiscreteMotionValidator(ck)
    st = torch.as_tensor(w.states.T.copy(), device="cuda")
    a = torch.as_tensor(w.s1.T.copy(), device="cuda")
    b = torch.as_tensor(w.s2.T.copy(), device="cuda")
    q = torch.as_tensor(w.queries.T.copy(), device="cuda")
    nn = B.NearestNeighborsGPU(space, capacity=len(w.states))
    nn.add(st, soa=True)

    def rate(fn, units, reps=20):
        fn()
        torch.cuda.synchronize()
        e0, e1 = _events()
        e0.record()
        for _ in range(reps):
            out = fn()
        e1.record()
        torch.cuda.synchronize()
        return units * reps / (e0.elapsed_time(e1) * 1e-3), out

    v_rate, valid = rate(lambda: ck.isValid(st, soa=True), len(w.states))
    plain, rp = rate(lambda: mv.checkMotions(a, b, schedule=capi.SCHEDULE_PLAIN, soa=True), len(w.s1))
    batched, rb = rate(lambda: mv.checkMotions(a, b, schedule=capi.SCHEDULE_AUTO, soa=True), len(w.s1))
    k_rate, (idx, dist) = rate(lambda: nn.nearestK(q, 10, soa=True), len(w.queries))
    sd = SpaceDesc(w.space_kind, 2, w.low, w.high, lvs_fraction=w.lvs_fraction)
    cd = CheckerDesc(w.checker_kind, w.obstacles)
    port.set_threads(os.cpu_count() or 1)
    v_ref = port.is_valid(sd, cd, w.states).astype(bool)
    m_ref = port.check_motion(sd, cd, w.s1, w.s2, want_state=False, want_bisect=False)
    i_ref, d_ref = port.knn(sd, w.states, w.queries, 10)
    rb = {k: v.cpu().numpy() for k, v in rb.items()}
    idx, dist = idx.cpu().numpy(), dist.cpu().numpy()
    parity = {"states_checked": len(w.states), "states_agree": int((valid.cpu().numpy().astype(bool) == v_ref).sum()),
              "edges_checked": len(w.s1),
              "edges_agree": int(((rb["ok"] == m_ref["ok"]) & (rb["first_j"] == m_ref["first_j"]) &
                                  (rb["nd"] == m_ref["nd"])).sum()),
              "knn_checked": len(w.queries),
              "knn_agree": int(((idx == i_ref).all(1) & (dist.view(np.uint64) == d_ref.view(np.uint64)).all(1)).sum())}
    checked = _checked_states({k: torch.as_tensor(v) for k, v in rb.items()})

    def cpu_motion(n, threads):
        port.set_threads(threads)
        port.check_motion(sd, cd, w.s1[:n], w.s2[:n], want_state=False, want_bisect=False)

    cpu = cpu_rates(len(w.s1), 2000, cpu_motion)
    port.set_threads(os.cpu_count() or 1)
    return {"workload": "circles2d: point robot in RealVector(2) on [0,1]^2, 100 circles, 10,000 states, 10,000 "
                        "random edges at segment fraction 0.01, nearestK k=10 for 1,000 queries, FP64",
            "states_per_s": v_rate, "plain_edges_per_s": plain, "batched_edges_per_s": batched,
            "knn_queries_per_s": k_rate, "checked_states_per_edge": checked / len(w.s1),
            "roofline": {"bound": "fp64 latency (tiny batch)", "note": "10,000 edges of ~1.6 checked states "
                         "finish in tens of microseconds: launch latency, not a roofline, bounds this size"},
            "cpu_baseline": {"unit": "edges/s", "kind": "port", **cpu},
            "parity": parity, "flip_rate": None}


def arm_workload(port, n_plain=16_384):
    """7-DoF DH arm among 4,096 spheres: 256k edges with 2..2000 interpolation steps, one launch each."""
    import torch

    from ompl_gb300 import base as B
    from ompl_gb300 import capi
    from ompl_gb300 import workloads as W
    from oracle.oracle import CheckerDesc, SpaceDesc
    w = W.config2()
    space = B.RealVectorStateSpace(7, w.low, w.high)
    space.setLongestValidSegmentFraction(w.lvs_fraction)
    checker = B.DHSphereArmValidityChecker(space, w.dh, w.obstacles, 8, 0.05)
    mv = B.DiscreteMotionValidator(checker)
    s1 = torch.as_tensor(w.s1.T.copy(), device="cuda")
    s2 = torch.as_tensor(w.s2.T.copy(), device="cuda")
    n = s1.shape[1]
    res, res_ms, outs = {}, {}, {}
    for prec, sch, name in (("fp32_guarded", capi.SCHEDULE_TILE, "tile"), ("fp32_guarded", capi.SCHEDULE_WARP, "warp"),
                            ("fp32_guarded", capi.SCHEDULE_AUTO, "batched"), ("fp64", capi.SCHEDULE_PLAIN, "plain_fp64")):
        checker.setPrecision(prec)
        m = n if name != "plain_fp64" else n_plain
        a, b = s1[:, :m].contiguous(), s2[:, :m].contiguous()
        mv.checkMotions(a, b, schedule=sch, soa=True)
        torch.cuda.synchronize()
        reps = 3 if name != "plain_fp64" else 1
        e0, e1 = _events()
        e0.record()
        for _ in range(reps):
            r = mv.checkMotions(a, b, schedule=sch, soa=True)
        e1.record()
        torch.cuda.synchronize()
        res[name] = reps * m / (e0.elapsed_time(e1) * 1e-3)
        res_ms[name] = e0.elapsed_time(e1) / reps
        outs[name] = (r, checker.stats())  # counters of the last call
    r, st = outs["batched"]
    checked = _checked_states(r)
    pairs = st.get("pairs")
    flop = checked * ARM_FLOP_PER_STATE + (pairs or 0) * NARROW_FLOP_PER_PAIR
    peak = _fp32_peak()
    achieved = flop / (res_ms["batched"] * 1e-3)
    sd = SpaceDesc(w.space_kind, 7, w.low, w.high, lvs_fraction=w.lvs_fraction)
    cd = CheckerDesc(w.checker_kind, w.obstacles, w.dh, 8, 0.05)
    port.set_threads(os.cpu_count() or 1)
    npar = 2000
    ref = port.check_motion(sd, cd, w.s1[:npar], w.s2[:npar], want_state=False, want_bisect=False)
    got = {k: r[k][:npar].cpu().numpy() for k in ("ok", "first_j", "nd")}
    agree = (got["ok"] == ref["ok"]) & (got["first_j"] == ref["first_j"]) & (got["nd"] == ref["nd"])

    def cpu_motion(k, threads):
        port.set_threads(threads)
        port.check_motion(sd, cd, w.s1[:k], w.s2[:k], want_state=False, want_bisect=False)

    cpu = cpu_rates(npar, 200, cpu_motion)
    port.set_threads(os.cpu_count() or 1)
    # precision statistics over every state the ordered validator would build for the first 1,000 edges
    # (RealVector interpolation from + (to - from) * t with t = j / nd, as RealVectorStateSpace.cpp:257-265)
    nd0 = ref["nd"][:1000].astype(np.int64)
    rows = np.repeat(np.arange(1000), np.maximum(nd0, 1))
    jj = np.concatenate([np.arange(1, max(k, 1) + 1) for k in nd0]).astype(np.float64)
    tt = jj / np.maximum(nd0[rows], 1)
    pstates = w.s1[rows] + (w.s2[rows] - w.s1[rows]) * tt[:, None]
    checker.setPrecision("fp32_guarded")
    precision = checker.precisionStats(pstates)
    checker.setPrecision("fp64")
    mv.checkMotions(s1[:, :n_plain].contiguous(), s2[:, :n_plain].contiguous(), schedule=capi.SCHEDULE_PLAIN, soa=True)
    hz_plain = checker.stats()["hazards"]
    checker.setPrecision("fp32_guarded")
    return {"workload": "dh_arm7: 7-DoF DH arm (8 spheres r 0.05 per link), 4,096 world spheres in a 64^3 grid, "
                        "256k edges of 2..2000 interpolation steps, one launch",
            "edges": n, "edges_per_s": res, "plain_edges_per_s": res["plain_fp64"],
            "batched_edges_per_s": res["batched"], "batched_vs_plain": res["batched"] / res["plain_fp64"],
            "plain_sample_edges": n_plain, "checked_states_per_edge": checked / n,
            "valid_fraction": float(r["ok"].float().mean().item()),
            "roofline": {"bound": "fp32", "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
                         "frac": achieved / peak,
                         "work": f"{ARM_FLOP_PER_STATE} flop x checked states ({checked}) + {NARROW_FLOP_PER_PAIR} "
                                 f"flop x narrow-phase pairs examined ({pairs})",
                         "peak_source": "FP32 FMA throughput measured in this run (gbo_measure_fp32_peak)"},
            "recheck": st, "cpu_baseline": {"unit": "edges/s", "kind": "port", **cpu},
            "parity": {"edges_checked": npar, "edges_agree": int(agree.sum())},
            "flip_rate": precision["flip_rate"],
            "precision": {**precision, "over": f"the {len(pstates)} states of the first 1,000 edges",
                          "hazards_batched": st.get("hazards"), "hazards_plain_fp64": hz_plain},
            "l2": "inputs (29 MB) fit in L2; each launch is compute-bound (3 ms)"}


def prm_workload(port, n=None, star=False):
    """Full PRM roadmap construction (2M uniform samples, validity filter, prefix nearestK k=10 in
    the wrap-L2 joint space, n->m edges at 0.01 rad) for the DH arm among 16,384 spheres; PRM* with
    KStarStrategy when star is set."""
    import hashlib

    import torch

    from ompl_gb300 import base as B
    from ompl_gb300 import capi
    from ompl_gb300 import prm
    from ompl_gb300 import workloads as W
    from oracle.oracle import CheckerDesc, SpaceDesc
    w = W.config4()
    n = int(n or w.extra["n_samples"])
    space = B.WrapL2StateSpace(7)
    space.setLongestValidSegmentFraction(w.lvs_fraction)
    checker = B.DHSphereArmValidityChecker(space, w.dh, w.obstacles, 8, 0.05)
    checker.setPrecision("fp32_guarded")
    seed = w.extra["sampler_seed"]
    small = 20_000
    prm.construct_roadmap(space, checker, seed, small, star=star)  # warm-up (autotune, allocations)
    # a sampling call of the roadmap's size on another stream prepares the jump polynomials of that
    # call size (once per process, on the host), as a planner that samples repeatedly would have them
    B.StateSampler(space, seed + 1).sampleUniform(n, soa=True, host=False)
    torch.cuda.synchronize()
    _, gpu_small_s = timed(lambda: (prm.construct_roadmap(space, checker, seed, small, star=star),
                                    torch.cuda.synchronize()))
    torch.cuda.synchronize()
    rm, total = timed(lambda: prm.construct_roadmap(space, checker, seed, n, star=star))
    nm = rm.milestones.shape[1]
    src, dst = rm.edge_src.cpu().numpy(), rm.edge_dst.cpu().numpy()
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components
    comps = connected_components(coo_matrix((np.ones(len(src)), (src, dst)), shape=(nm, nm)), directed=False)[0]
    # the motion phase: batched (persistent, FP32 + FP64 re-check) vs plain (one FP64 launch) on a sample
    mv = B.DiscreteMotionValidator(checker)
    m = min(200_000, int(rm.edge_src.numel()))
    a = rm.milestones[:, rm.edge_src[:m]].contiguous()
    b = rm.milestones[:, rm.edge_dst[:m]].contiguous()
    forms = {}
    for name, prec, sch in (("batched", "fp32_guarded", capi.SCHEDULE_AUTO), ("plain_fp64", "fp64", capi.SCHEDULE_PLAIN)):
        checker.setPrecision(prec)
        mv.checkMotions(a[:, :1000].contiguous(), b[:, :1000].contiguous(), schedule=sch, soa=True)
        torch.cuda.synchronize()
        e0, e1 = _events()
        e0.record()
        mv.checkMotions(a, b, schedule=sch, soa=True)
        e1.record()
        torch.cuda.synchronize()
        forms[name] = m / (e0.elapsed_time(e1) * 1e-3)
    checker.setPrecision("fp32_guarded")
    samples = B.StateSampler(space, seed).sampleUniform(min(n, 2_000_000), soa=True, host=False)
    precision = checker.precisionStats(samples, soa=True)
    del samples
    out = {"workload": "prm%s_dh_arm7: PRM roadmap from %d uniform samples, 7-DoF DH arm among 16,384 spheres, "
                       "wrap-L2 joint space, nearestK k=10 (prefix), edges at 0.01 rad" % ("_star" if star else "", n),
           "samples": n, "milestones": nm, "candidate_edges": rm.candidate_edges, "edges": int(len(src)),
           "components": int(comps), "total_s": total, "timings_ms": rm.timings_ms,
           "edges_per_s": rm.candidate_edges / (rm.timings_ms["motion"] * 1e-3),
           "knn_queries_per_s": nm / (rm.timings_ms["nn add+prefix kNN"] * 1e-3),
           "checked_states": rm.checked_states,
           "motion_sample_edges": m, "plain_edges_per_s": forms["plain_fp64"],
           "batched_edges_per_s": forms["batched"], "batched_vs_plain": forms["batched"] / forms["plain_fp64"],
           "flip_rate": precision["flip_rate"], "precision": {**precision, "over": "the uniform samples"}}
    if not star:
        dg = os.path.join(ROOT, "tests", "golden", "prm_dh_arm7_digest.json")
        ref = json.load(open(dg))["sizes"].get(str(n)) if os.path.exists(dg) else None
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from golden.make_prm_digest import roadmap_digest
        got = roadmap_digest(rm.sample_index.cpu().numpy(), src, dst, rm.candidate_edges)
        out["parity"] = {"digest_match": (got == ref) if ref else None, "edges": got["edges"],
                         "reference": "tests/golden/prm_dh_arm7_digest.json (oracle on the CPU)"}
        sd = SpaceDesc(w.space_kind, 7, lvs_fraction=w.lvs_fraction)
        cd = CheckerDesc(w.checker_kind, w.obstacles, w.dh, 8, 0.05)

        def cpu_prm(k, threads):
            port.set_threads(threads)
            port.prm_roadmap(sd, cd, seed, k, 10)

        cpu = cpu_rates(small, 4000, cpu_prm)
        port.set_threads(os.cpu_count() or 1)
        out["cpu_baseline"] = {"unit": "samples/s", "kind": "port", **cpu,
                               "gpu_same_sample_samples_per_s": small / gpu_small_s,
                               "note": "whole roadmap construction of the first 20,000 (all threads) / 4,000 (one "
                                       "thread) samples"}
    return out


def serve_workload(port, n_clients=512, n_req=2000):
    """Serving: n_clients clients, each with its own world (1,024..8,192 spheres, the 7-DoF DH arm) and
    roadmap (10k..200k joint states, nearestK k=10); Poisson arrivals of motion requests (16..65,536
    edges) and nearestK requests (1..4,096 queries). Reports saturation throughput and, at 70% of it,
    p50/p99; the plain form runs the same requests one at a time (FP64 plain motion schedule, FP64 exact
    nearestK). Parity: 24 served requests against the oracle."""
    import threading as th

    import torch

    from ompl_gb300 import base as B
    from ompl_gb300 import capi
    from ompl_gb300 import serve
    from ompl_gb300 import workloads as W
    from oracle.oracle import CheckerDesc, SpaceDesc
    rng = np.random.default_rng(3)
    dh = W.dh_arm(np.random.default_rng(2))
    lvs_fraction = 1.0 / 2500.0
    clients = []
    t_setup = time.perf_counter()

    def client_data(c):
        crng = np.random.default_rng(3 + 1000 * (c + 1))
        world = W.sphere_world(crng, int(crng.integers(1024, 8193)))
        nroad = int(np.exp(crng.uniform(np.log(10_000), np.log(200_000))))
        return world, crng.uniform(-math.pi, math.pi, size=(7, nroad))

    for c in range(n_clients):
        world, road = client_data(c)
        space = B.RealVectorStateSpace(7, -math.pi, math.pi)
        space.setLongestValidSegmentFraction(lvs_fraction)
        ck = B.DHSphereArmValidityChecker(space, dh, world, 8, 0.05)
        ck.setPrecision("fp32_guarded")
        wspace = B.WrapL2StateSpace(7)
        nn = B.NearestNeighborsGPU(wspace, capacity=road.shape[1])
        nn.add(torch.as_tensor(road, device="cuda"), soa=True)
        clients.append((ck, nn, road.shape[1]))
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
        results = [None] * len(reqs)
        tickets = [None] * len(reqs)
        done = th.Event()

        def waiter():
            for i in range(len(reqs)):
                while tickets[i] is None:
                    time.sleep(0.0002)
                results[i], lat[i] = srv.wait(tickets[i])
            done.set()

        wt = th.Thread(target=waiter)
        wt.start()
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
        wt.join()
        return wall, lat, results

    wall_sat, _, results = run(None)
    edges = sum(len(r[2]) for r in reqs if r[0] == "motion")
    queries = sum(len(r[2]) for r in reqs if r[0] == "knn")
    rate = 0.7 * len(reqs) / wall_sat
    wall, lat, _ = run(rate)

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
    # parity and the CPU baseline: 24 served requests replayed on the oracle (all threads, then one)
    port.set_threads(os.cpu_count() or 1)
    sd = SpaceDesc(0, 7, lo, hi, lvs_fraction=lvs_fraction)
    sdw = SpaceDesc(3, 7, lvs_fraction=lvs_fraction)
    pick = np.random.default_rng(4).choice(len(reqs), 24, replace=False)
    agree, cpu_t, cpu_units = 0, 0.0, 0
    for i in pick:
        kind, c, a, b = reqs[i]
        world, road = client_data(c)
        t = time.perf_counter()
        if kind == "motion":
            ref = port.check_motion(sd, CheckerDesc(3, world, dh, 8, 0.05), a, b, want_state=False, want_bisect=False)
            same = np.array_equal(ref["ok"], results[i]["ok"]) and np.array_equal(ref["first_j"], results[i]["first_j"])
        else:
            ri, _ = port.knn(sdw, road.T.copy(), a, 10)
            same = np.array_equal(ri, results[i]["idx"])
        cpu_t += time.perf_counter() - t
        cpu_units += len(a)
        agree += int(same)
    return {
        "workload": f"serving: {n_clients} clients, own worlds of 1,024..8,192 spheres and roadmaps of 10k..200k "
                    f"joint states, {n_req} Poisson requests (motion 16..65,536 edges / nearestK 1..4,096 queries)",
        "clients": n_clients, "requests": n_req, "setup_s": setup_s,
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
        "plain_edges_per_s": pe / plain_s if pe else None, "batched_edges_per_s": edges / wall_sat,
        "parity": {"requests_checked": len(pick), "requests_agree": agree},
        "cpu_baseline": {"unit": "work units/s (edges + queries)", "kind": "port", "all_core": cpu_units / cpu_t,
                         "cores": os.cpu_count() or 1, "sample": "the 24 parity requests replayed on all threads"},
        "server": st}


def rrt_workload(port, n_clients=64, iterations=100):
    """RRTConnect-shaped planner clients (ompl_gb300/rrt.py) on the request loop: each client plans
    between two valid states of its own world (1,024..8,192 spheres, the DH arm), each iteration one
    nearestK(1) request and one short checkMotion (plus isValid for the goal tree) per growTree, the
    clients' requests overlapping. Reports growTree rate, request latency percentiles per kind, and that
    four clients give the same trees alone as in the mix."""
    import torch

    from ompl_gb300 import base as B
    from ompl_gb300 import rrt
    from ompl_gb300 import serve
    from ompl_gb300 import workloads as W
    from oracle.oracle import CheckerDesc, SpaceDesc
    dh = W.dh_arm(np.random.default_rng(2))
    lo, hi = np.full(7, -math.pi), np.full(7, math.pi)
    lvs_fraction = 1.0 / 2500.0
    rng_range = 0.2 * math.sqrt(7 * (2 * math.pi) ** 2)
    port.set_threads(os.cpu_count() or 1)
    setups = []
    for c in range(n_clients):
        crng = np.random.default_rng(5000 + c)
        world = W.sphere_world(crng, int(crng.integers(1024, 8193)))
        cand = crng.uniform(-math.pi, math.pi, size=(400, 7))
        ok = port.is_valid(SpaceDesc(0, 7, lo, hi, lvs_fraction=lvs_fraction), CheckerDesc(3, world, dh, 8, 0.05),
                           cand).astype(bool)
        setups.append((world, cand[ok][0], cand[ok][1]))
    srv = serve.Server(n_streams=32, arena_bytes=2 << 30)
    checkers = []
    for world, _, _ in setups:
        space = B.RealVectorStateSpace(7, lo, hi)
        space.setLongestValidSegmentFraction(lvs_fraction)
        ck = B.DHSphereArmValidityChecker(space, dh, world, 8, 0.05)
        ck.setPrecision("fp32_guarded")
        checkers.append(ck)

    def clients(idx):
        return [rrt.RRTConnectClient(srv, checkers[i], setups[i][1], setups[i][2], 9000 + i, rng_range)
                for i in idx]

    warm = clients([0])
    rrt.run_clients(warm, 5, concurrent=False)
    mix = clients(range(n_clients))
    t = time.perf_counter()
    rrt.run_clients(mix, iterations, concurrent=True)
    wall = time.perf_counter() - t
    alone = clients(range(4))
    rrt.run_clients(alone, iterations, concurrent=False)
    same = sum(len(a.trace) == len(m.trace) and all(
        x[0] == y[0] and x[1] == y[1] and x[3] == y[3] and ((x[2] is None and y[2] is None) or
                                                          np.array_equal(x[2], y[2]))
        for x, y in zip(a.trace, m.trace)) for a, m in zip(alone, mix[:4]))
    grows = sum(len(c.trace) for c in mix)
    st = srv.stats()
    srv.close()
    torch.cuda.synchronize()
    return {"workload": f"RRTConnect clients: {n_clients} planners, each in its own world of 1,024..8,192 spheres "
                        f"with the DH arm, range 0.2 of the extent, up to {iterations} iterations, served "
                        "concurrently", "clients": n_clients, "wall_s": wall,
            "solved": sum(c.solution is not None for c in mix), "grow_steps": grows,
            "grow_steps_per_s": grows / wall, "requests": sum(len(c.log) for c in mix),
            "requests_per_s": sum(len(c.log) for c in mix) / wall,
            "latency_ms": {k: rrt.request_percentiles(mix, k) for k in ("knn", "motion", "validity")},
            "alone_equals_mix": {"clients_checked": 4, "clients_same": int(same)},
            "server": st}


def other_workloads(port):
    import torch
    out = {}
    for name, fn in (("circles2d", circles_workload), ("dh_arm7_4096", arm_workload),
                     ("prm_dh_arm7_2M", prm_workload), ("serve_512_clients", serve_workload),
                     ("rrtconnect_64_clients", rrt_workload)):
        t = time.perf_counter()
        out[name] = fn(port)
        out[name]["bench_wall_s"] = time.perf_counter() - t
        torch.cuda.empty_cache()
    return out


def main():
    args = parse()
    if args.workload != "chain" and not args.profile and args.impl == "ours":
        from oracle.oracle import Oracle
        port = Oracle.port()
        if args.workload == "serve":
            r = serve_workload(port, int(os.environ.get("SERVE_CLIENTS", 512)), int(os.environ.get("SERVE_REQUESTS", 2000)))
        elif args.workload == "arm":
            r = arm_workload(port)
        elif args.workload == "rrt":
            r = rrt_workload(port)
        else:
            r = prm_workload(port, os.environ.get("PRM_SAMPLES"), os.environ.get("PRM_STAR", "0") == "1")
        print(json.dumps(r))
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

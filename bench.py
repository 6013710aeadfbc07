#!/usr/bin/env python
"""Benchmark of the ABC-PMC hot path on GB300.

Workload (configuration 1): two-component lognormal mixture
(175/500 nm, sd 10/25 nm, weights 0.6/0.4, 5e14 m^-3), 50 videos x 300
frames, population 1024, epsilon = 50% quantile, histograms 301 x 128.  A
step is one ABC-PMC generation (batched rounds until every population slot
has accepted a proposal) of a sequence of such jobs run back to back, each
capped at the configuration's 12 generations.  The metric is
particle-steps/s (one walk step of one particle; initial placements count
as steps), whole job, all GPUs.

At N = 1 the line also carries, as extra keys, short runs of
configurations 2 (512-proposal rounds) and 3 (a 64-proposal slice of the
1e5-particles-per-video model), the PMC step's time at population 4096, and
`serve`: the 64-job serving stream (p50/p99 job latency, accepted
proposals/s) and the served / plain ratio of accepted proposals/s on equal
work, each with its own clock record (--headline-only leaves them out).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's CPU path (the Julia forward model of
src/cpu/simulate.jl, restated in C as oracle/cpu_baseline.c because Julia
is not installed) on all host cores, one bounded sample per step.  N > 1
runs independent replicas (the path does not shard: no collectives).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic thread-operations of the forward model, counted from the
# algorithm (not from the compiled code): a uniform costs 22 (a quarter of a
# Philox4x32-10 call at ~80 integer ops, plus ~2 to convert), a Box-Muller
# pair 12 (log, sqrt, sincos, three multiplies), a full step of the walk 21
# (position 3, wrap 9, detection 5, DE 4):
#   per-step walk, per particle-step: 3 uniforms (66) + 1.5 pairs (18) + the
#     step (21) = 105;
#   slab-split walk, per particle-step of the z pass: per group of four steps
#     6 uniforms (132) + 3 pairs (36) + four z steps (20) + summed x, y (10) =
#     198, i.e. 49.5 per step;
#   slab-split walk, per task (a group walked in x, y): 8 uniforms (176) + 4
#     pairs (48) + bridge means (12) + four x, y steps with detection and DE
#     (72) + track bookkeeping (12) = 320.
# The compiled per-step walk executes fewer thread instructions than its 105
# (~73 on a configuration-1 round, ncu): wide multiplies and fused
# multiply-adds do more than one of these operations each.
OPS_PER_STEP = 105
OPS_SPLIT_STEP = 49.5
OPS_SPLIT_TASK = 320
# bytes the distance kernel moves per histogram cell: read count, write zero,
# read the observed cumulative histogram
DIST_BYTES_PER_CELL = 12
WORKLOAD = ("config1: 2-component lognormal (175/500 nm, sd 10/25, w 0.6/0.4), 5e14 m^-3, "
            "50 videos x 300 frames, pop 1024, quantile-0.5 schedule, R x B = 301 x 128")
# generation cap of each configuration's jobs (prior pass not counted)
GENERATIONS = {0: 8, 1: 12, 2: 8, 3: 10}
STEP_SEQ = ("one ABC-PMC generation (the prior pass counts as one) of a sequence of jobs run back to back, seeds "
            "1, 2, ..., each ended by its cap of {g} generations or by the trial cap (500 trials per slot on "
            "average; that generation is discarded, as the reference discards it); every timed step ends a "
            "generation that did work")
WORKLOADS = {
    0: ("config0: 1-component lognormal (175 nm, sd 10), 2e14 m^-3, 20 videos x 200 frames, pop 256, "
        "quantile-0.5 schedule, R x B = 201 x 100", STEP_SEQ.format(g=GENERATIONS[0])),
    1: (WORKLOAD, STEP_SEQ.format(g=GENERATIONS[1])),
    2: ("config2: 2-component lognormal, diameters U(100,800) nm, concentration prior spanning 50..5000 "
        "particles per video, 20 videos x 200 frames, pop 512, 512 proposals per round, R x B = 201 x 100",
        STEP_SEQ.format(g=GENERATIONS[2]) + " (512-proposal rounds)"),
    3: ("config3: 3-component lognormal (100/250/600 nm, sd 5%, w 0.3/0.4/0.3), 1e5 particles per video, "
        "100 videos x 1000 frames, pop 4096, R x B = 1001 x 256",
        "one round of 64 prior-pass proposals (fixed slice; a full run is ~4e14 particle-steps)"),
}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(gpu_index)], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is not None:
            time.sleep(0.25)
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [l.strip().split(", ") for l in self.f.read().splitlines() if l.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows if len(r) >= 9 for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def device_sm_count(P, device: int) -> int:
    import ctypes
    import re
    buf = ctypes.create_string_buffer(1 << 16)
    P.lib().pcs_device_report(buf, len(buf))
    m = re.search(rf"^\s+{device + 1}: .*?, (\d+) SMs", buf.value.decode(), re.M)
    return int(m.group(1)) if m else 152


def dist_setup():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return rank, world, local


def allreduce(x: float, op: str, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_job_dict(truth):
    import part_conc_spt_abc_gb300.workloads as W
    return dict(C=len(truth["mu"]), lognormal=1, m=truth["mu"], s=truth["sd"], c=truth["conc_ml"], az=[W.DEPTH],
                temperature=W.T_K, viscosity=W.ETA, ax=W.AREA[0], ay=W.AREA[1], Lx=W.BOX[0], Ly=W.BOX[1],
                Lz=W.BOX[2], deltat=W.DT, ub_de=W.UB_DE, kmin=2, B=128)


def cpu_port_sample(target_s: float, threads: int):
    """The reference CPU forward model on config-1 proposals at the true
    parameters: a bounded sample sized to take about target_s seconds."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    truth = dict(mu=[175.0, 500.0], sd=[10.0, 25.0], conc_ml=[3e8, 2e8])
    job = cpu_job_dict(truth)
    frames = np.full(50, 300, np.uint32)
    steps, secs = O.cpu_forward_batch([job] * max(1, threads), frames, threads, seed=11)
    rate = steps / max(secs, 1e-9)
    per = steps / max(1, threads)
    n = max(threads, int(target_s * rate / per))
    return (lambda seed: O.cpu_forward_batch([job] * n, frames, threads, seed=seed)), n


def run_reference(args, rank, world):
    if rank != 0:
        barrier(world)
        return
    threads = os.cpu_count() or 1
    sample, n = cpu_port_sample(3.0, threads)
    for w in range(args.warmup):
        sample(100 + w)
    tot_steps, tot_s = 0, 0.0
    for k in range(args.steps):
        st, s = sample(200 + k)
        tot_steps += st
        tot_s += s
    value = tot_steps / tot_s
    line = {
        "impl": "reference", "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "parallelism": f"replicas x{world}"},
        "run": {"step": f"{n} configuration-1 forward simulations at the true parameters (a bounded sample of the "
                        "workload's forward-model work, timed on the host cores)"},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{n} config-1 forward simulations per step, Julia conventions, Float64"},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    barrier(world)


def serve_stream_run(P, ctx, jobs, arrivals):
    """Served form: jobs are submitted at their arrival offsets into the
    continuous-batching loop.  Returns latency percentiles and totals."""
    n = len(jobs)
    srv = P.Server(ctx)
    sims = [P.make_simulation(ctx, j[0], j[2]) for j in jobs]
    finish = [None] * n
    submitted = 0
    t0 = time.perf_counter()
    while True:
        now = time.perf_counter() - t0
        while submitted < n and arrivals[submitted] <= now:
            srv.submit(sims[submitted])
            submitted += 1
        active = srv.step()
        now = time.perf_counter() - t0
        for i in range(submitted):
            if finish[i] is None and srv.finished(sims[i]):
                finish[i] = now
        if submitted == n and active == 0:
            break
        if active == 0 and submitted < n:
            time.sleep(max(0.0, min(0.05, arrivals[submitted] - now)))
    makespan = max(finish)
    lat = np.array(finish) - np.asarray(arrivals[:n])
    acc = sum(s.info().accepted for s in sims)
    props = sum(s.info().simulations for s in sims)
    steps = sum(s.info().particle_steps for s in sims)
    for s in sims:
        s.close()
    return {"jobs": n, "makespan_s": makespan, "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)), "accepted": int(acc), "accepted_per_s": acc / makespan,
            "proposals_per_s": props / makespan, "particle_steps_per_s": steps / makespan}


def plain_stream_run(P, ctx, jobs, arrivals, budget_s, geometry):
    """Plain form: jobs one at a time in arrival order, each with the
    reference's per-proposal schedule (30 queues), until the budget is spent.
    The clock is simulated: a job starts at max(its arrival, the previous
    job's end)."""
    ctx.set_tuning(plain_launch=geometry)
    clock, lat, acc, props, steps, done = 0.0, [], 0, 0, 0, 0
    t_start = time.perf_counter()
    for i, (inp, truth, seed) in enumerate(jobs):
        if time.perf_counter() - t_start > budget_s:
            break
        sim = P.make_simulation(ctx, inp, seed)
        t = time.perf_counter()
        sim.run_plain(0, 30)
        dt = time.perf_counter() - t
        clock = max(clock, arrivals[i]) + dt
        lat.append(clock - arrivals[i])
        inf = sim.info()
        acc += inf.accepted
        props += inf.simulations
        steps += inf.particle_steps
        done += 1
        sim.close()
    ctx.set_tuning(plain_launch=1)
    return {"jobs": done, "makespan_s": clock, "p50_latency_s": float(np.percentile(lat, 50)) if lat else None,
            "p99_latency_s": float(np.percentile(lat, 99)) if lat else None, "accepted": int(acc),
            "accepted_per_s": acc / max(clock, 1e-9), "proposals_per_s": props / max(clock, 1e-9),
            "particle_steps_per_s": steps / max(clock, 1e-9)}


def serve_section(args, P, device: int):
    """The serving stream (configuration 4): jobs arrive as a Poisson
    process at 2 jobs/s.  The served form admits them into the
    continuous-batching loop as they arrive (p50/p99 latency and accepted
    proposals/s over the whole stream).  The plain form runs jobs one at a
    time with the reference's per-proposal schedule; it cannot finish the
    stream in minutes, so the served/plain ratio is taken on equal work at
    saturation: the first --cmp-jobs jobs of the stream, each capped at
    --cmp-generations generations after the prior pass, all submitted at
    time 0, run by the plain form (one job after another; the reference's
    launch geometry, and the library's persistent grid) and by the served
    form (all jobs at once).  Clocks are sampled throughout."""
    import part_conc_spt_abc_gb300.workloads as W
    ctx = P.Context(device)
    if args.job_order:
        ctx.set_tuning(job_order=args.job_order)
    ctx.set_tuning(walk=1 if args.walk == "split" else 2)
    jobs, arrivals = W.serve_stream(ctx, n_jobs=args.jobs, seed=args.seed)
    clocks = Clocks(device)
    t0 = time.perf_counter()
    res = {"served": serve_stream_run(P, ctx, jobs, arrivals), "job_order": ctx.tuning.job_order}
    cmp_jobs = []
    for inp, truth, seed in jobs[:args.cmp_jobs]:
        inp.params.max_generations = args.cmp_generations
        cmp_jobs.append((inp, truth, seed))
    cmp_arr = np.zeros(len(cmp_jobs))
    comparisons = {}
    for name, geometry in (("reference_launch", 1), ("persistent_grid", 2)):
        if not cmp_jobs:
            break
        plain = plain_stream_run(P, ctx, cmp_jobs, cmp_arr, args.plain_budget, geometry)
        J = plain["jobs"]
        if J == 0:
            comparisons[name] = {"plain": plain}
            continue
        served_j = serve_stream_run(P, ctx, cmp_jobs[:J], cmp_arr[:J])
        comparisons[name] = {"plain": plain, "served_same_jobs": served_j,
                             "served_over_plain_accepted_per_s":
                                 served_j["accepted_per_s"] / max(plain["accepted_per_s"], 1e-12)}
    res["equal_work"] = comparisons
    res["wall_s"] = time.perf_counter() - t0
    res["clocks"] = clocks.stop()
    res["config"] = {
        "workload": f"serving stream: {len(jobs)} jobs, Poisson arrivals 2/s, 1-3 lognormal components, 100-500 "
                    "frames, 64-256 DE bins, pop 256-4096, 6-12 generations",
        "equal_work": f"first {len(cmp_jobs)} jobs, {args.cmp_generations} generations after the prior pass "
                      f"each, all submitted at time 0, plain budget {args.plain_budget:.0f} s per form",
        "plain_forms": "reference_launch: ceil(V/4) CTAs x 128 threads per proposal, as the reference launches "
                       "its kernel; persistent_grid: the library's persistent grid"}
    ctx.close()
    return res


def pmc_at_pop4096(P, device: int):
    """The PMC step (accept, whiten, pairwise kernel sum, finalize) at
    population 4096, the largest of configuration 3 and the serving stream:
    a configuration-0-shaped job with N = 4096, its prior pass and two
    generations.  Reports the PMC step's CUDA-event span per ended
    generation next to the generations' whole GPU time."""
    import part_conc_spt_abc_gb300.workloads as W
    ctx = P.Context(device)
    inp, _ = W.make_problem(ctx, [175.0], [10.0], 2e14, [1.0], 20, 200, 100, 4096, 2, seed=0)
    sim = P.make_simulation(ctx, inp, 1)
    ctx.reset_kernel_stats()
    for _ in range(3):
        if sim.step():
            break
    ks = ctx.kernel_stats()
    sim.close()
    ctx.close()
    g = max(1, ks.generations)
    return {"population": 4096, "generations_ended": int(ks.generations), "rounds": int(ks.rounds),
            "pmc_ms_per_generation": ks.pmc_ms / g, "gpu_ms_per_generation": ks.round_ms / g,
            "pmc_share": ks.pmc_ms / max(ks.round_ms, 1e-9),
            "pair_tflops": ks.pmc_pair_flops / max(ks.pmc_ms, 1e-9) / 1e9,
            "workload": "configuration 0 shape (20 videos x 200 frames, 201 x 100 bins) with population 4096"}


def run_serve(args, rank, world):
    """--serve: the serving stream alone, as its own line."""
    import part_conc_spt_abc_gb300 as P
    res = serve_section(args, P, rank)
    line = {"metric": "serve p50/p99 job latency, accepted proposals/s (served vs plain)",
            "value": res["served"]["accepted_per_s"], "unit": "accepted proposals/s", "n_gpus": 1, **res}
    print(json.dumps(line), flush=True)


class JobSequence:
    """Estimation jobs of one configuration run back to back (seeds seed0,
    seed0 + 1, ...), each until its generation cap or the trial cap ends it.
    step() advances the current job by one generation (its prior pass counts
    as one; a generation that reaches the trial cap is discarded, as the
    reference discards it, and ends the job), then moves on to the next job,
    so every step ends a generation that did work.  `prepare` jobs are
    created up front (their observed data uploaded); later ones on demand."""

    def __init__(self, P, ctx, inp, seed0: int, prepare: int = 0):
        self.P, self.ctx, self.inp, self.seed0 = P, ctx, inp, seed0
        self.ready = [P.make_simulation(ctx, inp, seed0 + i) for i in range(prepare)]
        self.made = prepare
        self.cur = None
        self.sims = []
        self.jobs_finished = 0

    def step(self):
        if self.cur is None:
            if self.ready:
                self.cur = self.ready.pop(0)
            else:
                self.cur = self.P.make_simulation(self.ctx, self.inp, self.seed0 + self.made)
                self.made += 1
            self.sims.append(self.cur)
        sim = self.cur
        if sim.step():
            self.cur = None
            self.jobs_finished += 1
        return sim

    def totals(self):
        """(particle-steps, proposals, accepted) of every job started."""
        infos = [s.info() for s in self.sims]
        return (sum(i.particle_steps for i in infos), sum(i.simulations for i in infos),
                sum(i.accepted for i in infos))

    def close(self):
        for s in self.sims + self.ready:
            s.close()


def simulate_traffic(launch_ms: float):
    """DRAM bytes (read + write) of one k_simulate launch, from the ncu
    capture of a configuration-1 launch summarised in profiles/ (line
    'dram bytes per ms of launch: X'), scaled to this run's mean launch
    time; None when the summary is absent."""
    import re
    try:
        with open(os.path.join(ROOT, "profiles", "k_simulate_config1_ncu_full.md")) as f:
            m = re.search(r"dram bytes per ms of launch:\s*([0-9.eE+]+)", f.read())
    except OSError:
        return None
    return float(m.group(1)) * launch_ms if m else None


def run_plain_config(args, P, ctx, inp, workload, rank):
    """The plain form (reference schedule, 30 queues) on one configuration:
    prior pass plus --steps generations, wall-clock timed (host PMC)."""
    ctx.set_tuning(plain_launch=args.plain)
    inp.params.max_generations = args.steps
    sim = P.make_simulation(ctx, inp, seed=1 + rank)
    t0 = time.perf_counter()
    sim.run_plain(0, 30)
    dt = time.perf_counter() - t0
    inf = sim.info()
    sim.close()
    line = {"impl": "plain", "metric": "particle-steps/s", "value": inf.particle_steps / dt,
            "unit": "particle-steps/s", "n_gpus": 1, "steps": args.steps, "warmup": 0,
            "ms_per_step": 1e3 * dt / (args.steps + 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload, "step": "prior pass + generations, reference per-proposal schedule",
                       "plain_launch": {1: "reference ceil(V/4) x 128", 2: "persistent grid"}[args.plain]},
            "proposals_per_s": inf.simulations / dt, "accepted_per_s": inf.accepted / dt, "wall_s": dt}
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


def distance_case(args, local):
    """pcs_scan_distance on COUNT Poisson(0.7) histograms of ROWS x BINS
    against a cumulative Poisson(0.7) observed histogram: W untimed and K
    timed calls, wall clock per call including the host-device copies (the
    kernel's own time comes from the ncu capture this case exists for)."""
    import part_conc_spt_abc_gb300 as P
    R, B, n = args.distance_case
    rng = np.random.default_rng(5)
    hist = rng.poisson(0.7, (n, R, B)).astype(np.uint32)
    ref = np.cumsum(np.cumsum(rng.poisson(0.7, (R, B)), 0), 1).astype(np.uint32)
    ctx = P.Context(local)
    for _ in range(args.warmup):
        P.scan_distance(ctx, hist, ref)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        P.scan_distance(ctx, hist, ref)
    dt = (time.perf_counter() - t0) / max(1, args.steps)
    ctx.close()
    return {"metric": "pcs_scan_distance wall time per call (host copies included)", "value": dt * 1e3,
            "unit": "ms", "higher_is_better": False, "steps": args.steps, "warmup": args.warmup,
            "config": {"workload": f"{n} histograms of {R} x {B}", "cells": n * R * B}}


def config_input(P, ctx, cfg, args):
    """(input, workload text, step text) of configuration cfg on ctx, with the
    context tuned for it (walk, autotuner, round capacity)."""
    import part_conc_spt_abc_gb300.workloads as W
    workload, step_def = WORKLOADS[cfg]
    inp, _ = {0: W.config0, 1: W.config1, 2: W.config2, 3: W.config3}[cfg](ctx, seed=0, generations=GENERATIONS[cfg])
    ctx.set_tuning(walk=1 if args.walk == "split" else 2)
    if not args.no_autotune and cfg != 3:
        ctx.autotune(inp)
    if args.no_round_fill:
        ctx.set_tuning(round_fill=0xFFFFFFFF)
    if cfg == 2:
        ctx.set_tuning(round_capacity=512)
    if cfg == 3:
        ctx.set_tuning(round_capacity=64)
    return inp, workload, step_def


def e2e_run(P, ctx, inp, sequence, steps, rank, world):
    """The same steps end to end through the public API from host buffers:
    job creation (H2D of the observed data) inside the timing, the
    population read back after every step (D2H)."""
    barrier(world)
    t0 = time.perf_counter()
    seq2 = sequence(501 + 1000 * rank, 0)
    d2h_total = 0
    for _ in range(steps):
        sim2 = seq2.step()
        out = sim2.output()  # D2H: the population (m, s, c, az, dist, w)
        d2h_total += sum(a.nbytes for a in (out.m, out.c, out.az, out.dist, out.w, out.s) if a is not None)
    e2e_s = time.perf_counter() - t0
    e2e_steps = seq2.totals()[0]
    e2e_jobs = len(seq2.sims)
    seq2.close()
    e2e_s = allreduce(e2e_s, "max", world)
    e2e_value = allreduce(float(e2e_steps), "sum", world) / e2e_s
    h2d = e2e_jobs * (inp.K.nbytes + inp.DE.nbytes + inp.frames.nbytes) / steps
    d2h = d2h_total / steps

    return e2e_value, h2d, d2h


def measure_config(args, P, cfg, steps, warmup, rank, world, local, e2e=True):
    """One configuration's bench line: `steps` timed steps after `warmup`,
    on a fresh context (its own tuning)."""
    peaks, peak_src = measured_peaks()
    ctx = P.Context(local)
    inp, workload, step_def = config_input(P, ctx, cfg, args)
    t = ctx.tuning
    tune = dict(walk={1: "slab-split", 2: "per-step"}.get(t.walk, t.walk), round_fill=t.round_fill,
                block=t.block_size, ppt=t.particles_per_thread, tile_rows=t.hist_tile_rows,
                warp_aggregate=t.warp_aggregate, chunk=t.chunk_particles, capacity=t.round_capacity,
                autotuned=not args.no_autotune and cfg != 3)

    class SliceSteps:
        """configuration 3: one round of the fixed 64-proposal prior-pass slice per step"""

        def __init__(self, seed):
            self.sim = P.make_simulation(ctx, inp, seed)
            self.srv = P.Server(ctx)
            self.srv.submit(self.sim)
            self.sims = [self.sim]
            self.jobs_finished = 0

        def step(self):
            self.srv.step()
            return self.sim

        def totals(self):
            i = self.sim.info()
            return i.particle_steps, i.simulations, i.accepted

        def close(self):
            self.sim.close()

    def sequence(seed0, prepare):
        return SliceSteps(seed0) if cfg == 3 else JobSequence(P, ctx, inp, seed0, prepare)

    # ---- device-resident run: inputs already in HBM -----------------------
    # every job the warm-up and the timed steps can need is created (its
    # observed data uploaded) before the timed region
    seq = sequence(1 + 1000 * rank, warmup + steps)
    for _ in range(warmup):
        seq.step()
    barrier(world)
    ctx.reset_kernel_stats()
    t0_steps, t0_props, t0_acc = seq.totals()
    jobs0 = seq.jobs_finished
    clocks = Clocks(local)
    ctx.timer_start()
    for _ in range(steps):
        seq.step()
    ms = ctx.timer_stop()
    clk = clocks.stop()
    t1_steps, t1_props, t1_acc = seq.totals()
    jobs_ended = seq.jobs_finished - jobs0
    ks = ctx.kernel_stats()
    steps_local = t1_steps - t0_steps
    props_local = t1_props - t0_props
    acc_local = t1_acc - t0_acc
    ms_max = allreduce(ms, "max", world)
    steps_all = allreduce(float(steps_local), "sum", world)
    props_all = allreduce(float(props_local), "sum", world)
    acc_all = allreduce(float(acc_local), "sum", world)
    value = steps_all / (ms_max / 1e3)
    seq.close()

    # ---- end to end through the public API, host buffers ------------------
    # jobs are created inside the timed region here (H2D: observed K, DE,
    # frame counts); each step reads the population back (D2H)
    e2e_value, h2d, d2h = None, 0, 0
    if e2e:
        e2e_value, h2d, d2h = e2e_run(P, ctx, inp, sequence, steps, rank, world)

    # ---- roofline of the dominant kernel (forward model: issue bound) -----
    sim_ms = ks.simulate_ms / max(1, ks.simulate_launches)
    steps_per_launch = ks.particle_steps / max(1, ks.simulate_launches)
    split = t.walk == 1
    tasks_per_launch = ks.split_tasks / max(1, ks.simulate_launches)
    ops_per_launch = (steps_per_launch * OPS_SPLIT_STEP + tasks_per_launch * OPS_SPLIT_TASK if split
                      else steps_per_launch * OPS_PER_STEP)
    achieved = ops_per_launch / (sim_ms / 1e3) / 1e12
    sm_count = device_sm_count(P, local)
    peak = sm_count * 128 * float(peaks.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12
    traffic = simulate_traffic(sim_ms) if cfg == 1 else None
    dist_ms = ks.distance_ms / max(1, ks.distance_launches)
    dist_gbs = (ks.histogram_cells / max(1, ks.distance_launches)) * DIST_BYTES_PER_CELL / (dist_ms / 1e3) / 1e9

    pmc_s = max(ks.pmc_ms, 1e-9) / 1e3
    pmc_gbs = ks.pmc_bytes / pmc_s / 1e9
    pmc_tflops = ks.pmc_pair_flops / pmc_s / 1e12

    cells = ks.histogram_cells / max(1, ks.rounds)
    l2_note = (f"round histograms {cells * 4 / 1e6:.0f} MB per round + job state"
               + (" (above L2)" if cells * 4 > 129e6 else " (below L2; the kernels are issue-bound)"))
    line = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": steps, "warmup": warmup, "ms_per_step": ms_max / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        # the workload alone (the reference arm prints the same object);
        # what this run chose and saw is under "run"
        "config": {"workload": workload, "parallelism": f"replicas x{world}"},
        "run": {"step": step_def, "l2": l2_note, "tuning": tune,
                "timed_region": {"steps": steps, "generations_ended": int(ks.generations),
                                 "jobs_ended": jobs_ended, "generation_cap": GENERATIONS[cfg]}},
        "proposals_per_s": props_all / (ms_max / 1e3),
        "accepted_per_s": acc_all / (ms_max / 1e3),
        "e2e": ({"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": int(h2d),
                 "d2h_bytes_per_step": int(d2h)} if e2e else None),
        "gpu_launches": int(ks.kernel_launches),
        "roofline": {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "Tops/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": "k_simulate (fused forward model + histogram)",
                     "achieved_def": (f"({OPS_SPLIT_STEP} x particle-steps + {OPS_SPLIT_TASK} x x,y tasks) algorithmic "
                                      "thread-ops per launch / launch time" if split else
                                      f"{OPS_PER_STEP} algorithmic thread-ops per particle-step x steps per launch / "
                                      "launch time"),
                     "ops_per_particle_step": ops_per_launch / max(1.0, steps_per_launch),
                     "peak_def": f"{sm_count} SMs x 128 lanes x {peaks.get('sm_max_mhz', 2070.0)} MHz ({peak_src} clock)"},
        "roofline_distance": {"bound": "hbm", "achieved": dist_gbs, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                              "frac": dist_gbs / float(peaks.get("hbm_gbs", 6800.0)),
                              "kernel": "k_distance", "peak_src": peak_src},
        "roofline_pmc": {"bound": "hbm", "achieved": pmc_gbs, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                         "frac": pmc_gbs / float(peaks.get("hbm_gbs", 6800.0)),
                         "kernel": "k_accept + k_whiten + k_kernel_sum + k_finalize (the PMC step)",
                         "achieved_def": "(2 N P x 8 population read + write + N x 8 weights) per ended generation / "
                                         "PMC-step time of all rounds",
                         "pair_tflops": pmc_tflops, "generations": int(ks.generations),
                         "ms_per_generation": ks.pmc_ms / max(1, ks.generations), "peak_src": peak_src},
        "kernel_ms": {"simulate_per_launch": sim_ms, "distance_per_launch": dist_ms,
                      "rounds": int(ks.rounds), "round_ms_total": ks.round_ms},
        "clocks": clk,
    }
    ctx.close()
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--small", action="store_true", help="configuration 0 (pop 256): the case profiled under ncu")
    ap.add_argument("--plain", type=int, default=0, choices=[0, 1, 2],
                    help="time the plain form instead (1: reference launch geometry, 2: persistent grid) "
                         "over --steps generations")
    ap.add_argument("--walk", default="step", choices=["step", "split"],
                    help="forward-model walk on Philox streams: per step (default) or slab-split")
    ap.add_argument("--no-round-fill", action="store_true",
                    help="no extra trials for rounds that would underfill the GPU")
    ap.add_argument("--config", type=int, default=1, choices=[0, 1, 2, 3],
                    help="benchmark configuration (1 is the headline; 3 times a fixed 64-proposal slice)")
    ap.add_argument("--serve", action="store_true", help="the 64-job serving stream, served vs plain")
    ap.add_argument("--jobs", type=int, default=64)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--plain-budget", type=float, default=300.0, help="seconds allowed for each plain form")
    ap.add_argument("--job-order", type=int, default=0, choices=[0, 1, 2],
                    help="serve: capacity order among jobs (1 admission, 2 least remaining work; 0 library default)")
    ap.add_argument("--cmp-jobs", type=int, default=4, help="serve: jobs in the equal-work comparison")
    ap.add_argument("--cmp-generations", type=int, default=6, help="serve: generations per compared job")
    ap.add_argument("--pmc-pop4096", action="store_true",
                    help="only the PMC step's time per generation at population 4096, as its own line")
    ap.add_argument("--headline-only", action="store_true",
                    help="configuration 1 alone: no configuration 2 / 3 slices, PMC timing or serving stream")
    ap.add_argument("--distance-case", type=int, nargs=3, metavar=("ROWS", "BINS", "COUNT"),
                    help="the distance kernel alone through pcs_scan_distance on COUNT seeded histograms of "
                         "ROWS x BINS (the small case its ncu captures run on)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    rank, world, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.serve:
        run_serve(args, local, world)
        return
    if args.distance_case:
        if rank == 0:
            print(json.dumps(distance_case(args, local)), flush=True)
        return
    if args.pmc_pop4096:
        import part_conc_spt_abc_gb300 as P
        if rank == 0:
            print(json.dumps({"metric": "PMC step ms per generation at population 4096",
                              **pmc_at_pop4096(P, local)}), flush=True)
        return

    import part_conc_spt_abc_gb300 as P

    cfg = 0 if args.small else args.config
    if args.plain:
        ctx = P.Context(local)
        inp, workload, _ = config_input(P, ctx, cfg, args)
        run_plain_config(args, P, ctx, inp, workload, rank)
        return
    line = measure_config(args, P, cfg, args.steps, args.warmup, rank, world, local, e2e=True)
    if cfg != 1:
        line["config"]["headline"] = False
    if cfg == 1 and world == 1 and not args.headline_only:
        # other configurations as extra keys: short runs, not the headline
        for extra in (2, 3):
            x = measure_config(args, P, extra, 3, 3, rank, world, local, e2e=False)
            line[f"config{extra}"] = {k: x[k] for k in ("value", "unit", "steps", "ms_per_step", "proposals_per_s",
                                                          "accepted_per_s", "roofline", "roofline_distance",
                                                          "kernel_ms", "clocks") if k in x}
            line[f"config{extra}"]["workload"] = x["config"]["workload"]
            line[f"config{extra}"]["step"] = x["run"]["step"]
            line[f"config{extra}"]["tuning"] = x["run"]["tuning"]
        line["pmc_pop4096"] = pmc_at_pop4096(P, local)
        # the serving stream and the served / plain comparison (the batching target)
        line["serve"] = serve_section(args, P, local)
    if rank == 0 and world == 1 and not args.no_cpu_baseline and cfg == 1:
        threads = os.cpu_count() or 1
        sample, n = cpu_port_sample(10.0, threads)
        st, s = sample(7)
        line["cpu_baseline"] = {"value": st / s, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                                "sample": f"{n} config-1 forward simulations (Julia conventions, Float64), {s:.1f} s"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    barrier(world)


if __name__ == "__main__":
    main()

"""The ABC-PMC engine on the GPU: invariants of every generation, results
independent of how work is batched (round capacity, speculation, launch
shape, other jobs sharing the rounds), the accel drop-in end to end."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_input(pcs, seed=0, C=1, schedule=None, weighting=0, model=None, videos=6, frames=60, pop=96, de_bins=48):
    import part_conc_spt_abc_gb300.workloads as W
    ctx = pcs.Context(0)
    try:
        mu = [175.0, 500.0][:C]
        sd = [10.0, 25.0][:C]
        w = [0.6, 0.4][:C]
        inp, truth = W.make_problem(ctx, mu, sd, 3e14, w, videos, frames, de_bins, pop, 4, seed=seed)
    finally:
        ctx.close()
    p = inp.params
    p.avg_trial_count = 200
    p.weighting_scheme = weighting
    if schedule is not None:
        p.schedule = schedule
    return inp, truth


def run_job(pcs, ctx, inp, seed, steps):
    sim = pcs.make_simulation(ctx, inp, seed)
    for _ in range(steps):
        if sim.step():
            break
    out = sim.output()
    info = sim.info()
    sim.close()
    return out, info


def test_generation_invariants(pcs, ctx):
    inp, truth = small_input(pcs, C=2)
    sim = pcs.make_simulation(ctx, inp, 5)
    p = inp.params
    for g in range(4):
        done = sim.step()
        out = sim.output()
        info = sim.info()
        N = p.abc_sample_count
        assert out.w.shape == (N,) and abs(out.w.sum() - 1.0) < 1e-9 and (out.w > 0).all()
        m = out.m.reshape(N, 2)
        if g >= 1:  # the prior population (after the first step) is kept as drawn, like the reference's
            assert (np.diff(m, axis=1) >= 0).all(), "components sorted by mean diameter"
        assert (m >= p.lb_m).all() and (m <= p.ub_m).all()
        c = np.log10(out.c)
        assert (c >= np.log10(p.lb_c) - 1e-9).all() and (c <= np.log10(p.ub_c) + 1e-9).all()
        assert (out.az == 2.0).all(), "a parameter with equal bounds stays fixed"
        if g >= 1:
            assert np.isfinite(out.dist).all()
        if done:
            break
    assert info.iterations >= 2 and info.simulations > 0 and info.particle_steps > 0


@pytest.mark.parametrize("walk", [2, 1], ids=["step", "split"])
def test_results_do_not_depend_on_batching(pcs, ctx, walk):
    ctx.set_tuning(walk=walk)
    inp, _ = small_input(pcs, C=1, pop=64)
    fill0 = ctx.tuning.round_fill
    ref_out, ref_info = run_job(pcs, ctx, inp, 9, 3)
    settings = [dict(max_speculation=1), dict(max_speculation=3, block_size=128, particles_per_thread=2),
                dict(round_capacity=200, max_speculation=64),
                dict(block_size=128, particles_per_thread=8),
                dict(max_speculation=4096, block_size=256, particles_per_thread=4, hist_tile_rows=8,
                     warp_aggregate=1),
                dict(round_fill=0xFFFFFFFF), dict(round_fill=3000000), dict(job_order=2),
                # no shared-memory tile: each warp takes its own slices of the work items
                dict(hist_tile_rows=0xFFFFFFFF, block_size=256, particles_per_thread=1, warp_aggregate=0xFFFFFFFF),
                dict(hist_tile_rows=0xFFFFFFFF, block_size=1024, particles_per_thread=1, warp_aggregate=1)]
    try:
        for kw in settings:
            ctx.set_tuning(**kw)
            out, info = run_job(pcs, ctx, inp, 9, 3)
            for f in ["m", "c", "az", "dist", "w", "s"]:
                assert np.array_equal(getattr(out, f), getattr(ref_out, f)), (kw, f)
            assert info.trials == ref_info.trials and info.accepted == ref_info.accepted
            assert info.gamma == ref_info.gamma
    finally:
        ctx.set_tuning(max_speculation=4096, block_size=256, particles_per_thread=1, hist_tile_rows=64,
                       warp_aggregate=0xFFFFFFFF, round_capacity=2048, round_fill=fill0, walk=2, job_order=2)


@pytest.mark.parametrize("plain_launch", [1, 2], ids=["reference_launch", "persistent_grid"])
def test_plain_form_draws_the_batched_proposals(pcs, ctx, plain_launch):
    """The plain form (reference schedule, host PMC in FP64) and the batched
    engine draw the same proposals from the same streams: through the first
    generation after the prior pass the trial counts are identical and the
    accepted populations and distances agree to the last bits (the proposal
    construction runs in FP64 on the host in one and on the device in the
    other, whose log/exp/sin differ in the last place); the weights differ
    by the batched engine's FP32 kernel-density sums."""
    inp, _ = small_input(pcs, C=2, pop=64)
    inp.params.max_generations = 1
    sim = pcs.make_simulation(ctx, inp, 21)
    sim.run()
    a, ia = sim.output(), sim.info()
    sim.close()
    ctx.set_tuning(plain_launch=plain_launch)
    try:
        sim = pcs.make_simulation(ctx, inp, 21)
        sim.run_plain(0, 7)
        b, ib = sim.output(), sim.info()
        sim.close()
    finally:
        ctx.set_tuning(plain_launch=1)
    for f in ["m", "c", "az", "s"]:
        np.testing.assert_allclose(getattr(a, f), getattr(b, f), rtol=1e-9, err_msg=f)
    np.testing.assert_allclose(a.dist, b.dist, rtol=1e-6)
    np.testing.assert_allclose(a.w, b.w, rtol=1e-4)
    assert ia.trials == ib.trials and ia.accepted == ib.accepted and ia.iterations == ib.iterations


def test_serve_alone_equals_mix(pcs, ctx):
    jobs = [small_input(pcs, seed=s, C=1 + s % 2, pop=48 + 16 * s)[0] for s in range(3)]
    alone = []
    for i, inp in enumerate(jobs):
        out, _ = run_job(pcs, ctx, inp, 100 + i, 1000)
        alone.append(out)
    for order in (1, 2):  # admission order, least remaining work first
        ctx.set_tuning(job_order=order, round_capacity=256)  # a short round: jobs compete for it
        srv = pcs.Server(ctx)
        sims = [pcs.make_simulation(ctx, inp, 100 + i) for i, inp in enumerate(jobs)]
        for s in sims:
            srv.submit(s)
        for _ in range(100000):
            if srv.step() == 0:
                break
        for s, a in zip(sims, alone):
            assert srv.finished(s)
            b = s.output()
            for f in ["m", "c", "az", "dist", "w"]:
                assert np.array_equal(getattr(a, f), getattr(b, f)), (order, f)
            s.close()
    ctx.set_tuning(job_order=2, round_capacity=2048)


def test_serve_mixed_shapes_alone_equals_mix(pcs, ctx):
    """Jobs whose histograms differ in rows and bins (61 x 48, 91 x 37,
    46 x 64, 121 x 130) share the rounds: the distance kernel then moves from
    one proposal's shape to another's inside a launch, and every job's result
    is still the one it gets alone."""
    shapes = [(60, 48), (90, 37), (45, 64), (120, 130)]
    jobs = [small_input(pcs, seed=10 + i, C=1 + i % 2, pop=48, frames=f, de_bins=b)[0]
            for i, (f, b) in enumerate(shapes)]
    alone = [run_job(pcs, ctx, inp, 200 + i, 1000)[0] for i, inp in enumerate(jobs)]
    srv = pcs.Server(ctx)
    sims = [pcs.make_simulation(ctx, inp, 200 + i) for i, inp in enumerate(jobs)]
    for s in sims:
        srv.submit(s)
    for _ in range(100000):
        if srv.step() == 0:
            break
    for s, a in zip(sims, alone):
        assert srv.finished(s)
        b = s.output()
        for f in ["m", "c", "az", "dist", "w"]:
            assert np.array_equal(getattr(a, f), getattr(b, f)), f
        s.close()


def test_destroyed_served_job_gives_its_memory_back(pcs):
    """A served job destroyed before it finishes no longer counts against
    the memory cap: under a cap that holds one job, a second job is
    admitted after the first is destroyed mid-run."""
    c2 = pcs.Context(0)
    try:
        jobs = [small_input(pcs, seed=s, C=1, pop=48)[0] for s in range(2)]
        hist_b = c2.tuning.round_capacity * (61 * 48) * 4
        srv = pcs.Server(c2, memory_cap=hist_b + 48000)
        a = pcs.make_simulation(c2, jobs[0], 1)
        srv.submit(a)
        srv.step()
        assert not srv.finished(a)
        a.close()
        b = pcs.make_simulation(c2, jobs[1], 2)
        srv.submit(b)
        for _ in range(100000):
            if srv.step() == 0:
                break
        assert srv.finished(b)
        b.close()
    finally:
        c2.close()


def test_serve_memory_cap(pcs, ctx):
    """With a cap that holds one job's arena and the round histograms but not
    two, jobs are admitted one after another and give the same results as
    alone; a cap below one job's needs is an out-of-memory error."""
    jobs = [small_input(pcs, seed=s, C=1, pop=48)[0] for s in range(2)]
    alone = [run_job(pcs, ctx, inp, 200 + i, 1000)[0] for i, inp in enumerate(jobs)]
    hist_b = ctx.tuning.round_capacity * (61 * 48) * 4  # 60 frames + 1 rows x 48 bins
    cap = hist_b + 48000                                # one job's arena (32,088 B) fits, two do not
    srv = pcs.Server(ctx, memory_cap=cap)
    sims = [pcs.make_simulation(ctx, inp, 200 + i) for i, inp in enumerate(jobs)]
    for s in sims:
        srv.submit(s)
    for _ in range(100000):
        if srv.step() == 0:
            break
    for s, a in zip(sims, alone):
        assert srv.finished(s)
        b = s.output()
        for f in ["m", "c", "az", "dist", "w"]:
            assert np.array_equal(getattr(a, f), getattr(b, f)), f
        s.close()
    lib = pcs._lib.lib()
    pcs._lib.check(lib.pcs_serve_set_memory_cap(ctx.h, 1 << 20), "cap")
    srv2 = pcs.Server(ctx)
    s = pcs.make_simulation(ctx, jobs[0], 1)
    srv2.submit(s)
    with pytest.raises(pcs.PcsError):
        srv2.step()
    s.close()
    pcs._lib.check(lib.pcs_serve_set_memory_cap(ctx.h, 0), "cap")


def test_inverse_distance_weights(pcs, ctx):
    inp, _ = small_input(pcs, C=1, weighting=1)
    out, info = run_job(pcs, ctx, inp, 3, 3)
    w = 1.0 / out.dist ** 2
    np.testing.assert_allclose(out.w, w / w.sum(), rtol=1e-12)


def test_max_steps_semantics(pcs, ctx):
    """-S n stops when the iteration counter exceeds n (the counter then
    reads n + 1, as the reference's meta does)."""
    inp, _ = small_input(pcs, C=1, pop=32)
    inp.params.max_generations = 0
    sim = pcs.make_simulation(ctx, inp, 1)
    sim.run(2)
    info = sim.info()
    assert info.iterations == 3 and not info.converged
    sim.close()
    # run(0) keeps the cap the job's parameters carry
    inp.params.max_generations = 2
    for plain in (False, True):
        sim = pcs.make_simulation(ctx, inp, 1)
        sim.run_plain() if plain else sim.run()
        info = sim.info()
        assert info.iterations == 3 and not info.converged, plain
        sim.close()


def test_accel_end_to_end(pcs, ctx, tmp_path):
    inp, _ = small_input(pcs, C=2, pop=48)
    p = inp.params
    data = tmp_path / "data.xml"
    data.write_text("<data>\n\t<ax>%r</ax>\n\t<ay>%r</ay>\n\t<number_of_frames>%s</number_of_frames>\n\t<deltat>%r</deltat>\n"
                    "\t<K>%s</K>\n\t<DE>%s</DE>\n</data>" % (
                        inp.ax, inp.ay, ",".join(str(int(x)) for x in inp.frames), inp.deltat,
                        ",".join(str(int(x)) for x in inp.K), ",".join(repr(float(x)) for x in inp.DE)))
    xml = tmp_path / "input.xml"
    tags = dict(data_file_path=str(data), model="lognormal", number_of_components=2, weighting_scheme="pmc-standard",
                Lx=p.Lx, Ly=p.Ly, Lz=p.Lz, kmin=2, number_of_de_bins=p.de_bin_count, ub_de=p.ub_de, lb_m=p.lb_m,
                ub_m=p.ub_m, lb_s=p.lb_s, ub_s=p.ub_s, lb_c=p.lb_c, ub_c=p.ub_c, lb_az=p.lb_az, ub_az=p.ub_az,
                number_of_abc_samples=48, gamma_initial=15.0, gamma_adaptive="true", delta_gamma=0.05,
                ub_average_number_of_trials=50, output_file_path=str(tmp_path / "never.xml"))
    xml.write_text("<input>\n" + "".join(f"\t<{k}>{v}</{k}>\n" for k, v in tags.items()) + "</input>\n")
    out = tmp_path / "out.xml"
    r = subprocess.run([pcs._lib.ACCEL_PATH, "-i", str(xml), "-o", str(out), "-S", "2", "-F", "7", "-q"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    o = pcs.load_output(str(out))
    assert o.model == 2 and o.abc_sample_count == 48 and o.component_count == 2
    assert len(o.m) == 96 and len(o.s) == 96 and len(o.w) == 48
    meta = dict(o.meta)
    assert meta["iterations"] == "3" and meta["simulator"] == "gpu" and meta["gpu0_queues"] == "30"
    # same seed, same result
    out2 = tmp_path / "out2.xml"
    r = subprocess.run([pcs._lib.ACCEL_PATH, "-i", str(xml), "-o", str(out2), "-S", "2", "-F", "7", "-q"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0
    o2 = pcs.load_output(str(out2))
    assert np.array_equal(o.m, o2.m) and np.array_equal(o.w, o2.w)


def test_autotune(pcs, ctx):
    inp, _ = small_input(pcs, C=1, pop=64)
    t = ctx.autotune(inp)
    assert t.block_size in (128, 256, 512, 1024) and t.particles_per_thread in (1, 2, 4)
    ctx.set_tuning(block_size=256, particles_per_thread=1, hist_tile_rows=64, warp_aggregate=0xFFFFFFFF)


def test_kernel_stats_account_for_the_rounds(pcs, ctx):
    """The per-kernel accounting that the benchmark's rooflines divide by:
    every round is counted with its launches and timed spans, steps and
    proposals match the job's own counters, and each ended generation adds
    its population bytes (and, after the prior pass, its pairwise kernel-sum
    FLOPs under pmc-standard weights)."""
    inp, _ = small_input(pcs, C=2)
    p = inp.params
    ctx.reset_kernel_stats()
    sim = pcs.make_simulation(ctx, inp, 11)
    for _ in range(3):
        sim.step()
    info = sim.info()
    sim.close()
    ks = ctx.kernel_stats()
    N, P = p.abc_sample_count, info.param_count
    assert ks.rounds > 0
    assert ks.kernel_launches == 9 * ks.rounds
    assert ks.simulate_launches == ks.rounds == ks.distance_launches == ks.pmc_launches
    assert ks.simulate_ms > 0 and ks.distance_ms > 0 and ks.pmc_ms > 0
    assert ks.simulate_ms + ks.distance_ms + ks.pmc_ms <= ks.round_ms * (1 + 1e-6)
    assert ks.particle_steps == info.particle_steps
    assert ks.proposals == info.simulations
    assert ks.generations == 3  # the prior pass and two generations
    assert ks.pmc_bytes == 3 * (2 * N * P * 8 + N * 8)
    assert ks.pmc_pair_flops == 2 * N * N * (6 * P + 7)


def test_round_distances_equal_the_standalone_kernels(pcs, ctx, oracle):
    """Every proposal of served rounds that mix histogram shapes -- two with
    tensor maps (61 x 48, 46 x 64) and two copied cell by cell (91 x 37 and
    121 x 130: B not a multiple of 4) -- carries the distance that the
    standalone kernels give: its
    histogram rebuilt from its Philox coordinates (simulate_hist) and scanned
    against its job's observed cumulative histogram (scan_distance), bit for
    bit, as the oracle's K_distance restatement gives on the rebuilt
    histogram."""
    import part_conc_spt_abc_gb300.workloads as W
    shapes = [(60, 48), (90, 37), (45, 64), (120, 130)]
    seeds = [300 + i for i in range(len(shapes))]
    jobs = [small_input(pcs, seed=20 + i, C=1 + i % 2, pop=48, frames=f, de_bins=b)[0]
            for i, (f, b) in enumerate(shapes)]
    srv = pcs.Server(ctx)
    sims = [pcs.make_simulation(ctx, inp, s) for inp, s in zip(jobs, seeds)]
    refs = []
    for inp in jobs:
        R, B = int(inp.frames.max()) + 1, inp.params.de_bin_count
        refs.append(pcs.observed_sat(ctx, inp.K, inp.DE, R, B, inp.params.ub_de))
    for s in sims:
        srv.submit(s)
    checked = 0
    try:
        for _ in range(6):
            if srv.step() == 0:
                break
            for inp, sim, seed, ref in zip(jobs, sims, seeds, refs):
                if srv.finished(sim):
                    continue
                props, _, counts = sim.round_proposals()
                C, Z = sim.info().component_count, sim.info().z_component_count
                setup = W.forward_setup(inp.frames, inp.params.de_bin_count, C=C)
                for q, pr in enumerate(props[:24]):
                    run = pcs.ForwardRun(counts[q], np.array(pr.half_az[:Z], np.float32),
                                         np.array(pr.pre_comp_prob[:C], np.float32),
                                         np.array(pr.sd_scale[:C], np.float32), np.array(pr.sd_shape[:C], np.float32),
                                         slot=pr.slot, trial=pr.trial, generation=pr.generation)
                    hist = pcs.simulate_hist(ctx, setup, run, seed=seed)[0]
                    d = pcs.scan_distance(ctx, hist, ref)["dist_f32"][0]
                    assert np.float32(pr.distance).tobytes() == np.float32(d).tobytes(), \
                        (inp.params.de_bin_count, pr.slot, pr.trial, pr.generation, pr.distance, d)
                    dw, _, _ = oracle.distance_kdist(hist, ref)
                    assert np.float32(dw).tobytes() == np.float32(d).tobytes()
                    checked += 1
    finally:
        for s in sims:
            s.close()
    assert checked >= 4 * 24

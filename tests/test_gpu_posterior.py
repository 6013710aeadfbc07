"""Posterior-level parity: the GPU engine against an independent CPU run of
the same ABC-PMC algorithm (oracle/abc_oracle.c: its own random numbers,
the Julia Poisson sampler, double weights), ten seeds each, on the same
synthetic observation.  Seed-averaged posterior means and 5%/95% quantiles
must agree within 2% of the prior range, and both must recover the truth.

Three problems: a small lognormal one with the oracle run live; and, from
tests/golden/posterior_cases.npz (the oracle's ten seeds, made by
tests/golden/make_posterior_golden.py), benchmark configuration 0 and the
reference's own discrete fixed-depth model with its delta schedule, shaped
like its test_files/input.xml."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEEDS = 10
GENERATIONS = 8
TRUTH = dict(mu=300.0, sd=20.0, conc_ml=3e8)
PRIOR = dict(m=(100.0, 800.0), s=(1.0, 60.0), c=(1e7, 1e9))


def wstats(x, w):
    o = np.argsort(x)
    xs, cw = x[o], np.cumsum(w[o])
    q = lambda p: xs[min(len(xs) - 1, np.searchsorted(cw, p))]  # noqa: E731
    return np.array([np.sum(w * x), q(0.05), q(0.95)])


@pytest.mark.parametrize("walk", [2, 1], ids=["step", "split"])
def test_posterior_matches_independent_cpu_run(pcs, ctx, oracle, walk):
    ctx.set_tuning(walk=walk)
    try:
        _posterior_case(pcs, ctx, oracle)
    finally:
        ctx.set_tuning(walk=2)


def _posterior_case(pcs, ctx, oracle):
    import part_conc_spt_abc_gb300.workloads as W
    inp, truth = W.make_problem(ctx, [TRUTH["mu"]], [TRUTH["sd"]], TRUTH["conc_ml"] * 1e6, [1.0], 8, 80, 48, 512,
                                GENERATIONS, seed=0, prior_mu=PRIOR["m"], prior_sd=PRIOR["s"])
    p = inp.params
    R, B = int(inp.frames.max()) + 1, p.de_bin_count
    sat = oracle.observed_sat(inp.K, inp.DE, R, B, p.ub_de)
    gpu, cpu = [], []
    for seed in range(1, SEEDS + 1):
        sim = pcs.make_simulation(ctx, inp, seed)
        sim.run()
        o = sim.output()
        sim.close()
        gpu.append(np.stack([wstats(o.m, o.w), wstats(o.s, o.w), wstats(np.log10(o.c), o.w)]))
        pb = dict(C=1, N=p.abc_sample_count, generations=GENERATIONS, kmin=2, quantile=0.5, lb_m=p.lb_m,
                  ub_m=p.ub_m, lb_s=p.lb_s, ub_s=p.ub_s, lb_c=p.lb_c, ub_c=p.ub_c, az=2.0, Lx=p.Lx, Ly=p.Ly, Lz=p.Lz,
                  ax=inp.ax, ay=inp.ay, deltat=inp.deltat, ub_de=p.ub_de, temperature=p.temperature,
                  viscosity=p.viscosity)
        th, w, _ = oracle.abc_pmc(pb, inp.frames, sat, 1000 + seed, os.cpu_count() or 4)
        cpu.append(np.stack([wstats(th[:, 0], w), wstats(th[:, 1], w), wstats(th[:, 2], w)]))
    g, c = np.mean(gpu, 0), np.mean(cpu, 0)
    ranges = np.array([PRIOR["m"][1] - PRIOR["m"][0], PRIOR["s"][1] - PRIOR["s"][0],
                       np.log10(PRIOR["c"][1]) - np.log10(PRIOR["c"][0])])
    rel = np.abs(g - c) / ranges[:, None]
    assert (rel <= 0.02).all(), f"GPU {g}\nCPU {c}\nrelative differences {rel}"
    truth = np.array([TRUTH["mu"], TRUTH["sd"], np.log10(TRUTH["conc_ml"])])
    for est in (g, c):
        assert abs(est[0, 0] - truth[0]) <= 0.1 * ranges[0], est
        assert abs(est[2, 0] - truth[2]) <= 0.1 * ranges[2], est
        assert (est[:, 1] <= truth).all() and (truth <= est[:, 2]).all(), est


# ---------------------------------------------------------------------------
# benchmark configuration 0 and the reference's discrete model, against the
# oracle's committed posteriors

def _fixture_input(pcs, case, hist):
    import part_conc_spt_abc_gb300.workloads as W
    t, pr = case["truth"], case["prior"]
    if case["model"] == 2:
        inp, _ = W.problem_from_hist(hist, t["m"], t["s"], sum(t["c"]) * 1e6, [1.0] * case["C"], case["V"],
                                     case["F"], case["N"], case["generations"], prior_mu=pr["m"], prior_sd=pr["s"],
                                     prior_conc_m3=(pr["c"][0] * 1e6, pr["c"][1] * 1e6),
                                     avg_trials=case["avg_trials"], quantile=case["quantile"])
        return inp
    K, DE = W.observed_from_hist(hist, case["ub_de"])
    p = pcs.params_defaults()
    p.model = pcs.MODEL_DISCRETE_FIXED_DEPTH
    p.component_count = case["C"]
    p.kmin = case["kmin"]
    p.de_bin_count = case["B"]
    p.abc_sample_count = case["N"]
    p.avg_trial_count = case["avg_trials"]
    p.gamma_adaptive = 1
    p.delta_gamma = case["delta_gamma"]
    p.schedule = pcs.SCHEDULE_DELTA
    p.reference_initial_gamma = case["full_az_prior"]
    p.Lx, p.Ly, p.Lz = case["box"]
    p.ub_de = case["ub_de"]
    p.lb_m, p.ub_m = pr["m"]
    p.lb_c, p.ub_c = pr["c"]
    p.lb_az, p.ub_az = pr["az"]
    p.max_generations = case["generations"]
    fr = np.full(case["V"], case["F"], np.uint64)
    return pcs.Input(p, case["area"][0], case["area"][1], case["dt"], fr, K, DE)


def _theta(case, out):
    N, Cc = case["N"], case["C"]
    cols = [out.m.reshape(N, Cc)]
    if case["model"] == 2:
        cols.append(out.s.reshape(N, Cc))
    cols.append(np.log10(out.c.reshape(N, Cc)))
    cols.append(out.az.reshape(N, -1)[:, :1])
    return np.concatenate(cols, axis=1)


@pytest.mark.parametrize("walk", [2, 1], ids=["step", "split"])
@pytest.mark.parametrize("name", ["config0", "discrete_fixed_depth"])
def test_posterior_matches_oracle_fixture(pcs, ctx, name, walk):
    ctx.set_tuning(walk=walk)
    try:
        _fixture_case(pcs, ctx, name)
    finally:
        ctx.set_tuning(walk=2)


def _fixture_case(pcs, ctx, name):
    import sys
    from conftest import GOLDEN
    sys.path.insert(0, GOLDEN)
    import posterior_cases as PC
    case = PC.CASES[name]
    z = np.load(os.path.join(GOLDEN, "posterior_cases.npz"))
    hist = z[f"{name}__hist"]
    cpu = z[f"{name}__summaries"]
    assert cpu.shape[0] == PC.SEEDS
    inp = _fixture_input(pcs, case, hist)
    gpu = []
    for seed in range(1, PC.SEEDS + 1):
        sim = pcs.make_simulation(ctx, inp, seed)
        sim.run()
        o = sim.output()
        info = sim.info()
        sim.close()
        assert info.iterations >= 1
        gpu.append(PC.summaries(_theta(case, o), o.w))
    g, c = np.mean(gpu, 0), cpu.mean(0)
    ranges = PC.prior_ranges(case)
    free = ranges > 0
    rel = np.abs(g - c)[free] / ranges[free][:, None]
    names = np.array(PC.param_names(case))[free]
    assert (rel <= 0.02).all(), f"{names}\nGPU {g[free]}\nCPU {c[free]}\nrelative differences {rel}"
    truth = PC.truth_vector(case)
    for est in (g, c):
        inside = (est[free, 1] <= truth[free]) & (truth[free] <= est[free, 2])
        assert inside.all(), (names, est[free], truth[free])

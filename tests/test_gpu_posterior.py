"""Posterior-level parity: the GPU engine against an independent CPU run of
the same ABC-PMC algorithm (oracle/abc_oracle.c: its own random numbers,
the Julia Poisson sampler, double weights), ten seeds each, on the same
synthetic observation, eight generations after the prior pass.  Seed-averaged
posterior means and 5%/95% quantiles must agree within 2% of the prior range,
and both must recover the truth."""
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

"""The two estimation problems of the posterior fixtures (posterior_cases.npz)
and the pieces shared by their generator and the test.

  config0               one lognormal component (175 nm, sd 10 nm, 2e14 m^-3),
                        20 videos x 200 frames, 201 x 100 bins over DE in
                        [0, 20) um^2/s, box 200 x 160 x 20 um, detection area
                        100 x 80 um and depth 2 um, dt 1/30 s, kmin 2; priors
                        m 50-1000 nm, s 1-100 nm, c 1e13-1e15 m^-3; population
                        256, 8 generations, epsilon = 50% quantile of the
                        previous generation's distances
  discrete_fixed_depth  the reference's own model and schedule, shaped like its
                        test_files/input.xml: two diffusivities (0.5 and 4.0
                        um^2/s), 1e9 and 1.5e9 particles/ml, one known depth
                        of 2 um; box 80 x 80 x 20 um, detection area 61.6448
                        um square and dt 0.068 s (its data file's), kmin 3,
                        1000 DE bins over [0, 5), priors m 0.1-5 and c
                        5e8-5e9 (input.xml's), population 1000 (input.xml's);
                        25 videos x 200 frames; gamma_0 = the prior pass's
                        upper median, then gamma -= 0.2 per generation for 10
                        generations (gamma_0 ~ 12.9 and the distance at the
                        truth ~ 10 in log10 units), trial cap 500 per slot

The observed histogram of each problem is the oracle's forward model
(orc_simulate_philox: the library's Philox streams) at the true parameters,
seed 0, with numpy's Poisson counts per video; the fixture stores it, so the
GPU side estimates from exactly the oracle's observation.
"""
from __future__ import annotations

import math

import numpy as np

KB = 1.380649e-23
SEEDS = 10

CASES = {
    "config0": dict(model=2, C=1, truth=dict(m=[175.0], s=[10.0], c=[2e8], az=[2.0]), V=20, F=200, B=100,
                    ub_de=20.0, kmin=2, box=(200.0, 160.0, 20.0), area=(100.0, 80.0), dt=1.0 / 30.0,
                    prior=dict(m=(50.0, 1000.0), s=(1.0, 100.0), c=(1e7, 1e9), az=(2.0, 2.0)), N=256,
                    generations=8, schedule=1, quantile=0.5, delta_gamma=0.0, avg_trials=500, full_az_prior=0),
    "discrete_fixed_depth": dict(model=0, C=2, truth=dict(m=[0.5, 4.0], c=[1e9, 1.5e9], az=[2.0]), V=25, F=200,
                                 B=1000, ub_de=5.0, kmin=3, box=(80.0, 80.0, 20.0), area=(61.6448, 61.6448),
                                 dt=0.068, prior=dict(m=(0.1, 5.0), c=(5e8, 5e9), az=(2.0, 2.0)), N=1000,
                                 generations=10, schedule=0, quantile=0.5, delta_gamma=0.2, avg_trials=500,
                                 full_az_prior=1),
}


def param_names(case):
    C = case["C"]
    names = [f"m{i + 1}" for i in range(C)]
    if case["model"] == 2:
        names += [f"s{i + 1}" for i in range(C)]
    return names + [f"log10c{i + 1}" for i in range(C)] + ["az"]


def prior_ranges(case):
    """Width of each parameter's prior box (log10 for concentrations)."""
    C, pr = case["C"], case["prior"]
    r = [pr["m"][1] - pr["m"][0]] * C
    if case["model"] == 2:
        r += [pr["s"][1] - pr["s"][0]] * C
    r += [math.log10(pr["c"][1]) - math.log10(pr["c"][0])] * C
    return np.array(r + [pr["az"][1] - pr["az"][0]])


def truth_vector(case):
    t = case["truth"]
    v = list(t["m"]) + (list(t["s"]) if case["model"] == 2 else []) + [math.log10(x) for x in t["c"]]
    return np.array(v + list(t["az"]))


def observed_hist(O, case):
    """The oracle's forward model at the truth, seed 0: R x B counts."""
    C, V, F, B, dt = case["C"], case["V"], case["F"], case["B"], case["dt"]
    t = case["truth"]
    vol_ml = case["box"][0] * case["box"][1] * case["box"][2] / 1e12
    lam = sum(t["c"]) * vol_ml
    parts = np.random.default_rng(0).poisson(lam, V).astype(np.uint32)
    fr = np.full(V, F, np.uint32)
    pre = np.cumsum(np.array(t["c"]) / sum(t["c"])).astype(np.float32)
    pre[-1] = 2.0
    f32 = lambda x: float(np.float32(x))  # noqa: E731
    if case["model"] == 2:
        g = math.sqrt(2.0 * dt * KB * 298.0 * 1e21 / (3.0 * math.pi * 0.95e-3))
        sc, sh = [], []
        for mu, sd in zip(t["m"], t["s"]):
            sl2 = math.log1p(sd * sd / (mu * mu))
            sc.append(np.float32(g * math.exp(-0.5 * (math.log(mu) - 0.5 * sl2))))
            sh.append(np.float32(-0.5 * math.sqrt(sl2)))
        rw = np.zeros(C, np.float32)
    else:
        rw = np.array([np.float32(math.sqrt(2.0 * m * dt)) for m in t["m"]], np.float32)
    st = O.Setup(case["model"], C, fr, parts, case["kmin"], f32(np.float32(4.0) * np.float32(dt)),
                 tuple(f32(np.float32(0.5) * np.float32(x)) for x in case["box"]),
                 tuple(f32(np.float32(0.5) * np.float32(x)) for x in case["area"]),
                 np.array([np.float32(0.5) * np.float32(t["az"][0])], np.float32), pre, rw,
                 f32(case["ub_de"] / B), F + 1, B)
    if case["model"] == 2:
        st.ln_scale[:C] = sc
        st.ln_shape[:C] = sh
    hist, _ = O.simulate_philox(st, 0)
    return hist


def oracle_problem(case):
    pr = case["prior"]
    return dict(C=case["C"], N=case["N"], generations=case["generations"], kmin=case["kmin"],
                quantile=case["quantile"], lb_m=pr["m"][0], ub_m=pr["m"][1], lb_s=pr.get("s", (0.0, 0.0))[0],
                ub_s=pr.get("s", (0.0, 0.0))[1], lb_c=pr["c"][0], ub_c=pr["c"][1], az=case["truth"]["az"][0],
                Lx=case["box"][0], Ly=case["box"][1], Lz=case["box"][2], ax=case["area"][0], ay=case["area"][1],
                deltat=case["dt"], ub_de=case["ub_de"], temperature=298.0, viscosity=0.95e-3,
                model=case["model"], schedule=case["schedule"], avg_trials=case["avg_trials"],
                full_az_prior=case["full_az_prior"], delta_gamma=case["delta_gamma"], lb_az=pr["az"][0],
                ub_az=pr["az"][1])


def summaries(theta, w):
    """[P, 3]: weighted mean and 5% / 95% weighted quantiles per parameter."""
    out = []
    for p in range(theta.shape[1]):
        x = theta[:, p]
        o = np.argsort(x, kind="stable")
        xs, cw = x[o], np.cumsum(w[o])
        q = lambda a: xs[min(len(xs) - 1, int(np.searchsorted(cw, a)))]  # noqa: E731
        out.append([float(np.sum(w * x)), q(0.05), q(0.95)])
    return np.array(out)

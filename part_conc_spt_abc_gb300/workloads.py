"""Synthetic estimation problems with the shapes of the benchmark
configurations (seeded; no external data exists for them).

The observed data of each problem is the forward model's own output at the
problem's true parameters (GPU, Philox streams, seed 0), turned into
per-track (K, DE) lists with DE at the centre of its bin, so the observed
cumulative histogram is exactly the simulated one.

  config0  1 lognormal component (175 nm, sd 10), 2e14 m^-3, 20 videos x 200
           frames, pop 256, epsilon = 50% quantile, 8 generations
  config1  2 components 175/500 nm (sd 10/25, weights 0.6/0.4), 5e14 m^-3,
           50 videos x 300 frames, R x B = 301 x 128, pop 1024, 12 generations
  config2  2 components U(100,800) nm, concentration prior spanning a mean
           of 50..5000 particles per video, 20 videos x 200 frames, 201 x 100
           bins, pop 512 (one 512-proposal round per launch)
  config3  3 components 100/250/600 nm (sd 5%, weights 0.3/0.4/0.3), 1e5
           particles per video, 100 videos x 1000 frames, 1001 x 256 bins,
           pop 4096, 10 generations
  serve_stream  64 jobs with 1-3 components, means U(100,800) nm, conc
           U(1e13,1e15) m^-3, 100-500 frames, 64-256 DE bins, pop 256-4096,
           6-12 generations, Poisson arrivals at 2 jobs/s
Box 200 x 160 x 20 um, detection area 100 x 80 um, depth 2 um, T = 298 K,
eta = 0.95e-3 Pa s, dt = 1/30 s, DE range 0..20 um^2/s, kmin = 2.
Concentrations in m^-3 are converted to the reference's particles/ml (x 1e-6).
"""
from __future__ import annotations

import math

import numpy as np

from . import (MODEL_LOGNORMAL, SCHEDULE_QUANTILE, ForwardRun, ForwardSetup, Input, params_defaults,
               simulate_hist)

KB = 1.380649e-23
BOX = (200.0, 160.0, 20.0)
AREA = (100.0, 80.0)
DEPTH = 2.0
T_K = 298.0
ETA = 0.95e-3
DT = 1.0 / 30.0
UB_DE = 20.0


def lognormal_sd_params(mu_nm, sd_nm, temperature=T_K, viscosity=ETA, dt=DT):
    """Per-component step-sd scale and shape of the lognormal diameter model:
    sd_step = scale * exp(shape * z), z ~ N(0,1) (mirrors the device
    computation in kernels_pmc.cu)."""
    g = math.sqrt(2.0 * dt * KB * temperature * 1e21 / (3.0 * math.pi * viscosity))
    scale, shape = [], []
    for mu, sd in zip(mu_nm, sd_nm):
        sl2 = math.log1p((sd * sd) / (mu * mu))
        mul = math.log(mu) - 0.5 * sl2
        scale.append(np.float32(g * math.exp(-0.5 * mul)))
        shape.append(np.float32(-0.5 * math.sqrt(sl2)))
    return np.array(scale, np.float32), np.array(shape, np.float32)


def forward_setup(frames, de_bins, kmin=2, box=BOX, area=AREA, dt=DT, ub_de=UB_DE, C=1):
    frames = np.asarray(frames, np.uint32)
    return ForwardSetup(MODEL_LOGNORMAL, C, frames, kmin, float(np.float32(4.0) * np.float32(dt)),
                        tuple(float(np.float32(0.5) * np.float32(x)) for x in box),
                        tuple(float(np.float32(0.5) * np.float32(x)) for x in area),
                        float(np.float32(ub_de / de_bins)), int(frames.max()) + 1, de_bins)


def lognormal_run(particles, mu, sd, weights, depth=DEPTH, slot=0, trial=0, generation=0):
    scale, shape = lognormal_sd_params(mu, sd)
    pre = np.cumsum(np.asarray(weights, float)).astype(np.float32)
    pre[-1] = 2.0
    return ForwardRun(np.asarray(particles, np.uint32), np.array([np.float32(0.5) * np.float32(depth)], np.float32),
                      pre, scale, shape, slot, trial, generation)


def observed_from_hist(hist: np.ndarray, ub_de: float):
    """(K, DE) track lists whose binned histogram is `hist` (DE at bin centres)."""
    R, B = hist.shape
    w = ub_de / B
    ks, bs = np.nonzero(hist)
    counts = hist[ks, bs].astype(np.int64)
    K = np.repeat(ks.astype(np.uint64), counts)
    DE = np.repeat((bs.astype(np.float64) + 0.5) * w, counts)
    return K, DE


def make_problem(ctx, mu, sd, conc_m3, weights, videos, frames, de_bins, pop, generations, seed=0,
                 prior_mu=(50.0, 1000.0), prior_sd=(1.0, 100.0), prior_conc_m3=(1e13, 1e15), avg_trials=500,
                 quantile=0.5):
    """Input for one estimation problem with synthetic observed data."""
    C = len(mu)
    vol_ml = BOX[0] * BOX[1] * BOX[2] / 1e12
    lam = conc_m3 * 1e-6 * vol_ml
    rng = np.random.default_rng(seed)
    parts = rng.poisson(lam, videos).astype(np.uint32)
    fr = np.full(videos, frames, np.uint32)
    setup = forward_setup(fr, de_bins, C=C)
    run = lognormal_run(parts, mu, sd, np.asarray(weights) / np.sum(weights))
    hist = simulate_hist(ctx, setup, run, seed=seed)[0]
    return problem_from_hist(hist, mu, sd, conc_m3, weights, videos, frames, pop, generations, prior_mu, prior_sd,
                             prior_conc_m3, avg_trials, quantile)


def problem_from_hist(hist, mu, sd, conc_m3, weights, videos, frames, pop, generations, prior_mu=(50.0, 1000.0),
                      prior_sd=(1.0, 100.0), prior_conc_m3=(1e13, 1e15), avg_trials=500, quantile=0.5):
    """Input for one lognormal estimation problem whose observed histogram
    (R x B, DE over [0, UB_DE)) is given."""
    C = len(mu)
    de_bins = hist.shape[1]
    fr = np.full(videos, frames, np.uint32)
    K, DE = observed_from_hist(hist, UB_DE)
    p = params_defaults()
    p.model = MODEL_LOGNORMAL
    p.component_count = C
    p.kmin = 2
    p.de_bin_count = de_bins
    p.abc_sample_count = pop
    p.avg_trial_count = avg_trials
    p.gamma_adaptive = 1
    p.Lx, p.Ly, p.Lz = BOX
    p.ub_de = UB_DE
    p.lb_m, p.ub_m = prior_mu
    p.lb_s, p.ub_s = prior_sd
    p.lb_c, p.ub_c = prior_conc_m3[0] * 1e-6, prior_conc_m3[1] * 1e-6
    p.lb_az = p.ub_az = DEPTH
    p.temperature, p.viscosity = T_K, ETA
    p.schedule = SCHEDULE_QUANTILE
    p.quantile = quantile
    p.max_generations = generations
    inp = Input(p, AREA[0], AREA[1], DT, fr.astype(np.uint64), K, DE)
    truth = dict(mu=list(mu), sd=list(sd), conc_ml=[conc_m3 * 1e-6 * w / sum(weights) for w in weights])
    return inp, truth


def config0(ctx, seed=0, generations=8):
    return make_problem(ctx, [175.0], [10.0], 2e14, [1.0], 20, 200, 100, 256, generations, seed)


def config1(ctx, seed=0, generations=12):
    return make_problem(ctx, [175.0, 500.0], [10.0, 25.0], 5e14, [0.6, 0.4], 50, 300, 128, 1024, generations, seed)


def config2(ctx, seed=0, generations=8):
    """512-proposal rounds with uneven Poisson means: two components with
    diameters drawn U(100, 800) nm, concentration prior spanning a mean of
    50..5000 particles per video (each component 25..2500), 20 videos x 200
    frames, 201 x 100 bins, population 512."""
    rng = np.random.default_rng(1000 + seed)
    mu = sorted(rng.uniform(100.0, 800.0, 2).tolist())
    vol_ml = BOX[0] * BOX[1] * BOX[2] / 1e12
    lam_to_m3 = 1e6 / vol_ml
    return make_problem(ctx, mu, [0.05 * m for m in mu], 1000.0 * lam_to_m3, [0.5, 0.5], 20, 200, 100, 512,
                        generations, seed, prior_mu=(100.0, 800.0), prior_sd=(1.0, 100.0),
                        prior_conc_m3=(25.0 * lam_to_m3, 2500.0 * lam_to_m3))


def config3(ctx, seed=0, generations=10):
    """1e5 particles per video in total; each component's concentration prior
    spans 1e4..1e5 particles per video, so prior-pass proposals average about
    1.2e5 particles per video (1.2e10 particle-steps each)."""
    conc = 1e5 / (BOX[0] * BOX[1] * BOX[2] / 1e12) * 1e6
    return make_problem(ctx, [100.0, 250.0, 600.0], [5.0, 12.5, 30.0], conc, [0.3, 0.4, 0.3], 100, 1000, 256,
                        4096, generations, seed, prior_conc_m3=(conc / 10, conc))


def serve_stream(ctx, n_jobs=64, seed=0, rate_per_s=2.0, pop_range=(256, 4096), gen_range=(6, 12),
                 frames_range=(100, 500), bins_range=(64, 256), videos=20):
    """Jobs of the serving stream and their arrival offsets (seconds).  At
    least 64 arrival gaps are drawn before the jobs, so a shorter stream's
    jobs are the first jobs of the 64-job stream."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate_per_s, max(n_jobs, 64)))[:n_jobs]
    arrivals -= arrivals[0]
    jobs = []
    for j in range(n_jobs):
        C = int(rng.integers(1, 4))
        mu = sorted(rng.uniform(100.0, 800.0, C).tolist())
        sd = [0.05 * m for m in mu]
        conc = float(rng.uniform(1e13, 1e15))
        w = rng.dirichlet(np.ones(C)).tolist()
        frames = int(rng.integers(frames_range[0], frames_range[1] + 1))
        bins = int(rng.integers(bins_range[0], bins_range[1] + 1))
        pop = int(rng.integers(pop_range[0], pop_range[1] + 1))
        gens = int(rng.integers(gen_range[0], gen_range[1] + 1))
        inp, truth = make_problem(ctx, mu, sd, conc, w, videos, frames, bins, pop, gens, seed=1000 + j,
                                  prior_mu=(100.0, 800.0))
        jobs.append((inp, truth, int(rng.integers(0, 2**31))))
    return jobs, arrivals

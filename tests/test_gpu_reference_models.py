"""The reference's own models end to end on the GPU engine: discrete
diffusion-coefficient mixtures with a fixed depth (discrete-fixed-depth) and
with a depth per component (discrete-variable-depth), the reference's delta
schedule (gamma -= delta_gamma per generation after the prior pass, with
gamma_adaptive) and both weighting schemes, on synthetic observed data from
the forward model at known parameters (the shape of the reference's own
input.xml: 80 x 80 x 20 um box, kmin 3, DE up to 5 um^2/s)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = 1.0 / 30.0
BOX = (80.0, 80.0, 20.0)
AREA = (40.0, 40.0)


def discrete_input(pcs, ctx, model, weighting=0, V=10, F=100, B=64, N=96, seed=0):
    import part_conc_spt_abc_gb300.workloads as W
    C = 2
    m_true = [0.92, 2.6]               # D [um^2/s] of 500 nm and 175 nm particles
    c_true = [4e8, 6e8]                # particles / ml
    az_true = [2.0, 2.0] if model == pcs.MODEL_DISCRETE_FIXED_DEPTH else [1.6, 2.4]
    vol_ml = BOX[0] * BOX[1] * BOX[2] / 1e12
    rng = np.random.default_rng(seed)
    parts = rng.poisson(sum(c_true) * vol_ml, V).astype(np.uint32)
    fr = np.full(V, F, np.uint32)
    setup = pcs.ForwardSetup(model, C, fr, 3, float(np.float32(4.0) * np.float32(DT)),
                             tuple(float(np.float32(0.5) * np.float32(x)) for x in BOX),
                             tuple(float(np.float32(0.5) * np.float32(x)) for x in AREA),
                             float(np.float32(5.0 / B)), F + 1, B)
    Z = 1 if model == pcs.MODEL_DISCRETE_FIXED_DEPTH else C
    half_az = np.array([np.float32(0.5) * np.float32(a) for a in az_true[:Z]], np.float32)
    pre = np.array([c_true[0] / sum(c_true), 2.0], np.float32)
    rwsd = np.array([np.float32(np.sqrt(2.0 * m * DT)) for m in m_true], np.float32)
    hist = pcs.simulate_hist(ctx, setup, pcs.ForwardRun(parts, half_az, pre, rwsd), seed=seed)[0]
    K, DE = W.observed_from_hist(hist, 5.0)
    p = pcs.params_defaults()
    p.model = model
    p.component_count = C
    p.kmin = 3
    p.de_bin_count = B
    p.abc_sample_count = N
    p.avg_trial_count = 100
    p.gamma_adaptive = 1
    p.gamma_initial = 15.0
    p.delta_gamma = 0.05
    p.weighting_scheme = weighting
    p.Lx, p.Ly, p.Lz = BOX
    p.ub_de = 5.0
    p.lb_m, p.ub_m = 0.1, 5.0
    p.lb_c, p.ub_c = 5e7, 5e9
    p.lb_az, p.ub_az = 0.5, 5.0
    p.max_generations = 5
    return pcs.Input(p, AREA[0], AREA[1], DT, fr.astype(np.uint64), K, DE), dict(m=m_true, c=c_true, az=az_true)


@pytest.mark.parametrize("model,weighting", [(0, 0), (1, 0), (1, 1)],
                         ids=["fixed-depth", "variable-depth", "variable-depth-inv-dist-sq"])
def test_reference_model_generations(pcs, ctx, model, weighting):
    inp, truth = discrete_input(pcs, ctx, model, weighting)
    p = inp.params
    sim = pcs.make_simulation(ctx, inp, 4)
    N, C = p.abc_sample_count, 2
    Z = 1 if model == 0 else C
    gammas = []
    for g in range(6):
        done = sim.step()
        o, info = sim.output(), sim.info()
        assert o.w.shape == (N,) and abs(o.w.sum() - 1.0) < 1e-9 and (o.w > 0).all()
        m = o.m.reshape(N, C)
        if g >= 1:
            assert (np.diff(m, axis=1) >= 0).all(), "components sorted by m"
            assert np.isfinite(o.dist).all()
        assert (m >= p.lb_m).all() and (m <= p.ub_m).all()
        lc = np.log10(o.c)
        assert (lc >= np.log10(p.lb_c) - 1e-9).all() and (lc <= np.log10(p.ub_c) + 1e-9).all()
        assert o.az.shape == (N * Z,) and (o.az >= p.lb_az).all() and (o.az <= p.ub_az).all()
        if done:
            break  # the cap stops before the next decrement: the output gamma is the last one used
        gammas.append(info.gamma)
    # delta schedule: after the prior pass, gamma drops by delta_gamma per generation
    steps = np.diff(gammas)
    assert len(steps) >= 2 and np.allclose(steps, -p.delta_gamma, atol=1e-9), gammas
    assert info.iterations == p.max_generations + 1 or info.converged
    sim.close()

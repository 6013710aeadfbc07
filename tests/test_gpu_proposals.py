"""The device's proposal construction (k_propose) against the oracle's FP64
restatement of the reference's proposal loop (src/gpu/detail/
simulation_impl.inl:256-347) on the same counter-based streams, and the
initial threshold against the reference's rule (compute_initial_gamma_,
:750-830: gamma_0 = nth_element at N/2 of the prior population's distances).

The population, cumulative weights and perturbation factor a round's
proposals are built from are read from a checkpoint taken right before the
round; the round's proposals are read back through
pcs_debug_round_proposals.  Compared per proposal: the parameters after the
weighted parent pick, the reflected perturbation and the sort by m (FP64,
1e-12 relative: CUDA's and the C library's log / sin / pow differ in the last
bits), the per-video Poisson counts (exact), and the float forward-model
arguments (within one ulp)."""
import numpy as np
import pytest

from test_gpu_pmc import small_input
from test_gpu_reference_models import discrete_input

pytestmark = pytest.mark.gpu

HEADER, SCALARS = 64, 72  # checkpoint.cpp: CkptHeader, CkptScalars


def parse(blob, N, P):
    a = np.frombuffer(blob, np.uint8)
    sc = a[HEADER:HEADER + SCALARS].tobytes()
    st = {"gamma": np.frombuffer(sc[:8], np.float64)[0]}
    st["generation"], st["pending"], st["iterations"], st["converged"], st["done"] = \
        np.frombuffer(sc[48:68], np.uint32).tolist()
    off = HEADER + SCALARS

    def take(n, dt):
        nonlocal off
        x = np.frombuffer(a[off:off + n * np.dtype(dt).itemsize].tobytes(), dt)
        off += n * np.dtype(dt).itemsize
        return x
    st["theta"] = take(N * P, np.float64).reshape(N, P)
    st["theta_new"] = take(N * P, np.float64).reshape(N, P)
    st["w"] = take(N, np.float64)
    st["wcum"] = take(N, np.float64)
    st["dist"] = take(N, np.float64)
    st["dist_new"] = take(N, np.float64)
    st["factor"] = take(P * P, np.float64).reshape(P, P)
    return st


def check_rounds(pcs, ctx, oracle, inp, seed, rounds):
    """Runs the job in the serve loop past its prior pass, then checks the
    proposals of `rounds` consecutive rounds against the oracle.  Returns the
    number of proposals checked and the Poisson means seen."""
    p = inp.params
    N = p.abc_sample_count
    sim = pcs.make_simulation(ctx, inp, seed)
    srv = pcs.Server(ctx)
    srv.submit(sim)
    P = None
    job = oracle.prop_job(p, len(inp.frames), inp.deltat, seed)
    try:
        for _ in range(100):  # the prior pass
            srv.step()
            P = sim.info().param_count
            if parse(sim.checkpoint(), N, P)["generation"] >= 1:
                break
        assert P == job.P
        checked, lambdas = 0, []
        for _ in range(rounds):
            if srv.finished(sim):
                break
            st = parse(sim.checkpoint(), N, P)
            srv.step()
            if srv.finished(sim):
                break
            props, theta, counts = sim.round_proposals()
            assert len(props) > 0
            for q, pr in enumerate(props):
                assert pr.generation == st["generation"] >= 1
                th, cn, op = oracle.build_proposal(job, st["theta"], st["wcum"], st["factor"], pr.slot, pr.trial,
                                                   pr.generation)
                np.testing.assert_allclose(theta[q], th, rtol=1e-12, atol=0, err_msg=f"slot {pr.slot} trial {pr.trial}")
                assert np.array_equal(counts[q], cn), (pr.slot, pr.trial, op.lambda_)
                assert pr.total_particles == op.total_particles
                for f in ("pre_comp_prob", "sd_scale", "sd_shape", "half_az"):
                    np.testing.assert_array_max_ulp(np.array(getattr(pr, f), np.float32),
                                                    np.array(getattr(op, f), np.float32), maxulp=1)
                lambdas.append(op.lambda_)
                checked += 1
        return checked, np.array(lambdas)
    finally:
        sim.close()


@pytest.mark.parametrize("perturbation", [0, 1], ids=["diagonal", "cholesky"])
def test_lognormal_proposals_match_oracle(pcs, ctx, oracle, perturbation):
    inp, _ = small_input(pcs, C=2, pop=64)
    inp.params.perturbation = perturbation
    inp.params.lb_c = 1e6  # particles/ml: Poisson means from ~0.6 per video up
    n, lam = check_rounds(pcs, ctx, oracle, inp, 23, 4)
    assert n >= 64
    # both Poisson samplers ran: inversion below a mean of 12, PTRS above
    assert (lam < 12).any() and (lam >= 12).any(), (lam.min(), lam.max())


@pytest.mark.parametrize("model", [0, 1], ids=["fixed-depth", "variable-depth"])
def test_discrete_proposals_match_oracle(pcs, ctx, oracle, model):
    inp, _ = discrete_input(pcs, ctx, model, N=64)
    n, lam = check_rounds(pcs, ctx, oracle, inp, 29, 4)
    assert n >= 64 and (lam >= 12).any()


@pytest.mark.parametrize("N", [64, 63, 4097])
def test_initial_gamma_is_the_upper_median_of_prior_distances(pcs, ctx, N):
    """Delta schedule (the reference's): after the prior pass gamma_0 is the
    element of rank N/2 of the prior population's distances
    (simulation_impl.inl:819-829), and the first main iteration has already
    lowered it by delta_gamma (:202-219)."""
    inp, _ = discrete_input(pcs, ctx, 0, N=N)
    p = inp.params
    sim = pcs.make_simulation(ctx, inp, 41)
    try:
        sim.step()  # prior pass
        st = parse(sim.checkpoint(), N, sim.info().param_count)
        d = st["dist_new"]
        assert np.isfinite(d).all()
        g0 = np.sort(d)[N // 2]
        assert g0 == np.partition(d, N // 2)[N // 2]
        assert sim.info().gamma == g0 - p.delta_gamma
        assert st["generation"] == 1
    finally:
        sim.close()


@pytest.mark.parametrize("N,q", [(50, 0.5), (3001, 0.3)])
def test_quantile_threshold_after_prior_pass(pcs, ctx, N, q):
    """Quantile schedule: epsilon for generation 1 is the element of rank
    floor(q N) of the prior distances, with no delta step; so is the next
    generation's, from the committed distances."""
    inp, _ = small_input(pcs, C=1, pop=N)
    inp.params.quantile = q
    sim = pcs.make_simulation(ctx, inp, 43)
    try:
        sim.step()
        st = parse(sim.checkpoint(), N, sim.info().param_count)
        assert sim.info().gamma == np.sort(st["dist_new"])[min(N - 1, int(np.floor(q * N)))]
        if not sim.step():
            st = parse(sim.checkpoint(), N, sim.info().param_count)
            assert sim.info().gamma == np.sort(st["dist"])[min(N - 1, int(np.floor(q * N)))]
    finally:
        sim.close()

"""The oracle, pinned: against the reference's own kernel code (golden
fixtures made by tests/golden/make_golden.py from oracle/_ref), against
published Philox known-answer vectors, and against the restated distance."""
import numpy as np
import pytest

from conftest import load_replay_cases


def test_philox_known_answers(oracle):
    # Random123 known-answer vectors for Philox4x32-10
    assert [hex(x) for x in oracle.philox([0, 0, 0, 0], [0, 0])] == ["0x6627e8d5", "0xe169c58d", "0xbc57ac4c", "0x9b00dbd8"]
    assert [hex(x) for x in oracle.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)] == ["0x408f276d", "0x41c83b0e", "0xa20bc7c6", "0x6d5451fd"]
    assert [hex(x) for x in oracle.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0])] == \
        ["0xd16cfe09", "0x94fdcceb", "0x5001e420", "0x24126ea1"]


def test_replay_matches_reference_golden(oracle):
    cases = load_replay_cases(oracle)
    assert len(cases) >= 8
    for name, st, seed, gold in cases:
        u, z, _ = oracle.replay_draws(seed, st.n_particles, st.stride)
        hist, (closed, recorded) = oracle.simulate_replay(st, u, z)
        assert np.array_equal(hist, gold), name
        assert recorded >= hist.sum()  # records with k == 0 land in row 0 only when kmin == 0


def test_replay_matches_reference_kernel_random(oracle):
    """Fresh random configurations against the host-compiled reference kernel."""
    if not oracle.ref_available():
        pytest.skip("oracle/_ref not built (reference tree absent)")
    rng = np.random.default_rng(3)
    for trial in range(6):
        model = trial % 2
        C = 1 + trial % 3
        V = 1 + trial
        frames = rng.integers(1, 50, V).astype(np.uint32)
        parts = rng.integers(0, 60, V).astype(np.uint32)
        pc = np.cumsum(np.ones(C) / C).astype(np.float32)
        pc[-1] = 2
        Z = 1 if model == 0 else C
        st = oracle.Setup(model, C, frames, parts, trial % 4, float(np.float32(0.2)), (6.0, 5.0, 1.5), (3.0, 2.5),
                          np.linspace(0.4, 1.0, Z).astype(np.float32), pc,
                          np.linspace(0.2, 0.6, C).astype(np.float32), float(np.float32(0.25)),
                          int(frames.max()) + 1, 24)
        u, z, _ = oracle.replay_draws(100 + trial, st.n_particles, st.stride)
        h1, _ = oracle.simulate_replay(st, u, z)
        h2 = oracle.ref_simulate_replay(st, u, z)
        assert np.array_equal(h1, h2)


def test_distance_golden(oracle):
    """The oracle's K_distance restatement against the reference's own
    kernel (kernel-distance.inl:81-241) built without FMA contraction and run
    on a GPU (tests/golden/make_distance_golden.py): float and double sums
    bit for bit, on every case of distance_inputs.py."""
    import os
    import sys
    from conftest import GOLDEN
    sys.path.insert(0, GOLDEN)
    import distance_inputs as D
    z = np.load(os.path.join(GOLDEN, "distance_cases.npz"))
    assert int(z["count"][0]) == len(D.CASES)
    for i, case in enumerate(D.CASES):
        assert str(z[f"c{i}_name"]) == case[0]
        hist, ref = D.case_arrays(case)
        d, cum, ssd = oracle.distance_kdist(hist, ref)
        assert np.float32(d).tobytes() == z[f"c{i}_ref_f32_nofma"][0].tobytes(), case[0]
        assert oracle.distance_kdist_f64(hist, ref) == z[f"c{i}_ref_f64_nofma"][0], case[0]
        assert int(z[f"c{i}_zeroed"][0]) == 1, "the reference kernel resets the histogram"
        assert np.array_equal(cum, D.sat(hist))
        diff = cum.astype(np.int64) - ref.astype(np.int64)
        assert ssd == int(np.sum(diff.astype(object) ** 2)), case[0]


def test_distance_fma_build_within_bound(oracle):
    """The reference as shipped (nvcc's default FMA contraction) differs from
    the contraction-free contract only within the float-summation bound."""
    import os
    import sys
    from conftest import GOLDEN
    sys.path.insert(0, GOLDEN)
    import distance_inputs as D
    z = np.load(os.path.join(GOLDEN, "distance_cases.npz"))
    differs = 0
    for i, (name, R, B, *_rest) in enumerate(D.CASES):
        for bits, key in ((24, "f32"), (53, "f64")):
            a, b = float(z[f"c{i}_ref_{key}_nofma"][0]), float(z[f"c{i}_ref_{key}_fma"][0])
            assert abs(a - b) <= D.fma_bound(R, B, a, bits), (name, key, a, b)
            differs += a != b
    assert differs > 0, "the two builds are expected to differ somewhere"


def test_distance_properties(oracle):
    """Prefix sums equal numpy's; the exact sum of squares agrees with the
    float sum within float rounding."""
    rng = np.random.default_rng(11)
    for R, B in [(5, 7), (64, 64), (100, 33)]:
        h = rng.integers(0, 5, (R, B)).astype(np.uint32)
        ref = np.cumsum(np.cumsum(rng.integers(0, 5, (R, B)), 0), 1).astype(np.uint32)
        d, cum, ssd = oracle.distance_kdist(h, ref)
        want = np.cumsum(np.cumsum(h.astype(np.uint64), 1), 0).astype(np.uint32)
        assert np.array_equal(cum, want)
        exact = float(((cum.astype(np.int64) - ref.astype(np.int64)) ** 2).sum())
        assert ssd == int(exact)
        assert abs(float(d) - exact) <= 1e-5 * exact + 1


def test_observed_sat_matches_numpy(oracle):
    rng = np.random.default_rng(2)
    R, B, ub = 51, 40, 5.0
    K = rng.integers(2, 50, 3000)
    DE = rng.uniform(0, 6.0, 3000)
    sat = oracle.observed_sat(K, DE, R, B, ub)
    H = np.zeros((R, B), np.uint64)
    w = ub / B
    for k, de in zip(K, DE):
        if de >= ub:
            continue
        H[k, int(de / w)] += 1
    assert np.array_equal(sat, np.cumsum(np.cumsum(H, 0), 1).astype(np.uint32))


def test_pmc_pieces(oracle):
    rng = np.random.default_rng(4)
    N, P = 20, 3
    th = rng.normal(size=(N, P))
    ths = rng.normal(size=(N, P))
    w = rng.dirichlet(np.ones(N))
    tau = np.sqrt(2 * th.var(0))
    import ctypes as C
    out = np.zeros(N)
    P_ = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    oracle.lib().orc_weights_pmc_standard(P_(ths), P_(th), P_(w), P_(tau), None, N, P, P_(out))
    ref = np.array([1 / sum(w[i] * np.prod([np.exp(-0.5 * ((ths[a, p] - th[i, p]) / tau[p]) ** 2) /
                                             (np.sqrt(2 * np.pi) * tau[p]) for p in range(P)]) for i in range(N))
                    for a in range(N)])
    np.testing.assert_allclose(out, ref / ref.sum(), rtol=1e-12)
    assert oracle.lib().orc_displace(0.5, 0.7, 0.0, 1.0) == pytest.approx(0.8)
    assert oracle.lib().orc_displace(0.5, -0.9, 0.0, 1.0) == pytest.approx(0.4)


def test_observed_sat_julia_matches_numpy_restatement(oracle):
    """estimate.jl:32-40 restated with numpy (ceil binning, K = 1..kmax rows)
    against the C oracle, including DE = 0, DE on bin edges and DE > ub."""
    rng = np.random.default_rng(12)
    kmax, B, ub = 57, 40, 8.0
    K = rng.integers(1, kmax + 1, 5000)
    DE = np.concatenate([rng.uniform(0, 9.0, 4970), np.zeros(10), np.arange(1, 21) * (ub / B)])
    want = np.zeros((kmax, B), np.int64)
    for k, de in zip(K, DE):
        idx = int(np.ceil(de / (ub / B)))
        if 1 <= idx <= B:
            want[k - 1, idx - 1] += 1
    want = np.cumsum(np.cumsum(want, 0), 1)
    got = oracle.observed_sat_julia(K, DE, kmax, B, ub)
    assert np.array_equal(got, want)
    with pytest.raises(ValueError):
        oracle.observed_sat_julia(np.array([0]), np.array([1.0]), kmax, B, ub)


def _ln_setup(oracle, mu, sd, parts, V=20, F=200, B=100):
    import math
    dt, kB, T, eta = 1 / 30, 1.380649e-23, 298.0, 0.95e-3
    g = math.sqrt(2 * dt * kB * T * 1e21 / (3 * math.pi * eta))
    sl2 = math.log1p(sd * sd / (mu * mu))
    mul = math.log(mu) - 0.5 * sl2
    st = oracle.Setup(2, 1, np.full(V, F, np.uint32), np.full(V, parts, np.uint32), 2,
                      float(np.float32(4) * np.float32(dt)), (100.0, 80.0, 10.0), (50.0, 40.0),
                      np.array([1.0], np.float32), np.array([2.0], np.float32), np.zeros(1, np.float32),
                      float(np.float32(20.0 / B)), F + 1, B)
    st.ln_scale = np.array([np.float32(g * math.exp(-0.5 * mul))] + [0] * 7, np.float32)
    st.ln_shape = np.array([np.float32(-0.5 * math.sqrt(sl2))] + [0] * 7, np.float32)
    return st


@pytest.mark.parametrize("mu,F", [(175.0, 200), (60.0, 100)])
def test_split_walk_has_the_per_step_distribution(oracle, mu, F):
    """The slab-split walk (x, y drawn per group as a sum and, near the
    detection slab, as a Gaussian bridge) against the per-step walk on
    independent streams: histogram total, mean track length and mean DE bin
    within 4 Monte-Carlo standard errors over 48 replicas each."""
    st = _ln_setup(oracle, mu, 10.0, 128, F=F)

    def moments(h):
        R, B = h.shape
        n = h.sum()
        return np.array([n, (h * np.arange(R)[:, None]).sum() / n, (h * np.arange(B)[None, :]).sum() / n])

    reps = 48
    a = np.array([moments(oracle.simulate_philox(st, 3, slot=s)[0]) for s in range(reps)])
    b = np.array([moments(oracle.simulate_philox(st, 4, slot=s, split=True)[0]) for s in range(reps)])
    se = np.sqrt(a.var(0, ddof=1) / reps + b.var(0, ddof=1) / reps)
    z = np.abs(a.mean(0) - b.mean(0)) / se
    assert (z < 4.0).all(), (a.mean(0), b.mean(0), z)


def test_oracle_proposal_against_its_distributions(oracle):
    """orc_build_proposal on many (slot, trial) streams: parents drawn in
    proportion to the weights (chi-square), every parameter in its prior box,
    components sorted by m, Poisson counts with the right mean and variance
    for a mean below 12 (inversion) and above (PTRS), and the prior pass
    taking the slot's own parameters."""
    from types import SimpleNamespace
    rng = np.random.default_rng(3)
    N, Cc = 40, 2
    par = SimpleNamespace(component_count=Cc, model=oracle.MODEL_LOGNORMAL, abc_sample_count=N, perturbation=0,
                          reference_initial_gamma=0, Lx=200.0, Ly=160.0, Lz=20.0, lb_m=50.0, ub_m=1000.0, lb_s=1.0,
                          ub_s=100.0, lb_c=1e7, ub_c=1e9, lb_az=2.0, ub_az=2.0, temperature=298.0,
                          viscosity=0.95e-3)
    job = oracle.prop_job(par, 16, 1 / 30, 77)
    P = job.P
    lo, hi = np.array(job.lo[:P]), np.array(job.hi[:P])
    theta = lo + (hi - lo) * rng.uniform(size=(N, P))
    w = rng.uniform(0.2, 1.0, N)
    w /= w.sum()
    wcum = np.cumsum(w)
    factor = np.diag(0.3 * (hi - lo))
    parents = np.zeros(N)
    for t in range(4000):
        th, cn, op = oracle.build_proposal(job, theta, wcum, factor, t % N, t // N, 3)
        parents[op.parent] += 1
        assert (th >= lo).all() and (th <= hi).all()
        assert th[0] <= th[1], "components sorted by m"
        assert op.total_particles == cn.sum()
    chi2 = ((parents - 4000 * w) ** 2 / (4000 * w)).sum()
    assert chi2 < 80, chi2  # 39 degrees of freedom: p ~ 1e-4
    for lc in (np.log10(3e7), np.log10(8e8)):  # lambda ~ 5.8 and ~ 154 per video
        th0 = theta.copy()
        th0[:, 4:6] = lc - np.log10(2.0)  # two components of half the concentration each
        cs = []
        for s in range(N):
            th, cn, op = oracle.build_proposal(job, th0, wcum, factor, s, 0, 0)
            assert np.array_equal(th, th0[s]), "the prior pass simulates the slot's own parameters"
            cs.append(cn)
        cs = np.concatenate(cs).astype(float)
        lam = op.lambda_
        se = np.sqrt(lam / cs.size)
        assert abs(cs.mean() - lam) < 4 * se, (lam, cs.mean())
        assert abs(cs.var() / lam - 1) < 0.15, (lam, cs.var())


@pytest.mark.parametrize("name", ["config0", "discrete_fixed_depth"])
def test_posterior_fixture_observation(oracle, name):
    """The committed posterior fixture: ten oracle seeds per case, each
    posterior's 5-95% interval containing the synthetic truth, and the
    observed histogram it was estimated from is the one the oracle's forward
    model gives today (so the GPU side estimates from the same data)."""
    import os
    import sys
    from conftest import GOLDEN
    sys.path.insert(0, GOLDEN)
    import posterior_cases as PC
    z = np.load(os.path.join(GOLDEN, "posterior_cases.npz"))
    case = PC.CASES[name]
    np.testing.assert_array_equal(z[f"{name}__hist"], PC.observed_hist(oracle, case))
    summ = z[f"{name}__summaries"]
    assert summ.shape == (PC.SEEDS, len(PC.param_names(case)), 3)
    free = PC.prior_ranges(case) > 0
    truth = PC.truth_vector(case)
    mean = summ.mean(0)
    assert ((mean[free, 1] <= truth[free]) & (truth[free] <= mean[free, 2])).all(), (mean, truth)

"""Parity of the sm_103a kernels with the oracle, through the C ABI.

Bit-exact: forward-model histograms on replayed draws (golden fixtures made
by the reference's own kernel code), prefix sums, float and double distances
in the reference reduction order, exact sums of squares, observed cumulative
histograms, raw Philox words.  Statistical: histograms on the product's own
random streams against the oracle on the same streams."""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, load_replay_cases

pytestmark = pytest.mark.gpu


def fwd(pcs, st, lognormal=None):
    setup = pcs.ForwardSetup(st.model if lognormal is None else 2, st.C, st.frames, st.kmin, st.four_delta_t,
                             st.half_l, st.half_a, st.dde, st.R, st.B)
    run = pcs.ForwardRun(st.particles, st.half_az, st.pre_comp_prob, st.rwsd if lognormal is None else lognormal[0],
                         None if lognormal is None else lognormal[1])
    return setup, run


@pytest.mark.parametrize("tile_rows", [0, 16, 4096])
def test_replay_golden_bit_exact(pcs, ctx, oracle, tile_rows):
    ctx.set_tuning(hist_tile_rows=tile_rows if tile_rows else 0xFFFFFFFF)
    try:
        for name, st, seed, gold in load_replay_cases(oracle):
            u, z, _ = oracle.replay_draws(seed, st.n_particles, st.stride)
            setup, run = fwd(pcs, st)
            got = pcs.simulate_hist(ctx, setup, run, replay=(u, z, None))[0]
            assert np.array_equal(got, gold), (name, int(got.sum()), int(gold.sum()))
    finally:
        ctx.set_tuning(hist_tile_rows=64)


def test_replay_lognormal_bit_exact(pcs, ctx, oracle):
    st = oracle.Setup(2, 2, np.array([80, 64, 90], np.uint32), np.array([70, 0, 55], np.uint32), 2, 0.2,
                      (10.0, 8.0, 2.0), (5.0, 4.0), np.array([0.75], np.float32),
                      np.array([0.4, 2.0], np.float32), np.zeros(2, np.float32), 0.1, 91, 40)
    u, z, sig = oracle.replay_draws(17, st.n_particles, st.stride, with_sigmas=True, base_sigma=0.5)
    want, _ = oracle.simulate_replay(st, u, z, sig)
    setup, run = fwd(pcs, st, lognormal=(np.array([0.4, 0.4], np.float32), np.zeros(2, np.float32)))
    got = pcs.simulate_hist(ctx, setup, run, replay=(u, z, sig))[0]
    assert want.sum() > 0 and np.array_equal(got, want)


def _distance_cases():
    sys.path.insert(0, GOLDEN)
    import distance_inputs as D
    return D, np.load(os.path.join(GOLDEN, "distance_cases.npz"))


def test_distance_golden_bit_exact(pcs, ctx, oracle):
    """Against the reference's own K_distance (kernel-distance.inl:81-241)
    built without FMA contraction and run on a GPU: float and double
    distances bit for bit; prefix sums and the exact integer sum of squares
    against numpy and the oracle."""
    D, zf = _distance_cases()
    for i, case in enumerate(D.CASES):
        h, ref = D.case_arrays(case)
        r = pcs.scan_distance(ctx, h, ref, want_cum=True, want_f64=True, want_ssd=True)
        assert r["dist_f32"][0].tobytes() == zf[f"c{i}_ref_f32_nofma"][0].tobytes(), case[0]
        assert r["dist_f64"][0] == zf[f"c{i}_ref_f64_nofma"][0], case[0]
        assert np.array_equal(r["cum"][0], D.sat(h)), case[0]
        assert r["ssd"][0] == oracle.distance_kdist(h, ref)[2], case[0]
        # the PMC rounds' variant (float sum only) gives the same float
        assert pcs.scan_distance(ctx, h, ref)["dist_f32"][0] == r["dist_f32"][0], case[0]


def test_distance_within_bound_of_shipped_reference(pcs, ctx):
    """The reference as it ships is compiled with nvcc's default FMA
    contraction (premake5.lua:76), which fuses `a2 += dd*dd`; this library
    keeps every product and sum a separate rounding.  The two differ at most
    by the float-summation bound of distance_inputs.fma_bound."""
    D, zf = _distance_cases()
    for i, case in enumerate(D.CASES):
        name, R, B = case[:3]
        h, ref = D.case_arrays(case)
        r = pcs.scan_distance(ctx, h, ref, want_f64=True)
        for got, key, bits in ((float(r["dist_f32"][0]), "f32", 24), (float(r["dist_f64"][0]), "f64", 53)):
            want = float(zf[f"c{i}_ref_{key}_fma"][0])
            assert abs(got - want) <= D.fma_bound(R, B, want, bits), (name, key, got, want)


@pytest.mark.parametrize("want_f64,want_ssd", [(False, True), (False, False), (True, False), (True, True)])
def test_distance_batch_and_sizes(pcs, ctx, oracle, want_f64, want_ssd):
    """Every kernel variant (with and without the double and exact-integer sums,
    which the PMC rounds leave out) gives the oracle's float distance."""
    rng = np.random.default_rng(8)
    for R, B in [(301, 128), (513, 7), (1001, 256), (2, 300), (2001, 40)]:  # 2001 rows: the row-block kernel
        n = 3
        hist = rng.poisson(0.7, (n, R, B)).astype(np.uint32)
        ref = np.cumsum(np.cumsum(rng.poisson(0.7, (R, B)), 0), 1).astype(np.uint32)
        r = pcs.scan_distance(ctx, hist, ref, want_f64=want_f64, want_ssd=want_ssd)
        for q in range(n):
            d, _, ssd = oracle.distance_kdist(hist[q], ref)
            assert r["dist_f32"][q].tobytes() == np.float32(d).tobytes(), (R, B, q)
            if want_ssd:
                assert r["ssd"][q] == ssd
            if want_f64:
                assert r["dist_f64"][q] == oracle.distance_kdist_f64(hist[q], ref), (R, B, q)


@pytest.mark.parametrize("R,B", [(61, 48), (301, 128), (120, 130), (257, 33), (45, 256), (200, 100), (1001, 256),
                                 (640, 70)])
def test_distance_cluster_and_strip_modes(pcs, ctx, oracle, R, B):
    """Launches whose histograms each get a cluster, and launches of tall
    histograms (512 rows or more), spread each histogram's strips of 32 bins
    over a thread-block cluster (one strip per CTA, row carries and per-lane
    sums exchanged through distributed shared memory; tall histograms
    outnumbering the clusters are taken in turn); other launches walk the
    strips in one CTA.  Every histogram gets the oracle's float distance bit
    for bit either way: two to eight strips, ragged last strips, with tensor
    maps and cell-by-cell copies (B % 4 != 0)."""
    rng = np.random.default_rng(R * 1000 + B)
    ref = np.cumsum(np.cumsum(rng.poisson(0.7, (R, B)), 0), 1).astype(np.uint32)
    n = 340  # at least the CTAs of one launch (<= 2 per SM): the strip walk
    hist = rng.poisson(0.7, (n, R, B)).astype(np.uint32)
    want = np.array([np.float32(oracle.distance_kdist(hist[q], ref)[0]) for q in range(n)])
    for count in (3, 150, n):
        got = pcs.scan_distance(ctx, hist[:count], ref)["dist_f32"]
        assert got.tobytes() == want[:count].tobytes(), (R, B, count)


@pytest.mark.parametrize("want_f64,want_ssd", [(False, False), (True, True)])
def test_distance_large_counts(pcs, ctx, oracle, want_f64, want_ssd):
    """Cumulative counts at and beyond 2^22 (where the strip kernel leaves
    its integer-difference form for the reference's two conversions) and
    beyond 2^24 (where those conversions round), in the simulated or only in
    the observed histogram, with even and odd bin counts."""
    rng = np.random.default_rng(11)
    for R, B, lam_h, lam_r in [(301, 128, 200.0, 0.7), (301, 128, 0.7, 200.0), (257, 33, 2000.0, 2000.0),
                               (120, 96, 400.0, 1.0)]:
        n = 2
        hist = rng.poisson(lam_h, (n, R, B)).astype(np.uint32)
        ref = np.cumsum(np.cumsum(rng.poisson(lam_r, (R, B)), 0), 1).astype(np.uint32)
        r = pcs.scan_distance(ctx, hist, ref, want_f64=want_f64, want_ssd=want_ssd)
        for q in range(n):
            d, _, ssd = oracle.distance_kdist(hist[q], ref)
            assert r["dist_f32"][q].tobytes() == np.float32(d).tobytes(), (R, B, q)
            if want_ssd:
                assert r["ssd"][q] == ssd
            if want_f64:
                assert r["dist_f64"][q] == oracle.distance_kdist_f64(hist[q], ref), (R, B, q)


def test_observed_sat_matches_oracle(pcs, ctx, oracle):
    rng = np.random.default_rng(5)
    R, B, ub = 1001, 1000, 5.0
    K = rng.integers(3, 1000, 38302)
    DE = rng.gamma(2.0, 0.6, 38302)
    np.testing.assert_array_equal(pcs.observed_sat(ctx, K, DE, R, B, ub), oracle.observed_sat(K, DE, R, B, ub))


def test_observed_sat_julia_matches_oracle(pcs, ctx, oracle):
    rng = np.random.default_rng(6)
    kmax, B, ub = 300, 128, 20.0
    K = rng.integers(1, kmax + 1, 40000)
    DE = np.concatenate([rng.gamma(2.0, 2.0, 39970), np.zeros(10), np.arange(1, 21) * (ub / B)])
    np.testing.assert_array_equal(pcs.observed_sat(ctx, K, DE, kmax, B, ub, julia=True),
                                  oracle.observed_sat_julia(K, DE, kmax, B, ub))
    with pytest.raises(pcs.PcsError):
        pcs.observed_sat(ctx, np.array([kmax + 1]), np.array([1.0]), kmax, B, ub, julia=True)


def test_philox_stream_layout(pcs, ctx, oracle):
    for seed, slot, trial, gen, n, blk in [(0, 0, 0, 0, 0, 0), (0xDEADBEEF12345678, 17, 3, 5, 999, 2),
                                           (42, 4095, 0xFFFFF, 4095, 123456, 77)]:
        got = pcs.debug_particle_stream(ctx, seed, slot, trial, gen, n, blk)
        # fixed key; the seed enters counter words 2 and 3 through splitmix64 masks
        M = (1 << 64) - 1
        z = (seed + 0x9E3779B97F4A7C15) & M
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        z ^= z >> 31
        ctr = [n, (0 << 28) | blk, slot ^ (z & 0xFFFFFFFF), ((gen << 20) | trial) ^ (z >> 32)]
        want = oracle.philox(ctr, [0xA4093822, 0x299F31D0])
        assert np.array_equal(got, want)


def _cfg0_setup(oracle, V=20, frames=200, parts=128, C=1):
    pc = np.array([2.0] if C == 1 else [0.6, 2.0], np.float32)
    rw = np.array([np.float32(np.sqrt(2 * 2.626 / 30))] + ([np.float32(np.sqrt(2 * 0.919 / 30))] if C == 2 else []),
                  np.float32)
    return oracle.Setup(0, C, np.full(V, frames, np.uint32), np.full(V, parts, np.uint32), 2,
                        float(np.float32(4) * np.float32(1 / 30)), (100.0, 80.0, 10.0), (50.0, 40.0),
                        np.array([1.0], np.float32), pc, rw, float(np.float32(20.0 / 100)), frames + 1, 100)


@pytest.fixture(params=[1, 2], ids=["split", "step"])
def walk(request, ctx):
    ctx.set_tuning(walk=request.param)
    yield request.param
    ctx.set_tuning(walk=2)


def test_philox_forward_model_matches_oracle_streams(pcs, ctx, oracle, walk):
    """Same Philox streams on both sides, for both walks; the GPU's fast-math
    Box-Muller differs in the last bits, so the histograms agree to a
    fraction of a percent, far inside Monte-Carlo noise."""
    st = _cfg0_setup(oracle, C=2)
    setup, run = fwd(pcs, st)
    runs = []
    for s in range(4):
        r = pcs.ForwardRun(st.particles, st.half_az, st.pre_comp_prob, st.rwsd, slot=s, trial=1, generation=2)
        runs.append(r)
    got = pcs.simulate_hist(ctx, setup, runs, seed=12345)
    for s in range(4):
        want, _ = oracle.simulate_philox(st, 12345, slot=s, trial=1, generation=2, split=walk == 1)
        tot = want.sum()
        assert tot > 1000
        assert abs(int(got[s].sum()) - int(tot)) <= 0.005 * tot + 5
        assert np.abs(got[s].astype(np.int64) - want).sum() <= 0.02 * tot + 10


def _moments(h):
    R, B = h.shape
    k = np.arange(R)[:, None]
    b = np.arange(B)[None, :]
    n = h.sum()
    return n, (h * k).sum() / n, (h * b).sum() / n


def test_lognormal_streams_match_oracle(pcs, ctx, oracle, walk):
    """Lognormal diameters (per-particle step sd from the size stream), both
    walks, ragged frame counts (every partial last group, a one-frame video)."""
    import part_conc_spt_abc_gb300.workloads as W
    frames = np.array([80, 1, 59, 2, 130], np.uint32)
    parts = np.array([900, 60, 750, 30, 1200], np.uint32)
    B = 48
    setup = W.forward_setup(frames, B, C=2)
    sc, sh = W.lognormal_sd_params([150.0, 400.0], [15.0, 30.0])
    pre = np.array([0.55, 2.0], np.float32)
    runs = [pcs.ForwardRun(parts, np.array([1.0], np.float32), pre, sc, sh, slot=s, trial=2, generation=1)
            for s in range(3)]
    got = pcs.simulate_hist(ctx, setup, runs, seed=99)
    st = oracle.Setup(2, 2, frames, parts, 2, setup.four_delta_t, setup.half_l, setup.half_a,
                      np.array([1.0], np.float32), pre, np.zeros(2, np.float32), setup.dde, setup.rows, B)
    st.ln_scale = np.array(list(sc) + [0] * 6, np.float32)
    st.ln_shape = np.array(list(sh) + [0] * 6, np.float32)
    for s in range(3):
        want, _ = oracle.simulate_philox(st, 99, slot=s, trial=2, generation=1, split=walk == 1)
        tot = want.sum()
        assert tot > 300
        assert abs(int(got[s].sum()) - int(tot)) <= 0.005 * tot + 5
        assert np.abs(got[s].astype(np.int64) - want).sum() <= 0.02 * tot + 10


def test_fresh_draws_moments_within_3_se(pcs, ctx, oracle, walk):
    """Histogram moments of the GPU path (either walk) within 3 Monte-Carlo
    standard errors of the oracle's per-step walk on independent draws at
    the same parameters: for the slab-split walk this checks it against the
    reference's step-by-step model."""
    st = _cfg0_setup(oracle)
    setup, run = fwd(pcs, st)
    reps = 24
    runs = [pcs.ForwardRun(st.particles, st.half_az, st.pre_comp_prob, st.rwsd, slot=s) for s in range(reps)]
    g = pcs.simulate_hist(ctx, setup, runs, seed=1)
    o = np.stack([oracle.simulate_philox(st, 99, slot=s)[0] for s in range(reps)])
    for stat in range(3):
        a = np.array([_moments(x)[stat] for x in g], float)
        b = np.array([_moments(x)[stat] for x in o], float)
        se = np.sqrt(a.var(ddof=1) / reps + b.var(ddof=1) / reps)
        assert abs(a.mean() - b.mean()) <= 3 * se + 1e-9, (stat, a.mean(), b.mean(), se)


def test_philox_determinism_and_independence(pcs, ctx, oracle, walk):
    st = _cfg0_setup(oracle, V=5, frames=120, parts=300)
    setup, run = fwd(pcs, st)
    a = pcs.simulate_hist(ctx, setup, [run, run], seed=7)
    b = pcs.simulate_hist(ctx, setup, [run], seed=7)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], a[0])
    c = pcs.simulate_hist(ctx, setup, [run], seed=8)
    assert not np.array_equal(b[0], c[0])
    # independent of the launch shape
    for kw in [dict(block_size=128, particles_per_thread=1), dict(block_size=512, particles_per_thread=2),
               dict(block_size=256, particles_per_thread=4, warp_aggregate=1),
               dict(block_size=256, particles_per_thread=8),
               dict(block_size=256, particles_per_thread=1, hist_tile_rows=0xFFFFFFFF),  # warp slices
               dict(block_size=1024, particles_per_thread=1, hist_tile_rows=0xFFFFFFFF, warp_aggregate=1)]:
        ctx.set_tuning(**kw)
        d = pcs.simulate_hist(ctx, setup, [run], seed=7)
        assert np.array_equal(d[0], b[0]), kw
    ctx.set_tuning(block_size=256, particles_per_thread=1, warp_aggregate=0xFFFFFFFF, hist_tile_rows=64)


def test_bad_arguments_raise(pcs, ctx, oracle):
    st = _cfg0_setup(oracle, V=2, frames=10, parts=5)
    setup, run = fwd(pcs, st)
    setup.rows = 5  # rows must exceed the frame count
    with pytest.raises(pcs.PcsError):
        pcs.simulate_hist(ctx, setup, run)
    # a launch shape the build for that walker count cannot run is refused
    # up front, not at launch
    with pytest.raises(pcs.PcsError, match="walkers per thread"):
        ctx.set_tuning(block_size=1024, particles_per_thread=2)
    with pytest.raises(pcs.PcsError, match="1, 2, 4 or 8"):
        ctx.set_tuning(particles_per_thread=3)
    ctx.set_tuning(block_size=256, particles_per_thread=1)

"""The device PMC step against the oracle's FP64 restatement, on the
populations the engine itself produced (read back from checkpoints taken
after consecutive generations): the perturbation factor (tau = sqrt(2 var)
per parameter, simulation_impl.inl:733-749, or the Cholesky factor of 2 x
the weighted covariance), the pmc-standard weights
(simulation_impl.inl:832-871; the device sums the kernel densities in FP32
log-sum-exp) and the cumulative weights."""
import ctypes as C

import numpy as np
import pytest

from test_gpu_pmc import small_input

pytestmark = pytest.mark.gpu

HEADER = 64   # magic, version, N, P, C, Z, V, R, B, model, pad, seed, bytes
SCALARS = 72  # gamma, 5 counters, 6 x u32


def parse(blob, N, P):
    a = np.frombuffer(blob, np.uint8)
    off = HEADER + SCALARS

    def take(n, dt):
        nonlocal off
        x = np.frombuffer(a[off:off + n * np.dtype(dt).itemsize].tobytes(), dt)
        off += n * np.dtype(dt).itemsize
        return x
    st = {}
    st["theta"] = take(N * P, np.float64).reshape(N, P)
    st["theta_new"] = take(N * P, np.float64).reshape(N, P)
    st["w"] = take(N, np.float64)
    st["wcum"] = take(N, np.float64)
    st["dist"] = take(N, np.float64)
    st["dist_new"] = take(N, np.float64)
    st["factor"] = take(P * P, np.float64).reshape(P, P)
    assert off + 3 * N * 4 == len(blob)
    return st


def _p(a):
    return np.ascontiguousarray(a, np.float64).ctypes.data_as(C.POINTER(C.c_double))


def run_two(pcs, ctx, perturbation):
    inp, _ = small_input(pcs, C=2, pop=64)
    inp.params.perturbation = perturbation
    sim = pcs.make_simulation(ctx, inp, 17)
    sim.step()  # prior pass
    sim.step()  # generation 1
    before = sim.checkpoint()
    sim.step()  # generation 2
    after = sim.checkpoint()
    sim.close()
    P = 7  # m1 m2 s1 s2 log10c1 log10c2 az
    return parse(before, 64, P), parse(after, 64, P), [6]


def test_diagonal_factor_and_weights(pcs, ctx, oracle):
    a, b, fixed = run_two(pcs, ctx, pcs.PERTURB_DIAGONAL)
    N, P = b["theta"].shape
    free = [p for p in range(P) if p not in fixed]
    L = oracle.lib()
    for p in range(P):
        col = np.ascontiguousarray(b["theta"][:, p])
        want = 0.0 if p in fixed else np.sqrt(2.0 * L.orc_var_uncorrected(_p(col), N, 1))
        assert b["factor"][p, p] == pytest.approx(want, rel=1e-12, abs=0.0), p
    assert np.count_nonzero(b["factor"] - np.diag(np.diag(b["factor"]))) == 0
    # weights of generation 2 from generation 1's population, weights and tau
    tau = np.ascontiguousarray(np.diag(a["factor"]))
    fx = (C.c_int * P)(*[1 if p in fixed else 0 for p in range(P)])
    w = np.zeros(N)
    L.orc_weights_pmc_standard(_p(b["theta"]), _p(a["theta"]), _p(a["w"]), _p(tau), fx, N, P, _p(w))
    np.testing.assert_allclose(b["w"], w, rtol=5e-4)
    np.testing.assert_allclose(b["wcum"], np.cumsum(b["w"]), rtol=1e-12)
    assert abs(b["w"].sum() - 1.0) < 1e-12 and free


def test_cholesky_factor(pcs, ctx, oracle):
    a, b, fixed = run_two(pcs, ctx, pcs.PERTURB_CHOLESKY)
    N, P = b["theta"].shape
    free = [p for p in range(P) if p not in fixed]
    th = np.ascontiguousarray(b["theta"][:, free])
    cov = np.zeros((len(free), len(free)))
    chol = np.zeros_like(cov)
    rc = oracle.lib().orc_weighted_cov_cholesky(_p(th), _p(b["w"]), N, len(free), 2.0, _p(cov), _p(chol))
    assert rc == 0
    got = b["factor"][np.ix_(free, free)]
    np.testing.assert_allclose(got, chol, rtol=1e-9, atol=1e-12)
    for p in fixed:
        assert not b["factor"][p].any() and not b["factor"][:, p].any()

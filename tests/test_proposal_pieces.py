"""The pieces of proposal construction that the host's plain path and
k_propose share (pcs_proposal.h), built from the library's header into a
small harness.  The Poisson sampler (inversion below lambda = 12, PTRS
transformed rejection above) follows the Poisson distribution (mean,
variance and a chi-square test against the pmf, seeded, so the outcome is
fixed), and computing its constants once per proposal gives the same draws
as computing them per draw; the Box-Muller pair is standard normal and
uncorrelated; the reflection is the reference's displace_ (the oracle's
restatement) wherever that terminates, and stays in the box beyond; the
parent pick is std::lower_bound clamped to N - 1.  The PTRS iteration's
FP32 filter decides exactly as the FP64 iteration wherever it decides (on
Philox draws and on draws placed at the tests' thresholds), so the filtered
sampler's draws equal the FP64 sampler's; a copy built with margins at 1%
of the library's shows that the comparison finds narrow margins."""
import ctypes as C
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "part_conc_spt_abc_gb300", "csrc")


def build_harness(tmp_path_factory, defines=()):
    cxx = shutil.which("g++")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if not cxx or not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA headers are missing")
    out = str(tmp_path_factory.mktemp("proposal") / "libproposal_pieces.so")
    subprocess.check_call([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", *defines, "-I", CSRC, "-I", cuda_inc,
                           os.path.join(ROOT, "tests", "harness", "proposal_pieces.cpp"), "-o", out])
    lib = C.CDLL(out)
    lib.ptrs_check.argtypes = [C.c_double, C.c_uint32, C.c_uint64, C.c_int, C.POINTER(C.c_uint64)]
    lib.ptrs_check.restype = None
    lib.poisson_filter_diffs.argtypes = [C.c_double, C.c_uint32, C.c_uint64]
    lib.poisson_filter_diffs.restype = C.c_uint32
    lib.draw_poisson.argtypes = [C.c_double, C.c_uint32, C.c_uint64, C.POINTER(C.c_uint32)]
    lib.draw_poisson.restype = None
    lib.draw_poisson_one.argtypes = [C.c_double, C.c_uint32, C.c_uint32, C.c_uint64]
    lib.draw_poisson_one.restype = C.c_uint32
    lib.reflect.argtypes = [C.c_double, C.c_double, C.c_double]
    lib.reflect.restype = C.c_double
    lib.pick.argtypes = [C.POINTER(C.c_double), C.c_uint32, C.c_double]
    lib.pick.restype = C.c_uint32
    lib.normals.argtypes = [C.c_uint32, C.c_uint64, C.POINTER(C.c_double)]
    lib.normals.restype = None
    return lib


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    return build_harness(tmp_path_factory)


def ptrs_check(lib, lam, n, seed, with_table=1):
    out = (C.c_uint64 * 4)()
    lib.ptrs_check(lam, n, seed, with_table, out)
    return dict(decided=out[0] / n, mismatches=int(out[1]), accepts=out[2] / n, filter_accepts=out[3] / n)


def draws(lib, lam, n, seed):
    out = np.zeros(n, np.uint32)
    lib.draw_poisson(lam, n, seed, out.ctypes.data_as(C.POINTER(C.c_uint32)))
    return out.astype(np.int64)


def log_pmf(k, lam):
    return k * math.log(lam) - lam - math.lgamma(k + 1)


@pytest.mark.parametrize("lam", [0.7, 4.0, 11.9, 12.0, 30.0, 320.0, 5000.0])
def test_draws_follow_the_poisson_distribution(harness, lam):
    n = 200_000
    x = draws(harness, lam, n, seed=17)
    se = math.sqrt(lam / n)
    assert abs(x.mean() - lam) < 5 * se, (x.mean(), lam)
    # variance: relative standard error ~ sqrt(2 / n) for large lambda
    assert abs(x.var() / lam - 1.0) < 6 * math.sqrt((2 + 1 / lam) / n), x.var()
    # chi-square against the pmf over the cells with expected count >= 20
    lo, hi = int(max(0, lam - 6 * math.sqrt(lam) - 2)), int(lam + 6 * math.sqrt(lam) + 3)
    ks = np.arange(lo, hi + 1)
    exp = n * np.exp([log_pmf(int(k), lam) for k in ks])
    keep = exp >= 20
    obs = np.bincount(np.clip(x - lo, 0, hi - lo + 1), minlength=hi - lo + 2)[:hi - lo + 1]
    chi2 = float((((obs - exp) ** 2) / exp)[keep].sum())
    dof = int(keep.sum()) - 1
    # 5-sigma upper bound of a chi-square with dof degrees of freedom
    assert chi2 < dof + 5 * math.sqrt(2 * dof), (chi2, dof)


def test_constants_once_per_proposal_give_the_same_draws(harness):
    for lam in (3.0, 12.0, 320.0, 2500.0):
        x = draws(harness, lam, 4096 * 3, seed=5)
        for i in (0, 1, 77, 4095, 4096, 4096 * 2 + 13):
            assert harness.draw_poisson_one(lam, i & 4095, i >> 12, 5) == x[i], (lam, i)


def test_non_positive_mean_draws_zero(harness):
    assert (draws(harness, 0.0, 100, seed=1) == 0).all()
    assert (draws(harness, -3.0, 100, seed=1) == 0).all()


def test_normal_pairs_are_standard_normal(harness):
    n = 100_000
    z = np.zeros(2 * n)
    harness.normals(n, 9, z.ctypes.data_as(C.POINTER(C.c_double)))
    a, b = z[0::2], z[1::2]
    for v in (a, b):
        assert abs(v.mean()) < 5 / math.sqrt(n) and abs(v.var() - 1) < 5 * math.sqrt(2 / n)
        # Kolmogorov-Smirnov distance to the standard normal cdf
        s = np.sort(v)
        cdf = 0.5 * (1 + np.vectorize(math.erf)(s / math.sqrt(2)))
        d = max(np.max(np.arange(1, n + 1) / n - cdf), np.max(cdf - np.arange(n) / n))
        assert d < 1.95 / math.sqrt(n), d  # 0.1% critical value
    assert abs(np.corrcoef(a, b)[0, 1]) < 5 / math.sqrt(n)


def test_reflection_matches_displace(harness, oracle):
    rng = np.random.default_rng(2)
    for _ in range(2000):
        lo = rng.uniform(-10, 10)
        hi = lo + rng.uniform(0.1, 5)
        x = rng.uniform(lo - 30, hi + 30)
        got = harness.reflect(x, lo, hi)
        assert lo <= got <= hi
        assert got == pytest.approx(oracle.lib().orc_displace(x, 0.0, lo, hi), abs=1e-9)
    # far outside the box: the bounded loop hands over to the closed-form fold
    for x in (1e6, -1e6, 123456.789):
        got = harness.reflect(x, 0.0, 1.0)
        assert 0.0 <= got <= 1.0


def test_parent_pick_is_lower_bound(harness):
    rng = np.random.default_rng(3)
    for N in (1, 2, 7, 1024, 1025):
        w = rng.choice([0.0, 1.0, 2.0], N)
        w[-1] += 1.0
        wcum = np.cumsum(w / w.sum())
        p = wcum.ctypes.data_as(C.POINTER(C.c_double))
        for u in list(rng.random(200)) + [0.0, float(wcum[0]), float(wcum[-1])]:
            want = min(int(np.searchsorted(wcum, u, side="left")), N - 1)
            assert harness.pick(p, N, u) == want, (N, u)


LAMS_PTRS = [12.0, 12.7, 55.5, 320.0, 1000.0, 4096.0, 25000.0, 1.0e5, 1.3e5, 1.0e6, 5.0e6]


@pytest.mark.parametrize("lam", LAMS_PTRS)
def test_ptrs_fp32_filter_decides_as_fp64(harness, lam):
    n = 2_000_000
    r = ptrs_check(harness, lam, n, seed=7)
    assert r["mismatches"] == 0, r
    if lam <= 1.0e5:
        # the filter carries most iterations (a quarter of the draws sit at thresholds)
        assert r["decided"] > 0.6, r
    # the same without the log-factorial table: the slow test stays in FP64
    r = ptrs_check(harness, lam, n // 4, seed=8, with_table=0)
    assert r["mismatches"] == 0, r
    assert harness.poisson_filter_diffs(lam, n // 4, 11) == 0


def test_ptrs_check_finds_narrow_margins(tmp_path_factory):
    weak = build_harness(tmp_path_factory, defines=("-DPCS_PTRS_MARGIN=0.01f",))
    bad = sum(ptrs_check(weak, lam, 1_000_000, seed=7)["mismatches"] for lam in (320.0, 4096.0, 1.0e5))
    assert bad > 0

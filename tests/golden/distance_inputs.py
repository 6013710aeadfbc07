"""Inputs of the distance fixtures (distance_cases.npz).

Every histogram is made from an integer hash (splitmix64) of its case seed
and cell index, so it is the same on every machine and numpy version and the
fixture stores only the case parameters and the reference kernel's results.

A case is (name, rows, bins, seed, hist, ref) with hist / ref each
(kind, max count, density in 1/256):
  kind "hist"  independent counts per cell, row 0 empty as in the forward
               model's histograms (no track has K = 0)
  kind "dense" the same without the empty row
  kind "zero"  all zero
  kind "same"  (ref only) the cumulative histogram of this case's histogram,
               so every difference is 0
The observed input to the distance is the 2-D inclusive prefix sum of the
ref counts, as the reference builds it (src/gpu/detail/simulation_impl.inl
:605-629).
"""
from __future__ import annotations

import numpy as np

M64 = np.uint64(0xFFFFFFFFFFFFFFFF)

# (name, rows, bins, seed, hist spec, ref spec)
CASES = [
    # the benchmark configurations' histogram shapes
    ("cfg0_201x100", 201, 100, 11, ("hist", 5, 80), ("hist", 3, 128)),
    ("cfg1_301x128", 301, 128, 12, ("hist", 7, 96), ("hist", 4, 128)),
    ("cfg3_1001x256", 1001, 256, 13, ("hist", 3, 64), ("hist", 3, 96)),
    # the reference data fixture's binning (test_files/input.xml: kmax 1000, 1000 DE bins)
    ("fixture_1001x1000", 1001, 1000, 14, ("hist", 2, 40), ("hist", 2, 60)),
    # ragged: bins and rows not multiples of 32, single row / column, taller than one strip tile
    ("ragged_37x5", 37, 5, 15, ("dense", 9, 200), ("dense", 9, 200)),
    ("ragged_65x33", 65, 33, 16, ("hist", 4, 128), ("dense", 4, 128)),
    ("exact_33x64", 33, 64, 17, ("dense", 3, 160), ("hist", 3, 160)),
    ("single_1x1", 1, 1, 18, ("dense", 50, 256), ("dense", 20, 256)),
    ("column_17x1", 17, 1, 19, ("dense", 6, 200), ("dense", 6, 200)),
    ("row_2x300", 2, 300, 20, ("dense", 6, 200), ("dense", 6, 200)),
    ("narrow_513x7", 513, 7, 21, ("hist", 5, 160), ("hist", 5, 160)),
    ("tall_1001x40", 1001, 40, 22, ("hist", 4, 128), ("hist", 4, 128)),
    ("taller_than_strip_2001x40", 2001, 40, 23, ("hist", 4, 128), ("hist", 4, 128)),
    # large counts: cumulative sums above 2^24, where float(cum) rounds
    ("large_counts_1001x256", 1001, 256, 24, ("dense", 200, 256), ("dense", 200, 256)),
    # edge cases: nothing simulated; simulated equal to observed
    ("empty_hist_301x128", 301, 128, 25, ("zero", 0, 0), ("hist", 4, 128)),
    ("equal_201x100", 201, 100, 26, ("hist", 5, 128), ("same", 0, 0)),
]


def splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser (Steele, Lea, Flood 2014) on uint64 arrays."""
    with np.errstate(over="ignore"):
        z = (x + np.uint64(0x9E3779B97F4A7C15)) & M64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & M64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & M64
        return z ^ (z >> np.uint64(31))


def counts(rows: int, bins: int, seed: int, salt: int, spec) -> np.ndarray:
    kind, vmax, density = spec
    if kind == "zero":
        return np.zeros((rows, bins), np.uint32)
    idx = np.arange(rows * bins, dtype=np.uint64)
    h = splitmix64(idx ^ np.uint64((seed << 40) | (salt << 32)))
    val = (h >> np.uint64(32)) % np.uint64(vmax + 1)
    keep = (h & np.uint64(0xFF)) < np.uint64(density)
    c = np.where(keep, val, np.uint64(0)).astype(np.uint32).reshape(rows, bins)
    if kind == "hist":
        c[0, :] = 0
    return c


def sat(c: np.ndarray) -> np.ndarray:
    """2-D inclusive prefix sum, wrapping like 32-bit unsigned arithmetic."""
    return (np.cumsum(np.cumsum(c.astype(np.uint64), 0), 1) & np.uint64(0xFFFFFFFF)).astype(np.uint32)


def case_arrays(case):
    """(histogram, observed cumulative histogram) of one case."""
    _, rows, bins, seed, hspec, rspec = case
    hist = counts(rows, bins, seed, 1, hspec)
    ref = sat(hist) if rspec[0] == "same" else sat(counts(rows, bins, seed, 2, rspec))
    return hist, ref


def fma_bound(rows: int, bins: int, dist: float, real_bits: int = 24) -> float:
    """Bound on |a - b| for two evaluations of K_distance's sum, one with
    every `a2 += dd*dd` rounded twice (multiply, add) and one contracted to
    a fused multiply-add.  The differences dd are the same in both.  All
    terms are non-negative, so each evaluation is within gamma_n * S of the
    exact sum S (Higham, Accuracy and Stability of Numerical Algorithms, 2nd
    ed., section 4.2), n being the most roundings a term passes through: its
    product, a column's ceil(rows/32) additions into a2, a lane's
    ceil(bins/32) additions into acc and two 5-step shuffle trees.  Hence
    |a - b| <= 2 gamma_n S, and S <= dist / (1 - gamma_n)."""
    u = 2.0 ** -real_bits
    n = 1 + -(-rows // 32) + -(-bins // 32) + 10
    g = n * u / (1 - n * u)
    return 2 * g * abs(dist) / (1 - g)

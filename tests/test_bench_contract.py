"""Host-side pieces of bench.py that its JSON line depends on and that a
CPU can check: the DRAM traffic figure parsed from the committed ncu summary
of the simulate kernel, the peaks fallback, and the algorithmic-operation
constants of the roofline."""
import importlib.util
import os

from conftest import ROOT


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_simulate_traffic_is_read_from_the_profile_summary():
    b = load_bench()
    per_ms = b.simulate_traffic(1.0)
    assert per_ms is not None and 1e5 < per_ms < 1e8  # bytes per ms of launch: well under 0.1% of HBM
    assert b.simulate_traffic(2.0) == 2 * per_ms


def test_peaks_and_roofline_constants():
    b = load_bench()
    peaks, src = b.measured_peaks()
    assert src in ("measured", "fallback") and peaks.get("hbm_gbs", 0) > 0
    # 0.75 Philox calls x 80 + 1.5 Box-Muller pairs x 14 + 32 walk operations
    assert b.OPS_PER_STEP == 0.75 * 80 + 1.5 * 14 + 32
    assert b.DIST_BYTES_PER_CELL == 12

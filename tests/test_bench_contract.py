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
    # per particle-step: 3 uniforms x 22 + 1.5 Box-Muller pairs x 12 + a 21-op step
    assert b.OPS_PER_STEP == 3 * 22 + 1.5 * 12 + 21
    # slab-split walk: (6 uniforms + 3 pairs + four z steps + summed x, y) / 4 steps;
    # a task: 8 uniforms + 4 pairs + bridge means + four x, y steps + bookkeeping
    assert b.OPS_SPLIT_STEP == (6 * 22 + 3 * 12 + 20 + 10) / 4
    assert b.OPS_SPLIT_TASK == 8 * 22 + 4 * 12 + 12 + 72 + 12
    assert b.DIST_BYTES_PER_CELL == 12


def test_job_sequence_steps_only_jobs_with_work():
    """Each step of the bench's job sequence advances a job that has not
    finished; a finished job hands over to the next seed, created on
    demand once the prepared ones are used."""
    from types import SimpleNamespace
    b = load_bench()
    made = []

    class FakeSim:
        def __init__(self, ctx, inp, seed):
            self.seed, self.left, self.closed = seed, 3 + seed % 2, False
            made.append(self)

        def step(self):
            assert self.left > 0, "stepped a finished job"
            self.left -= 1
            return self.left == 0

        def info(self):
            return SimpleNamespace(particle_steps=10 * (3 + self.seed % 2 - self.left), simulations=0, accepted=0)

        def close(self):
            self.closed = True

    P = SimpleNamespace(make_simulation=FakeSim)
    seq = b.JobSequence(P, None, None, seed0=1, prepare=2)
    assert len(made) == 2
    for _ in range(11):
        seq.step()
    assert seq.jobs_finished == 3 and len(made) == 3  # seeds 1 (4 steps), 2 (3), 3 (4): 11 steps
    seq.step()  # the fourth job, made on demand
    assert len(made) == 4 and seq.jobs_finished == 3
    assert seq.totals()[0] == 120
    seq.close()
    assert all(s.closed for s in made)

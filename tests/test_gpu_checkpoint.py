"""Checkpoint / resume of estimation jobs: a job restored from a checkpoint
continues exactly as the original (same populations, weights, distances,
counters), alone or inside the serve loop, and a checkpoint is refused by a
job of another shape or seed, or by one that has already run."""
import numpy as np
import pytest

from test_gpu_pmc import small_input

pytestmark = pytest.mark.gpu

FIELDS = ["m", "c", "az", "dist", "w", "s"]


def counters(info):
    return (info.iterations, info.trials, info.simulations, info.accepted, info.particle_steps, info.gamma,
            info.converged)


def test_resume_continues_exactly(pcs, ctx):
    inp, _ = small_input(pcs, C=2, pop=64)
    a = pcs.make_simulation(ctx, inp, 7)
    a.step()
    a.step()
    ck = a.checkpoint()
    a.step()
    a.step()
    want, want_info = a.output(), a.info()
    a.close()
    b = pcs.make_simulation(ctx, inp, 7)
    b.restore(ck)
    b.step()
    b.step()
    got, got_info = b.output(), b.info()
    b.close()
    for f in FIELDS:
        assert np.array_equal(getattr(want, f), getattr(got, f)), f
    assert counters(want_info) == counters(got_info)


def test_resume_inside_serve_loop(pcs, ctx):
    inp, _ = small_input(pcs, C=1, pop=48)
    other, _ = small_input(pcs, seed=3, C=2, pop=40)
    a = pcs.make_simulation(ctx, inp, 11)
    a.step()
    ck = a.checkpoint()
    a.run()
    want = a.output()
    a.close()
    srv = pcs.Server(ctx)
    b = pcs.make_simulation(ctx, inp, 11)
    b.restore(ck)
    o = pcs.make_simulation(ctx, other, 5)
    srv.submit(o)
    srv.submit(b)
    for _ in range(100000):
        if srv.step() == 0:
            break
    assert srv.finished(b)
    got = b.output()
    for f in FIELDS:
        assert np.array_equal(getattr(want, f), getattr(got, f)), f
    b.close()
    o.close()


def test_checkpoint_refusals(pcs, ctx):
    inp, _ = small_input(pcs, C=1, pop=32)
    fresh = pcs.make_simulation(ctx, inp, 1)
    with pytest.raises(pcs.PcsError):
        fresh.checkpoint()  # nothing has run
    fresh.step()
    ck = fresh.checkpoint()
    with pytest.raises(pcs.PcsError):
        fresh.restore(ck)  # already ran
    fresh.close()
    wrong_seed = pcs.make_simulation(ctx, inp, 2)
    with pytest.raises(pcs.PcsError):
        wrong_seed.restore(ck)
    wrong_seed.close()
    other, _ = small_input(pcs, C=2, pop=32)
    wrong_shape = pcs.make_simulation(ctx, other, 1)
    with pytest.raises(pcs.PcsError):
        wrong_shape.restore(ck)
    with pytest.raises(pcs.PcsError):
        wrong_shape.restore(ck[:100])
    wrong_shape.close()


def test_checkpoint_refused_by_other_parameters_or_observed_data(pcs, ctx):
    """Same shape and seed, but other prior bounds, frame interval,
    weighting, schedule quantile or observed data: refused.  Another
    generation cap is accepted (the resumed job obeys its own)."""
    import copy
    inp, _ = small_input(pcs, C=1, pop=32)
    a = pcs.make_simulation(ctx, inp, 3)
    a.step()
    ck = a.checkpoint()
    a.close()

    def variant(edit):
        v = copy.copy(inp)
        v.params = copy.copy(inp.params)
        edit(v)
        return v

    def set_param(name, value):
        return lambda v: setattr(v.params, name, value)

    refused = [set_param("ub_m", inp.params.ub_m * 1.01), set_param("lb_c", inp.params.lb_c * 2),
               set_param("weighting_scheme", 1), set_param("quantile", 0.4),
               lambda v: setattr(v, "deltat", inp.deltat * 1.001),
               lambda v: setattr(v, "DE", np.asarray(inp.DE) * 1.0000001)]
    for edit in refused:
        b = pcs.make_simulation(ctx, variant(edit), 3)
        with pytest.raises(pcs.PcsError, match="other parameters or observed data"):
            b.restore(ck)
        b.close()
    c = pcs.make_simulation(ctx, variant(set_param("max_generations", 2)), 3)
    c.restore(ck)
    c.close()

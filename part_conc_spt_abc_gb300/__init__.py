"""GB300-native ABC-PMC for nanoparticle size distribution and concentration
from single-particle tracking.

A thin Python mirror of the reference's interface over the C ABI in
``include/pcs.h`` (libpcs.so, sm_103a kernels + C++ runtime):

  load_input / write_output / load_output   accel's XML formats
                                            (src/gpu/shared/input.cpp, output.cpp)
  make_simulation(...).run() / .output()     Simulation (src/gpu/simulation.hpp:45-62)
  Server                                     continuous batching of jobs
  simulate_hist / scan_distance / observed_sat
                                             the hot-path kernels one call at a time
                                             (K_simulate_system, K_distance)

Every call goes to the CUDA library; nothing here computes on the CPU.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import (CudaError, PcsError, XMLLoadError, MODEL_DISCRETE_FIXED_DEPTH, MODEL_DISCRETE_VARIABLE_DEPTH,
                   MODEL_LOGNORMAL, WEIGHTING_PMC_STANDARD, WEIGHTING_INVERSE_DIST_SQ, SCHEDULE_DELTA,
                   SCHEDULE_QUANTILE, PERTURB_DIAGONAL, PERTURB_CHOLESKY, MAX_COMPONENTS, build, check, lib)

__all__ = [
    "Context", "Input", "Simulation", "Server", "load_input", "write_output", "load_output",
    "make_simulation", "simulate_hist", "scan_distance", "observed_sat", "params_defaults",
    "PcsError", "XMLLoadError", "CudaError", "build",
]

MODEL_NAMES = {MODEL_DISCRETE_FIXED_DEPTH: "discrete-fixed-depth",
               MODEL_DISCRETE_VARIABLE_DEPTH: "discrete-variable-depth", MODEL_LOGNORMAL: "lognormal"}
WEIGHTING_NAMES = {WEIGHTING_PMC_STANDARD: "pmc-standard", WEIGHTING_INVERSE_DIST_SQ: "inverse-distance-squared"}


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


def params_defaults() -> _lib.Params:
    p = _lib.Params()
    lib().pcs_params_defaults(C.byref(p))
    return p


class Context:
    """One GPU (pcs_open).  ``inflight`` is accel's -g queue count."""

    def __init__(self, device: int = 0, inflight: int = 0):
        h = C.c_void_p()
        check(lib().pcs_open(device, inflight, C.byref(h)), "pcs_open")
        self.h = h

    def close(self):
        if self.h:
            check(lib().pcs_close(self.h), "pcs_close")
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def tuning(self) -> _lib.Tuning:
        t = _lib.Tuning()
        check(lib().pcs_get_tuning(self.h, C.byref(t)), "pcs_get_tuning")
        return t

    def set_tuning(self, **kw):
        t = _lib.Tuning()
        for k, v in kw.items():
            setattr(t, k, v)
        check(lib().pcs_set_tuning(self.h, C.byref(t)), "pcs_set_tuning")

    def timer_start(self) -> None:
        check(lib().pcs_timer_start(self.h), "pcs_timer_start")

    def timer_stop(self) -> float:
        """Milliseconds on the context's stream since timer_start()."""
        ms = C.c_double(0)
        check(lib().pcs_timer_stop(self.h, C.byref(ms)), "pcs_timer_stop")
        return ms.value

    def kernel_stats(self) -> _lib.KernelStats:
        s = _lib.KernelStats()
        check(lib().pcs_get_kernel_stats(self.h, C.byref(s)), "pcs_get_kernel_stats")
        return s

    def reset_kernel_stats(self) -> None:
        check(lib().pcs_reset_kernel_stats(self.h), "pcs_reset_kernel_stats")

    def autotune(self, inp: "Input") -> _lib.Tuning:
        t = _lib.Tuning()
        obs, keep = inp.observed()
        check(lib().pcs_autotune(self.h, C.byref(inp.params), C.byref(obs), C.byref(t)), "pcs_autotune")
        del keep
        return t


# --------------------------------------------------------------------------
# inputs / outputs
# --------------------------------------------------------------------------

@dataclass
class Input:
    """input.xml + data.xml (input::Parameters, shared/input.hpp:27-53)."""
    params: _lib.Params
    ax: float
    ay: float
    deltat: float
    frames: np.ndarray          # uint64 [V]
    K: np.ndarray               # uint64 [n]
    DE: np.ndarray              # float64 [n]
    output_file_path: str = ""

    def observed(self):
        fr = np.ascontiguousarray(self.frames, np.uint64)
        K = np.ascontiguousarray(self.K, np.uint64)
        DE = np.ascontiguousarray(self.DE, np.float64)
        o = _lib.Observed(self.ax, self.ay, self.deltat, _p(fr, C.c_uint64), len(fr), _p(K, C.c_uint64),
                          _p(DE, C.c_double), len(K))
        return o, (fr, K, DE)


def load_input(input_path: str, data_path: str | None = None) -> Input:
    h = C.c_void_p()
    check(lib().pcs_input_load(input_path.encode(), data_path.encode() if data_path else None, C.byref(h)),
          "input::load")
    try:
        p = _lib.Params()
        o = _lib.Observed()
        out = C.c_char_p()
        check(lib().pcs_input_params(h, C.byref(p), C.byref(o), C.byref(out)), "pcs_input_params")
        fr = np.ctypeslib.as_array(o.frame_counts, (o.video_count,)).copy() if o.video_count else np.zeros(0, np.uint64)
        K = np.ctypeslib.as_array(o.K, (o.track_count,)).copy() if o.track_count else np.zeros(0, np.uint64)
        DE = np.ctypeslib.as_array(o.DE, (o.track_count,)).copy() if o.track_count else np.zeros(0, np.float64)
        return Input(p, o.ax, o.ay, o.deltat, fr, K, DE, out.value.decode())
    finally:
        lib().pcs_input_free(h)


@dataclass
class Output:
    """output::Output (shared/output.hpp:16-34); m/c/az flattened sample-major."""
    model: int
    weighting_scheme: int
    abc_sample_count: int
    component_count: int
    z_component_count: int
    m: np.ndarray
    c: np.ndarray
    az: np.ndarray
    dist: np.ndarray
    w: np.ndarray
    converged: bool
    gamma: float
    s: np.ndarray | None = None
    meta: list = field(default_factory=list)


def write_output(path: str, o: Output) -> None:
    keep = [(k.encode(), v.encode()) for k, v in o.meta]
    meta = (_lib.OutputMeta * max(1, len(keep)))(*[_lib.OutputMeta(k, v) for k, v in keep])
    arrs = [np.ascontiguousarray(x, np.float64) if x is not None else None for x in (o.m, o.s, o.c, o.az, o.dist, o.w)]
    args = []
    for a in arrs:
        args += [_p(a, C.c_double), 0 if a is None else len(a)]
    check(lib().pcs_output_write(path.encode(), o.model, o.weighting_scheme, o.abc_sample_count, o.component_count,
                                 o.z_component_count, meta, len(keep), int(bool(o.converged)), float(o.gamma), *args),
          "output::write")


def load_output(path: str) -> Output:
    h = C.c_void_p()
    check(lib().pcs_output_load(path.encode(), C.byref(h)), "output::load")
    try:
        v = _lib.OutputView()
        check(lib().pcs_output_get(h, C.byref(v)), "pcs_output_get")

        def arr(ptr, n):
            return np.ctypeslib.as_array(ptr, (n,)).copy() if n else np.zeros(0)

        meta = [(v.meta[i].key.decode(), v.meta[i].value.decode()) for i in range(v.meta_count)]
        return Output(v.model, v.weighting, v.abc_sample_count, v.component_count, v.z_component_count,
                      arr(v.m, v.nm), arr(v.c, v.nc), arr(v.az, v.naz), arr(v.dist, v.nd), arr(v.w, v.nw),
                      bool(v.converged), v.gamma, arr(v.s, v.ns) if v.ns else None, meta)
    finally:
        lib().pcs_output_free(h)


# --------------------------------------------------------------------------
# estimation jobs
# --------------------------------------------------------------------------

class Simulation:
    """make_simulation() result: run() / step() / output() (simulation.hpp:45-62)."""

    def __init__(self, ctx: Context, inp: Input, seed: int):
        self.ctx = ctx
        self.input = inp
        obs, keep = inp.observed()
        h = C.c_void_p()
        check(lib().pcs_job_create(ctx.h, C.byref(inp.params), C.byref(obs), seed, C.byref(h)), "make_simulation")
        del keep
        self.h = h

    def run(self, max_steps: int = 0) -> None:
        check(lib().pcs_job_run(self.h, max_steps), "Simulation::run")

    def run_plain(self, max_steps: int = 0, queues: int = 30) -> None:
        """The reference's one-proposal-per-launch schedule on these kernels."""
        check(lib().pcs_job_run_plain(self.h, max_steps, queues), "pcs_job_run_plain")

    def step(self) -> bool:
        done = C.c_int(0)
        check(lib().pcs_job_step(self.h, C.byref(done)), "pcs_job_step")
        return bool(done.value)

    def info(self) -> _lib.JobInfo:
        i = _lib.JobInfo()
        check(lib().pcs_job_info_get(self.h, C.byref(i)), "pcs_job_info_get")
        return i

    def output(self) -> Output:
        i = self.info()
        N, Cc, Z = i.abc_sample_count, i.component_count, i.z_component_count
        m = np.zeros(N * Cc)
        s = np.zeros(N * Cc)
        c = np.zeros(N * Cc)
        az = np.zeros(N * Z)
        d = np.zeros(N)
        w = np.zeros(N)
        check(lib().pcs_job_output(self.h, _p(m, C.c_double), _p(s, C.c_double), _p(c, C.c_double),
                                   _p(az, C.c_double), _p(d, C.c_double), _p(w, C.c_double)), "Simulation::output")
        p = self.input.params
        meta = [("simulator", "gpu"), ("iterations", str(i.iterations)), ("simulations", str(i.simulations))]
        return Output(p.model, p.weighting_scheme, N, Cc, Z, m, c, az, d, w, bool(i.converged), i.gamma,
                      s if p.model == MODEL_LOGNORMAL else None, meta)

    def checkpoint(self) -> bytes:
        """The job's state after its last round (exact resume point)."""
        n = C.c_size_t(0)
        check(lib().pcs_job_checkpoint(self.h, None, 0, C.byref(n)), "pcs_job_checkpoint")
        buf = C.create_string_buffer(n.value)
        check(lib().pcs_job_checkpoint(self.h, buf, n.value, C.byref(n)), "pcs_job_checkpoint")
        return buf.raw[:n.value]

    def restore(self, data: bytes) -> None:
        """Load a checkpoint into this job (created with the same parameters,
        observed data and seed, not yet run)."""
        buf = C.create_string_buffer(bytes(data), len(data))
        check(lib().pcs_job_restore(self.h, buf, len(data)), "pcs_job_restore")

    def round_proposals(self):
        """This job's proposals in the context's last round: (list of
        pcs_debug_proposal, theta [n, P], counts [n, V])."""
        n = C.c_uint32(0)
        check(lib().pcs_debug_round_proposals(self.h, 0, C.byref(n), None, None, None), "pcs_debug_round_proposals")
        i = self.info()
        P, V = i.param_count, len(self.input.frames)
        props = (_lib.DebugProposal * max(1, n.value))()
        theta = np.zeros((max(1, n.value), P))
        counts = np.zeros((max(1, n.value), V), np.uint32)
        check(lib().pcs_debug_round_proposals(self.h, n.value, C.byref(n), props, _p(theta, C.c_double),
                                              _p(counts, C.c_uint32)), "pcs_debug_round_proposals")
        return list(props)[:n.value], theta[:n.value], counts[:n.value]

    def close(self):
        if self.h:
            check(lib().pcs_job_destroy(self.h), "pcs_job_destroy")
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_simulation(ctx: Context, inp: Input, seed: int = 0) -> Simulation:
    return Simulation(ctx, inp, seed)


class Server:
    """Continuous batching: jobs are admitted as device memory allows and
    their generations share batched launches."""

    def __init__(self, ctx: Context, memory_cap: int = 0):
        self.ctx = ctx
        if memory_cap:
            check(lib().pcs_serve_set_memory_cap(ctx.h, memory_cap), "pcs_serve_set_memory_cap")

    def submit(self, sim: Simulation) -> None:
        check(lib().pcs_serve_submit(self.ctx.h, sim.h), "pcs_serve_submit")

    def step(self) -> int:
        n = C.c_uint32(0)
        check(lib().pcs_serve_step(self.ctx.h, C.byref(n)), "pcs_serve_step")
        return n.value

    def finished(self, sim: Simulation) -> bool:
        f = C.c_int(0)
        check(lib().pcs_serve_poll(self.ctx.h, sim.h, C.byref(f)), "pcs_serve_poll")
        return bool(f.value)


# --------------------------------------------------------------------------
# hot-path entry points
# --------------------------------------------------------------------------

@dataclass
class ForwardSetup:
    """SimulateSetup + recorder of one forward-model configuration."""
    model: int
    component_count: int
    frames: np.ndarray
    kmin: int
    four_delta_t: float
    half_l: tuple
    half_a: tuple
    dde: float
    rows: int
    de_bins: int

    def struct(self):
        fr = np.ascontiguousarray(self.frames, np.uint32)
        s = _lib.Setup(self.model, self.component_count, len(fr), self.kmin, self.four_delta_t, self.half_l[0],
                       self.half_l[1], self.half_l[2], self.half_a[0], self.half_a[1], self.dde, self.rows,
                       self.de_bins, _p(fr, C.c_uint32))
        return s, fr


@dataclass
class ForwardRun:
    """SimulateRun of one proposal plus its random-stream coordinates."""
    particles: np.ndarray
    half_az: np.ndarray
    pre_comp_prob: np.ndarray
    sd_scale: np.ndarray
    sd_shape: np.ndarray | None = None
    slot: int = 0
    trial: int = 0
    generation: int = 0


def simulate_hist(ctx: Context, setup: ForwardSetup, runs, seed: int = 0, replay=None) -> np.ndarray:
    """Forward model of each run; returns uint32 [len(runs), R, B]."""
    if isinstance(runs, ForwardRun):
        runs = [runs]
    s, keep_fr = setup.struct()
    arr = (_lib.Run * len(runs))()
    keep = []
    for i, r in enumerate(runs):
        parts = np.ascontiguousarray(r.particles, np.uint32)
        keep.append(parts)
        arr[i].particles = _p(parts, C.c_uint32)
        for k in range(MAX_COMPONENTS):
            arr[i].half_az[k] = float(r.half_az[k]) if k < len(r.half_az) else 0.0
            arr[i].pre_comp_prob[k] = float(r.pre_comp_prob[k]) if k < len(r.pre_comp_prob) else 2.0
            arr[i].sd_scale[k] = float(r.sd_scale[k]) if k < len(r.sd_scale) else 0.0
            arr[i].sd_shape[k] = float(r.sd_shape[k]) if r.sd_shape is not None and k < len(r.sd_shape) else 0.0
        arr[i].slot, arr[i].trial, arr[i].generation = r.slot, r.trial, r.generation
    rp = None
    if replay is not None:
        u, z, sig = replay
        u = np.ascontiguousarray(u, np.float32)
        z = np.ascontiguousarray(z, np.float32)
        sig = np.ascontiguousarray(sig, np.float32) if sig is not None else None
        keep += [u, z, sig]
        rp = _lib.Replay(_p(u, C.c_float), _p(z, C.c_float), z.shape[1], _p(sig, C.c_float) if sig is not None else None)
    out = np.zeros((len(runs), setup.rows, setup.de_bins), np.uint32)
    check(lib().pcs_simulate_hist(ctx.h, C.byref(s), arr, len(runs), seed, C.byref(rp) if rp is not None else None,
                                  _p(out, C.c_uint32)), "pcs_simulate_hist")
    return out


def scan_distance(ctx: Context, hist: np.ndarray, ref_sat: np.ndarray, want_cum: bool = False,
                  want_f64: bool = False, want_ssd: bool = False):
    """K_distance on each histogram (uint32 [n, R, B] or [R, B])."""
    h = np.ascontiguousarray(hist, np.uint32)
    if h.ndim == 2:
        h = h[None]
    n, R, B = h.shape
    ref = np.ascontiguousarray(ref_sat, np.uint32)
    cum = np.zeros_like(h) if want_cum else None
    d32 = np.zeros(n, np.float32)
    d64 = np.zeros(n, np.float64) if want_f64 else None
    ssd = np.zeros((n, 2), np.uint64) if want_ssd else None
    check(lib().pcs_scan_distance(ctx.h, _p(h, C.c_uint32), _p(ref, C.c_uint32), R, B, n,
                                  _p(cum, C.c_uint32) if cum is not None else None, _p(d32, C.c_float),
                                  _p(d64, C.c_double) if d64 is not None else None,
                                  _p(ssd, C.c_uint64) if ssd is not None else None), "pcs_scan_distance")
    res = {"dist_f32": d32}
    if cum is not None:
        res["cum"] = cum
    if d64 is not None:
        res["dist_f64"] = d64
    if ssd is not None:
        res["ssd"] = [(int(a) << 64) | int(b) for a, b in ssd]
    return res


def observed_sat(ctx: Context, K, DE, rows: int, bins: int, ub_de: float, julia: bool = False) -> np.ndarray:
    """Observed cumulative histogram on the device; julia=True uses the Julia
    path's conventions (rows = kmax for K = 1..kmax, ceil binning)."""
    K = np.ascontiguousarray(K, np.uint32)
    DE = np.ascontiguousarray(DE, np.float64)
    out = np.zeros((rows, bins), np.uint32)
    fn = lib().pcs_observed_sat_julia if julia else lib().pcs_observed_sat
    check(fn(ctx.h, _p(K, C.c_uint32), _p(DE, C.c_double), len(K), rows, bins, ub_de, _p(out, C.c_uint32)),
          "pcs_observed_sat")
    return out


def debug_particle_stream(ctx: Context, seed: int, slot: int, trial: int, generation: int, particle: int,
                          block: int) -> np.ndarray:
    out = np.zeros(4, np.uint32)
    check(lib().pcs_debug_particle_stream(ctx.h, seed, slot, trial, generation, particle, block,
                                          _p(out, C.c_uint32)), "pcs_debug_particle_stream")
    return out

"""ctypes bindings for the CPU oracle (oracle/liborcl.so) and, where it was
built, the host-compiled reference (oracle/_ref/libpcsref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the ``cpu_baseline`` leg of ``bench.py``, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liborcl.so")
REF_SO = os.path.join(HERE, "_ref", "libpcsref.so")

MAXC = 8
MODEL_FIXED_Z, MODEL_VARIABLE_Z, MODEL_LOGNORMAL = 0, 1, 2

_u32p = C.POINTER(C.c_uint32)
_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)
_u64p = C.POINTER(C.c_uint64)


class OrcSetup(C.Structure):
    _fields_ = [
        ("model", C.c_uint32), ("component_count", C.c_uint32), ("video_count", C.c_uint32),
        ("kmin", C.c_uint32), ("four_delta_t", C.c_float), ("half_lx", C.c_float),
        ("half_ly", C.c_float), ("half_lz", C.c_float), ("half_ax", C.c_float),
        ("half_ay", C.c_float), ("dde", C.c_float), ("rows", C.c_uint32), ("de_bins", C.c_uint32),
    ]


class OrcRun(C.Structure):
    _fields_ = [
        ("frames", _u32p), ("particles", _u32p), ("half_az", C.c_float * MAXC),
        ("pre_comp_prob", C.c_float * MAXC), ("rand_walk_stddev", C.c_float * MAXC),
        ("ln_scale", C.c_float * MAXC), ("ln_shape", C.c_float * MAXC),
    ]


class OrcReplay(C.Structure):
    _fields_ = [("uniforms", _f32p), ("normals", _f32p), ("normal_stride", C.c_uint32),
                ("sigmas", _f32p)]


class OrcCounts(C.Structure):
    _fields_ = [("closed", C.c_uint64), ("recorded", C.c_uint64)]


class OrcCpuJob(C.Structure):
    _fields_ = [
        ("C", C.c_uint32), ("lognormal", C.c_int32), ("m", C.c_double * MAXC), ("s", C.c_double * MAXC),
        ("c", C.c_double * MAXC), ("az", C.c_double * MAXC), ("temperature", C.c_double),
        ("viscosity", C.c_double), ("ax", C.c_double), ("ay", C.c_double), ("Lx", C.c_double),
        ("Ly", C.c_double), ("Lz", C.c_double), ("deltat", C.c_double), ("ub_de", C.c_double),
        ("kmin", C.c_uint32), ("B", C.c_uint32), ("V", C.c_uint32), ("frames", _u32p),
    ]


def build(quiet: bool = True) -> None:
    """Compile the oracle (and, when the reference tree is present, oracle/_ref)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-s", "-C", HERE], check=True, stdout=out)
    subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], check=True, stdout=out)
    subprocess.run(["bash", os.path.join(HERE, "build_ref_kdist.sh"), "prepare"], check=True, stdout=out)


def reference_root():
    """The reference tree: $PCS_REFERENCE_ROOT, else the tree build_ref.sh
    compiled oracle/_ref from (recorded in oracle/_ref/reference_root), else
    None.  Only fixture scripts and host-side tests use it."""
    env = os.environ.get("PCS_REFERENCE_ROOT")
    if env:
        return env
    try:
        with open(os.path.join(HERE, "_ref", "reference_root")) as f:
            root = f.read().strip()
    except OSError:
        return None
    return root if root and os.path.isdir(root) else None


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = C.CDLL(ORACLE_SO)
        L.orc_philox4x32_10.argtypes = [_u32p, _u32p, _u32p]
        L.orc_replay_draws.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, _f32p, _f32p, _f32p, C.c_float]
        L.orc_simulate_replay.argtypes = [C.POINTER(OrcSetup), C.POINTER(OrcRun), C.POINTER(OrcReplay), _u32p, C.POINTER(OrcCounts)]
        L.orc_simulate_replay.restype = C.c_int
        L.orc_simulate_philox.argtypes = [C.POINTER(OrcSetup), C.POINTER(OrcRun), C.c_uint64, C.c_uint32,
                                          C.c_uint32, C.c_uint32, _u32p, C.POINTER(OrcCounts)]
        L.orc_simulate_philox.restype = C.c_int
        L.orc_simulate_philox_split.argtypes = L.orc_simulate_philox.argtypes
        L.orc_simulate_philox_split.restype = C.c_int
        L.orc_observed_sat.argtypes = [_u32p, _f64p, C.c_size_t, C.c_uint32, C.c_uint32, C.c_double, _u32p]
        L.orc_observed_sat_julia.argtypes = L.orc_observed_sat.argtypes
        L.orc_observed_sat_julia.restype = C.c_int
        L.orc_observed_sat.restype = C.c_int
        L.orc_distance_kdist.argtypes = [_u32p, _u32p, C.c_uint32, C.c_uint32, _u32p, _u64p, _u64p]
        L.orc_distance_kdist.restype = C.c_float
        L.orc_distance_kdist_f64.argtypes = [_u32p, _u32p, C.c_uint32, C.c_uint32]
        L.orc_distance_kdist_f64.restype = C.c_double
        L.orc_var_uncorrected.argtypes = [_f64p, C.c_size_t, C.c_size_t]
        L.orc_var_uncorrected.restype = C.c_double
        L.orc_normpdf.argtypes = [C.c_double, C.c_double, C.c_double]
        L.orc_normpdf.restype = C.c_double
        L.orc_displace.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double]
        L.orc_displace.restype = C.c_double
        L.orc_weights_pmc_standard.argtypes = [_f64p, _f64p, _f64p, _f64p, C.POINTER(C.c_int), C.c_size_t, C.c_size_t, _f64p]
        L.orc_weights_inv_dist_sq.argtypes = [_f64p, C.c_size_t, _f64p]
        L.orc_weighted_cov_cholesky.argtypes = [_f64p, _f64p, C.c_size_t, C.c_size_t, C.c_double, _f64p, _f64p]
        L.orc_weighted_cov_cholesky.restype = C.c_int
        L.orc_simulate_julia.argtypes = [C.c_uint32, _f64p, _f64p, C.c_double, C.c_double, _f64p,
                                         C.c_double, C.c_double, C.c_double, _u32p, _u32p, C.c_uint32,
                                         C.c_double, C.c_uint32, C.c_uint32, C.c_double, C.c_void_p, _i64p]
        L.orc_simulate_julia.restype = C.c_int
        L.orc_distance_julia.argtypes = [_i64p, _i64p, C.c_uint32, C.c_uint32]
        L.orc_distance_julia.restype = C.c_double
        L.orc_cpu_forward_batch.argtypes = [C.POINTER(OrcCpuJob), C.c_uint32, C.c_uint32, C.c_uint64,
                                            C.POINTER(C.c_double), C.POINTER(C.c_uint64)]
        L.orc_cpu_forward_batch.restype = C.c_uint64
        _lib = L
    return _lib


def cpu_forward_batch(jobs, frames, nthreads: int, seed: int = 1):
    """Times the Julia-convention forward model over `jobs` (list of dicts
    with C, lognormal, m, s, c, az, temperature, viscosity, ax, ay, Lx, Ly,
    Lz, deltat, ub_de, kmin, B) on nthreads threads.  Returns (steps, seconds)."""
    fr = np.ascontiguousarray(frames, np.uint32)
    arr = (OrcCpuJob * len(jobs))()
    for i, j in enumerate(jobs):
        a = arr[i]
        a.C, a.lognormal = j["C"], int(j.get("lognormal", 0))
        for k in range(j["C"]):
            a.m[k], a.c[k] = j["m"][k], j["c"][k]
            a.s[k] = j.get("s", [0.0] * MAXC)[k]
        for k, v in enumerate(j["az"]):
            a.az[k] = v
        for f in ["temperature", "viscosity", "ax", "ay", "Lx", "Ly", "Lz", "deltat", "ub_de"]:
            setattr(a, f, float(j.get(f, 0.0)))
        a.kmin, a.B, a.V = j["kmin"], j["B"], len(fr)
        a.frames = ptr(fr, C.c_uint32)
    secs = C.c_double(0)
    cs = C.c_uint64(0)
    steps = lib().orc_cpu_forward_batch(arr, len(jobs), nthreads, seed, C.byref(secs), C.byref(cs))
    return int(steps), float(secs.value)


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_SO)
        R.ref_simulate_replay.argtypes = [C.c_int, C.c_uint, C.c_uint, C.c_uint, C.c_float, _f32p, _f32p,
                                          _u32p, _u32p, _f32p, _f32p, _f32p, C.c_float, C.c_uint,
                                          C.c_uint, _f32p, _f32p, C.c_uint, _u32p, C.c_char_p, C.c_size_t]
        R.ref_simulate_replay.restype = C.c_int
        _ref = R
    return _ref


def ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


# --------------------------------------------------------------------------
# Problem description shared by the oracle, the reference harness and tests
# --------------------------------------------------------------------------

@dataclass
class Setup:
    """One forward-model call: SimulateSetup + SimulateRun + recorder."""
    model: int
    C: int
    frames: np.ndarray          # uint32 [V]
    particles: np.ndarray       # uint32 [V]
    kmin: int
    four_delta_t: float
    half_l: tuple
    half_a: tuple
    half_az: np.ndarray         # float32 [Z]
    pre_comp_prob: np.ndarray   # float32 [C]
    rwsd: np.ndarray            # float32 [C]
    dde: float
    R: int
    B: int
    ln_scale: np.ndarray = field(default_factory=lambda: np.zeros(MAXC, np.float32))
    ln_shape: np.ndarray = field(default_factory=lambda: np.zeros(MAXC, np.float32))

    @property
    def V(self) -> int:
        return int(len(self.frames))

    @property
    def n_particles(self) -> int:
        return int(np.sum(self.particles, dtype=np.uint64))

    @property
    def stride(self) -> int:
        return max(1, int(np.max(self.frames)) - 1) if len(self.frames) else 1


def replay_draws(seed: int, n: int, stride: int, with_sigmas: bool = False, base_sigma: float = 0.4):
    u = np.zeros((max(n, 1), 4), np.float32)
    z = np.zeros((max(n, 1), stride, 3), np.float32)
    s = np.zeros(max(n, 1), np.float32) if with_sigmas else None
    lib().orc_replay_draws(seed, n, stride, ptr(u, C.c_float), ptr(z, C.c_float),
                           ptr(s, C.c_float) if s is not None else None, base_sigma)
    return u, z, s


def _structs(st: Setup):
    s = OrcSetup(st.model, st.C, st.V, st.kmin, st.four_delta_t, st.half_l[0], st.half_l[1],
                 st.half_l[2], st.half_a[0], st.half_a[1], st.dde, st.R, st.B)
    frames = np.ascontiguousarray(st.frames, np.uint32)
    parts = np.ascontiguousarray(st.particles, np.uint32)
    r = OrcRun()
    r.frames = ptr(frames, C.c_uint32)
    r.particles = ptr(parts, C.c_uint32)
    for i, v in enumerate(st.half_az):
        r.half_az[i] = float(v)
    for i in range(st.C):
        r.pre_comp_prob[i] = float(st.pre_comp_prob[i])
        r.rand_walk_stddev[i] = float(st.rwsd[i])
        r.ln_scale[i] = float(st.ln_scale[i])
        r.ln_shape[i] = float(st.ln_shape[i])
    return s, r, (frames, parts)


def simulate_replay(st: Setup, u, z, sig=None):
    s, r, keep = _structs(st)
    rp = OrcReplay(ptr(u, C.c_float), ptr(z, C.c_float), z.shape[1],
                   ptr(sig, C.c_float) if sig is not None else None)
    hist = np.zeros((st.R, st.B), np.uint32)
    cnt = OrcCounts()
    rc = lib().orc_simulate_replay(C.byref(s), C.byref(r), C.byref(rp), ptr(hist, C.c_uint32), C.byref(cnt))
    if rc != 0:
        raise RuntimeError(f"orc_simulate_replay failed: {rc}")
    return hist, (cnt.closed, cnt.recorded)


def simulate_philox(st: Setup, seed: int, slot: int = 0, trial: int = 0, generation: int = 0, split: bool = False):
    """Forward model on the product's Philox streams; split=True is the
    slab-split walk, False the per-step walk."""
    s, r, keep = _structs(st)
    hist = np.zeros((st.R, st.B), np.uint32)
    cnt = OrcCounts()
    fn = lib().orc_simulate_philox_split if split else lib().orc_simulate_philox
    rc = fn(C.byref(s), C.byref(r), seed, slot, trial, generation, ptr(hist, C.c_uint32), C.byref(cnt))
    if rc != 0:
        raise RuntimeError(f"orc_simulate_philox failed: {rc}")
    return hist, (cnt.closed, cnt.recorded)


def ref_simulate_replay(st: Setup, u, z):
    hist = np.zeros((st.R, st.B), np.uint32)
    err = C.create_string_buffer(512)
    frames = np.ascontiguousarray(st.frames, np.uint32)
    parts = np.ascontiguousarray(st.particles, np.uint32)
    hl = np.asarray(st.half_l, np.float32)
    ha = np.asarray(st.half_a, np.float32)
    hz = np.ascontiguousarray(st.half_az, np.float32)
    pc = np.ascontiguousarray(st.pre_comp_prob, np.float32)
    rw = np.ascontiguousarray(st.rwsd, np.float32)
    rc = ref().ref_simulate_replay(st.model, st.C, st.V, st.kmin, st.four_delta_t, ptr(hl, C.c_float),
                                   ptr(ha, C.c_float), ptr(frames, C.c_uint32), ptr(parts, C.c_uint32),
                                   ptr(hz, C.c_float), ptr(pc, C.c_float), ptr(rw, C.c_float), st.dde,
                                   st.R, st.B, ptr(u, C.c_float), ptr(z, C.c_float), z.shape[1],
                                   ptr(hist, C.c_uint32), err, 512)
    if rc != 0:
        raise RuntimeError(err.value.decode())
    return hist


def observed_sat(K, DE, R, B, ub_de):
    K = np.ascontiguousarray(K, np.uint32)
    DE = np.ascontiguousarray(DE, np.float64)
    sat = np.zeros((R, B), np.uint32)
    rc = lib().orc_observed_sat(ptr(K, C.c_uint32), ptr(DE, C.c_double), len(K), R, B, ub_de, ptr(sat, C.c_uint32))
    if rc != 0:
        raise ValueError("observed track outside the histogram")
    return sat


def observed_sat_julia(K, DE, kmax, B, ub_de):
    """Observed cumulative histogram in the Julia path's conventions."""
    K = np.ascontiguousarray(K, np.uint32)
    DE = np.ascontiguousarray(DE, np.float64)
    sat = np.zeros((kmax, B), np.uint32)
    rc = lib().orc_observed_sat_julia(ptr(K, C.c_uint32), ptr(DE, C.c_double), len(K), kmax, B, ub_de,
                                      ptr(sat, C.c_uint32))
    if rc != 0:
        raise ValueError("observed track length outside 1..kmax")
    return sat


def distance_kdist(hist, ref_sat):
    hist = np.ascontiguousarray(hist, np.uint32)
    ref_sat = np.ascontiguousarray(ref_sat, np.uint32)
    R, B = hist.shape
    cum = np.zeros_like(hist)
    hi, lo = C.c_uint64(0), C.c_uint64(0)
    d = lib().orc_distance_kdist(ptr(hist, C.c_uint32), ptr(ref_sat, C.c_uint32), R, B,
                                 ptr(cum, C.c_uint32), C.byref(hi), C.byref(lo))
    return np.float32(d), cum, (int(hi.value) << 64) | int(lo.value)


def distance_kdist_f64(hist, ref_sat):
    hist = np.ascontiguousarray(hist, np.uint32)
    ref_sat = np.ascontiguousarray(ref_sat, np.uint32)
    R, B = hist.shape
    return lib().orc_distance_kdist_f64(ptr(hist, C.c_uint32), ptr(ref_sat, C.c_uint32), R, B)


def philox(ctr, key):
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    lib().orc_philox4x32_10(ptr(c, C.c_uint32), ptr(k, C.c_uint32), ptr(out, C.c_uint32))
    return out


class OrcAbcProblem(C.Structure):
    _fields_ = [
        ("C", C.c_uint32), ("N", C.c_uint32), ("generations", C.c_uint32), ("kmin", C.c_uint32),
        ("V", C.c_uint32), ("R", C.c_uint32), ("B", C.c_uint32), ("quantile", C.c_double),
        ("lb_m", C.c_double), ("ub_m", C.c_double), ("lb_s", C.c_double), ("ub_s", C.c_double),
        ("lb_c", C.c_double), ("ub_c", C.c_double), ("az", C.c_double), ("Lx", C.c_double), ("Ly", C.c_double),
        ("Lz", C.c_double), ("ax", C.c_double), ("ay", C.c_double), ("deltat", C.c_double), ("ub_de", C.c_double),
        ("temperature", C.c_double), ("viscosity", C.c_double), ("frames", _u32p), ("ref_sat", _u32p),
        ("model", C.c_uint32), ("schedule", C.c_uint32), ("avg_trials", C.c_uint32), ("full_az_prior", C.c_uint32),
        ("delta_gamma", C.c_double), ("lb_az", C.c_double), ("ub_az", C.c_double),
    ]


def abc_pmc(problem: dict, frames, ref_sat, seed: int, nthreads: int, full: bool = False):
    """Whole ABC-PMC estimation on the CPU (abc_oracle.c).  `problem` holds
    OrcAbcProblem fields; model defaults to lognormal and schedule to the
    quantile one.  Returns (theta [N, P] with layout m | s | log10c | az
    (lognormal) or m | log10c | az (discrete), w [N], trials), plus
    (generations committed, converged) when full."""
    L = lib()
    L.orc_abc_pmc.argtypes = [C.POINTER(OrcAbcProblem), C.c_uint64, C.c_uint32, _f64p, _f64p,
                              C.POINTER(C.c_uint32), C.POINTER(C.c_int)]
    L.orc_abc_pmc.restype = C.c_uint64
    fr = np.ascontiguousarray(frames, np.uint32)
    sat = np.ascontiguousarray(ref_sat, np.uint32)
    pb = OrcAbcProblem()
    pb.model, pb.schedule = MODEL_LOGNORMAL, 1
    for k, v in problem.items():
        setattr(pb, k, v)
    pb.V, pb.R, pb.B = len(fr), sat.shape[0], sat.shape[1]
    pb.frames = ptr(fr, C.c_uint32)
    pb.ref_sat = ptr(sat, C.c_uint32)
    P = (3 if pb.model == MODEL_LOGNORMAL else 2) * problem["C"] + 1
    th = np.zeros((problem["N"], P))
    w = np.zeros(problem["N"])
    gens, conv = C.c_uint32(0), C.c_int(0)
    trials = L.orc_abc_pmc(C.byref(pb), seed, nthreads, ptr(th, C.c_double), ptr(w, C.c_double), C.byref(gens),
                           C.byref(conv))
    if full:
        return th, w, int(trials), int(gens.value), bool(conv.value)
    return th, w, int(trials)


class OrcPropJob(C.Structure):
    _fields_ = [("model", C.c_uint32), ("C", C.c_uint32), ("Z", C.c_uint32), ("P", C.c_uint32),
                ("N", C.c_uint32), ("V", C.c_uint32), ("perturbation", C.c_uint32), ("full_az_prior", C.c_uint32),
                ("seed", C.c_uint64), ("lo", C.c_double * 32), ("hi", C.c_double * 32),
                ("volume_factor", C.c_double), ("delta_t", C.c_double), ("sd_const", C.c_double)]


class OrcProposal(C.Structure):
    _fields_ = [("parent", C.c_uint32), ("total_particles", C.c_uint32), ("lambda_", C.c_double),
                ("half_az", C.c_float * MAXC), ("pre_comp_prob", C.c_float * MAXC),
                ("sd_scale", C.c_float * MAXC), ("sd_shape", C.c_float * MAXC)]


def prop_job(params, V: int, deltat: float, seed: int) -> OrcPropJob:
    """orc_prop_job of a job with pcs_params-like `params` (attributes model,
    component_count, abc_sample_count, perturbation, reference_initial_gamma,
    Lx, Ly, Lz, lb_/ub_ m, s, c, az, temperature, viscosity)."""
    import math
    Cc = int(params.component_count)
    model = int(params.model)
    Z = Cc if model == MODEL_VARIABLE_Z else 1
    lo, hi = [], []
    lo += [params.lb_m] * Cc
    hi += [params.ub_m] * Cc
    if model == MODEL_LOGNORMAL:
        lo += [params.lb_s] * Cc
        hi += [params.ub_s] * Cc
    lo += [math.log10(params.lb_c)] * Cc
    hi += [math.log10(params.ub_c)] * Cc
    lo += [params.lb_az] * Z
    hi += [params.ub_az] * Z
    j = OrcPropJob()
    j.model, j.C, j.Z, j.P, j.N, j.V = model, Cc, Z, len(lo), int(params.abc_sample_count), V
    j.perturbation = int(params.perturbation)
    j.full_az_prior = 1 if (params.reference_initial_gamma and model != MODEL_LOGNORMAL) else 0
    j.seed = seed
    for i, (a, b) in enumerate(zip(lo, hi)):
        j.lo[i], j.hi[i] = a, b
    j.volume_factor = params.Lx * params.Ly * params.Lz / 1e12
    j.delta_t = deltat
    if model == MODEL_LOGNORMAL:
        kB = 1.380649e-23
        j.sd_const = math.sqrt(2.0 * deltat * kB * params.temperature * 1e21 / (3.0 * math.pi * params.viscosity))
    return j


def build_proposal(job: OrcPropJob, theta, wcum, factor, slot: int, trial: int, generation: int):
    """(theta [P], counts [V], OrcProposal) of one proposal."""
    L = lib()
    if not getattr(L, "_prop_bound", False):
        L.orc_build_proposal.argtypes = [C.POINTER(OrcPropJob), _f64p, _f64p, _f64p, C.c_uint32, C.c_uint32,
                                         C.c_uint32, _f64p, _u32p, C.POINTER(OrcProposal)]
        L.orc_build_proposal.restype = C.c_int
        L._prop_bound = True
    th = np.ascontiguousarray(theta, np.float64)
    wc = np.ascontiguousarray(wcum, np.float64)
    fa = np.ascontiguousarray(factor, np.float64)
    out = np.zeros(job.P)
    counts = np.zeros(max(1, job.V), np.uint32)
    prop = OrcProposal()
    rc = L.orc_build_proposal(C.byref(job), ptr(th, C.c_double), ptr(wc, C.c_double), ptr(fa, C.c_double), slot,
                              trial, generation, ptr(out, C.c_double), ptr(counts, C.c_uint32), C.byref(prop))
    if rc != 0:
        raise ValueError(f"orc_build_proposal: {rc}")
    return out, counts[:job.V], prop

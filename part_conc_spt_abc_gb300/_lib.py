"""ctypes binding of libpcs.so (include/pcs.h).

The library is built in-tree by ``build()`` (``make -C csrc``) and loaded
from this package directory.  There is no fallback: when the library is
missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpcs.so")
ACCEL_PATH = os.path.join(HERE, "bin", "accel")
COMPARE_PATH = os.path.join(HERE, "bin", "compare")
CSRC = os.path.join(HERE, "csrc")

MAX_COMPONENTS = 8

# pcs_status
OK, ERR_INVALID_ARGUMENT, ERR_CUDA, ERR_OUT_OF_MEMORY, ERR_XML, ERR_UNSUPPORTED, ERR_DEVICE, ERR_BUSY, ERR_NOT_FOUND = range(9)
MODEL_DISCRETE_FIXED_DEPTH, MODEL_DISCRETE_VARIABLE_DEPTH, MODEL_LOGNORMAL = 0, 1, 2
WEIGHTING_PMC_STANDARD, WEIGHTING_INVERSE_DIST_SQ = 0, 1
SCHEDULE_DELTA, SCHEDULE_QUANTILE = 0, 1
PERTURB_DIAGONAL, PERTURB_CHOLESKY = 0, 1

_u32p = C.POINTER(C.c_uint32)
_u64p = C.POINTER(C.c_uint64)
_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)


class Params(C.Structure):
    _fields_ = [
        ("model", C.c_int32), ("weighting_scheme", C.c_int32), ("component_count", C.c_uint32),
        ("kmin", C.c_uint32), ("de_bin_count", C.c_uint32), ("abc_sample_count", C.c_uint32),
        ("avg_trial_count", C.c_uint32), ("gamma_adaptive", C.c_int32),
        ("Lx", C.c_double), ("Ly", C.c_double), ("Lz", C.c_double),
        ("gamma_initial", C.c_double), ("delta_gamma", C.c_double), ("ub_de", C.c_double),
        ("lb_m", C.c_double), ("ub_m", C.c_double), ("lb_s", C.c_double), ("ub_s", C.c_double),
        ("lb_c", C.c_double), ("ub_c", C.c_double), ("lb_az", C.c_double), ("ub_az", C.c_double),
        ("temperature", C.c_double), ("viscosity", C.c_double),
        ("schedule", C.c_int32), ("perturbation", C.c_int32), ("quantile", C.c_double),
        ("max_generations", C.c_uint32), ("reference_initial_gamma", C.c_int32),
        ("distance_double", C.c_int32),
    ]


class Observed(C.Structure):
    _fields_ = [
        ("ax", C.c_double), ("ay", C.c_double), ("deltat", C.c_double),
        ("frame_counts", _u64p), ("video_count", C.c_size_t),
        ("K", _u64p), ("DE", _f64p), ("track_count", C.c_size_t),
    ]


class Tuning(C.Structure):
    _fields_ = [
        ("block_size", C.c_uint32), ("particles_per_thread", C.c_uint32), ("hist_tile_rows", C.c_uint32),
        ("warp_aggregate", C.c_uint32), ("chunk_particles", C.c_uint32), ("round_capacity", C.c_uint32),
        ("max_speculation", C.c_uint32), ("use_graphs", C.c_uint32), ("plain_launch", C.c_uint32),
        ("round_fill", C.c_uint32), ("walk", C.c_uint32),
        ("job_order", C.c_uint32),
    ]


class JobInfo(C.Structure):
    _fields_ = [
        ("component_count", C.c_uint32), ("z_component_count", C.c_uint32), ("param_count", C.c_uint32),
        ("abc_sample_count", C.c_uint32), ("iterations", C.c_uint32), ("converged", C.c_uint32),
        ("simulations", C.c_uint64), ("trials", C.c_uint64), ("accepted", C.c_uint64),
        ("particle_steps", C.c_uint64), ("gamma", C.c_double), ("device_ms", C.c_double),
    ]


class KernelStats(C.Structure):
    _fields_ = [
        ("rounds", C.c_uint64), ("kernel_launches", C.c_uint64), ("simulate_launches", C.c_uint64),
        ("simulate_ms", C.c_double), ("distance_launches", C.c_uint64), ("distance_ms", C.c_double),
        ("round_ms", C.c_double), ("proposals", C.c_uint64), ("particle_steps", C.c_uint64),
        ("histogram_cells", C.c_uint64), ("split_tasks", C.c_uint64), ("pmc_launches", C.c_uint64),
        ("pmc_ms", C.c_double), ("generations", C.c_uint64), ("pmc_bytes", C.c_uint64),
        ("pmc_pair_flops", C.c_uint64),
    ]


class Setup(C.Structure):
    _fields_ = [
        ("model", C.c_int32), ("component_count", C.c_uint32), ("video_count", C.c_uint32),
        ("kmin", C.c_uint32), ("four_delta_t", C.c_float), ("half_lx", C.c_float), ("half_ly", C.c_float),
        ("half_lz", C.c_float), ("half_ax", C.c_float), ("half_ay", C.c_float), ("dde", C.c_float),
        ("rows", C.c_uint32), ("de_bins", C.c_uint32), ("frames", _u32p),
    ]


class Run(C.Structure):
    _fields_ = [
        ("particles", _u32p), ("half_az", C.c_float * MAX_COMPONENTS),
        ("pre_comp_prob", C.c_float * MAX_COMPONENTS), ("sd_scale", C.c_float * MAX_COMPONENTS),
        ("sd_shape", C.c_float * MAX_COMPONENTS), ("slot", C.c_uint32), ("trial", C.c_uint32),
        ("generation", C.c_uint32),
    ]


class Replay(C.Structure):
    _fields_ = [("uniforms", _f32p), ("normals", _f32p), ("normal_stride", C.c_uint32), ("sigmas", _f32p)]


class DebugProposal(C.Structure):
    _fields_ = [
        ("slot", C.c_uint32), ("trial", C.c_uint32), ("generation", C.c_uint32), ("total_particles", C.c_uint32),
        ("half_az", C.c_float * MAX_COMPONENTS), ("pre_comp_prob", C.c_float * MAX_COMPONENTS),
        ("sd_scale", C.c_float * MAX_COMPONENTS), ("sd_shape", C.c_float * MAX_COMPONENTS),
        ("distance", C.c_float),
    ]


class OutputMeta(C.Structure):
    _fields_ = [("key", C.c_char_p), ("value", C.c_char_p)]


class OutputView(C.Structure):
    _fields_ = [
        ("model", C.c_int32), ("weighting", C.c_int32), ("abc_sample_count", C.c_uint64),
        ("component_count", C.c_uint64), ("z_component_count", C.c_uint64), ("converged", C.c_int),
        ("gamma", C.c_double), ("m", _f64p), ("s", _f64p), ("c", _f64p), ("az", _f64p), ("dist", _f64p),
        ("w", _f64p), ("nm", C.c_size_t), ("ns", C.c_size_t), ("nc", C.c_size_t), ("naz", C.c_size_t),
        ("nd", C.c_size_t), ("nw", C.c_size_t), ("meta_count", C.c_size_t), ("meta", C.POINTER(OutputMeta)),
    ]


# every exported symbol and its (restype, argtypes); checked against include/pcs.h by the tests
SIGNATURES = {
    "pcs_abi_version": (C.c_int, []),
    "pcs_last_error": (C.c_char_p, []),
    "pcs_status_string": (C.c_char_p, [C.c_int]),
    "pcs_device_report": (C.c_size_t, [C.c_char_p, C.c_size_t]),
    "pcs_params_defaults": (None, [C.POINTER(Params)]),
    "pcs_open": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "pcs_close": (C.c_int, [C.c_void_p]),
    "pcs_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "pcs_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "pcs_autotune": (C.c_int, [C.c_void_p, C.POINTER(Params), C.POINTER(Observed), C.POINTER(Tuning)]),
    "pcs_timer_start": (C.c_int, [C.c_void_p]),
    "pcs_timer_stop": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "pcs_get_kernel_stats": (C.c_int, [C.c_void_p, C.POINTER(KernelStats)]),
    "pcs_reset_kernel_stats": (C.c_int, [C.c_void_p]),
    "pcs_job_create": (C.c_int, [C.c_void_p, C.POINTER(Params), C.POINTER(Observed), C.c_uint64, C.POINTER(C.c_void_p)]),
    "pcs_job_destroy": (C.c_int, [C.c_void_p]),
    "pcs_job_run": (C.c_int, [C.c_void_p, C.c_uint32]),
    "pcs_job_run_plain": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32]),
    "pcs_job_step": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "pcs_job_info_get": (C.c_int, [C.c_void_p, C.POINTER(JobInfo)]),
    "pcs_job_output": (C.c_int, [C.c_void_p, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p]),
    "pcs_job_checkpoint": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "pcs_job_restore": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "pcs_serve_submit": (C.c_int, [C.c_void_p, C.c_void_p]),
    "pcs_serve_step": (C.c_int, [C.c_void_p, _u32p]),
    "pcs_serve_poll": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]),
    "pcs_serve_set_memory_cap": (C.c_int, [C.c_void_p, C.c_uint64]),
    "pcs_input_load": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p)]),
    "pcs_input_free": (C.c_int, [C.c_void_p]),
    "pcs_input_params": (C.c_int, [C.c_void_p, C.POINTER(Params), C.POINTER(Observed), C.POINTER(C.c_char_p)]),
    "pcs_output_write": (C.c_int, [C.c_char_p, C.c_int32, C.c_int32, C.c_uint64, C.c_uint64, C.c_uint64,
                                   C.POINTER(OutputMeta), C.c_size_t, C.c_int, C.c_double,
                                   _f64p, C.c_size_t, _f64p, C.c_size_t, _f64p, C.c_size_t, _f64p, C.c_size_t,
                                   _f64p, C.c_size_t, _f64p, C.c_size_t]),
    "pcs_output_load": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "pcs_output_free": (C.c_int, [C.c_void_p]),
    "pcs_output_get": (C.c_int, [C.c_void_p, C.POINTER(OutputView)]),
    "pcs_simulate_hist": (C.c_int, [C.c_void_p, C.POINTER(Setup), C.POINTER(Run), C.c_uint32, C.c_uint64,
                                    C.POINTER(Replay), _u32p]),
    "pcs_scan_distance": (C.c_int, [C.c_void_p, _u32p, _u32p, C.c_uint32, C.c_uint32, C.c_uint32, _u32p,
                                    _f32p, _f64p, _u64p]),
    "pcs_scan_distance_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                            C.c_void_p, C.c_void_p]),
    "pcs_observed_sat": (C.c_int,[C.c_void_p, _u32p, _f64p, C.c_size_t, C.c_uint32, C.c_uint32, C.c_double, _u32p]),
    "pcs_observed_sat_julia": (C.c_int, [C.c_void_p, _u32p, _f64p, C.c_size_t, C.c_uint32, C.c_uint32, C.c_double,
                                         _u32p]),
    "pcs_debug_particle_stream": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32,
                                            C.c_uint32, C.c_uint32, _u32p]),
    "pcs_debug_round_proposals": (C.c_int, [C.c_void_p, C.c_uint32, _u32p, C.c_void_p, _f64p, _u32p]),
}


class PcsError(RuntimeError):
    """A failed C-ABI call; ``status`` is the pcs_status code."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


class XMLLoadError(PcsError):
    """error::XMLLoadError of the reference (shared/errors.hpp:21-42)."""


class CudaError(PcsError):
    """error::CudaError of the reference (support/cuda_error.hpp)."""


def build(quiet: bool = True, jobs: int = 0) -> None:
    """Compile libpcs.so and bin/accel in-tree for sm_103a."""
    n = jobs or max(1, min(8, os.cpu_count() or 1))
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-s", "-j", str(n), "-C", CSRC], check=True, stdout=out)


_lib = None
_lock = threading.Lock()


def lib():
    """The loaded library (raises when it is missing: there is no fallback)."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if not os.path.exists(LIB_PATH):
                    raise ImportError(f"{LIB_PATH} is not built; run __graft_entry__.build() or make -C {CSRC}")
                L = C.CDLL(LIB_PATH)
                for name, (res, args) in SIGNATURES.items():
                    fn = getattr(L, name)
                    fn.restype = res
                    fn.argtypes = args
                _lib = L
    return _lib


def check(status: int, what: str = "") -> None:
    if status == OK:
        return
    msg = lib().pcs_last_error().decode(errors="replace")
    text = f"{what}: {lib().pcs_status_string(status).decode()}: {msg}" if what else msg
    if status == ERR_XML:
        raise XMLLoadError(status, text)
    if status in (ERR_CUDA, ERR_DEVICE):
        raise CudaError(status, text)
    raise PcsError(status, text)

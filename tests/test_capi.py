"""The C-ABI library loads on a CPU-only machine and exports every entry
point include/pcs.h declares; no call here needs a GPU."""
import ctypes as C
import os
import re
import subprocess

from conftest import ROOT


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "pcs.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pcs_[a-z0-9_]+)\s*\(", src)))


def test_header_parses_and_lists_entry_points():
    syms = declared_symbols()
    for s in ["pcs_open", "pcs_job_run", "pcs_simulate_hist", "pcs_scan_distance", "pcs_serve_step", "pcs_input_load"]:
        assert s in syms


def test_library_exports_every_declared_symbol(pcs):
    L = C.CDLL(pcs._lib.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing
    assert set(declared_symbols()) == set(pcs._lib.SIGNATURES)
    out = subprocess.run(["nm", "-D", "--defined-only", pcs._lib.LIB_PATH], capture_output=True, text=True).stdout
    for s in declared_symbols():
        assert re.search(rf"\bT {s}\b", out), s


def test_host_only_calls(pcs):
    L = pcs.lib()
    assert L.pcs_abi_version() == 3
    assert L.pcs_status_string(0) == b"ok"
    p = pcs.params_defaults()
    assert p.delta_gamma == 0.01 and p.reference_initial_gamma == 1 and p.quantile == 0.5


def test_open_without_gpu_fails_cleanly(pcs):
    import pytest
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    st = pcs.lib().pcs_open(0, 0, C.byref(h))
    assert st != 0 and not h.value
    assert pcs.lib().pcs_last_error()

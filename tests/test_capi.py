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
    assert L.pcs_abi_version() == 4
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


STRUCTS = {"Params": "pcs_params", "Observed": "pcs_observed", "Tuning": "pcs_tuning", "JobInfo": "pcs_job_info",
           "KernelStats": "pcs_kernel_stats", "Setup": "pcs_setup", "Run": "pcs_run", "Replay": "pcs_replay",
           "OutputMeta": "pcs_output_meta", "OutputView": "pcs_output_view"}


def test_ctypes_mirrors_match_the_header_layout(pcs, tmp_path):
    """Every ctypes structure of the Python binding has the size and field
    offsets that a C compiler gives the struct of include/pcs.h."""
    import shutil
    import pytest
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "pcs.h"', "int main(void) {"]
    for py, cname in STRUCTS.items():
        cls = getattr(pcs._lib, py)
        lines.append(f'  printf("{py} size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'  printf("{py} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        py, field, value = line.split()
        got[(py, field)] = int(value)
    for py in STRUCTS:
        cls = getattr(pcs._lib, py)
        assert got[(py, "size")] == C.sizeof(cls), py
        for f, _ in cls._fields_:
            assert got[(py, f)] == getattr(cls, f).offset, (py, f)

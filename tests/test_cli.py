"""accel command line: flags, help, errors (src/gpu/main.cpp:61-327).  No GPU."""
import os
import subprocess

import pytest

from conftest import GOLDEN


def run(pcs, *args):
    return subprocess.run([pcs._lib.ACCEL_PATH, *args], capture_output=True, text=True, timeout=60)


def test_help(pcs):
    r = run(pcs, "-h")
    assert r.returncode == 0
    for flag in ["--input, -i", "--data, -d", "--output, -o", "--gpus, -g", "--host-scalar, -hs", "--dev-scalar, -ds",
                 "--dist-type, -dt", "--max-steps, -S", "--fixed-seed, -F", "--quiet, -q", "--verbose, -v",
                 "--list-devices"]:
        assert flag in r.stdout


@pytest.mark.parametrize("args,msg", [
    (["-x"], "Unknown command line argument '-x'"),
    (["-S"], "requires an additional integer argument"),
    (["-S", "abc"], "positive integer argument"),
    (["-F", "1x"], "requires an additional integer argument and not 1x"),
    (["-hs", "q"], "Scalar type must be either 'f' (float) or 'd' (double)"),
    (["-ds", "d"], "not supported"),
    (["-g", "zz"], "Don't understand provided gpuspec"),
])
def test_bad_flags(pcs, args, msg):
    r = run(pcs, *args)
    assert r.returncode == 1
    assert "Top-level exception" in r.stderr and msg in r.stderr


def test_missing_input_is_xml_error(pcs, tmp_path):
    r = run(pcs, "-i", str(tmp_path / "nope.xml"))
    assert r.returncode == 1
    assert "XMLLoadError" in r.stderr


def test_list_devices(pcs):
    r = run(pcs, "--list-devices")
    assert r.returncode == 0 and "CUDA device" in r.stdout


def test_compare_tool(pcs, tmp_path):
    """compare prints the population means of two output files and their
    differences in the format of the reference's compare tool."""
    import numpy as np
    outs = []
    for k, (m0, g) in enumerate([(100.0, 1.5), (130.0, 1.25)]):
        o = pcs.Output(0, 0, 4, 1, 1, np.array([m0, m0 + 2, m0 + 4, m0 + 6]), np.array([1e8, 2e8, 3e8, 4e8]),
                       np.full(4, 2.0), np.array([0.5, 0.25, 0.125, 1.0]), np.full(4, 0.25), False, g)
        path = str(tmp_path / f"o{k}.xml")
        pcs.write_output(path, o)
        outs.append(path)
    r = subprocess.run([pcs._lib.COMPARE_PATH, *outs], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    assert lines[0] == "m    : %18g vs %18g (δ = %18g)" % (103.0, 133.0, 30.0)
    assert lines[1].startswith("c    : ") and lines[5] == "eps  : %18g vs %18g (δ = %18g)" % (1.5, 1.25, 0.25)
    r = subprocess.run([pcs._lib.COMPARE_PATH, outs[0]], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "need exactly two command line args" in r.stderr
    r = subprocess.run([pcs._lib.COMPARE_PATH, outs[0], str(tmp_path / "missing.xml")], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 1 and r.stderr.startswith("Top-level exception: error::")

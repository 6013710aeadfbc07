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

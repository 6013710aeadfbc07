"""Generates distance_cases.npz from the reference's own distance kernel.

cusim::K_distance (src/gpu/cusim/kernel-distance.inl:81-241) is built for
sm_103a by oracle/build_ref_kdist.sh in two forms, without FMA contraction
(-fmad=false) and with nvcc's defaults as the reference ships it
(premake5.lua:76), and run, one 32 x 32 block per histogram as the
reference launches it, in float and in double (K_distance<float,unsigned>,
K_distance<double,unsigned>, kernel-distance.cu:5-8) on the cases of
distance_inputs.py.  Needs a GPU and the prepared kernel copy under
oracle/_ref/kdist/ (made where the reference tree is present, by
`bash oracle/build_ref_kdist.sh prepare`):

    python tests/golden/make_distance_golden.py [--out PATH]

Stored per case i: c{i}_name, c{i}_shape (rows, bins), and the reference
kernel's results c{i}_ref_f32_nofma, c{i}_ref_f64_nofma, c{i}_ref_f32_fma,
c{i}_ref_f64_fma, c{i}_zeroed (1 if every build reset the histogram to
zero).  The inputs are regenerated from distance_inputs.CASES.
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import distance_inputs as D  # noqa: E402

KDIST = os.path.join(ROOT, "oracle", "_ref", "kdist")


def load(variant: str):
    L = C.CDLL(os.path.join(KDIST, f"libkdist_{variant}.so"))
    for name, real in (("ref_kdist_f32", C.c_float), ("ref_kdist_f64", C.c_double)):
        f = getattr(L, name)
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_void_p, C.POINTER(C.c_int),
                      C.c_char_p, C.c_size_t]
        f.restype = C.c_int
    return L


def run(L, name, hist, ref, dtype):
    out = np.zeros(1, dtype)
    zeroed = C.c_int(0)
    err = C.create_string_buffer(512)
    h = np.ascontiguousarray(hist, np.uint32)
    r = np.ascontiguousarray(ref, np.uint32)
    rc = getattr(L, name)(h.ctypes.data, r.ctypes.data, hist.shape[0], hist.shape[1], 1, out.ctypes.data,
                          C.byref(zeroed), err, 512)
    if rc != 0:
        raise RuntimeError(err.value.decode())
    return out[0], zeroed.value


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "distance_cases.npz"))
    args = ap.parse_args()
    subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref_kdist.sh")], check=True)
    if not os.path.exists(os.path.join(KDIST, "libkdist_nofma.so")):
        sys.exit("the reference distance kernel was not built (see oracle/build_ref_kdist.sh)")
    libs = {v: load(v) for v in ("nofma", "fma")}
    import oracle as O
    O.build()
    out = {"count": np.array([len(D.CASES)])}
    for i, case in enumerate(D.CASES):
        name = case[0]
        hist, ref = D.case_arrays(case)
        zeroed = 1
        for v, L in libs.items():
            d32, z32 = run(L, "ref_kdist_f32", hist, ref, np.float32)
            d64, z64 = run(L, "ref_kdist_f64", hist, ref, np.float64)
            zeroed &= z32 & z64
            out[f"c{i}_ref_f32_{v}"] = np.array([d32], np.float32)
            out[f"c{i}_ref_f64_{v}"] = np.array([d64], np.float64)
        out[f"c{i}_name"] = np.array(name)
        out[f"c{i}_shape"] = np.array(hist.shape, np.int64)
        out[f"c{i}_zeroed"] = np.array([zeroed], np.int32)
        o32, _, _ = O.distance_kdist(hist, ref)
        o64 = O.distance_kdist_f64(hist, ref)
        n32, n64 = out[f"c{i}_ref_f32_nofma"][0], out[f"c{i}_ref_f64_nofma"][0]
        f32, f64 = out[f"c{i}_ref_f32_fma"][0], out[f"c{i}_ref_f64_fma"][0]
        print(f"{name:28s} nofma f32 {n32!r:>14} f64 {n64!r:>22}  fma f32 {f32!r:>14} f64 {f64!r:>22}  "
              f"oracle {'=' if np.float32(o32) == n32 and o64 == n64 else '!='}  zeroed {zeroed}")
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    np.savez_compressed(args.out, **out)
    print("distance cases:", len(D.CASES), "->", args.out)


if __name__ == "__main__":
    main()

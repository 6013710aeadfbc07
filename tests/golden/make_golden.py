"""Generates the golden fixtures in this directory from the reference's own
code, compiled for the host by oracle/build_ref.sh (oracle/_ref/libpcsref.so):

  replay_cases.npz   forward-model histograms of cusim::K_simulate_system
                     (src/gpu/cusim/kernel-simulate.inl) on replayed draws;
                     the draws are regenerated from the stored seed by
                     orc_replay_draws (oracle/pcs_oracle.h)
  (distance_cases.npz comes from the reference's distance kernel run on a
   GPU: make_distance_golden.py)
  xml_cases.json     input::load (src/gpu/shared/input.cpp) on the XML files
                     in tests/golden/xml/: parsed values or the error type
  output_cases.json  output::write (src/gpu/shared/output.cpp) bytes for
                     seeded populations

Run here (the reference tree must be present):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import glob
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402


def f32(x):
    return float(np.float32(x))


def make_setup(model, Cc, frames, parts, kmin, L, A, az, D, B, ub, dt, probs=None):
    frames = np.asarray(frames, np.uint32)
    parts = np.asarray(parts, np.uint32)
    Z = 1 if model == 0 else Cc
    if probs is None:
        probs = np.ones(Cc) / Cc
    pc = np.cumsum(probs).astype(np.float32)
    pc[-1] = 2.0
    rw = np.array([np.float32(np.sqrt(2 * D[i] * dt)) for i in range(Cc)], np.float32)
    half_az = np.array([np.float32(0.5) * np.float32(a) for a in az[:Z]], np.float32)
    return O.Setup(model, Cc, frames, parts, kmin, f32(np.float32(4) * np.float32(dt)),
                   tuple(f32(np.float32(0.5) * np.float32(x)) for x in L),
                   tuple(f32(np.float32(0.5) * np.float32(x)) for x in A), half_az, pc, rw,
                   f32(ub / B), int(frames.max()) + 1, B)


def replay_cases():
    rng = np.random.default_rng(20240601)
    cases = []
    # the configuration-0 shape: 20 videos x 200 frames, 175 nm particles
    cases.append(("cfg0_shape", make_setup(0, 1, [200] * 20, rng.poisson(128, 20), 2, (200, 160, 20), (100, 80),
                                           (2.0,), (2.626,), 100, 20.0, 1 / 30)))
    # two components, variable depth, small box so particles wrap often
    cases.append(("two_comp_variable_z", make_setup(1, 2, [60, 75, 40], [90, 70, 110], 3, (12, 10, 3), (6, 5),
                                                    (1.2, 0.6), (3.0, 1.0), 48, 12.0, 0.05, [0.6, 0.4])))
    # three components (binary-search component pick), fixed depth
    cases.append(("three_comp_fixed_z", make_setup(0, 3, [50] * 4, [64, 0, 33, 96], 2, (20, 16, 4), (10, 8),
                                                   (2.0,), (0.5, 2.6, 9.2), 64, 20.0, 1 / 30, [0.3, 0.4, 0.3])))
    # kmin 0 and 1 (the recorder divides by k-1 = 0 and wraps k-1 for k = 0)
    cases.append(("kmin0", make_setup(0, 1, [30, 17], [40, 25], 0, (8, 8, 2), (4, 4), (1.0,), (1.5,), 32, 10.0, 0.05)))
    cases.append(("kmin1", make_setup(1, 2, [30, 1, 9], [40, 5, 7], 1, (8, 8, 2), (4, 4), (1.0, 0.5), (1.5, 0.3),
                                      32, 10.0, 0.05)))
    # few DE bins: most tracks fall beyond the last bin and are dropped
    cases.append(("narrow_de", make_setup(0, 2, [120] * 3, [50, 60, 70], 2, (30, 30, 6), (20, 20), (3.0,),
                                          (4.0, 8.0), 8, 2.0, 0.04)))
    # single-frame videos and empty videos
    cases.append(("degenerate_frames", make_setup(1, 1, [1, 2, 3, 1], [10, 10, 0, 3], 2, (5, 5, 5), (5, 5),
                                                  (5.0,), (1.0,), 16, 5.0, 0.1)))
    # the reference test script's setup (test/test_part_conc_spt_abc.jl:22-34): 250 frames
    cases.append(("ref_script_shape", make_setup(0, 2, [250] * 6, rng.poisson(36, 6), 2, (60, 60, 10), (40, 40),
                                                 (2.0,), (1.0, 3.0), 200, 12.0, 0.05)))
    out = {}
    for i, (name, st) in enumerate(cases):
        seed = 7000 + i
        u, z, _ = O.replay_draws(seed, st.n_particles, st.stride)
        hist = O.ref_simulate_replay(st, u, z)
        orc, _ = O.simulate_replay(st, u, z)
        assert np.array_equal(hist, orc), f"oracle disagrees with the reference kernel on {name}"
        pre = f"{name}__"
        out[pre + "seed"] = np.uint64(seed)
        out[pre + "scalars"] = np.array([st.model, st.C, st.kmin, st.R, st.B], np.int64)
        out[pre + "floats"] = np.array([st.four_delta_t, *st.half_l, *st.half_a, st.dde], np.float32)
        out[pre + "frames"] = st.frames
        out[pre + "particles"] = st.particles
        out[pre + "half_az"] = st.half_az
        out[pre + "pre_comp_prob"] = st.pre_comp_prob
        out[pre + "rwsd"] = st.rwsd
        out[pre + "hist"] = hist
    out["names"] = np.array([n for n, _ in cases])
    np.savez_compressed(os.path.join(HERE, "replay_cases.npz"), **out)
    print("replay cases:", len(cases))


# ---------------------------------------------------------------- XML ------

class RefParams(C.Structure):
    _fields_ = [
        ("model", C.c_int), ("weighting_scheme", C.c_int), ("component_count", C.c_uint64), ("kmin", C.c_uint64),
        ("de_bin_count", C.c_uint64), ("abc_sample_count", C.c_uint64), ("avg_trial_count", C.c_uint64),
        ("Lx", C.c_double), ("Ly", C.c_double), ("Lz", C.c_double), ("gamma", C.c_double),
        ("delta_gamma", C.c_double), ("adaptive_gamma", C.c_int), ("de_lower", C.c_double),
        ("de_upper", C.c_double), ("m_lower", C.c_double), ("m_upper", C.c_double), ("s_lower", C.c_double),
        ("s_upper", C.c_double), ("c_lower", C.c_double), ("c_upper", C.c_double), ("az_lower", C.c_double),
        ("az_upper", C.c_double), ("ax", C.c_double), ("ay", C.c_double), ("delta_t", C.c_double),
        ("n_frames", C.c_uint64), ("n_K", C.c_uint64), ("n_DE", C.c_uint64), ("output_file_path", C.c_char * 1024),
    ]


def ref_input_load(inp, data):
    R = C.CDLL(O.REF_SO)
    R.ref_input_load.restype = C.c_int
    p = RefParams()
    cap = 1 << 20
    fr = np.zeros(cap, np.uint64)
    K = np.zeros(cap, np.uint64)
    DE = np.zeros(cap, np.float64)
    err = C.create_string_buffer(4096)
    rc = R.ref_input_load(inp.encode(), data.encode() if data else None, C.byref(p),
                          fr.ctypes.data_as(C.c_void_p), C.c_size_t(cap), K.ctypes.data_as(C.c_void_p),
                          C.c_size_t(cap), DE.ctypes.data_as(C.c_void_p), C.c_size_t(cap), err, C.c_size_t(4096))
    if rc != 0:
        return {"error": err.value.decode()}
    d = {k: getattr(p, k) for k, _ in RefParams._fields_ if k not in ("output_file_path", "s_lower", "s_upper")}
    d["output_file_path"] = p.output_file_path.decode()
    d["frames"] = fr[: p.n_frames].tolist()
    d["K_sum"] = int(K[: p.n_K].sum())
    d["K_head"] = K[: min(20, p.n_K)].tolist()
    d["DE_sum"] = float(DE[: p.n_DE].sum())
    d["DE_head"] = DE[: min(20, p.n_DE)].tolist()
    return d


def xml_cases():
    xdir = os.path.join(HERE, "xml")
    res = {}
    for inp in sorted(glob.glob(os.path.join(xdir, "input_*.xml"))):
        name = os.path.basename(inp)
        data = os.path.join(xdir, "data_ok.xml")
        alt = inp.replace("input_", "datafor_")
        if os.path.exists(alt):
            data = alt
        if name == "input_empty_list.xml":
            # a whitespace-only list has no text node; input.cpp:241-260 then
            # hands a null pointer to strtoull and the reference crashes, so
            # there is nothing to record (the library reports an XML error)
            res[name] = {"data": os.path.basename(data), "ref": {"crash": True}}
            continue
        ref = ref_input_load(inp, data)
        if "error" in ref:
            # the message names the files: record them relative to the repository
            ref["error"] = ref["error"].replace(xdir + os.sep, "tests/golden/xml/")
        res[name] = {"data": os.path.basename(data), "ref": ref}
    # the reference's own fixture (test_files/), when the tree is present
    ref_root = O.reference_root()
    tf = os.path.join(ref_root, "test_files") if ref_root else ""
    if tf and os.path.isdir(tf):
        res["test_files/input.xml"] = {"data": "test_files/data_20171018_175nm_500nm.xml",
                                       "ref": ref_input_load(os.path.join(tf, "input.xml"),
                                                             os.path.join(tf, "data_20171018_175nm_500nm.xml"))}
    with open(os.path.join(HERE, "xml_cases.json"), "w") as f:
        json.dump(res, f, indent=1, sort_keys=True)
    print("xml cases:", len(res))


def output_cases():
    R = C.CDLL(O.REF_SO)
    R.ref_output_write.restype = C.c_int
    rng = np.random.default_rng(5)
    res = []
    for i, (model, ws, N, Cc, Z) in enumerate([(0, 0, 4, 1, 1), (1, 1, 3, 2, 2), (0, 1, 5, 3, 1)]):
        m = rng.uniform(0.1, 5, N * Cc)
        c = 10 ** rng.uniform(8, 9, N * Cc)
        az = rng.uniform(0.5, 5, N * Z)
        dist = rng.normal(3, 1, N)
        w = rng.dirichlet(np.ones(N))
        gamma = float(rng.normal(2, 1))
        conv = i % 2
        meta_k = (C.c_char_p * 1)(b"simulator")
        meta_v = (C.c_char_p * 1)(b"gpu")
        with tempfile.NamedTemporaryFile(suffix=".xml", delete=False) as tf:
            path = tf.name
        dp = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        rc = R.ref_output_write(path.encode(), model, ws, C.c_uint64(N), C.c_uint64(Cc), C.c_uint64(Z), dp(m),
                                C.c_size_t(len(m)), dp(c), C.c_size_t(len(c)), dp(az), C.c_size_t(len(az)),
                                dp(dist), C.c_size_t(len(dist)), dp(w), C.c_size_t(len(w)), conv,
                                C.c_double(gamma), meta_k, meta_v, C.c_size_t(1))
        assert rc == 0
        with open(path, "rb") as f:
            text = f.read().decode()
        os.unlink(path)
        res.append({"model": model, "weighting": ws, "N": N, "C": Cc, "Z": Z, "m": m.tolist(), "c": c.tolist(),
                    "az": az.tolist(), "dist": dist.tolist(), "w": w.tolist(), "gamma": gamma, "converged": conv,
                    "meta": [["simulator", "gpu"]], "text": text})
    with open(os.path.join(HERE, "output_cases.json"), "w") as f:
        json.dump(res, f, indent=1)
    print("output cases:", len(res))


if __name__ == "__main__":
    O.build()
    if not O.ref_available():
        sys.exit("oracle/_ref/libpcsref.so is missing: the reference tree is needed to make the fixtures")
    replay_cases()
    xml_cases()
    output_cases()

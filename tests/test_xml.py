"""accel's file formats against the reference's own loader and writer
(golden fixtures from src/gpu/shared/input.cpp and output.cpp compiled for
the host)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

XML = os.path.join(GOLDEN, "xml")
CASES = json.load(open(os.path.join(GOLDEN, "xml_cases.json")))


def _reference_root():
    import sys
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    return oracle.reference_root()


def _paths(name, case):
    if name.startswith("test_files/"):
        root = _reference_root()
        if root is None:
            return "", ""
        return os.path.join(root, name), os.path.join(root, case["data"])
    return os.path.join(XML, name), os.path.join(XML, case["data"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_input_load_matches_reference(pcs, name):
    case = CASES[name]
    inp, data = _paths(name, case)
    if not os.path.exists(inp):
        pytest.skip("reference fixture not present")
    ref = case["ref"]
    if ref.get("crash") or "error" in ref:
        with pytest.raises(pcs.XMLLoadError) as e:
            pcs.load_input(inp, data)
        if "error" in ref:
            want = ref["error"].split("| nested ")[-1].split(":")[0]
            assert want in str(e.value), (want, str(e.value))
        return
    got = pcs.load_input(inp, data)
    p = got.params
    assert p.model == ref["model"] and p.weighting_scheme == ref["weighting_scheme"]
    for a, b in [("component_count", "component_count"), ("kmin", "kmin"), ("de_bin_count", "de_bin_count"),
                 ("abc_sample_count", "abc_sample_count"), ("avg_trial_count", "avg_trial_count"),
                 ("gamma_adaptive", "adaptive_gamma")]:
        assert int(getattr(p, a)) == int(ref[b]), a
    for a, b in [("Lx", "Lx"), ("Ly", "Ly"), ("Lz", "Lz"), ("gamma_initial", "gamma"), ("delta_gamma", "delta_gamma"),
                 ("ub_de", "de_upper"), ("lb_m", "m_lower"), ("ub_m", "m_upper"), ("lb_c", "c_lower"),
                 ("ub_c", "c_upper"), ("lb_az", "az_lower"), ("ub_az", "az_upper")]:
        assert getattr(p, a) == ref[b], a
    assert (got.ax, got.ay, got.deltat) == (ref["ax"], ref["ay"], ref["delta_t"])
    assert got.output_file_path == ref["output_file_path"]
    assert got.frames.tolist() == ref["frames"]
    assert int(got.K.sum()) == ref["K_sum"] and got.K[:20].tolist() == ref["K_head"]
    assert got.DE[:20].tolist() == ref["DE_head"]
    assert float(got.DE.sum()) == pytest.approx(ref["DE_sum"], rel=0, abs=0)


@pytest.mark.parametrize("i", range(3))
def test_output_write_bytes_match_reference(pcs, tmp_path, i):
    case = json.load(open(os.path.join(GOLDEN, "output_cases.json")))[i]
    o = pcs.Output(case["model"], case["weighting"], case["N"], case["C"], case["Z"], np.array(case["m"]),
                   np.array(case["c"]), np.array(case["az"]), np.array(case["dist"]), np.array(case["w"]),
                   bool(case["converged"]), case["gamma"], None, [tuple(x) for x in case["meta"]])
    path = str(tmp_path / "out.xml")
    pcs.write_output(path, o)
    assert open(path).read() == case["text"]
    back = pcs.load_output(path)
    assert back.model == o.model and back.abc_sample_count == o.abc_sample_count
    assert back.converged == o.converged and back.gamma == o.gamma
    for f in ["m", "c", "az", "dist", "w"]:
        assert np.array_equal(getattr(back, f), getattr(o, f)), f
    assert back.meta == o.meta


def test_lognormal_input_and_output(pcs, tmp_path):
    src = open(os.path.join(XML, "input_ok_fixed.xml")).read()
    src = src.replace("discrete-fixed-depth", "lognormal").replace("</input>",
        "\t<lb_s>1.0</lb_s>\n\t<ub_s>100.0</ub_s>\n\t<temperature>298</temperature>\n"
        "\t<viscosity>0.95e-3</viscosity>\n\t<schedule>quantile</schedule>\n\t<quantile>0.5</quantile>\n"
        "\t<perturbation>cholesky</perturbation>\n</input>")
    p = tmp_path / "in.xml"
    p.write_text(src)
    got = pcs.load_input(str(p), os.path.join(XML, "data_ok.xml"))
    assert got.params.model == pcs.MODEL_LOGNORMAL
    assert (got.params.lb_s, got.params.ub_s) == (1.0, 100.0)
    assert got.params.schedule == pcs.SCHEDULE_QUANTILE and got.params.perturbation == pcs.PERTURB_CHOLESKY
    # lognormal needs the s bounds
    p.write_text(src.replace("<lb_s>1.0</lb_s>", ""))
    with pytest.raises(pcs.XMLLoadError):
        pcs.load_input(str(p), os.path.join(XML, "data_ok.xml"))
    o = pcs.Output(2, 0, 2, 1, 1, np.array([175.0, 180.0]), np.array([1e8, 2e8]), np.array([2.0, 2.0]),
                   np.array([1.0, 2.0]), np.array([0.5, 0.5]), False, 1.5, np.array([10.0, 12.0]), [])
    out = str(tmp_path / "o.xml")
    pcs.write_output(out, o)
    txt = open(out).read()
    assert "<model>lognormal</model>" in txt and "<s>10, 12\t</s>" in txt
    assert np.array_equal(pcs.load_output(out).s, o.s)


def test_missing_files(pcs):
    with pytest.raises(pcs.XMLLoadError) as e:
        pcs.load_input("/nonexistent/input.xml", None)
    assert "XMLLoadError" in str(e.value)

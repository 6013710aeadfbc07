"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on a
CPU-only machine (the library is cross-compiled and loaded, but no CUDA call
that needs a device is made)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def pcs():
    import part_conc_spt_abc_gb300 as P
    if not os.path.exists(P._lib.LIB_PATH):
        P.build()
    P.lib()
    return P


@pytest.fixture(scope="session")
def ctx(pcs):
    c = pcs.Context(0)
    yield c
    c.close()


def load_replay_cases(oracle):
    z = np.load(os.path.join(GOLDEN, "replay_cases.npz"))
    out = []
    for name in z["names"]:
        p = f"{name}__"
        sc = z[p + "scalars"]
        fl = z[p + "floats"]
        st = oracle.Setup(int(sc[0]), int(sc[1]), z[p + "frames"], z[p + "particles"], int(sc[2]), float(fl[0]),
                          (float(fl[1]), float(fl[2]), float(fl[3])), (float(fl[4]), float(fl[5])),
                          z[p + "half_az"], z[p + "pre_comp_prob"], z[p + "rwsd"], float(fl[6]), int(sc[3]),
                          int(sc[4]))
        out.append((str(name), st, int(z[p + "seed"]), z[p + "hist"]))
    return out

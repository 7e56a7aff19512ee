import glob
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")
if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libclv.so)")


def golden_files():
    return sorted(glob.glob(os.path.join(GOLDEN, "ref4_*d_*.npz")))


def load_golden(path):
    g = np.load(path)
    X, Y, Z, T, Cn = (int(v) for v in g["dims"])
    return g, dict(nx=X, ny=Y, nz=Z, nt=T, ncomp=Cn, eps=float(g["eps"]), a_x=float(g["a_x"]),
                   G=float(g["G"]), Q=float(g["Q"]), P=float(g["P"]), mu=float(g["MU"]),
                   DT=float(g["DT"]))


def large_golden_files():
    return sorted(glob.glob(os.path.join(GOLDEN, "ref4l_*.npz")))


def load_large_golden(path):
    """A larger golden configuration: the fixture, its parameters, and its inputs
    (regenerated from tests/golden/detinputs.py)."""
    import detinputs
    g, kw = load_golden(path)
    X, Y, Z, T, Cn = (int(v) for v in g["dims"])
    seed = int(g["seed"])
    psi0, psic0 = detinputs.ref4_inputs((Cn, T, X, Y, Z), seed)
    noise = detinputs.noise((Cn, X, Y, Z, T, 2), seed + 10)
    return g, kw, psi0, psic0, noise


def rel_err(a, b):
    """max |a-b| / max(|b|, rms(b)) -- floored relative error."""
    a = np.asarray(a)
    b = np.asarray(b)
    scale = max(float(np.sqrt(np.mean(np.abs(b) ** 2))), 1e-300)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), scale)))


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.build()
    return pyoracle

"""The drop-in main program (cl_var_dt_gb300/clv_main, the engine's main.cu)
run end to end from params.txt + Parameters.h, checked against the same run
driven through the Python binding: same trajectory, same snapshot values, the
reference's file layout."""
import os
import subprocess

import numpy as np
import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu

PARAMS_H = dict(COMPONENTS=4, XSIZE=64, YSIZE=1, ZSIZE=1, TAUSIZE=16, EPS=0.02, a_x=1.0, G=0.15,
                Q=0.02, STEPS=250, DT=0.002, SNAPSHOT_TRIGGER=100, EVALUATE_TRIGGER=50)
MU, P, SEED = -0.5, 0.1, 12345


@pytest.fixture(scope="module")
def clv():
    import cl_var_dt_gb300 as m
    m.build()
    return m


def test_drop_in_main_matches_engine_run(clv, tmp_path):
    with open(tmp_path / "Parameters.h", "w") as f:
        for k, v in PARAMS_H.items():
            f.write(f"#define {k} {v}\n")
    with open(tmp_path / "params.txt", "w") as f:
        f.write(f"mu={MU}\nP={P}\nrun=0\nseed={SEED}\nseed2=7\n")
    exe = os.path.join(REPO, "cl_var_dt_gb300", "clv_main")
    r = subprocess.run([exe, "0"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    base = tmp_path / "DATA" / f"BoseCL_Sim_mu_{MU:g}_P_{P:g}"
    run = base / "Run1"
    assert (run / "rawdata").is_dir() and (run / "Parameters.txt").is_file()
    skal = [[float(x) for x in line.strip().split("\t") if x] for line in open(base / "Skalars.txt")]
    Fx = [[float(x) for x in line.strip().split("\t") if x] for line in open(run / "F_x.txt")]

    # the same loop through the binding (main.cu:144-158)
    p = PARAMS_H
    c = clv.ChainParams(nx=p["XSIZE"], nt=p["TAUSIZE"], eps=p["EPS"], a_x=p["a_x"], G=p["G"], Q=p["Q"],
                        DT=p["DT"], mu=MU, P=P, seed=SEED)
    snaps = []
    with clv.Engine(c, model=clv.MODEL_REF4, noise=clv.NOISE_PHILOX) as e:
        e.set_mean_field(0, 0.0, 0.0)
        e.set_mean_field(1, 0.0, 0.0)
        steps = p["STEPS"]
        for i in range(steps):
            if (i % p["SNAPSHOT_TRIGGER"] == 0 and i not in (0, steps - 1)) or i == 1:
                snaps.append(e.ref_observables(0))
            e.step(1)
            if i % p["EVALUATE_TRIGGER"] == 0:
                e.evaluate()
        snaps.append(e.ref_observables(0))
    assert len(skal) == len(snaps) == len(Fx) == 4
    for row, (n, F) in zip(skal, snaps):
        assert np.allclose(row, n, rtol=0, atol=1e-6 + 1e-6 * np.abs(n).max())
    for row, (n, F) in zip(Fx, snaps):
        assert np.allclose(row, F[0], rtol=1e-5, atol=1e-5)

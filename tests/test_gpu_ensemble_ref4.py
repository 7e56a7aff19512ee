"""Ensemble agreement of the engine's plain FP64 drop-in with the reference's own
GPU build, over full runs with independent noise.

Model and rule: the reference's (4 components, linear px^2 kinetic term, mean/max
step rule), on a 32-site line with N_tau = 16 (EPS = 0.05, G = 0.1, DT = 0.002,
mu = -1.5, P = 0), from main.cu's zero start (set_mean_field(0, 0)).  Each side
runs NCHAIN independent chains: the reference build (its kernels compiled
unchanged, cuFFT, cuRAND XORWOW seeded per chain like Propagator's constructor)
one chain at a time, the engine all chains in one batch with its Philox noise.
After THERM steps, the observables of Observables::evaluate are taken every 10
steps for MEAS steps: n_tot, n_11, n_12, n_21, n_22 (Observables_without_cutoff.cu
:1322-1382) and the site means of F_x, F_y, F_z (:1274-1306), in the normalisation
of the reference's write_* methods (per site and imaginary time).  Per observable,
the chain means give an ensemble mean and standard error on each side; the two
means must agree within 2 sigma of their combined standard error.

The lattice's step-size reduction has two blocks, so the reference's atomicAdd of
block sums is order-free and both sides are reproducible run to run.  Set
CLV_ENSEMBLE_REPORT to a file path to get the table as JSON.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NAME = "1d_x32_t16_ens"
NCHAIN = 32
THERM = 500
MEAS = 2000
EVERY = 10
SEED = 20261203
OBS = ("n_tot", "n_11", "n_12", "n_21", "n_22", "F_x", "F_y", "F_z")


@pytest.fixture(scope="module")
def clv():
    import cl_var_dt_gb300 as m
    m.build()
    return m


@pytest.fixture(scope="module")
def refgpu():
    import refgpu as r
    r.build_runner()
    if not r.have_cubin(NAME):
        pytest.skip("reference cubins not built: run oracle/refgpu.py where the reference sources are")
    return r


def _reference_means(refgpu):
    X, T = 32, 16
    out = np.zeros((NCHAIN, len(OBS)))
    for i in range(NCHAIN):
        with refgpu.RefGpu(NAME, seed=SEED + 7919 * i) as r:
            r.set_mean_field(0.0, 0.0)
            for _ in range(THERM):
                r.propagate()
            acc = np.zeros(len(OBS))
            for _ in range(MEAS // EVERY):
                for _ in range(EVERY):
                    r.propagate()
                n, F = r.observables()
                acc += np.concatenate([n / (T * X), F.mean(axis=1) / T])
            out[i] = acc / (MEAS // EVERY)
    return out


def _engine_means(clv, refgpu):
    m = refgpu.macros(NAME)
    chains = [clv.ChainParams(nx=32, ny=1, nz=1, nt=16, eps=float(m["EPS"]), a_x=float(m["a_x"]),
                              G=float(m["G"]), Q=float(m["Q"]), P=0.0, mu=-1.5, DT=float(m["DT"]),
                              seed=SEED + 1) for _ in range(NCHAIN)]
    with clv.Engine(chains, model=clv.MODEL_REF4, noise=clv.NOISE_PHILOX, precision=clv.PREC_F64) as e:
        e.set_mean_field(0, 0.0, 0.0)
        e.set_mean_field(1, 0.0, 0.0)
        e.step(THERM)
        for _ in range(MEAS // EVERY):
            e.step(EVERY)
            e.evaluate()
        assert e.counter == MEAS // EVERY
        out = np.zeros((NCHAIN, len(OBS)))
        for i in range(NCHAIN):
            n, F = e.ref_observables(i)  # cumulative means over the evaluations
            out[i] = np.concatenate([n, F.mean(axis=1)])
        assert not any(f & clv.FLAG_NONFINITE for f in e.chain_flags())
    return out


def test_dropin_ensemble_within_two_sigma_of_reference_gpu_build(clv, refgpu):
    ref = _reference_means(refgpu)
    eng = _engine_means(clv, refgpu)
    report = {}
    for j, name in enumerate(OBS):
        mr, sr = ref[:, j].mean(), ref[:, j].std(ddof=1) / np.sqrt(NCHAIN)
        me, se = eng[:, j].mean(), eng[:, j].std(ddof=1) / np.sqrt(NCHAIN)
        report[name] = dict(reference=mr, reference_err=sr, engine=me, engine_err=se,
                            deviation_sigma=abs(me - mr) / np.hypot(sr, se))
    path = os.environ.get("CLV_ENSEMBLE_REPORT")
    if path:
        with open(path, "w") as f:
            json.dump(dict(lattice="32 x 16, 4 components", chains=NCHAIN, therm=THERM, meas=MEAS, every=EVERY,
                           report=report), f, indent=1)
    for name, r in report.items():
        assert np.isfinite(r["engine"]) and np.isfinite(r["reference"]), name
        assert r["reference_err"] > 0 and r["engine_err"] > 0, name
        assert r["deviation_sigma"] < 2.0, (name, r)

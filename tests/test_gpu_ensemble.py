"""Ensemble agreement of the FP32-mixed path with the plain FP64 path.

Workload: the single-chain spin-1 case (1D Nx = 64, N_tau = 64, beta = 4,
c0 = 0.5, c1 = -0.1, q = 0.05, mu = 1, start sqrt(1/3) + N(0, 0.01), K = 0.05,
dt_max = 1e-3; 2000 thermalisation steps, then 8000 steps with the observables
every 10), run as 16 independent chains (Philox streams of one seed) in each
precision.  For density, F_z, <F^2> and energy the chain means give an ensemble
mean and standard error per precision; the FP32-mixed mean must lie within 2
sigma (combined standard error) of the FP64 mean.  Set CLV_ENSEMBLE_REPORT to
a file path to get the table as JSON.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NCHAIN = 16
SEED = 20261203
NAMES = ("density", "F_z", "F^2", "energy")


@pytest.fixture(scope="module")
def clv():
    import cl_var_dt_gb300 as m
    m.build()
    return m


def _run(clv, precision, seed=SEED):
    chains = [clv.ChainParams(nx=64, nt=64, eps=4.0 / 64, mu=1.0, c0=0.5, c1=-0.1, q=0.05, K=0.05,
                              dt_max=1e-3, seed=seed) for _ in range(NCHAIN)]
    with clv.Engine(chains, model=clv.MODEL_SPIN1, precision=precision) as e:
        e.init_spin1(np.sqrt(1 / 3), 0.01)
        e.step(2000)
        for _ in range(800):
            e.step(10)
            e.evaluate()
        flags = e.chain_flags()
        samples = np.stack([e.spin1_samples(i) for i in range(NCHAIN)])  # (chain, 800, 8)
        info = e.step_info()
    assert not any(f & 1 for f in flags), flags
    return samples, info


def test_fp32_mixed_within_two_sigma_of_fp64(clv):
    s64, i64 = _run(clv, clv.PREC_F64)
    s32, i32 = _run(clv, clv.PREC_F32)
    s32b, _ = _run(clv, clv.PREC_F32, seed=SEED + 1)
    assert s64.shape == s32.shape == s32b.shape == (NCHAIN, 800, 8)

    def stat(s, j):
        m = s[:, :, 2 * j].mean(axis=1)  # real part, per-chain means
        return m.mean(), m.std(ddof=1) / np.sqrt(NCHAIN)

    report = {}
    for j, name in enumerate(NAMES):
        mean64, se64 = stat(s64, j)
        mean32, se32 = stat(s32, j)
        mean32b, se32b = stat(s32b, j)
        report[name] = dict(fp64=mean64, fp64_err=se64, fp32=mean32, fp32_err=se32,
                            deviation_sigma=abs(mean32 - mean64) / np.hypot(se64, se32),
                            fp32_other_seed=mean32b, fp32_other_seed_err=se32b,
                            other_seed_deviation_sigma=abs(mean32b - mean64) / np.hypot(se64, se32b))
    path = os.environ.get("CLV_ENSEMBLE_REPORT")
    if path:
        with open(path, "w") as f:
            json.dump(dict(report=report, langevin_time64=i64["t"].tolist(),
                           langevin_time32=i32["t"].tolist()), f, indent=1)
    for name, r in report.items():
        assert np.isfinite(r["fp64"]) and np.isfinite(r["fp32"]), name
        assert r["deviation_sigma"] < 2.0, (name, r)
        assert r["other_seed_deviation_sigma"] < 3.0, (name, r)

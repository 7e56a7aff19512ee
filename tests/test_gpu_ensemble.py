"""Ensemble agreement of the FP32-mixed path with the plain FP64 path.

Workload: the single-chain spin-1 case (1D Nx = 64, N_tau = 64, beta = 4,
c0 = 0.5, c1 = -0.1, q = 0.05, mu = 1, start sqrt(1/3) + N(0, 0.01), K = 0.05,
dt_max = 1e-3; 2000 thermalisation steps, then 8000 steps with the observables
every 10), run as NCHAIN = 64 independent chains in each precision.

* Independent ensembles: FP64 from Philox seed SEED, FP32-mixed from seed
  SEED + 1 (different noise and start).  Per chain, the time series of density,
  F_z, <F^2> and energy gives a mean and a block error (16 blocks, autocorrelated
  series); the ensemble mean is the mean over chains.  Its error is the larger of
  sqrt(sum of block errors^2) / NCHAIN and the chain-to-chain spread / sqrt(NCHAIN):
  F_z (the magnetisation, conserved but for the noise) relaxes over far more
  steps than a block, so its block errors come out several times too small and
  only the spread measures its fluctuation.  The two precisions' means must lie
  within 2 sigma of their combined error.
* Same noise: FP32-mixed from seed SEED tracks the FP64 run trajectory by
  trajectory; its ensemble means lie within 0.05 sigma of the FP64 means.

Set CLV_ENSEMBLE_REPORT to a file path to get the table as JSON.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NCHAIN = 64
NBLOCK = 16
SEED = 20261203
NAMES = ("density", "F_z", "F^2", "energy")


@pytest.fixture(scope="module")
def clv():
    import cl_var_dt_gb300 as m
    m.build()
    return m


def _run(clv, precision, seed):
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


def _stats(s, j):
    from cl_var_dt_gb300.secant import block_error
    x = s[:, :, 2 * j]  # real parts
    means = x.mean(axis=1)
    berr = np.array([block_error(c, NBLOCK) for c in x])
    block = np.sqrt((berr ** 2).sum()) / NCHAIN
    spread = means.std(ddof=1) / np.sqrt(NCHAIN)
    return means.mean(), max(block, spread), block, spread


def test_fp32_mixed_within_two_sigma_of_fp64(clv):
    s64, i64 = _run(clv, clv.PREC_F64, SEED)
    s32, i32 = _run(clv, clv.PREC_F32, SEED + 1)
    s32s, _ = _run(clv, clv.PREC_F32, SEED)
    assert s64.shape == s32.shape == s32s.shape == (NCHAIN, 800, 8)
    report = {}
    for j, name in enumerate(NAMES):
        m64, e64, b64, c64 = _stats(s64, j)
        m32, e32, b32, c32 = _stats(s32, j)
        ms, es, _, _ = _stats(s32s, j)
        report[name] = dict(fp64=m64, fp64_err=e64, fp64_block_err=b64, fp64_spread_err=c64,
                            fp32_independent=m32, fp32_independent_err=e32, fp32_independent_block_err=b32,
                            fp32_independent_spread_err=c32,
                            deviation_sigma=abs(m32 - m64) / np.hypot(e64, e32),
                            fp32_same_noise=ms, same_noise_deviation_sigma=abs(ms - m64) / np.hypot(e64, es))
    path = os.environ.get("CLV_ENSEMBLE_REPORT")
    if path:
        with open(path, "w") as f:
            json.dump(dict(chains=NCHAIN, blocks=NBLOCK, report=report, langevin_time64=float(i64["t"].mean()),
                           langevin_time32=float(i32["t"].mean())), f, indent=1)
    for name, r in report.items():
        assert np.isfinite(r["fp64"]) and np.isfinite(r["fp32_independent"]), name
        assert r["deviation_sigma"] < 2.0, (name, r)
        assert r["same_noise_deviation_sigma"] < 0.05, (name, r)
        assert r["fp64_err"] > 0 and r["fp32_independent_err"] > 0, (name, r)

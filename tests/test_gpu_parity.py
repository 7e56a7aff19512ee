"""Parity of the CUDA engine (through the C ABI of libclv.so) with the
reference's kernels (golden vectors) and with the CPU oracle.

Tolerances (floored relative error max|a-b| / max(|b|, rms b)):
  FP64: 1e-12 per site, FP32-mixed: 1e-5 per site (single step, same noise).
"""
import os

import numpy as np
import pytest

from conftest import golden_files, load_golden, rel_err

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5


@pytest.fixture(scope="module")
def clv():
    import cl_var_dt_gb300 as m
    m.build()
    return m


def _chain(m, kw, **extra):
    return m.ChainParams(nx=kw["nx"], ny=kw["ny"], nz=kw["nz"], nt=kw["nt"], eps=kw["eps"],
                         a_x=kw["a_x"], G=kw["G"], Q=kw["Q"], P=kw["P"], mu=kw["mu"], DT=kw["DT"],
                         **extra)


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.split("/")[-1][5:-4])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_ref4_matches_reference_kernels(clv, path, prec):
    g, kw = load_golden(path)
    precision = clv.PREC_F64 if prec == "f64" else clv.PREC_F32
    tol = TOL64 if prec == "f64" else TOL32
    with clv.Engine(_chain(clv, kw), model=clv.MODEL_REF4, noise=clv.NOISE_EXTERNAL,
                    precision=precision) as e:
        e.set_fields(0, g["psi0"], g["psic0"])
        e.evaluate()
        n, F = e.ref_observables(0)
        T, V = kw["nt"], kw["nx"] * kw["ny"] * kw["nz"]
        assert rel_err(n, g["n0"] / T / V) < tol
        assert rel_err(F, g["F0"] / T) < tol
        for s in range(len(g["dt"])):
            e.step_with_noise(g["noise"][s])
            info = e.step_info()
            assert abs(info["dt"][0] - g["dt"][s]) <= tol * g["dt"][s]
            psi, psic = e.get_fields(0)
            if prec == "f64" or s == 0:
                assert rel_err(psi, g["psi"][s]) < tol
                assert rel_err(psic, g["psic"][s]) < tol
        assert info["steps"][0] == len(g["dt"])


def test_ref4_zero_start_and_set_mean_field(clv):
    """main.cu's start: set_mean_field(0, 0); first step takes dt = DT."""
    g, kw = load_golden([f for f in golden_files() if f.endswith("1d_x16_t16_zero.npz")][0])
    with clv.Engine(_chain(clv, kw), model=clv.MODEL_REF4, noise=clv.NOISE_EXTERNAL) as e:
        e.set_fields(0, np.ones((4, 16, 16, 1, 1)), np.ones((4, 16, 16, 1, 1)))
        e.set_mean_field(0, 0.0, 0.0)
        e.set_mean_field(1, 0.0, 0.0)
        for s in range(len(g["dt"])):
            e.step_with_noise(g["noise"][s])
            assert e.step_info()["dt"][0] == pytest.approx(g["dt"][s], rel=TOL64)
        psi, psic = e.get_fields(0)
        assert rel_err(psi, g["psi"][-1]) < TOL64


def _spin1_chain(m, **kw):
    base = dict(nx=16, ny=1, nz=1, nt=16, eps=4 / 16, mu=1.0, c0=0.5, c1=-0.1, q=0.05, K=0.05,
                dt_max=1e-3, seed=20261203)
    base.update(kw)
    return m.ChainParams(**base)


def _orc_params(oracle, c):
    return oracle.spin1_params(nx=c.nx, ny=c.ny, nz=c.nz, nt=c.nt, eps=c.eps, mu=c.mu, c0=c.c0,
                               c1=c.c1, q=c.q, Kc=c.K, dt_max=c.dt_max)


SPIN1_SHAPES = [
    dict(nx=64, nt=64),                    # 1D (config 1 shape)
    dict(nx=16, ny=8, nt=8),               # 2D
    dict(nx=8, ny=6, nz=4, nt=4),          # 3D, radix 3
    dict(nx=96, nt=8),                     # radix 3 line
    dict(nx=80, ny=5, nt=6),               # radix 5
    dict(nx=32, ny=32, nt=16, K=0.5),      # K/max binding (dt below dt_max)
]


@pytest.mark.parametrize("shape", SPIN1_SHAPES, ids=lambda d: "x".join(f"{k}{v}" for k, v in d.items()))
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_spin1_philox_matches_oracle(clv, oracle, shape, prec):
    c = _spin1_chain(clv, **shape)
    p = _orc_params(oracle, c)
    precision = clv.PREC_F64 if prec == "f64" else clv.PREC_F32
    tol = TOL64 if prec == "f64" else TOL32
    with clv.Engine(c, model=clv.MODEL_SPIN1, precision=precision) as e:
        e.init_spin1(np.sqrt(1 / 3), 0.01)
        psi0, psic0 = oracle.spin1_init(p, c.seed, 0)
        psi, psic = e.get_fields(0)
        assert rel_err(psi, psi0) < tol and rel_err(psic, psic0) < tol
        # one step with the engine's own Philox noise
        e.step(1)
        ref_psi, ref_psic, dt, mx, _ = oracle.step(p, psi0, psic0, noise=None, seed=c.seed, chain=0,
                                                  step_index=0)
        info = e.step_info()
        assert abs(info["dt"][0] - dt) <= tol * dt
        psi, psic = e.get_fields(0)
        assert rel_err(psi, ref_psi) < tol
        assert rel_err(psic, ref_psic) < tol
        # observables of that configuration
        e.evaluate()
        got = e.spin1_samples(0)[0]
        want = oracle.spin1_observables(p, psi, psic)
        assert np.max(np.abs(got - want)) < tol * max(1.0, np.max(np.abs(want)))


@pytest.mark.parametrize("model", ["spin1", "ref4"])
def test_graph_steps_equal_single_steps(clv, model):
    """clv_step(n) replays graphs of 16 steps and of one step (37 = 2 x 16 + 5):
    the same fields, time and step count as 37 single steps."""
    if model == "spin1":
        c, m = _spin1_chain(clv, nx=32, ny=16, nt=16), clv.MODEL_SPIN1
    else:
        c, m = clv.ChainParams(nx=64, nt=16, mu=-0.5, G=0.15, P=0.1, seed=9), clv.MODEL_REF4
    outs = []
    for graph in (False, True):
        with clv.Engine(c, model=m) as e:
            if model == "spin1":
                e.init_spin1()
            else:
                e.set_mean_field(0, 0.3, 0.1)
                e.set_mean_field(1, 0.3, 0.1)
            if graph:
                e.step(37)
            else:
                for _ in range(37):
                    e.step(1)
            info = e.step_info()
            outs.append(e.get_fields(0) + (info["t"][0], info["steps"][0]))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    assert outs[0][2] == outs[1][2] and outs[0][3] == outs[1][3] == 37


def test_spin1_multistep_matches_oracle(clv, oracle):
    c = _spin1_chain(clv, nx=32, ny=8, nt=16)
    p = _orc_params(oracle, c)
    with clv.Engine(c, model=clv.MODEL_SPIN1) as e:
        e.init_spin1()
        e.step(6)
        psi, psic = oracle.spin1_init(p, c.seed, 0)
        t = 0.0
        for k in range(6):
            psi, psic, dt, _, _ = oracle.step(p, psi, psic, seed=c.seed, chain=0, step_index=k)
            t += dt
        gpsi, gpsic = e.get_fields(0)
        assert rel_err(gpsi, psi) < 1e-11
        assert abs(e.step_info()["t"][0] - t) < 1e-12 * t


def test_batched_uneven_chains_match_oracle(clv, oracle):
    rng = np.random.default_rng(11)
    chains = [
        _spin1_chain(clv, nx=32, ny=32, nt=8, mu=0.4, c1=-0.2, seed=1),
        _spin1_chain(clv, nx=64, ny=1, nt=16, mu=1.2, c0=0.3, seed=2),
        _spin1_chain(clv, nx=24, ny=24, nt=4, mu=0.8, q=0.0, seed=3),
        _spin1_chain(clv, nx=16, ny=8, nz=4, nt=8, mu=0.2, K=0.2, seed=4),
    ]
    with clv.Engine(chains, model=clv.MODEL_SPIN1) as e:
        e.init_spin1()
        e.step(3)
        info = e.step_info()
        for i, c in enumerate(chains):
            p = _orc_params(oracle, c)
            psi, psic = oracle.spin1_init(p, c.seed, i)
            for k in range(3):
                psi, psic, dt, _, _ = oracle.step(p, psi, psic, seed=c.seed, chain=i, step_index=k)
            gpsi, gpsic = e.get_fields(i)
            assert rel_err(gpsi, psi) < 1e-11, i
            assert rel_err(gpsic, psic) < 1e-11, i
            assert info["dt"][i] == pytest.approx(dt, rel=1e-12)


def test_determinism_same_seed_bitwise(clv):
    c = _spin1_chain(clv, nx=64, ny=64, nt=16)
    res = []
    for _ in range(2):
        with clv.Engine(c, model=clv.MODEL_SPIN1, precision=clv.PREC_F32) as e:
            e.init_spin1()
            e.step(4)
            res.append(e.get_fields(0))
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])


@pytest.mark.parametrize("shape", [dict(nx=32, ny=8, nt=8), dict(nx=64, ny=32, nt=8)],
                         ids=["fused", "tiled"])
def test_checkpoint_round_trip(clv, tmp_path, shape):
    c = _spin1_chain(clv, **shape)
    path = str(tmp_path / "ck.bin")
    with clv.Engine(c, model=clv.MODEL_SPIN1) as a:
        a.init_spin1()
        a.step(3)
        a.evaluate()
        a.save_checkpoint(path)
        a.step(4)
        a.evaluate()
        want = a.get_fields(0), a.spin1_samples(0), a.step_info()
    with clv.Engine(c, model=clv.MODEL_SPIN1) as b:
        b.load_checkpoint(path)
        b.step(4)
        b.evaluate()
        got = b.get_fields(0), b.spin1_samples(0), b.step_info()
    assert np.array_equal(got[0][0], want[0][0]) and np.array_equal(got[0][1], want[0][1])
    # the observable sums are reduced in a fixed order: equal bit for bit
    assert np.array_equal(got[1], want[1])
    assert got[2]["steps"][0] == want[2]["steps"][0] == 7


def test_nonfinite_flag(clv):
    c = _spin1_chain(clv, nx=16, nt=8)
    with clv.Engine(c, model=clv.MODEL_SPIN1, noise=clv.NOISE_EXTERNAL) as e:
        psi = np.full((3, 8, 16, 1, 1), 0.5 + 0j)
        psi[1, 3, 5, 0, 0] = np.nan
        e.set_fields(0, psi, np.conj(psi))
        e.step_with_noise(np.zeros((3, 16, 1, 1, 8, 2)))
        f = e.chain_flags()
        assert f[0] & clv.FLAG_NONFINITE
        with pytest.raises(clv.ClvError):
            e.chain_flags(raise_on_nonfinite=True)


def test_invalid_configs_rejected(clv):
    with pytest.raises(clv.ClvError):
        clv.Engine(_spin1_chain(clv, nx=7, nt=4), model=clv.MODEL_SPIN1)   # prime 7
    with pytest.raises(clv.ClvError):
        clv.Engine(_spin1_chain(clv, nx=1, nt=4), model=clv.MODEL_SPIN1)

"""The step loop (k_loop.cu): many steps of a small problem under the reference's
step rule in one cooperative launch.  Its trajectory must be the two-kernel
form's bit for bit (filter/drift/reduce pass, then the update; CLV_NO_LOOP=1):
fields, step sizes and Langevin time after odd and even step counts, at FP64
and FP32, on the reference's own 256 x 32 lattice (field and component-half
CTAs), shorter lines and two chains in one launch.  Its grid barrier waits are
bounded: with CLV_TEST_WITHHOLD_COPY the first CTA never arrives, the others'
waits run out after 0.5 s, every chain reports CLV_FLAG_TIMEOUT and the context
stays usable."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def clv():
    import cl_var_dt_gb300 as m
    m.build()
    return m


def _chains(clv, nx, nt, n):
    return [clv.ChainParams(nx=nx, nt=nt, eps=0.01 + 0.005 * i, a_x=1.0, G=0.1, Q=0.02, P=0.05 * i,
                            mu=-1.5 + 0.3 * i, DT=0.002, seed=77 + i) for i in range(n)]


def _run(clv, monkeypatch, chains, prec, loop, counts=(1, 16, 20)):
    monkeypatch.delenv("CLV_TEST_WITHHOLD_COPY", raising=False)
    if loop:
        monkeypatch.delenv("CLV_NO_LOOP", raising=False)
    else:
        monkeypatch.setenv("CLV_NO_LOOP", "1")
    rng = np.random.default_rng(5)
    with clv.Engine(chains, model=clv.MODEL_REF4, precision=prec) as e:
        assert (e.plan()[1] == ["loop_step"]) == loop, e.plan()
        for i in range(len(chains)):
            shape = e.shape(i)
            psi = 1.0 + 0.2 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
            e.set_fields(i, psi, np.conj(psi) + 0.05 * rng.standard_normal(shape))
        for n in counts:
            e.step(n)
        info = e.step_info()
        assert not any(e.chain_flags())
        return [e.get_fields(i) for i in range(len(chains))], info


@pytest.mark.parametrize("case", [(256, 32, 1), (64, 16, 1), (128, 8, 1), (64, 16, 2)],
                         ids=["256x32", "64x16", "128x8", "2x64x16"])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_step_loop_equals_two_kernel_form(clv, monkeypatch, case, prec):
    nx, nt, n = case
    p = clv.PREC_F64 if prec == "f64" else clv.PREC_F32
    chains = _chains(clv, nx, nt, n)
    got, gi = _run(clv, monkeypatch, chains, p, loop=True)
    want, wi = _run(clv, monkeypatch, chains, p, loop=False)
    assert np.array_equal(gi["steps"], wi["steps"]) and all(gi["steps"] == 37)
    for k in ("dt", "max", "mean", "t"):
        assert np.array_equal(gi[k], wi[k]), k
    for (a, b), (c, d) in zip(got, want):
        assert np.array_equal(a, c) and np.array_equal(b, d)


def test_step_loop_barrier_wait_runs_out(clv, monkeypatch):
    chains = _chains(clv, 256, 32, 1)
    monkeypatch.delenv("CLV_NO_LOOP", raising=False)
    monkeypatch.setenv("CLV_TEST_WITHHOLD_COPY", "1")
    t0 = time.time()
    with clv.Engine(chains, model=clv.MODEL_REF4, precision=clv.PREC_F64) as e:
        assert e.plan()[1] == ["loop_step"]
        e.set_mean_field(0, 0.5, 0.0)
        e.set_mean_field(1, 0.5, 0.0)
        e.step(3)
        flags = e.chain_flags()
        import ctypes as C
        f = np.zeros(1, np.int32)
        rc = clv.lib().clv_get_chain_flags(e.h, f.ctypes.data_as(C.POINTER(C.c_int)))
    assert time.time() - t0 < 30
    assert flags[0] & clv._native.FLAG_TIMEOUT
    assert rc == clv._native.ERR_TIMEOUT
    # the context is usable: a normal run afterwards is the two-kernel form's
    got, _ = _run(clv, monkeypatch, chains, clv.PREC_F64, loop=True, counts=(5,))
    want, _ = _run(clv, monkeypatch, chains, clv.PREC_F64, loop=False, counts=(5,))
    assert np.array_equal(got[0][0], want[0][0]) and np.array_equal(got[0][1], want[0][1])


def _spin1_chains(clv, nx, nt, n):
    # the FP64 single-chain workload (1D 64, N_tau 64, beta 4) and variations of it
    return [clv.ChainParams(nx=nx, nt=nt, eps=4.0 / nt, mu=1.0 + 0.2 * i, c0=0.5, c1=-0.1, q=0.05, K=0.05,
                            dt_max=1e-3, seed=11 + i) for i in range(n)]


def _run_spin1(clv, monkeypatch, chains, prec, loop, counts=(1, 16, 20)):
    monkeypatch.delenv("CLV_TEST_WITHHOLD_COPY", raising=False)
    if loop:
        monkeypatch.delenv("CLV_NO_LOOP", raising=False)
    else:
        monkeypatch.setenv("CLV_NO_LOOP", "1")
    with clv.Engine(chains, model=clv.MODEL_SPIN1, precision=prec) as e:
        if loop:
            assert e.plan()[1] == ["loop_step"], e.plan()
        else:
            assert e.plan()[1] == ["fused_step", "fused_redo"], e.plan()
        e.init_spin1()
        for n in counts:
            e.step(n)
        info = e.step_info()
        assert not any(e.chain_flags())
        return [e.get_fields(i) for i in range(len(chains))], info


@pytest.mark.parametrize("case", [(64, 64, 1), (128, 16, 2), (256, 32, 1)], ids=["64x64", "2x128x16", "256x32"])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_step_loop_kmax_equals_speculative_step(clv, monkeypatch, case, prec):
    """Under the K/max rule the loop computes dt before any update (no speculation);
    against the production kernel's speculative step with its redo pass: bit for bit
    (FP64 lines of 256 excepted: the loop's field CTAs filter them on warp pairs, 1e-13)."""
    nx, nt, n = case
    p = clv.PREC_F64 if prec == "f64" else clv.PREC_F32
    chains = _spin1_chains(clv, nx, nt, n)
    got, gi = _run_spin1(clv, monkeypatch, chains, p, loop=True)
    want, wi = _run_spin1(clv, monkeypatch, chains, p, loop=False)
    assert all(gi["steps"] == 37) and all(wi["steps"] == 37)
    exact = not (prec == "f64" and nx == 256)
    for k in ("dt", "max", "t"):
        if exact:
            assert np.array_equal(gi[k], wi[k]), k
        else:
            assert np.allclose(gi[k], wi[k], rtol=1e-13, atol=0), k
    for (a, b), (c, d) in zip(got, want):
        if exact:
            assert np.array_equal(a, c) and np.array_equal(b, d)
        else:
            assert np.abs(a - c).max() < 1e-13 * np.abs(c).max() and np.abs(b - d).max() < 1e-13 * np.abs(d).max()

"""Failure detection without a GPU fault: the fused kernel's waits on its bulk
copies are bounded (0.5 s), after which the CTA records CLV_FLAG_TIMEOUT,
issues nothing more and leaves.  With CLV_TEST_WITHHOLD_COPY the first CTA
never issues its first copy, so its wait runs out; the host reads the status,
the other chains' results are those of a normal run, and the context stays
usable."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def clv():
    import cl_var_dt_gb300 as m
    m.build()
    return m


def chains(clv):
    return [clv.ChainParams(nx=256, nt=16, eps=6 / 128, mu=0.5 + 0.4 * i, c0=0.5, c1=-0.1, q=0.05,
                            K=0.05, dt_max=1e-3, seed=5) for i in range(3)]


def one_step(clv, monkeypatch, withhold):
    for k in ("CLV_FUSED", "CLV_TILED", "CLV_NO_TMA", "CLV_CHUNK", "CLV_TEST_WITHHOLD_COPY"):
        monkeypatch.delenv(k, raising=False)
    monkeypatch.setenv("CLV_NO_LOOP", "1")  # the fused kernel's copy waits (the loop's: test_gpu_loop.py)
    if withhold:
        monkeypatch.setenv("CLV_TEST_WITHHOLD_COPY", "1")
    with clv.Engine(chains(clv), model=clv.MODEL_SPIN1, precision=clv.PREC_F32) as e:
        assert e.plan()[0] == "fused"
        e.init_spin1()
        e.step(1)
        flags = e.chain_flags()
        import ctypes as C
        f = np.zeros(3, np.int32)
        rc = clv.lib().clv_get_chain_flags(e.h, f.ctypes.data_as(C.POINTER(C.c_int)))
        return flags, rc, [e.get_fields(i) for i in range(3)]


def test_bounded_wait_runs_out_and_is_reported(clv, monkeypatch):
    t0 = time.time()
    flags, rc, out = one_step(clv, monkeypatch, withhold=True)
    assert time.time() - t0 < 30
    assert flags[0] & clv._native.FLAG_TIMEOUT
    assert rc == clv._native.ERR_TIMEOUT
    assert not (flags[1] & clv._native.FLAG_TIMEOUT) and not (flags[2] & clv._native.FLAG_TIMEOUT)
    # the context is usable and the other chains match a normal run bit for bit
    flags_ok, rc_ok, ref = one_step(clv, monkeypatch, withhold=False)
    assert rc_ok == clv._native.OK and not flags_ok.any()
    for i in (1, 2):
        assert np.array_equal(out[i][0], ref[i][0]) and np.array_equal(out[i][1], ref[i][1])

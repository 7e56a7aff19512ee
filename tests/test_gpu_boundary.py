"""Field transfers across the C ABI in both element types (complex128, the
reference's, and complex64 with CLV_C64), host and device buffers, one chain or
all chains at once."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def clv():
    import cl_var_dt_gb300 as m
    m.build()
    return m


def chains(clv):
    return [clv.ChainParams(nx=64, ny=8, nt=6, seed=1), clv.ChainParams(nx=32, nt=10, seed=2)]


def rand(shape, rng):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_complex64_and_complex128_transfers(clv, prec):
    rng = np.random.default_rng(3)
    precision = clv.PREC_F32 if prec == "f32" else clv.PREC_F64
    with clv.Engine(chains(clv), model=clv.MODEL_SPIN1, precision=precision) as e:
        for i in range(2):
            a, b = rand(e.shape(i), rng), rand(e.shape(i), rng)
            e.set_fields(i, a, b)
            p128, q128 = e.get_fields(i)
            p64, q64 = e.get_fields(i, np.complex64)
            assert np.array_equal(p64, p128.astype(np.complex64))
            assert np.array_equal(q64, q128.astype(np.complex64))
            if prec == "f64":
                assert np.array_equal(p128, a) and np.array_equal(q128, b)
            # complex64 in
            a32, b32 = a.astype(np.complex64), b.astype(np.complex64)
            e.set_fields(i, a32, b32)
            p128, q128 = e.get_fields(i)
            assert np.array_equal(p128, a32.astype(np.complex128))
            assert np.array_equal(q128, b32.astype(np.complex128))
        # every chain at once, complex64 host buffers
        total = sum(int(np.prod(e.shape(i))) for i in range(2))
        hp = np.zeros(total, np.complex64)
        hq = np.zeros(total, np.complex64)
        L = clv.lib()
        assert L.clv_get_fields(e.h, -1, hp.ctypes.data_as(C.c_void_p), hq.ctypes.data_as(C.c_void_p),
                                clv.HOST | clv.C64) == 0
        n0 = int(np.prod(e.shape(0)))
        assert np.array_equal(hp[n0:], e.get_fields(1, np.complex64)[0].ravel())
        hp2 = (hp * 2).astype(np.complex64)
        assert L.clv_set_fields(e.h, -1, hp2.ctypes.data_as(C.c_void_p), hq.ctypes.data_as(C.c_void_p),
                                clv.HOST | clv.C64) == 0
        assert np.array_equal(e.get_fields(0, np.complex64)[0].ravel(), hp2[:n0])
        # an unknown flag is rejected before any transfer
        assert L.clv_set_fields(e.h, -1, hp2.ctypes.data_as(C.c_void_p), hq.ctypes.data_as(C.c_void_p),
                                8) == clv._native.ERR_ARG


def test_device_buffers_complex64(clv):
    import torch
    with clv.Engine(chains(clv), model=clv.MODEL_SPIN1, precision=clv.PREC_F32) as e:
        e.init_spin1()
        n = int(np.prod(e.shape(0)))
        dp = torch.zeros(n, dtype=torch.complex64, device="cuda")
        dq = torch.zeros(n, dtype=torch.complex64, device="cuda")
        L = clv.lib()
        assert L.clv_get_fields(e.h, 0, C.c_void_p(dp.data_ptr()), C.c_void_p(dq.data_ptr()),
                                clv.DEVICE | clv.C64) == 0
        torch.cuda.synchronize()
        p, q = e.get_fields(0, np.complex64)
        assert np.array_equal(dp.cpu().numpy(), p.ravel()) and np.array_equal(dq.cpu().numpy(), q.ravel())


@pytest.mark.parametrize("c64", [True, False], ids=["complex64", "complex128"])
def test_async_transfers_complete_after_synchronize(clv, c64):
    """Asynchronous transfers of all chains' fields around steps: complex64 (the FP32
    engine's own element type, copied as is) and complex128 (the reference's, converted
    on the device through the staging buffer, which both fields share in stream order)."""
    rng = np.random.default_rng(9)
    dt = np.complex64 if c64 else np.complex128
    flag = clv.C64 if c64 else 0
    with clv.Engine(chains(clv), model=clv.MODEL_SPIN1, precision=clv.PREC_F32) as e:
        total = sum(int(np.prod(e.shape(i))) for i in range(2))
        a = rand(total, rng).astype(dt)
        b = rand(total, rng).astype(dt)
        L = clv.lib()
        w = clv.HOST | flag | clv.ASYNC
        assert L.clv_set_fields(e.h, -1, a.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p), w) == 0
        assert L.clv_step(e.h, 2) == 0
        pa = np.zeros(total, dt)
        pb = np.zeros(total, dt)
        assert L.clv_get_fields(e.h, -1, pa.ctypes.data_as(C.c_void_p), pb.ctypes.data_as(C.c_void_p), w) == 0
        assert L.clv_synchronize(e.h) == 0
        qa = np.zeros(total, dt)
        qb = np.zeros(total, dt)
        assert L.clv_get_fields(e.h, -1, qa.ctypes.data_as(C.c_void_p), qb.ctypes.data_as(C.c_void_p),
                                clv.HOST | flag) == 0
        assert np.array_equal(pa, qa) and np.array_equal(pb, qb)
        assert not np.array_equal(pa, a)  # two steps moved the fields

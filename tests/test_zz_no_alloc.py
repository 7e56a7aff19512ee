"""clv_ref_observables_noalloc (the allocation-free observables entry point)
against the engine path (clv_evaluate + clv_read_ref_observables) on the same
field configurations, through the C ABI.  Two calls in a row on each lattice,
with different fields, check that the shared scratch left by one call does not
leak into the next.  Kept last in collection order and self-contained, so it
passes alone in a fresh process and after the other tests.

Tolerance: 1e-12 relative (FP64; the two paths sum the CTA partials in a
different order)."""
import ctypes

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-12
MAX_SITES = 1 << 20


@pytest.fixture(scope="module")
def clv():
    import cl_var_dt_gb300 as m
    m.build()
    return m


def _fields(rng, shape):
    f = lambda: (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) * 0.5 + 0.3
    return f(), f()


def _engine_obs(clv, chain, psi, psic):
    with clv.Engine(chain, model=clv.MODEL_REF4, precision=clv.PREC_F64) as e:
        e.set_fields(0, psi, psic)
        e.evaluate()
        return e.ref_observables(0)


def _noalloc_obs(clv, chain, psi, psic):
    import torch
    dev = torch.device("cuda", 0)
    d_psi = torch.from_numpy(np.ascontiguousarray(psi)).to(dev)
    d_psic = torch.from_numpy(np.ascontiguousarray(psic)).to(dev)
    V = chain.nx * chain.ny * chain.nz
    # garbage in the outputs: the entry point must overwrite them, not add to them
    d_n = torch.full((5,), 7.0, dtype=torch.float64, device=dev)
    d_F = torch.full((3 * V,), -3.0, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = clv.lib().clv_ref_observables_noalloc(
        ctypes.c_void_p(d_psi.data_ptr()), ctypes.c_void_p(d_psic.data_ptr()), chain.nx, chain.ny,
        chain.nz, chain.nt, chain.a_x, ctypes.c_void_p(d_n.data_ptr()),
        ctypes.c_void_p(d_F.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, clv.lib().clv_last_error().decode()
    torch.cuda.synchronize(dev)
    return d_n.cpu().numpy(), d_F.cpu().numpy().reshape(3, V)


# (45, 9, 5, 3): 2025 sites, 8 CTAs of 256 with a partial last one (233 sites)
@pytest.mark.parametrize("dims", [(16, 4, 2, 8), (64, 8, 4, 4), (32, 32, 30, 2), (256, 1, 1, 32), (45, 9, 5, 3)],
                         ids=lambda d: "x".join(map(str, d)))
def test_noalloc_matches_engine_two_calls_in_a_row(clv, dims):
    nx, ny, nz, nt = dims
    chain = clv.ChainParams(nx=nx, ny=ny, nz=nz, nt=nt, a_x=0.7)
    rng = np.random.default_rng(nx * 1000 + nt)
    for call in range(2):
        psi, psic = _fields(rng, (4, nt, nx, ny, nz))
        n_ref, F_ref = _engine_obs(clv, chain, psi, psic)
        n, F = _noalloc_obs(clv, chain, psi, psic)
        assert rel_err(n, n_ref) < TOL, (call, n, n_ref)
        for k in range(3):
            assert rel_err(F[k], F_ref[k]) < TOL, (call, k)


def test_noalloc_rejects_lattices_above_its_limit(clv):
    import torch
    dev = torch.device("cuda", 0)
    buf = torch.zeros(64, dtype=torch.float64, device=dev)
    p = ctypes.c_void_p(buf.data_ptr())
    rc = clv.lib().clv_ref_observables_noalloc(p, p, MAX_SITES + 1, 1, 1, 2, 1.0, p, p, None)
    assert rc == clv._native.ERR_ARG
    assert "exceeds its maximum" in clv.lib().clv_last_error().decode()
    # the limit itself is accepted by the argument checks (not run: no buffers that large here)
    assert MAX_SITES == 1048576

"""Parity with the reference's own GPU build.

The reference's kernels, compiled unchanged from its sources into sm_103a cubins
(oracle/ref_gpu_build.sh, one per lattice configuration of oracle/refgpu.py),
run with the real cuFFT and cuRAND in the order of Propagator::propagate
(Propagator_without_cutoff.cu:406-442) by oracle/ref_gpu_runner.cpp.  With the
same injected noise, one step of the engine matches that build per site:

  FP64 (the plain drop-in): 1e-12, floored relative error max|a-b| / max(|b|, rms b);
  FP32-mixed: 1e-5 after the first step, 1e-5 x (s + 1) after step s (the FP32
  rounding accumulates over steps; the bound is stated per step).

The reference build is also checked against the golden vectors (its kernels run
on the host with numpy's DFT for cuFFT): that pins the host restatement of cuFFT.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, large_golden_files, load_golden, load_large_golden, rel_err

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5
NSTEPS = 3


@pytest.fixture(scope="module")
def clv():
    import cl_var_dt_gb300 as m
    m.build()
    return m


@pytest.fixture(scope="module")
def refgpu():
    import refgpu as r
    r.build_runner()
    missing = [n for n in r.CONFIGS if not r.have_cubin(n)]
    if missing:
        pytest.skip(f"reference cubins not built ({missing}): run oracle/refgpu.py where the reference "
                    "sources are (CLV_REFERENCE_DIR)")
    return r


def _inputs(refgpu, name, nsteps):
    """psi0, psic0 and nsteps noise buffers of a configuration: the golden vectors'
    where a fixture exists, else reproducible inputs of tests/golden/detinputs.py."""
    import detinputs
    small = os.path.join(GOLDEN, f"ref4_{name}.npz")
    large = os.path.join(GOLDEN, f"ref4l_{name}.npz")
    X, Y, Z, T, Cn = (int(refgpu.macros(name)[k]) for k in ("XSIZE", "YSIZE", "ZSIZE", "TAUSIZE", "COMPONENTS"))
    nshape = (Cn, X, Y, Z, T, 2)
    if os.path.exists(small):
        g, _ = load_golden(small)
        noise = [g["noise"][s] for s in range(len(g["dt"]))]
        psi0, psic0 = g["psi0"], g["psic0"]
    elif os.path.exists(large):
        _, _, psi0, psic0, n0 = load_large_golden(large)
        noise = [n0]
    else:
        psi0, psic0 = detinputs.ref4_inputs((Cn, T, X, Y, Z), 303)
        noise = []
    seed = 1000
    while len(noise) < nsteps:
        noise.append(detinputs.noise(nshape, seed + len(noise)))
    return psi0, psic0, noise[:nsteps]


def _chain(clv, refgpu, name):
    m = refgpu.macros(name)
    P, MU = refgpu.CONFIGS[name][1], refgpu.CONFIGS[name][2]
    return clv.ChainParams(nx=int(m["XSIZE"]), ny=int(m["YSIZE"]), nz=int(m["ZSIZE"]), nt=int(m["TAUSIZE"]),
                           eps=float(m["EPS"]), a_x=float(m["a_x"]), G=float(m["G"]), Q=float(m["Q"]),
                           P=P, mu=MU, DT=float(m["DT"]))


NAMES = ["1d_x16_t16", "1d_x32_t8_pq", "2d_x16_y4_t8", "3d_x8_y4_z2_t8", "1d_x16_t16_zero", "1d_x64_t32",
         "1d_x256_t32", "1d_x64_t64", "1d_x256_t128"]


@pytest.mark.parametrize("name", NAMES[:6])
def test_reference_gpu_build_matches_golden(refgpu, name):
    """cuFFT + the reference's kernels on the GPU against the host pin (numpy DFT)."""
    g, kw = load_golden(os.path.join(GOLDEN, f"ref4_{name}.npz"))
    with refgpu.RefGpu(name) as r:
        if name.endswith("zero"):
            r.set_fields(np.ones_like(g["psi0"]), np.ones_like(g["psic0"]))
            r.set_mean_field(0.0, 0.0)
        else:
            r.set_fields(g["psi0"], g["psic0"])
        n, F = r.observables()
        assert rel_err(n, g["n0"]) < TOL64 and rel_err(F, g["F0"]) < TOL64
        for s in range(len(g["dt"])):
            dt, mx, mean = r.propagate(g["noise"][s])
            assert abs(dt - g["dt"][s]) <= TOL64 * g["dt"][s]
            psi, psic = r.get_fields()
            assert rel_err(psi, g["psi"][s]) < TOL64
            assert rel_err(psic, g["psic"][s]) < TOL64


@pytest.mark.parametrize("path", large_golden_files(), ids=lambda p: p.split("/")[-1][6:-4])
def test_reference_gpu_build_matches_large_golden(refgpu, path):
    g, kw, psi0, psic0, noise = load_large_golden(path)
    name = os.path.basename(path)[6:-4]
    with refgpu.RefGpu(name) as r:
        r.set_fields(psi0, psic0)
        n, F = r.observables()
        assert rel_err(n, g["n0"]) < TOL64 and rel_err(F, g["F0"]) < TOL64
        dt, mx, mean = r.propagate(noise)
        assert abs(dt - g["dt"][0]) <= TOL64 * g["dt"][0]
        psi, psic = r.get_fields()
        assert rel_err(psi.reshape(-1)[g["idx"]], g["psi"]) < TOL64
        assert rel_err(psic.reshape(-1)[g["idx"]], g["psic"]) < TOL64


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_engine_matches_reference_gpu_build(clv, refgpu, name, prec):
    """NSTEPS steps from the same start with the same injected noise, compared per
    site after every step, plus the step sizes."""
    psi0, psic0, noise = _inputs(refgpu, name, NSTEPS)
    precision = clv.PREC_F64 if prec == "f64" else clv.PREC_F32
    with refgpu.RefGpu(name) as r, clv.Engine(_chain(clv, refgpu, name), model=clv.MODEL_REF4,
                                               noise=clv.NOISE_EXTERNAL, precision=precision) as e:
        if name.endswith("zero"):
            r.set_fields(np.ones_like(psi0), np.ones_like(psic0))
            r.set_mean_field(0.0, 0.0)
            psi0, psic0 = r.get_fields()
        r.set_fields(psi0, psic0)
        e.set_fields(0, psi0, psic0)
        for s in range(NSTEPS):
            dt, mx, mean = r.propagate(noise[s])
            e.step_with_noise(noise[s])
            info = e.step_info()
            tol = TOL64 if prec == "f64" else TOL32 * (s + 1)
            assert abs(info["dt"][0] - dt) <= tol * dt, s
            assert abs(info["max"][0] - mx) <= tol * max(mx, 1e-300), s
            want, wantc = r.get_fields()
            got, gotc = e.get_fields(0)
            assert rel_err(got, want) < tol, s
            assert rel_err(gotc, wantc) < tol, s


@pytest.mark.parametrize("name", ["1d_x32_t8_pq", "2d_x16_y4_t8", "3d_x8_y4_z2_t8", "1d_x256_t32"])
def test_engine_observables_match_reference_gpu_build(clv, refgpu, name):
    """n_tot, n_11..n_22 and the F profiles of Observables::evaluate (per call sums
    of the reference; the engine reports them divided by T (and V for n))."""
    psi0, psic0, _ = _inputs(refgpu, name, 1)
    c = _chain(clv, refgpu, name)
    with refgpu.RefGpu(name) as r, clv.Engine(c, model=clv.MODEL_REF4, noise=clv.NOISE_EXTERNAL) as e:
        r.set_fields(psi0, psic0)
        e.set_fields(0, psi0, psic0)
        e.evaluate()
        n, F = e.ref_observables(0)
        rn, rF = r.observables()
        assert rel_err(n, rn / c.nt / c.vol) < TOL64
        assert rel_err(F, rF / c.nt) < TOL64

"""The tiled path (per-axis kinetic filter kernels, then the tau-streaming step
kernel) used for slices too large for the fused kernel: against the reference's
kernels (golden vectors), the oracle, the separate-kernel path, and invariance
under its internal choices (chunking, speculation).

Tolerances: FP64 1e-12, FP32-mixed 1e-5 relative per site (single step, same noise).
"""
import numpy as np
import pytest

from conftest import golden_files, load_golden, rel_err

pytestmark = pytest.mark.gpu

ENV = ("CLV_FUSED", "CLV_TILED", "CLV_NO_TMA", "CLV_NO_SPECULATE", "CLV_CHUNK", "CLV_NO_STATIC_PLAN",
       "CLV_NO_PLANE")


@pytest.fixture(scope="module")
def clv():
    import cl_var_dt_gb300 as m
    m.build()
    return m


@pytest.fixture
def env(monkeypatch):
    for k in ENV:
        monkeypatch.delenv(k, raising=False)

    def set_(**kw):
        for k, v in kw.items():
            monkeypatch.setenv(k, v)
    return set_


def spin1(clv, **kw):
    base = dict(nx=64, ny=32, nz=1, nt=16, eps=8 / 128, mu=0.8, c0=0.3, c1=-0.05, q=0.02, K=0.05,
                dt_max=1e-3, seed=20261203)
    base.update(kw)
    return clv.ChainParams(**base)


def run(clv, chains, steps, precision, model=None):
    with clv.Engine(chains, model=model if model is not None else clv.MODEL_SPIN1,
                    precision=precision) as e:
        e.init_spin1()
        e.step(steps)
        return [e.get_fields(i) for i in range(len(chains))], e.step_info(), e.plan()


def test_large_slices_take_the_tiled_path(clv, env):
    with clv.Engine(spin1(clv, nx=128, ny=128, nt=8), model=clv.MODEL_SPIN1,
                    precision=clv.PREC_F32) as e:
        path, phases = e.plan()
        assert path == "tiled" and phases == ["plane01_n128", "tiled_step", "tiled_redo"]
    with clv.Engine(spin1(clv, nx=8, ny=64, nz=64, nt=4), model=clv.MODEL_SPIN1,
                    precision=clv.PREC_F64) as e:
        assert e.plan()[1] == ["axis0_n8", "plane12_n64", "tiled_step", "tiled_redo"]
    env(CLV_NO_PLANE="1")
    with clv.Engine(spin1(clv, nx=128, ny=128, nt=8), model=clv.MODEL_SPIN1,
                    precision=clv.PREC_F32) as e:
        path, phases = e.plan()
        assert path == "tiled" and phases == ["axis0_n128", "axis1_n128", "tiled_step", "tiled_redo"]
    with clv.Engine(spin1(clv, nx=256, ny=1, nt=8), model=clv.MODEL_SPIN1) as e:
        assert e.plan()[0] == "fused"


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.split("/")[-1][5:-4])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_ref4_tiled_matches_reference_kernels(clv, env, path, prec):
    env(CLV_FUSED="0")
    g, kw = load_golden(path)
    tol = 1e-12 if prec == "f64" else 1e-5
    c = clv.ChainParams(nx=kw["nx"], ny=kw["ny"], nz=kw["nz"], nt=kw["nt"], eps=kw["eps"], a_x=kw["a_x"],
                        G=kw["G"], Q=kw["Q"], P=kw["P"], mu=kw["mu"], DT=kw["DT"])
    with clv.Engine(c, model=clv.MODEL_REF4, noise=clv.NOISE_EXTERNAL,
                    precision=clv.PREC_F64 if prec == "f64" else clv.PREC_F32) as e:
        assert e.plan()[0] == "tiled"
        e.set_fields(0, g["psi0"], g["psic0"])
        for s in range(len(g["dt"])):
            e.step_with_noise(g["noise"][s])
            info = e.step_info()
            assert abs(info["dt"][0] - g["dt"][s]) <= tol * g["dt"][s]
            psi, psic = e.get_fields(0)
            if prec == "f64" or s == 0:
                assert rel_err(psi, g["psi"][s]) < tol and rel_err(psic, g["psic"][s]) < tol


SHAPES = [
    dict(nx=64, ny=32, nt=8),            # 2D, compile-time plans, full tiles
    dict(nx=48, ny=40, nt=6),            # 2D, runtime plans (radix 3, 5), partial tiles
    dict(nx=96, ny=32, nt=4),            # 2D, compile-time mixed-radix plans (8 4 3; 8 4)
    dict(nx=128, ny=16, nt=4),           # 2D, radix-16 plan for 128-site lines (16 8)
    dict(nx=16, ny=12, nz=10, nt=4),     # 3D, three axes, partial tiles
    dict(nx=2048, nt=4),                 # long 1D line: beyond the axis filter's 512
    dict(nx=32, ny=32, nt=16, K=1e-4),   # K/max binding: speculative update redone
    dict(nx=64, ny=64, nt=4),            # 2D square: plane filter (64)
    dict(nx=128, ny=128, nt=2),          # 2D square: plane filter (128; FP64 by axes)
    dict(nx=96, ny=96, nt=2),            # 2D square: plane filter (96 = 8 4 3)
    dict(nx=4, ny=64, nz=64, nt=2),      # 3D: x axis, then the (y, z) planes
    dict(nx=64, ny=8, nz=8, nt=2),       # 3D: x lines of 64 strided by 64 (lines in registers / in-place tiles)
    dict(nx=256, ny=8, nt=2),            # 2D: lines of 256 strided by 8 (in-place tiles, 8 8 4)
    dict(nx=512, ny=4, nt=2),            # 2D: lines of 512 strided by 4 (in-place tiles at FP64, 8 8 8)
]


@pytest.mark.parametrize("shape", SHAPES, ids=lambda d: "x".join(f"{k}{v}" for k, v in d.items()))
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_spin1_tiled_matches_oracle(clv, oracle, env, shape, prec):
    env(CLV_FUSED="0")
    c = spin1(clv, **shape)
    tol = 1e-12 if prec == "f64" else 1e-5
    p = oracle.spin1_params(nx=c.nx, ny=c.ny, nz=c.nz, nt=c.nt, eps=c.eps, mu=c.mu, c0=c.c0, c1=c.c1,
                            q=c.q, Kc=c.K, dt_max=c.dt_max)
    with clv.Engine(c, model=clv.MODEL_SPIN1,
                    precision=clv.PREC_F64 if prec == "f64" else clv.PREC_F32) as e:
        expect = "unfused" if c.nx > 512 else "tiled"
        assert e.plan()[0] == expect
        e.init_spin1()
        psi, psic = oracle.spin1_init(p, c.seed, 0)
        for k in range(2):
            e.step(1)
            psi, psic, dt, _, _ = oracle.step(p, psi, psic, seed=c.seed, chain=0, step_index=k)
            info = e.step_info()
            assert abs(info["dt"][0] - dt) <= tol * dt
            gp, gc = e.get_fields(0)
            assert rel_err(gp, psi) < tol and rel_err(gc, psic) < tol
            psi, psic = gp, gc  # continue from the engine's state (FP32 rounding stays local)


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_tiled_equals_separate_kernels(clv, env, prec):
    p = clv.PREC_F64 if prec == "f64" else clv.PREC_F32
    chains = [spin1(clv), spin1(clv, nx=32, ny=48, nt=12, mu=0.5, seed=5)]
    env(CLV_FUSED="0")
    a, ia, pa = run(clv, chains, 4, p)
    env(CLV_TILED="0")
    b, ib, pb = run(clv, chains, 4, p)
    assert pa[0] == "tiled" and pb[0] == "unfused"
    tol = 1e-13 if prec == "f64" else 2e-6
    for (x, xc), (y, yc) in zip(a, b):
        assert rel_err(x, y) < tol and rel_err(xc, yc) < tol
    assert np.allclose(ia["dt"], ib["dt"], rtol=tol)


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_plane_filter_equals_axis_filters(clv, env, prec):
    """Both axes of square planes in one launch against one launch per axis (planes of
    64, 96 and 128; 240 planes of 128, more than one wave of CTAs)."""
    p = clv.PREC_F64 if prec == "f64" else clv.PREC_F32
    chains = [spin1(clv, nx=64, ny=64, nt=6), spin1(clv, nx=6, ny=64, nz=64, nt=3, mu=0.5, seed=5),
              spin1(clv, nx=128, ny=128, nt=40, mu=1.1, seed=9), spin1(clv, nx=96, ny=96, nt=4, seed=3)]
    a, ia, pa = run(clv, chains, 3, p)
    env(CLV_NO_PLANE="1")
    b, ib, pb = run(clv, chains, 3, p)
    assert any(x.startswith("plane") for x in pa[1]) and not any(x.startswith("plane") for x in pb[1])
    tol = 1e-13 if prec == "f64" else 2e-6
    for (x, xc), (y, yc) in zip(a, b):
        assert rel_err(x, y) < tol and rel_err(xc, yc) < tol
    assert np.allclose(ia["dt"], ib["dt"], rtol=tol)


def test_tiled_speculation_and_two_pass_are_bitwise_equal(clv, env):
    chains = [spin1(clv, seed=s, mu=0.3 + 0.2 * s, K=0.05 if s % 2 else 1e-4) for s in range(4)]
    a, ia, _ = run(clv, chains, 5, clv.PREC_F32)
    env(CLV_NO_SPECULATE="1")
    b, ib, _ = run(clv, chains, 5, clv.PREC_F32)
    for (x, xc), (y, yc) in zip(a, b):
        assert np.array_equal(x, y) and np.array_equal(xc, yc)
    assert np.array_equal(ia["t"], ib["t"])


@pytest.mark.parametrize("chunk", ["1", "5", "64"])
def test_tiled_chunking_does_not_change_results(clv, env, chunk):
    chains = [spin1(clv, nt=24), spin1(clv, nx=128, ny=16, nt=10, seed=3)]
    a, _, _ = run(clv, chains, 2, clv.PREC_F64)
    env(CLV_CHUNK=chunk)
    b, _, _ = run(clv, chains, 2, clv.PREC_F64)
    for (x, xc), (y, yc) in zip(a, b):
        assert np.array_equal(x, y) and np.array_equal(xc, yc)


def test_mixed_batch_uneven_sizes(clv, oracle, env):
    """Chains of different 2D sizes and imaginary-time extents in one engine."""
    chains = [spin1(clv, nx=64, ny=64, nt=8, seed=1), spin1(clv, nx=96, ny=96, nt=4, mu=1.2, seed=2),
              spin1(clv, nx=32, ny=64, nt=12, mu=0.4, seed=3)]
    out, info, plan = run(clv, chains, 1, clv.PREC_F64)
    assert plan[0] == "tiled"
    for i, c in enumerate(chains):
        p = oracle.spin1_params(nx=c.nx, ny=c.ny, nz=c.nz, nt=c.nt, eps=c.eps, mu=c.mu, c0=c.c0,
                                c1=c.c1, q=c.q, Kc=c.K, dt_max=c.dt_max)
        psi, psic = oracle.spin1_init(p, c.seed, i)
        psi, psic, dt, _, _ = oracle.step(p, psi, psic, seed=c.seed, chain=i, step_index=0)
        assert rel_err(out[i][0], psi) < 1e-12 and rel_err(out[i][1], psic) < 1e-12


@pytest.mark.parametrize("shape", [dict(nx=64, ny=32, nt=8), dict(nx=16, ny=12, nz=10, nt=4)], ids=["2d", "3d"])
def test_tiled_stored_drift_equals_apply_pass(clv, env, shape):
    """Reference rule on the tiled path at FP64: the reduce pass storing the drift and
    the site-parallel update applying it (the default: FP64 arithmetic is scarce) give
    the same steps, bit for bit, as a second drift pass."""
    env(CLV_FUSED="0")
    c = clv.ChainParams(**shape, eps=0.02, a_x=1.0, G=0.1, Q=0.02, P=0.05, mu=-0.5, DT=0.002, seed=7)
    out = []
    for sd in ("1", "0"):
        env(CLV_STORE_DRIFT=sd)
        with clv.Engine(c, model=clv.MODEL_REF4, precision=clv.PREC_F64) as e:
            assert e.plan()[0] == "tiled"
            assert e.plan()[1][-1] == ("stored_drift_update" if sd == "1" else "tiled_apply")
            rng = np.random.default_rng(2)
            f = (rng.standard_normal(e.shape(0)) + 1j * rng.standard_normal(e.shape(0))) * 0.3 + 0.5
            e.set_fields(0, f, np.conj(f))
            e.step(3)
            out.append((e.get_fields(0), e.step_info()))
    (a, ia), (b, ib) = out
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(ia["dt"], ib["dt"]) and np.array_equal(ia["t"], ib["t"])

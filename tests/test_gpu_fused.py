"""The fused tau-streaming step against the unfused kernels and the oracle, and
invariance of its results under its internal choices (chunking, TMA, speculation).
"""
import numpy as np
import pytest

from conftest import golden_files, load_golden, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def clv():
    import cl_var_dt_gb300 as m
    m.build()
    return m


def spin1(clv, **kw):
    base = dict(nx=256, ny=1, nz=1, nt=32, eps=6 / 128, mu=1.1, c0=0.5, c1=-0.15, q=0.05, K=0.05,
                dt_max=1e-3, seed=77)
    base.update(kw)
    return clv.ChainParams(**base)


def run(clv, chains, steps, precision, monkeypatch, env=None, model=None):
    for k in ("CLV_FUSED", "CLV_TILED", "CLV_NO_TMA", "CLV_NO_SPECULATE", "CLV_CHUNK",
              "CLV_NO_STATIC_PLAN", "CLV_FUSED_SPLIT", "CLV_NO_LOOP"):
        monkeypatch.delenv(k, raising=False)
    for k, v in (env or {}).items():
        monkeypatch.setenv(k, v)
    with clv.Engine(chains, model=model if model is not None else clv.MODEL_SPIN1,
                    precision=precision) as e:
        e.init_spin1()
        e.step(steps)
        out = [e.get_fields(i) for i in range(len(chains))]
        return out, e.step_info()


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_fused_equals_unfused(clv, monkeypatch, prec):
    p = clv.PREC_F64 if prec == "f64" else clv.PREC_F32
    chains = [spin1(clv), spin1(clv, nx=64, ny=4, nt=16, mu=0.7, seed=5)]
    a, ia = run(clv, chains, 4, p, monkeypatch)
    b, ib = run(clv, chains, 4, p, monkeypatch, {"CLV_FUSED": "0", "CLV_TILED": "0"})
    tol = 1e-13 if prec == "f64" else 2e-6
    for (x, xc), (y, yc) in zip(a, b):
        assert rel_err(x, y) < tol and rel_err(xc, yc) < tol
    assert np.allclose(ia["dt"], ib["dt"], rtol=tol)


def test_speculation_and_two_pass_are_bitwise_equal(clv, monkeypatch):
    chains = [spin1(clv, seed=s, mu=0.3 + 0.2 * s) for s in range(4)]
    a, ia = run(clv, chains, 5, clv.PREC_F32, monkeypatch)
    b, ib = run(clv, chains, 5, clv.PREC_F32, monkeypatch, {"CLV_NO_SPECULATE": "1"})
    for (x, xc), (y, yc) in zip(a, b):
        assert np.array_equal(x, y) and np.array_equal(xc, yc)
    assert np.array_equal(ia["t"], ib["t"])


def test_rejected_speculation_matches_oracle(clv, oracle, monkeypatch):
    """K small enough that K/max|drift| < dt_max: every speculative update is redone
    (the two-kernel form: the step loop, which takes this small problem by default,
    computes dt before updating and never speculates)."""
    c = spin1(clv, nx=64, nt=16, K=1e-5)
    out, info = run(clv, [c], 3, clv.PREC_F64, monkeypatch, {"CLV_NO_LOOP": "1"})
    p = oracle.spin1_params(nx=64, nt=16, eps=c.eps, mu=c.mu, c0=c.c0, c1=c.c1, q=c.q, Kc=c.K,
                            dt_max=c.dt_max)
    psi, psic = oracle.spin1_init(p, c.seed, 0)
    for k in range(3):
        psi, psic, dt, _, _ = oracle.step(p, psi, psic, seed=c.seed, chain=0, step_index=k)
    assert dt < c.dt_max
    assert rel_err(out[0][0], psi) < 1e-11 and rel_err(out[0][1], psic) < 1e-11
    assert info["dt"][0] == pytest.approx(dt, rel=1e-12)


def test_plain_loads_equal_tma(clv, monkeypatch):
    chains = [spin1(clv), spin1(clv, nx=96, nt=12, seed=9)]
    a, _ = run(clv, chains, 3, clv.PREC_F32, monkeypatch)
    b, _ = run(clv, chains, 3, clv.PREC_F32, monkeypatch, {"CLV_NO_TMA": "1"})
    for (x, xc), (y, yc) in zip(a, b):
        assert np.array_equal(x, y) and np.array_equal(xc, yc)


@pytest.mark.parametrize("chunk", ["1", "3", "64"])
def test_chunking_does_not_change_results(clv, monkeypatch, chunk):
    chains = [spin1(clv, nt=24), spin1(clv, nx=128, nt=10, seed=3)]
    a, _ = run(clv, chains, 2, clv.PREC_F64, monkeypatch)
    b, _ = run(clv, chains, 2, clv.PREC_F64, monkeypatch, {"CLV_CHUNK": chunk})
    for (x, xc), (y, yc) in zip(a, b):
        assert np.array_equal(x, y) and np.array_equal(xc, yc)


@pytest.mark.parametrize("path", [f for f in golden_files() if "_1d_" in f or "_2d_" in f][:3],
                         ids=lambda p: p.split("/")[-1][5:-4])
def test_ref4_unfused_path_matches_reference_kernels(clv, monkeypatch, path):
    monkeypatch.setenv("CLV_FUSED", "0")
    monkeypatch.setenv("CLV_TILED", "0")
    g, kw = load_golden(path)
    c = clv.ChainParams(nx=kw["nx"], ny=kw["ny"], nz=kw["nz"], nt=kw["nt"], eps=kw["eps"], a_x=kw["a_x"],
                        G=kw["G"], Q=kw["Q"], P=kw["P"], mu=kw["mu"], DT=kw["DT"])
    with clv.Engine(c, model=clv.MODEL_REF4, noise=clv.NOISE_EXTERNAL) as e:
        e.set_fields(0, g["psi0"], g["psic0"])
        for s in range(len(g["dt"])):
            e.step_with_noise(g["noise"][s])
            psi, psic = e.get_fields(0)
            assert rel_err(psi, g["psi"][s]) < 1e-12 and rel_err(psic, g["psic"][s]) < 1e-12


@pytest.mark.parametrize("nx", [64, 256])
def test_static_plan_equals_runtime_plan(clv, monkeypatch, nx):
    chains = [spin1(clv, nx=nx, seed=s, mu=0.5 + 0.3 * s) for s in range(3)]
    a, _ = run(clv, chains, 3, clv.PREC_F32, monkeypatch)
    b, _ = run(clv, chains, 3, clv.PREC_F32, monkeypatch, {"CLV_NO_STATIC_PLAN": "1"})
    for (x, xc), (y, yc) in zip(a, b):
        assert np.array_equal(x, y) and np.array_equal(xc, yc)


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_stored_drift_equals_recomputed_drift(clv, monkeypatch, prec):
    """Reference dt rule on the fused path: the reduce pass storing the drift and a
    streaming update give the same step, bit for bit, as a second filter + drift pass
    (the two-kernel forms: the step loop, which takes this problem by default, is
    tested against them in test_gpu_loop.py)."""
    p = clv.PREC_F64 if prec == "f64" else clv.PREC_F32
    chains = [clv.ChainParams(nx=64, nt=16, mu=-0.5 + 0.3 * i, G=0.15, Q=0.02, P=0.1, seed=3 + i)
              for i in range(3)]
    monkeypatch.setenv("CLV_NO_LOOP", "1")
    out = []
    for sd in ("1", "0"):
        monkeypatch.setenv("CLV_STORE_DRIFT", sd)
        with clv.Engine(chains, model=clv.MODEL_REF4, precision=p) as e:
            path, phases = e.plan()
            assert path == "fused"
            assert phases[1] == ("stored_drift_update" if sd == "1" else "fused_apply")
            rng = np.random.default_rng(1)
            for i in range(3):
                a = (rng.standard_normal(e.shape(i)) + 1j * rng.standard_normal(e.shape(i))) * 0.3 + 0.5
                e.set_fields(i, a, np.conj(a))
            e.step(3)
            out.append(([e.get_fields(i) for i in range(3)], e.step_info()))
    (a, ia), (b, ib) = out
    for (x, xc), (y, yc) in zip(a, b):
        assert np.array_equal(x, y) and np.array_equal(xc, yc)
    assert np.array_equal(ia["dt"], ib["dt"]) and np.array_equal(ia["t"], ib["t"])


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_split_fields_equal_joint_step(clv, monkeypatch, prec):
    """Problems with fewer chunks than SMs step psi and psibar in separate CTAs: the same
    fields as one CTA for both (bit for bit under the K/max rule at FP32; at FP64 the
    split CTAs filter their 256-site lines on warp pairs with radix-4 passes, which round
    differently from the joint kernel's radix-8 passes: 1e-13; the reference rule's mean
    also regroups its FP64 partial sums, 1e-13)."""
    p = clv.PREC_F64 if prec == "f64" else clv.PREC_F32
    chains = [spin1(clv, nt=16, seed=s, mu=0.4 + 0.3 * s) for s in range(2)]
    a, ia = run(clv, chains, 4, p, monkeypatch, {"CLV_FUSED_SPLIT": "1"})
    b, ib = run(clv, chains, 4, p, monkeypatch, {"CLV_FUSED_SPLIT": "0"})
    for (x, xc), (y, yc) in zip(a, b):
        if prec == "f32":
            assert np.array_equal(x, y) and np.array_equal(xc, yc)
        else:
            assert rel_err(x, y) < 1e-13 and rel_err(xc, yc) < 1e-13
    if prec == "f32":
        assert np.array_equal(ia["dt"], ib["dt"])
    else:
        assert np.allclose(ia["dt"], ib["dt"], rtol=1e-13)
    chains = [clv.ChainParams(nx=64, nt=16, mu=-0.5 + 0.3 * i, G=0.15, Q=0.02, P=0.1, seed=3 + i)
              for i in range(2)]
    out = []
    for split in ("1", "0"):
        monkeypatch.setenv("CLV_FUSED_SPLIT", split)
        with clv.Engine(chains, model=clv.MODEL_REF4, precision=p) as e:
            assert e.plan()[0] == "fused"
            rng = np.random.default_rng(4)
            for i in range(2):
                f = (rng.standard_normal(e.shape(i)) + 1j * rng.standard_normal(e.shape(i))) * 0.3 + 0.5
                e.set_fields(i, f, np.conj(f))
            e.step(3)
            out.append(([e.get_fields(i) for i in range(2)], e.step_info()))
    (a, ia), (b, ib) = out
    tol = 1e-13 if prec == "f64" else 2e-6
    for (x, xc), (y, yc) in zip(a, b):
        assert rel_err(x, y) < tol and rel_err(xc, yc) < tol
    assert np.allclose(ia["dt"], ib["dt"], rtol=tol)

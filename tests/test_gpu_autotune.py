"""clv_autotune: times the candidate plans, keeps the fastest and leaves the
simulation exactly where it was (fields, dt, Langevin time and step counter
equal bit for bit to a run without the call)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def clv():
    import cl_var_dt_gb300 as m
    m.build()
    return m


@pytest.fixture(autouse=True)
def clean_env(monkeypatch):
    for k in ("CLV_FUSED", "CLV_TILED", "CLV_NO_TMA", "CLV_NO_SPECULATE", "CLV_CHUNK", "CLV_NO_STATIC_PLAN"):
        monkeypatch.delenv(k, raising=False)


def chains(clv, **kw):
    out = []
    for i in range(3):
        base = dict(nx=256, ny=1, nz=1, nt=32, eps=6 / 128, mu=0.4 + 0.3 * i, c0=0.5, c1=-0.1, q=0.05,
                    K=0.05, dt_max=1e-3, seed=11)
        base.update(kw)
        out.append(clv.ChainParams(**base))
    return out


def run(clv, cs, tune, precision):
    with clv.Engine(cs, model=clv.MODEL_SPIN1, precision=precision) as e:
        e.init_spin1()
        e.step(3)
        report = e.autotune(3) if tune else ""
        e.step(3)
        return [e.get_fields(i) for i in range(len(cs))], e.step_info(), report, e.plan()[0]


@pytest.mark.parametrize("shape", [dict(), dict(nx=64, ny=32, nt=16)], ids=["fused-1d", "tiled-2d"])
def test_autotune_keeps_the_trajectory(clv, shape):
    cs = chains(clv, **shape)
    a, ia, rep, path = run(clv, cs, True, clv.PREC_F64)
    b, ib, _, _ = run(clv, cs, False, clv.PREC_F64)
    assert path == ("fused" if not shape else "tiled")
    lines = rep.splitlines()
    assert len(lines) >= 3 and lines[-1].startswith("chosen:"), rep
    for (x, xc), (y, yc) in zip(a, b):
        assert np.array_equal(x, y) and np.array_equal(xc, yc)
    assert np.array_equal(ia["t"], ib["t"]) and np.array_equal(ia["steps"], ib["steps"])
    assert np.array_equal(ia["dt"], ib["dt"])


def test_autotune_without_a_tunable_plan(clv):
    with clv.Engine(chains(clv, nx=2048, nt=4), model=clv.MODEL_SPIN1) as e:
        assert e.plan()[0] == "unfused"
        assert "no tunable plan" in e.autotune(2)

"""Secant mu-tuning on the engine (FP32-mixed spin-1, 1D 32 x 32 lattices):
the density responds monotonically to mu, and the batched driver admits queued
chains, feeds the engine's measured densities into the secant rule and gives
every sampling block its own noise stream."""
from dataclasses import replace

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def clv():
    import cl_var_dt_gb300 as m
    m.build()
    return m


def _chain(clv, mu, seed):
    return clv.ChainParams(nx=32, nt=32, eps=0.1, mu=mu, c0=1.0, c1=0.0, q=0.0, K=0.05,
                           dt_max=1e-3, seed=seed)


def test_density_rises_with_mu(clv):
    from cl_var_dt_gb300 import secant
    run = secant.engine_sampler(therm_steps=1000, meas_steps=2000, obs_every=50)
    res = run([_chain(clv, mu, 11 + i) for i, mu in enumerate((-0.5, 0.5, 1.5))], [None] * 3)
    dens = [r[0] for r in res]
    assert all(np.isfinite(dens))
    assert dens[0] < dens[1] < dens[2], dens
    for n, err, (psi, psic) in res:
        assert np.isfinite(err) and err > 0
        assert psi.shape == (3, 32, 32, 1, 1)


def test_secant_driver_on_engine(clv):
    from cl_var_dt_gb300 import secant
    run = secant.engine_sampler(therm_steps=200, meas_steps=500, obs_every=50)
    seeds = []

    def sampler(chains, warm):
        seeds.append([c.seed for c in chains])
        return run(chains, warm)

    targets = [secant.TuneTarget(_chain(clv, 0.3, 100 + i), target=t, mu_step=0.3, tol=1e-6)
               for i, t in enumerate((0.5, 1.5, 0.7))]
    states = secant.tune(targets, sampler, max_active=2, max_rounds=3)
    # two active chains, the third stays queued (nothing converges at tol 1e-6)
    assert [len(s.mus) for s in states] == [3, 3, 0]
    for s in states[:2]:
        assert np.isfinite(s.dens).all()
        # second guess: mu_step towards the target; third: the safeguarded secant
        assert s.mus[0] == pytest.approx(0.3)
        assert s.mus[1] == pytest.approx(0.3 + np.copysign(0.3, s.target.target - s.dens[0]))
        assert s.mus[2] == pytest.approx(
            secant.safeguarded_next(s.mus[:2], s.dens[:2], s.target.target, s.target.mu_step))
    assert len({sd for rnd in seeds for sd in rnd}) == 6  # a new noise stream every block


def test_batch_sampler_reuses_one_engine(clv):
    """EngineBatchSampler: the rounds of a batch run on one engine with each chain's
    mu set in place (test_chemical_potential_set_in_place_equals_new_engine checks
    that this equals an engine built with that mu); a round measures only the new
    samples; a queued chain joining forces one re-batch."""
    from cl_var_dt_gb300 import secant
    sampler = secant.EngineBatchSampler(therm_steps=200, meas_steps=400, obs_every=50)
    targets = [secant.TuneTarget(_chain(clv, 0.5, 200 + i), target=t, mu_step=0.3, tol=1e-6)
               for i, t in enumerate((0.6, 0.9, 1.2, 1.5, 1.0))]
    try:
        states = secant.tune(targets, sampler, max_active=4, max_rounds=3)
        assert sampler.builds == 1  # nothing converges at tol 1e-6: the same four chains throughout
        assert [len(s.mus) for s in states] == [3, 3, 3, 3, 0]
        for k, i in enumerate(sampler.ids):
            assert sampler.mu[k] == pytest.approx(states[i].mus[-1])
            assert sampler.engine.chains[k].mu == pytest.approx(states[i].mus[-1])
        # 8 samples per round and chain, 3 rounds
        assert len(sampler.engine.spin1_samples(0)) == 24
        # a queued chain joins: the batch is rebuilt with the continuing chains' fields
        states[0].converged = True
        sampler.sample([1, 2, 3, 4], [replace(states[i].target.chain, mu=0.7) for i in (1, 2, 3, 4)],
                       [None] * 4)
        assert sampler.builds == 2 and sampler.ids == [1, 2, 3, 4]
    finally:
        sampler.close()
    for s in states[:4]:
        assert np.isfinite(s.dens).all() and np.isfinite(s.errs).all() and all(e > 0 for e in s.errs)
    assert sampler.site_updates > 0


@pytest.mark.parametrize("shape", [dict(nx=32, nt=32), dict(nx=256, nt=32), dict(nx=64, ny=32, nt=8)],
                         ids=["fused-runtime-plan", "fused-line", "tiled"])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_chemical_potential_set_in_place_equals_new_engine(clv, shape, prec, tmp_path):
    """clv_set_chemical_potential on a running engine: the steps after it equal, bit
    for bit, those of an engine built with that mu and resumed from the same state
    (the captured step graphs read the chain constants at run time)."""
    p = clv.PREC_F64 if prec == "f64" else clv.PREC_F32
    base = dict(eps=0.1, c0=1.0, c1=-0.1, q=0.05, K=0.05, dt_max=1e-3, seed=31)
    ck = str(tmp_path / "state.bin")
    with clv.Engine(clv.ChainParams(**shape, **base, mu=0.2), model=clv.MODEL_SPIN1, precision=p) as a:
        a.init_spin1()
        a.step(2)  # graphs captured with mu = 0.2
        a.save_checkpoint(ck)
        a.set_chemical_potential(0, 1.4)
        a.step(5)
        got = a.get_fields(0)
    with clv.Engine(clv.ChainParams(**shape, **base, mu=1.4), model=clv.MODEL_SPIN1, precision=p) as b:
        b.load_checkpoint(ck)
        b.step(5)
        want = b.get_fields(0)
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])

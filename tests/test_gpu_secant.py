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
    """EngineBatchSampler: the rounds of a batch run on one engine with mu set in
    place; the engine is rebuilt only when the active chains fall below half of its
    slots; the tuned chains still converge to their targets' densities."""
    from cl_var_dt_gb300 import secant
    sampler = secant.EngineBatchSampler(therm_steps=600, meas_steps=600, obs_every=50)
    # (dt_max 5e-3: a Langevin time of 6 per round, so the density settles within a round)
    targets = [secant.TuneTarget(replace(_chain(clv, 0.5, 200 + i), dt_max=5e-3), target=t, mu_step=0.3,
                                 tol=0.08) for i, t in enumerate((0.6, 0.9, 1.2, 1.5))]
    try:
        states = secant.tune(targets, sampler, max_active=4, max_rounds=12)
    finally:
        sampler.close()
    rounds = max(len(s.mus) for s in states)
    assert rounds >= 2
    assert sampler.builds <= 2, sampler.builds  # the first engine, at most one re-batch
    assert sampler.site_updates > 0
    for s in states:
        assert np.isfinite(s.dens).all() and np.isfinite(s.errs).all()
        assert s.converged, (s.target.target, s.mus, s.dens)

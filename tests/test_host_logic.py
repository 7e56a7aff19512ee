"""Host-side logic on the CPU: rank sharding over gloo (world size 2), the
secant mu-tuning driver on a synthetic density curve, block errors, and the
params.txt / Parameters.h readers (Python side)."""
import math
import os
import socket

import numpy as np
import pytest

from cl_var_dt_gb300 import dist, secant


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_range_partitions():
    for n in (0, 1, 7, 64, 256, 257):
        for world in (1, 2, 3, 8):
            got = [list(dist.shard_range(n, r, world)) for r in range(world)]
            flat = [i for g in got for i in g]
            assert flat == list(range(n))
            assert max(map(len, got)) - min(map(len, got)) <= 1
    with pytest.raises(ValueError):
        dist.shard_range(4, 2, 2)


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as td
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    td.init_process_group("gloo", rank=rank, world_size=world)
    mine = dist.shard(list(range(10)), rank, world)
    out = [None] * world
    td.all_gather_object(out, mine)
    t = dist.max_over_ranks(float(rank + 1) * 1.5)
    td.barrier()
    td.destroy_process_group()
    q.put((rank, out, t))


def test_gloo_two_ranks_shard_and_max():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, out, t in res:
        assert sorted(i for part in out for i in part) == list(range(10))
        assert t == 3.0  # max over ranks of 1.5 * (rank + 1)


def test_secant_next_root_and_limits():
    assert secant.secant_next(0.0, 1.0, 0.5, 1.5, 1.0) == pytest.approx(0.5)
    # flat secant: bounded step towards the target
    assert secant.secant_next(0.0, 1.0, 2.0, 2.0, 1.0) == pytest.approx(0.5)
    # long jumps are limited
    assert secant.secant_next(0.0, 0.1, 1.0, 1.0001, 5.0, max_jump=1.0) == pytest.approx(1.1)


def test_block_error_of_white_noise():
    rng = np.random.default_rng(1)
    x = rng.normal(0, 1, 8000)
    assert secant.block_error(x) == pytest.approx(1 / math.sqrt(8000), rel=0.6)


class _Chain:
    def __init__(self, mu):
        self.mu = mu


def test_tune_converges_with_admission():
    from dataclasses import dataclass

    @dataclass
    class C:
        mu: float
        k: float

    rng = np.random.default_rng(3)
    # synthetic density curves n(mu) = k * softplus(mu) with small noise
    def sampler(chains, warm):
        return [(c.k * math.log1p(math.exp(c.mu)) + rng.normal(0, 0.002), 0.002, ("f", c.mu))
                for c in chains]

    targets = [secant.TuneTarget(C(mu=0.0, k=1.0 + 0.1 * i), target=0.5 + 0.2 * i, tol=0.01)
               for i in range(10)]
    states = secant.tune(targets, sampler, max_active=4, max_rounds=30)
    assert all(s.converged for s in states)
    for s in states:
        assert abs(s.dens[-1] - s.target.target) < 0.01
        assert s.fields is not None  # warm start carried between rounds


def test_safeguarded_secant_brackets_and_bisects():
    # a falling secant (a chain still relaxing) inside a bracket: bisection
    assert secant.safeguarded_next([0.5, 0.8, 1.4], [0.9, 1.5, 1.3], 1.2, 0.2) == pytest.approx(0.65)
    # points older than the window do not bracket: with the stale lo = 0.5 the secant root
    # 0.4 would be rejected for bisection (0.575); without it the root is taken
    assert secant.safeguarded_next([0.5, 0.8, 0.7, 0.65], [1.0, 1.6, 1.5, 1.45], 1.2, 0.2) == \
        pytest.approx(0.4)
    # the secant's root inside the bracket is taken
    mu = secant.safeguarded_next([0.0, 1.0], [0.5, 1.5], 1.0, 0.2)
    assert mu == pytest.approx(0.5)
    # no bracket, flat response below the target: doubling steps upwards
    assert secant.safeguarded_next([-2.0, -1.8], [0.01, 0.01], 0.7, 0.2) == pytest.approx(-1.8 + 0.4)
    assert secant.safeguarded_next([-2.0, -1.8, -1.4], [0.01, 0.01, 0.01], 0.7, 0.2) == pytest.approx(-1.4 + 0.8)


def test_tune_recovers_from_a_relaxing_chain():
    """Densities that lag mu (a chain relaxing between rounds) make the plain secant
    oscillate; the safeguarded step still converges."""
    from dataclasses import dataclass

    @dataclass
    class C:
        mu: float

    state = {"n": 0.9}

    def sampler(chains, warm):
        out = []
        for c in chains:
            eq = 1.0 + c.mu  # equilibrium density
            state["n"] += 0.6 * (eq - state["n"])  # relaxes 60 % of the way per round
            out.append((state["n"], 0.001, None))
        return out

    st = secant.tune([secant.TuneTarget(C(mu=0.5), target=1.2, mu_step=0.3, tol=0.02)], sampler,
                     max_active=1, max_rounds=30)[0]
    assert st.converged, (st.mus, st.dens)


def test_settling_of_a_series():
    rng = np.random.default_rng(5)
    flat = 1.0 + rng.normal(0, 0.01, 600)
    ok, est, rest = secant.settling(flat, tol=0.05)
    assert ok and rest == 0.0 and abs(est - 1.0) < 0.005
    # an exponential approach to 1.5 (time constant 300 samples) seen over 600 samples:
    # Aitken's extrapolation recovers the equilibrium
    k = np.arange(600)
    relax = 1.5 - 0.5 * np.exp(-k / 300.0) + rng.normal(0, 0.002, 600)
    ok, est, rest = secant.settling(relax, tol=0.05)
    assert not ok and est == pytest.approx(1.5, abs=0.03) and rest > 0.025
    # a straight ramp has no visible end: unsettled, drift to come 3 x the last step
    ramp = 1.0 + np.linspace(0, 0.3, 600) + rng.normal(0, 0.002, 600)
    ok, est, rest = secant.settling(ramp, tol=0.05)
    assert not ok and rest == pytest.approx(0.3, abs=0.03)
    # a trend below half the tolerance counts as settled
    assert secant.settling(1.0 + 0.01 * np.exp(-k / 100.0), tol=0.1)[0]


def test_tune_waits_for_chains_that_lag_mu():
    """Densities that relax towards n_eq(mu) = mu / c0 over about two rounds (the
    sampler returns each round's series, as EngineBatchSampler does).  Every chain
    converges, and only on a settled round: the equilibrium density at the final mu
    is within the tolerance of the target."""
    from dataclasses import dataclass

    @dataclass
    class C:
        mu: float
        c0: float

    rng = np.random.default_rng(11)
    M, tau = 200, 400.0  # samples per round (half thermalisation before them), relaxation in samples
    state = {}

    def sampler(ids, chains, warm):
        out = []
        for i, c in zip(ids, chains):
            eq = c.mu / c.c0
            n = state.get(i, 1.0)
            n = eq + (n - eq) * math.exp(-M / tau)  # thermalisation half
            k = np.arange(1, M + 1)
            series = eq + (n - eq) * np.exp(-k / tau) + rng.normal(0, 0.01, M)
            state[i] = eq + (n - eq) * math.exp(-M / tau)
            out.append((float(series.mean()), secant.block_error(series), None, series))
        return out

    class S:
        sample = staticmethod(sampler)

    c0s = [0.15, 0.3, 0.45, 0.6] * 4
    targets = [0.6 + 0.1 * i for i in range(16)]
    # first guesses off by up to 25 % (the mean-field mu = c0 n of the workload, plus an error)
    tt = [secant.TuneTarget(C(mu=c0 * n * (1.0 + 0.25 * math.sin(3.0 * i)), c0=c0), target=n, mu_step=0.2,
                            tol=0.05, max_jump=0.5) for i, (c0, n) in enumerate(zip(c0s, targets))]
    states = secant.tune(tt, S(), max_active=16, max_rounds=30)
    for s in states:
        assert s.converged, (s.mus, s.dens, s.settled)
        assert s.settled[-1]
        c = s.target.chain
        assert abs(s.mus[-1] / c.c0 - s.target.target) < 0.075, (s.mus, s.dens)
    # the lag made some rounds keep mu
    assert any(not all(s.settled) for s in states)


def test_damped_newton_with_a_prior_slope():
    """A chain whose density responds steeply (dn/dmu = 6) and with noise: the
    damped Newton step with a prior slope converges where the secant through close,
    noisy points would not; the prior may be off by a factor of two."""
    from dataclasses import dataclass

    @dataclass
    class C:
        mu: float

    rng = np.random.default_rng(2)

    def sampler(chains, warm):
        return [(6.0 * c.mu + rng.normal(0, 0.01), 0.01, None) for c in chains]

    for prior in (6.0, 3.0, 12.0):
        st = secant.tune([secant.TuneTarget(C(mu=0.1), target=1.5, tol=0.03, max_jump=0.5, slope=prior)],
                         sampler, max_active=1, max_rounds=20)[0]
        assert st.converged, (prior, st.mus, st.dens)
        assert abs(st.mus[-1] - 0.25) < 0.01


def test_no_convergence_before_a_slow_chain_shows_its_trend():
    """A chain that starts at its target density with a mean-field mu that is off
    (equilibrium 0.3 above the target) and relaxes over about eight rounds: its first
    rounds look flat, so the driver must not declare it converged before the window
    at that mu reveals the trend; the mu it converges at gives the target density."""
    from dataclasses import dataclass

    @dataclass
    class C:
        mu: float
        c0: float

    rng = np.random.default_rng(4)
    M = 300
    tau = 8 * M * 5 / 3  # samples: eight rounds of 2 M / 3 thermalisation and M measured samples
    state = {}

    def sampler(ids, chains, warm):
        out = []
        for i, c in zip(ids, chains):
            eq = c.mu / c.c0 + 0.3
            n = state.get(i, 1.5)
            n = eq + (n - eq) * math.exp(-(2 * M / 3) / tau)
            k = np.arange(1, M + 1)
            series = eq + (n - eq) * np.exp(-k / tau) + rng.normal(0, 0.01, M)
            state[i] = eq + (n - eq) * math.exp(-M / tau)
            out.append((float(series.mean()), secant.block_error(series), None, series))
        return out

    class S:
        sample = staticmethod(sampler)

    t = secant.TuneTarget(C(mu=0.15 * 1.5, c0=0.15), target=1.5, tol=0.05, max_jump=0.5, slope=1 / 0.15)
    st = secant.tune([t], S(), max_active=1, max_rounds=40)[0]
    assert st.converged and len(st.mus) >= 4, (st.mus, st.dens)
    assert abs(st.mus[-1] / 0.15 + 0.3 - 1.5) < 0.075, (st.mus, st.dens)


def test_newton_gain_halves_on_overshoot():
    """A prior slope three times too small: the damped Newton step (factor 0.7) would
    overshoot by more than the error it corrects and oscillate without end; halving the
    factor at every overshoot makes it converge."""
    from dataclasses import dataclass

    @dataclass
    class C:
        mu: float

    def sampler(chains, warm):
        return [(3.0 * c.mu, 0.001, None) for c in chains]

    st = secant.tune([secant.TuneTarget(C(mu=0.0), target=1.5, tol=0.01, max_jump=2.0, slope=1.0)],
                     sampler, max_active=1, max_rounds=40)[0]
    assert st.converged, (st.mus, st.dens)
    assert abs(st.mus[-1] - 0.5) < 0.01 and st.gain < 0.7


def test_batch_sampler_frozen_rounds_and_restarts():
    """EngineBatchSampler's runaway handling on a stand-in engine: a round over which a
    chain's mean dt stayed below frozen_frac * dt_max reports NaN (the driver keeps its
    mu) and restarts nothing; a second frozen round in a row restarts the chain from its
    start density (amplitude sqrt(n / 3)); a healthy chain reports its samples."""
    from types import SimpleNamespace

    class FakeEngine:
        def __init__(self):
            self.chains = [SimpleNamespace(nx=4, ny=1, nz=1, nt=2, dt_max=1e-3) for _ in range(2)]
            self.t = np.zeros(2)
            self.rate = np.array([1e-3, 1e-3])  # dt per step of each chain
            self.samples = [[], []]
            self.starts = []

        def set_chemical_potential(self, k, mu):
            pass

        def step(self, n):
            self.t += n * self.rate

        def evaluate(self):
            for k in range(2):
                self.samples[k].append([1.0 + 0.1 * k] + [0.0] * 7)

        def spin1_samples(self, k):
            return np.array(self.samples[k]) if self.samples[k] else np.zeros((0, 8))

        def step_info(self):
            return {"dt": self.rate.copy(), "t": self.t.copy()}

        def shape(self, k):
            return (3, 2, 4, 1, 1)

        def set_fields(self, k, psi, psic):
            self.starts.append((k, float(np.mean(np.abs(psi)))))

    s = secant.EngineBatchSampler(therm_steps=10, meas_steps=20, obs_every=5, start_density={0: 0.75, 1: 1.2})
    e = FakeEngine()
    s.engine, s.ids, s.mu = e, [0, 1], [0.1, 0.2]
    chains = [SimpleNamespace(mu=0.1), SimpleNamespace(mu=0.2)]
    e.rate[0] = 1e-6  # chain 0 frozen (mean dt 1e-6 < 0.05 * 1e-3)
    out = s.sample([0, 1], chains, [None, None])
    assert np.isnan(out[0][0]) and out[0][3] is None and s.restarts == 0
    assert out[1][0] == pytest.approx(1.1) and len(out[1][3]) == 4
    out = s.sample([0, 1], chains, [None, None])
    assert np.isnan(out[0][0]) and s.restarts == 1
    assert e.starts and e.starts[-1][0] == 0 and e.starts[-1][1] == pytest.approx(math.sqrt(0.75 / 3), rel=0.05)
    e.rate[0] = 1e-3  # recovered
    out = s.sample([0, 1], chains, [None, None])
    assert out[0][0] == pytest.approx(1.0) and s.restarts == 1 and s.frozen[0] == 0

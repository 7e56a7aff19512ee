"""Secant tuning of the chemical potential to a target density, over batched chains.

The reference tunes mu with a secant iteration driven through SLURM jobs
(``Secant_method_function``, ``step``, ``new_mu``; mylib.py:511-580, 599-706):
two runs at mu_1, mu_2, then mu_{k+1} = mu_k - (r_k - r*) (mu_k - mu_{k-1}) /
(r_k - r_{k-1}) until |r - r*| < err, with r the measured ratio.  Here the
measured quantity is the spin-1 density and every chain of a batch is a
separate tuning problem: all active chains step together on one GPU, each
updates its own mu after every sampling block, converged chains leave the batch
and queued chains are admitted in their place.

Samplers: ``engine_sampler`` builds one engine per round (continuing chains keep
their fields, the dt state restarts); ``EngineBatchSampler`` keeps one engine
across rounds, sets each chain's mu in place (clv_set_chemical_potential) and
rebuilds the engine only when the active chains fall below a fraction of its
slots or a queued chain is admitted.

A chain's density relaxes slowly after mu changes (its long-wavelength modes
over thousands of steps, tens of thousands at small couplings), so a round's
mean can lag its mu.  A sampler that returns the round's sample series lets the
driver see that (``settling``): the series of the rounds at one mu are read as
one window, its trend is extrapolated to an equilibrium estimate, a chain
converges only on a settled window of at least three rounds, an unsettled chain
keeps its mu for a few rounds, and the estimate, not the lagging mean, is the
point the next mu is computed from.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace
from typing import Callable, List, Optional, Sequence

import numpy as np


@dataclass
class TuneTarget:
    """One tuning problem: a chain and the density it should reach."""
    chain: object              # ChainParams (mu is the starting guess)
    target: float
    mu_step: float = 0.2       # second guess mu_2 = mu_1 +- mu_step (towards the target)
    tol: float = 0.02          # convergence: |n - target| < tol (absolute)
    max_jump: float = 1.0      # largest change of mu from one round to the next
    slope: Optional[float] = None  # a prior dn/dmu (e.g. 1 / c0 of the mean field): damped Newton
    damping: float = 0.7           # fraction of the Newton step taken with the prior slope
    min_rounds: int = 3            # rounds at one mu before the chain may count as converged
    max_holds: int = 4             # rounds an unsettled chain keeps its mu before it moves anyway


@dataclass
class TuneState:
    target: TuneTarget
    mus: List[float] = field(default_factory=list)      # every round's mu ...
    dens: List[float] = field(default_factory=list)     # ... its mean density ...
    errs: List[float] = field(default_factory=list)     # ... and standard error
    settled: List[bool] = field(default_factory=list)   # the round's density had settled
    pmus: List[float] = field(default_factory=list)     # the points the secant steps from
    pdens: List[float] = field(default_factory=list)
    holds: int = 0          # consecutive rounds that kept mu for a chain still on its way
    gain: Optional[float] = None  # the damped Newton step's current factor (halved on overshoot)
    converged: bool = False
    fields: Optional[tuple] = None
    window: List[np.ndarray] = field(default_factory=list)  # the series of the rounds at the current mu

    @property
    def mu(self) -> float:
        """mu of the next round."""
        if not self.mus:
            return self.target.chain.mu
        if self.holds:
            return self.mus[-1]
        t = self.target
        if t.slope:
            # damped Newton with the prior slope: a secant through nearby points that
            # still lag their mu gives slopes of either sign and makes mu oscillate; the
            # factor halves whenever the last two points lie on opposite sides of the
            # target (an overshoot: the prior slope too small, or the response lagging)
            if self.gain is None:
                self.gain = t.damping
            step = self.gain * (t.target - self.pdens[-1]) / t.slope
            return self.pmus[-1] + max(-t.max_jump, min(t.max_jump, step))
        if len(self.pmus) == 1:
            return self.pmus[0] + math.copysign(self.target.mu_step, self.target.target - self.pdens[0])
        return safeguarded_next(self.pmus, self.pdens, self.target.target, self.target.mu_step,
                                self.target.max_jump)

    def record(self, mu: float, n: float, err: float, series=None):
        """Add one round's measurement and decide what the next round does.

        With a sample series, the rounds spent at the same mu are read as one window
        (a chain relaxing over many rounds shows its trend only over several), and
        the window's equilibrium estimate (``settling``) drives the decision (with the
        target's ``min_rounds`` and ``max_holds``): the
        chain converges when the window is settled, at least ``min_rounds`` long and
        both the last round's mean and the estimate lie within the tolerance; a
        settled window near the target but shorter than ``min_rounds`` (a trend
        slower than one round may not show in it yet), or an unsettled window for at
        most ``max_holds`` rounds, keeps mu; otherwise the estimate at mu becomes the
        next point of the mu update.  Without a series every round is a settled
        point."""
        t = self.target
        min_rounds, max_holds = t.min_rounds, t.max_holds
        if self.window and self.mus and mu != self.mus[-1]:
            self.window = []
        self.mus.append(mu)
        self.dens.append(n)
        self.errs.append(err)
        if not math.isfinite(n):  # no measurement this round (the chain restarted): keep mu
            self.settled.append(False)
            self.window = []
            self.holds = max(self.holds, 1)
            return
        if series is None:
            ok, est, rounds = True, n, min_rounds
        else:
            self.window.append(np.asarray(series, dtype=float))
            ok, est, _ = settling(np.concatenate(self.window), t.tol)
            rounds = len(self.window)
        self.settled.append(ok)
        if ok and rounds >= min_rounds and abs(n - t.target) < t.tol and abs(est - t.target) < t.tol:
            self.converged = True
            return
        near = abs(est - t.target) < t.tol
        if (ok and near and rounds < min_rounds) or (not ok and self.holds < max_holds):
            self.holds += 1  # confirm a settled window near the target, or wait for the trend
            return
        self.holds = 0
        self.window = []
        if self.pdens and self.gain is not None and (self.pdens[-1] - t.target) * (est - t.target) < 0:
            self.gain = max(0.1 * t.damping, 0.5 * self.gain)
        self.pmus.append(mu)
        self.pdens.append(est)


def safeguarded_next(mus: Sequence[float], dens: Sequence[float], target: float, mu_step: float,
                     max_jump: float = 1.0, window: int = 3) -> float:
    """The next mu of one chain from all its (mu, density) points so far.

    The density rises with mu, so the points give a bracket: lo, the largest mu
    measured below the target, and hi, the smallest measured above it (from the
    latest measurement at each mu, among the last ``window`` rounds: a chain that
    is still relaxing makes older points stale, and a bracket kept from them
    would pin mu while the density drifts away).  The secant of the last two points
    (``secant_next``) is taken when its slope is positive and its root lies
    strictly inside the bracket; otherwise, with a bracket, its midpoint
    (bisection); without one, a step away from the known side that doubles with
    every round spent on that side (a flat or falling secant comes from
    measurement noise or a chain still relaxing, where the plain secant of
    mylib.py:561-580 can jump back and forth)."""
    last = {}
    for m, n in list(zip(mus, dens))[-window:]:
        if math.isfinite(n):
            last[m] = n
    lo = max((m for m, n in last.items() if n < target), default=None)
    hi = min((m for m, n in last.items() if n > target), default=None)
    m1, m2, r1, r2 = mus[-2], mus[-1], dens[-2], dens[-1]
    slope_ok = all(map(math.isfinite, (r1, r2))) and m2 != m1 and (r2 - r1) / (m2 - m1) > 0
    cand = secant_next(m1, m2, r1, r2, target, max_jump) if slope_ok else None
    if lo is not None and hi is not None and lo < hi:
        if cand is not None and lo < cand < hi:
            return cand
        return 0.5 * (lo + hi)
    if cand is not None and (lo is None or cand > lo) and (hi is None or cand < hi):
        return cand
    # one-sided: expand away from the measured side
    same_side = 0
    for n in reversed(dens):
        if math.isfinite(n) and (n < target) == (r2 < target):
            same_side += 1
        else:
            break
    step = min(max_jump, mu_step * 2.0 ** max(0, same_side - 1))
    if lo is not None:
        return lo + step
    if hi is not None:
        return hi - step
    return m2 + math.copysign(step, target - r2)


def secant_next(mu1: float, mu2: float, r1: float, r2: float, target: float,
                max_jump: float = 1.0) -> float:
    """new_mu of mylib.py:561-580 for a general target: the root of the line
    through (mu1, r1), (mu2, r2); a flat secant or a jump beyond max_jump is
    limited to a bounded step in the direction that reduces |r - target|."""
    if r2 == r1 or not math.isfinite(r1) or not math.isfinite(r2):
        return mu2 + math.copysign(0.5 * max_jump, target - r2)
    mu = mu2 - (r2 - target) * (mu2 - mu1) / (r2 - r1)
    if abs(mu - mu2) > max_jump:
        mu = mu2 + math.copysign(max_jump, mu - mu2)
    return mu


def block_error(x: np.ndarray, nblocks: int = 8) -> float:
    """Standard error of the mean from block averages (autocorrelated samples)."""
    x = np.asarray(x, dtype=float)
    nb = min(nblocks, len(x))
    if nb < 2:
        return float("inf")
    blocks = np.array_split(x, nb)
    means = np.array([b.mean() for b in blocks])
    return float(means.std(ddof=1) / math.sqrt(nb))


def settling(series, tol: float, nblocks: int = 4):
    """(settled, equilibrium estimate, drift still to come) of one round's sample series.

    The series is cut in thirds with means m1, m2, m3 and differences d1 = m2 - m1,
    d2 = m3 - m2, each compared with twice its standard error (block errors of the
    thirds).  No significant difference: no trend, the estimate is the mean of the
    last two thirds.  A significant d2 of the same sign as a larger d1: an
    exponential approach, extrapolated by Aitken's delta-squared process (ratio
    q = d2 / d1, capped at 0.9; drift to come d2 q / (1 - q)).  A significant d2
    that is not decaying: the drift to come is taken as 3 d2 (the trend has no
    visible end yet).  Settled when the drift to come is below half the tolerance."""
    x = np.asarray(series, dtype=float)
    if len(x) < 6 or not np.all(np.isfinite(x)):
        return True, float(np.mean(x)) if len(x) else float("nan"), 0.0
    k = len(x) // 3
    t = (x[:k], x[k:2 * k], x[2 * k:])
    m = [float(v.mean()) for v in t]
    e = [block_error(v, nblocks) for v in t]
    e = [v if math.isfinite(v) else 0.0 for v in e]
    d1, d2 = m[1] - m[0], m[2] - m[1]
    sig1 = abs(d1) > 2.0 * math.hypot(e[0], e[1])
    sig2 = abs(d2) > 2.0 * math.hypot(e[1], e[2])
    if not sig2:
        rest = d2 if sig1 else 0.0
        est = m[2] + rest if sig1 else float(x[k:].mean())
    elif d1 * d2 > 0 and abs(d2) < abs(d1):
        q = min(d2 / d1, 0.9)
        rest = d2 * q / (1.0 - q)
        est = m[2] + rest
    else:
        rest = 3.0 * d2
        est = m[2] + rest
    return abs(rest) < 0.5 * tol, est, rest


Sampler = Callable[[List[object], Sequence[Optional[tuple]]], List[tuple]]


def engine_sampler(therm_steps: int, meas_steps: int, obs_every: int, precision=None, device=0) -> Sampler:
    """Sampler on the GB300 engine: one batched run per round.  Returns, per chain,
    (density mean, standard error, fields)."""
    import cl_var_dt_gb300 as clv

    prec = clv.PREC_F32 if precision is None else precision

    def run(chains, warm):
        with clv.Engine(list(chains), model=clv.MODEL_SPIN1, precision=prec, device=device) as e:
            e.init_spin1()
            for i, f in enumerate(warm):
                if f is not None:
                    e.set_fields(i, *f)
            e.step(therm_steps)
            for _ in range(meas_steps // obs_every):
                e.step(obs_every)
                e.evaluate()
            out = []
            for i in range(len(chains)):
                s = e.spin1_samples(i)[:, 0]
                out.append((float(s.mean()), block_error(s), e.get_fields(i)))
            return out

    return run


class EngineBatchSampler:
    """Sampler that reuses one engine across rounds.

    Called as ``sample(ids, chains, warm)`` by ``tune`` (ids: the targets' indices).
    While every requested chain sits in the current engine and they fill at least
    ``min_fill`` of its slots, a round sets the chains' mu in place, steps the whole
    engine (converged chains in it keep stepping at their final mu) and reads the
    new samples; the fields stay on the device and the step counters run on, so
    every round draws fresh noise.  Otherwise the engine is rebuilt for the
    requested chains, continuing chains taking their fields from the old engine.
    ``start_density`` (target index -> density) sets the spin-1 start of a chain to
    that density (amplitude sqrt(n / 3) per component) instead of n = 1, so that a
    chain tuned to a density far from 1 does not first relax over the slow
    density mode.  A round over which a chain's step size stayed collapsed (a
    complex-Langevin spike: the K/max rule shrinks dt to follow it; its mean dt over
    the round below ``frozen_frac`` of dt_max, or, when ``restart_dt`` is set, its
    last dt below it) reports a NaN density (the driver keeps the chain's mu): the
    chain hardly moved, so its samples say nothing.  Most spikes decay by
    themselves; a chain frozen for ``frozen_rounds`` rounds in a row starts again
    from its start at its current mu (``restarts`` counts them).
    Returns, per chain, (density mean, standard error, None, the round's density
    samples)."""

    def __init__(self, therm_steps: int, meas_steps: int, obs_every: int, precision=None, device=0,
                 min_fill: float = 0.5, restart_dt: Optional[float] = None, frozen_frac: float = 0.05,
                 frozen_rounds: int = 2, start_density=None):
        import cl_var_dt_gb300 as clv
        self.clv = clv
        self.therm, self.meas, self.every = therm_steps, meas_steps, obs_every
        self.prec = clv.PREC_F32 if precision is None else precision
        self.device, self.min_fill = device, min_fill
        self.engine = None
        self.ids: List[int] = []
        self.mu: List[float] = []
        self.builds = 0
        self.site_updates = 0
        self.last_dt = {}  # target index -> the chain's step size after its last round
        self.restart_dt = restart_dt
        self.frozen_frac = frozen_frac
        self.frozen_rounds = frozen_rounds
        self.frozen = {}  # target index -> consecutive frozen rounds
        self.start_density = start_density or {}
        self.restarts = 0

    def close(self):
        if self.engine is not None:
            self.engine.close()
            self.engine = None

    def _rebuild(self, ids, chains, warm):
        clv = self.clv
        old, old_slot = self.engine, {i: k for k, i in enumerate(self.ids)}
        fields = []
        for i, w in zip(ids, warm):
            if old is not None and i in old_slot:
                fields.append(old.get_fields(old_slot[i]))
            else:
                fields.append(w)
        self.close()
        e = clv.Engine(list(chains), model=clv.MODEL_SPIN1, precision=self.prec, device=self.device)
        e.init_spin1()
        for k, (i, f) in enumerate(zip(ids, fields)):
            if f is not None:
                e.set_fields(k, *f)
            elif i in self.start_density:
                self._start(e, k, i)
        self.engine, self.ids, self.mu = e, list(ids), [c.mu for c in chains]
        self.builds += 1

    def _start(self, e, k, i):
        """Spin-1 start of slot k (target i) at its start density (default 1)."""
        amp = math.sqrt(self.start_density.get(i, 1.0) / 3.0)
        rng = np.random.default_rng(1000003 * (i + 1) + self.restarts)
        shape = e.shape(k)
        start = amp + 0.01 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
        e.set_fields(k, start, np.conj(start))

    def sample(self, ids, chains, warm):
        slot = {i: k for k, i in enumerate(self.ids)}
        reuse = (self.engine is not None and all(i in slot for i in ids)
                 and len(ids) >= self.min_fill * len(self.ids))
        if reuse:
            for i, c in zip(ids, chains):
                k = slot[i]
                if c.mu != self.mu[k]:
                    self.engine.set_chemical_potential(k, c.mu)
                    self.mu[k] = c.mu
        else:
            self._rebuild(ids, chains, warm)
            slot = {i: k for k, i in enumerate(self.ids)}
        e = self.engine
        before = [len(e.spin1_samples(k)) for k in range(len(self.ids))]
        t0 = e.step_info()["t"]
        nsteps = self.therm + self.meas // self.every * self.every
        e.step(self.therm)
        for _ in range(self.meas // self.every):
            e.step(self.every)
            e.evaluate()
        self.site_updates += sum(c.nx * c.ny * c.nz * c.nt for c in e.chains) * nsteps
        info = e.step_info()
        dts, mean_dt = info["dt"], (info["t"] - t0) / nsteps
        out = []
        for i in ids:
            k = slot[i]
            smp = e.spin1_samples(k)[before[k]:, 0]
            self.last_dt[i] = float(dts[k])
            stuck = self.restart_dt is not None and dts[k] < self.restart_dt
            if stuck or mean_dt[k] < self.frozen_frac * e.chains[k].dt_max:
                self.frozen[i] = self.frozen.get(i, 0) + 1
                if self.frozen[i] >= self.frozen_rounds:
                    self._start(e, k, i)
                    self.restarts += 1
                    self.frozen[i] = 0
                out.append((float("nan"), float("nan"), None, None))
            else:
                self.frozen[i] = 0
                out.append((float(smp.mean()), block_error(smp), None, smp))
        return out


def _round_chain(st: TuneState):
    """The chain for the next sampling block: the current mu and, when the chain
    carries a noise seed, a seed of its own for every block (a new engine starts
    its step counter at zero, so reusing the seed would replay the noise)."""
    c = replace(st.target.chain, mu=st.mu)
    if hasattr(c, "seed"):
        c = replace(c, seed=(st.target.chain.seed + 0x9E3779B97F4A7C15 * len(st.mus)) % (1 << 64))
    return c


def tune(targets: Sequence[TuneTarget], sampler: Sampler, max_active: int = 64,
         max_rounds: int = 20, log: Optional[Callable[[str], None]] = None) -> List[TuneState]:
    """Tune every target's mu; returns the final state of each target."""
    states = [TuneState(t) for t in targets]
    queue = list(range(len(states)))
    active: List[int] = []
    for rnd in range(max_rounds):
        while queue and len(active) < max_active:
            active.append(queue.pop(0))
        if not active:
            break
        chains = [_round_chain(states[i]) for i in active]
        warm = [states[i].fields for i in active]
        res = sampler.sample(active, chains, warm) if hasattr(sampler, "sample") else sampler(chains, warm)
        still = []
        for i, c, r in zip(active, chains, res):
            n, err, fld = r[:3]
            st = states[i]
            st.record(c.mu, n, err, r[3] if len(r) > 3 else None)
            if fld is not None:
                st.fields = fld
            if not st.converged:
                still.append(i)
        if log:
            log(f"round {rnd}: {len(active) - len(still)} converged, {len(still)} active, {len(queue)} queued")
        active = still
    return states

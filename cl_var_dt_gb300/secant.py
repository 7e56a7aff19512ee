"""Secant tuning of the chemical potential to a target density, over batched chains.

The reference tunes mu with a secant iteration driven through SLURM jobs
(``Secant_method_function``, ``step``, ``new_mu``; mylib.py:511-580, 599-706):
two runs at mu_1, mu_2, then mu_{k+1} = mu_k - (r_k - r*) (mu_k - mu_{k-1}) /
(r_k - r_{k-1}) until |r - r*| < err, with r the measured ratio.  Here the
measured quantity is the spin-1 density and every chain of a batch is a
separate tuning problem: all active chains step together on one GPU, each
updates its own mu after every sampling block, converged chains leave the batch
and queued chains are admitted in their place (the engine is rebuilt for the new
active set; continuing chains keep their fields and dt state is restarted).
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
    mu_step: float = 0.2       # second guess mu_2 = mu_1 + mu_step
    tol: float = 0.02          # convergence: |n - target| < tol (absolute)


@dataclass
class TuneState:
    target: TuneTarget
    mus: List[float] = field(default_factory=list)
    dens: List[float] = field(default_factory=list)
    errs: List[float] = field(default_factory=list)
    converged: bool = False
    fields: Optional[tuple] = None

    @property
    def mu(self) -> float:
        if not self.mus:
            return self.target.chain.mu
        if len(self.mus) == 1:
            return self.mus[0] + self.target.mu_step
        return secant_next(self.mus[-2], self.mus[-1], self.dens[-2], self.dens[-1], self.target.target)


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
        res = sampler(chains, [states[i].fields for i in active])
        still = []
        for i, c, (n, err, fld) in zip(active, chains, res):
            st = states[i]
            st.mus.append(c.mu)
            st.dens.append(n)
            st.errs.append(err)
            st.fields = fld
            if abs(n - st.target.target) < st.target.tol:
                st.converged = True
            else:
                still.append(i)
        if log:
            log(f"round {rnd}: {len(active) - len(still)} converged, {len(still)} active, {len(queue)} queued")
        active = still
    return states

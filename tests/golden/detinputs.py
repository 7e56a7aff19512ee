"""Platform-independent inputs for the larger golden configurations.

Values come from a splitmix64 hash of (seed, index) in integer arithmetic,
mapped to a uniform distribution on [-sqrt(3), sqrt(3)) (mean 0, variance 1),
so the same arrays arise on any machine and numpy version without storing
them: only the outputs at sampled sites are kept in the fixtures.
"""
import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def det_uniform(seed: int, n: int) -> np.ndarray:
    """n values, uniform on [-sqrt 3, sqrt 3), from 53 bits of each hash."""
    with np.errstate(over="ignore"):
        idx = np.arange(n, dtype=np.uint64) + np.uint64(seed) * np.uint64(0x100000001B3)
    u = (_splitmix64(idx) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return (2.0 * u - 1.0) * np.sqrt(3.0)


def ref4_inputs(shape, seed: int):
    """psi, psibar start of the random golden configurations (as make_golden's)."""
    n = int(np.prod(shape))
    a, b, c, d = (det_uniform(seed + k, n).reshape(shape) for k in range(4))
    psi = 0.8 * (1 + 0.3 * a) + 0.3j * b
    psic = np.conj(psi) + 0.05 * (c + 1j * d)
    return np.ascontiguousarray(psi), np.ascontiguousarray(psic)


def noise(shape, seed: int):
    return np.ascontiguousarray(det_uniform(seed, int(np.prod(shape))).reshape(shape))

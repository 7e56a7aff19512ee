"""Unit tests of the oracle's building blocks against independent restatements:
numpy FFT, Philox known-answer vectors, and the spin-1 drift against numerical
derivatives of an independently written action."""
import numpy as np
import pytest

from conftest import rel_err


@pytest.mark.parametrize("n", [2, 3, 4, 5, 6, 8, 12, 16, 30, 32, 64, 80, 96, 128, 256])
def test_fft_line_matches_numpy(oracle, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    assert rel_err(oracle.fft_line(x, -1), np.fft.fft(x)) < 1e-13
    assert rel_err(oracle.fft_line(x, +1), np.fft.ifft(x, norm="forward")) < 1e-13


# Published known-answer vectors of Philox4x32-10 (Salmon et al., SC'11).
KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,out", KAT)
def test_philox_known_answers(oracle, ctr, key, out):
    assert tuple(oracle.philox4x32_10(ctr, key)) == out


def test_philox_normals_statistics(oracle):
    # 393k normals: 5-sigma bounds on mean, variance and fourth moment
    p = oracle.spin1_params(nx=256, nt=256)
    z = oracle.philox_noise(p, seed=20261203, chain=0, step=0)
    v = z.reshape(-1)
    assert abs(v.mean()) < 0.008
    assert abs(v.var() - 1.0) < 0.012
    assert abs(np.mean(v ** 4) - 3.0) < 0.08
    z2 = oracle.philox_noise(p, seed=20261203, chain=0, step=1)
    assert abs(np.corrcoef(v, z2.reshape(-1))[0, 1]) < 0.008


def _numpy_kinetic_exp(p, f):
    """exp(-eps (k^2/2 - mu - q m^2)) applied in Fourier space per (c, tau) slice."""
    C, T, X, Y, Z = f.shape
    def k(L):
        j = np.arange(L)
        return np.where((j < L // 2) | (L == 1), 2 * np.pi * j / L, -2 * np.pi * (L - j) / L)
    k2 = k(X)[:, None, None] ** 2 + k(Y)[None, :, None] ** 2 + k(Z)[None, None, :] ** 2
    out = np.empty_like(f)
    for c in range(C):
        m = 1 - c
        E = np.exp(-p.eps * (0.5 * k2 - p.mu - p.q * m * m))
        out[c] = np.fft.ifftn(E[None] * np.fft.fftn(f[c], axes=(1, 2, 3)), axes=(1, 2, 3))
    return out


def _action(p, psi, psic):
    """S = sum_tau [psibar_tau.psi_tau - psibar_tau.E psi_{tau-1} + eps V(psibar_tau, psi_{tau-1})]."""
    Epsi = _numpy_kinetic_exp(p, psi)
    ket = np.roll(psi, 1, axis=1)       # psi(tau-1)
    Eket = np.roll(Epsi, 1, axis=1)
    bar = psic
    n = np.sum(bar * ket, axis=0)
    Fz = bar[0] * ket[0] - bar[2] * ket[2]
    Fp = np.sqrt(2) * (bar[0] * ket[1] + bar[1] * ket[2])
    Fm = np.sqrt(2) * (bar[1] * ket[0] + bar[2] * ket[1])
    V = 0.5 * p.c0 * n ** 2 + 0.5 * p.c1 * (Fz ** 2 + Fp * Fm)
    return np.sum(bar * psi) - np.sum(bar * Eket) + p.eps * np.sum(V)


def test_spin1_drift_is_minus_action_gradient(oracle):
    rng = np.random.default_rng(7)
    p = oracle.spin1_params(nx=6, ny=4, nz=1, nt=5, eps=0.07, mu=0.8, c0=0.4, c1=-0.3, q=0.1)
    shape = p.shape
    psi = 0.6 + 0.2 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    psic = np.conj(psi) + 0.1 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    kin, kinc = oracle.kinetic(p, psi, psic)
    d, dc = oracle.drift(p, psi, psic, kin, kinc)
    h = 1e-5
    for idx in [(0, 0, 0, 0, 0), (1, 2, 3, 1, 0), (2, 4, 5, 3, 0), (1, 0, 2, 2, 0)]:
        for field, target in ((psic, d), (psi, dc)):
            a = field.copy(); a[idx] += h
            b = field.copy(); b[idx] -= h
            if field is psic:
                g = (_action(p, psi, a) - _action(p, psi, b)) / (2 * h)
            else:
                g = (_action(p, a, psic) - _action(p, b, psic)) / (2 * h)
            assert abs(-g - target[idx]) < 1e-7 * max(1.0, abs(target[idx])), (idx, -g, target[idx])


def test_spin1_exp_kinetic_matches_numpy(oracle):
    rng = np.random.default_rng(3)
    p = oracle.spin1_params(nx=8, ny=6, nz=4, nt=3, eps=0.1, mu=0.5, q=0.2)
    psi = rng.standard_normal(p.shape) + 1j * rng.standard_normal(p.shape)
    psic = rng.standard_normal(p.shape) + 1j * rng.standard_normal(p.shape)
    kin, kinc = oracle.kinetic(p, psi, psic)
    assert rel_err(kin, _numpy_kinetic_exp(p, psi)) < 1e-13
    assert rel_err(kinc, _numpy_kinetic_exp(p, psic)) < 1e-13


def test_spin1_observables_match_numpy(oracle):
    rng = np.random.default_rng(5)
    p = oracle.spin1_params(nx=8, ny=4, nt=4, c0=0.3, c1=-0.05, q=0.02)
    psi = 0.5 + 0.1 * (rng.standard_normal(p.shape) + 1j * rng.standard_normal(p.shape))
    psic = np.conj(psi) + 0.05 * rng.standard_normal(p.shape)
    out = oracle.spin1_observables(p, psi, psic)
    bar = np.roll(psic, -1, axis=1)  # psibar(tau+1)
    ket = psi
    n = np.sum(bar * ket, axis=0)
    Fz = bar[0] * ket[0] - bar[2] * ket[2]
    Fp = np.sqrt(2) * (bar[0] * ket[1] + bar[1] * ket[2])
    Fm = np.sqrt(2) * (bar[1] * ket[0] + bar[2] * ket[1])
    F2 = Fz ** 2 + Fp * Fm
    C, T, X, Y, Z = p.shape
    j = np.arange(X); kx = np.where(j < X // 2, 2 * np.pi * j / X, -2 * np.pi * (X - j) / X)
    j = np.arange(Y); ky = np.where(j < Y // 2, 2 * np.pi * j / Y, -2 * np.pi * (Y - j) / Y)
    k2 = kx[:, None, None] ** 2 + ky[None, :, None] ** 2
    tk = np.fft.ifftn(0.5 * k2[None, None] * np.fft.fftn(ket, axes=(2, 3, 4)), axes=(2, 3, 4))
    m2 = np.array([1.0, 0.0, 1.0])[:, None, None, None, None]
    e = np.sum(bar * (tk - p.q * m2 * ket), axis=0) + 0.5 * p.c0 * n ** 2 + 0.5 * p.c1 * F2
    ref = [n.mean(), Fz.mean(), F2.mean(), e.mean()]
    got = [out[0] + 1j * out[1], out[2] + 1j * out[3], out[4] + 1j * out[5], out[6] + 1j * out[7]]
    for a, b in zip(got, ref):
        assert abs(a - b) < 1e-12 * max(1, abs(b))


def test_ref_set_mean_field(oracle):
    p = oracle.Params(nx=16, nt=16)
    f = oracle.set_mean_field(p, 0.3, 0.2, False)
    fc = oracle.set_mean_field(p, 0.3, 0.2, True)
    assert np.all(f[0] == 0.3 + 0.2j) and np.all(f[3] == 0.3 + 0.2j)
    assert np.allclose(f[1], (2 / 3) * (0.3 + 0.2j), rtol=1e-15)
    assert np.all(fc[0] == 0.3 - 0.2j)

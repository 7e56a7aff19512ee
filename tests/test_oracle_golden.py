"""Pin the CPU oracle to the reference's own kernels.

The golden vectors in tests/golden/ come from the reference's kernel sources
(Propagator_without_cutoff.cu, Lattice.cu, Observables_without_cutoff.cu)
compiled for the host by oracle/ref_build.sh and driven in the order of
Propagator::propagate with injected noise (tests/golden/make_golden.py).
"""
import numpy as np
import pytest

from conftest import golden_files, large_golden_files, load_golden, load_large_golden, rel_err

FILES = golden_files()


def test_golden_present():
    assert len(FILES) >= 6


@pytest.mark.parametrize("path", FILES, ids=lambda p: p.split("/")[-1][5:-4])
def test_oracle_matches_reference_kernels(oracle, path):
    g, kw = load_golden(path)
    p = oracle.Params(**kw)
    kin, kinc = oracle.kinetic(p, g["psi0"], g["psic0"])
    assert rel_err(kin, g["kin0"]) < 1e-13 or np.abs(g["kin0"]).max() == 0
    assert rel_err(kinc, g["kinc0"]) < 1e-13 or np.abs(g["kinc0"]).max() == 0
    d, dc = oracle.drift(p, g["psi0"], g["psic0"], g["kin0"], g["kinc0"])
    assert np.array_equal(d, g["drift0"]) or rel_err(d, g["drift0"]) < 1e-14
    assert np.array_equal(dc, g["driftc0"]) or rel_err(dc, g["driftc0"]) < 1e-14
    psi, psic = g["psi0"], g["psic0"]
    for s in range(len(g["dt"])):
        psi, psic, dt, mx, mean = oracle.step(p, psi, psic, noise=g["noise"][s])
        assert abs(dt - g["dt"][s]) <= 1e-13 * g["dt"][s]
        assert abs(mx - g["max"][s]) <= 1e-13 * max(g["max"][s], 1e-300)
        assert abs(mean - g["mean"][s]) <= 1e-13 * max(g["mean"][s], 1e-300)
        assert rel_err(psi, g["psi"][s]) < 1e-13
        assert rel_err(psic, g["psic"][s]) < 1e-13
    for tag, fields in (("0", (g["psi0"], g["psic0"])), ("1", (g["psi"][-1], g["psic"][-1]))):
        F, n = oracle.ref_observables(p, *fields)
        assert rel_err(F, g["F" + tag]) < 1e-13
        assert rel_err(n, g["n" + tag]) < 1e-13


def test_dt_rule_table(oracle):
    t = np.load("tests/golden/ref4_dt_table.npz")
    p = oracle.Params(DT=float(t["DT"]))
    for mean, mx, dt in t["table"]:
        got, _ = oracle.new_dt(p, mean, mx)
        assert got == dt, (mean, mx, got, dt)


def test_zero_start_takes_base_step(oracle):
    """main.cu starts from exactly zero fields: max|K| = 0 gives dt = DT."""
    path = [f for f in FILES if f.endswith("1d_x16_t16_zero.npz")][0]
    g, kw = load_golden(path)
    assert g["dt"][0] == pytest.approx(kw["DT"], rel=1e-15)


@pytest.mark.parametrize("path", large_golden_files(), ids=lambda p: p.split("/")[-1][6:-4])
def test_oracle_matches_reference_kernels_large(oracle, path):
    """The reference's shipped 256 x 32 lattice and a 64 x 64 line: one step, the
    outputs compared at the fixture's 4096 sampled sites."""
    g, kw, psi0, psic0, noise = load_large_golden(path)
    assert len(large_golden_files()) >= 2
    p = oracle.Params(**kw)
    idx = g["idx"]
    kin, kinc = oracle.kinetic(p, psi0, psic0)
    assert rel_err(kin.reshape(-1)[idx], g["kin0"]) < 1e-13
    assert rel_err(kinc.reshape(-1)[idx], g["kinc0"]) < 1e-13
    d, dc = oracle.drift(p, psi0, psic0, kin, kinc)
    assert rel_err(d.reshape(-1)[idx], g["drift0"]) < 1e-13
    assert rel_err(dc.reshape(-1)[idx], g["driftc0"]) < 1e-13
    psi, psic, dt, mx, mean = oracle.step(p, psi0, psic0, noise=noise)
    assert abs(dt - g["dt"][0]) <= 1e-13 * g["dt"][0]
    assert abs(mx - g["max"][0]) <= 1e-13 * g["max"][0]
    assert abs(mean - g["mean"][0]) <= 1e-13 * g["mean"][0]
    assert rel_err(psi.reshape(-1)[idx], g["psi"]) < 1e-13
    assert rel_err(psic.reshape(-1)[idx], g["psic"]) < 1e-13
    F, n = oracle.ref_observables(p, psi0, psic0)
    assert rel_err(F, g["F0"]) < 1e-13
    assert rel_err(n, g["n0"]) < 1e-13

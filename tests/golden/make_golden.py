"""Generate the golden vectors that pin the oracle (and the CUDA engine) to the
reference's own kernels.

Run where the reference sources are (CLV_REFERENCE_DIR, default ../reference
beside the repository):

    python tests/golden/make_golden.py

For every configuration below it builds the reference's kernel sources for the
host with oracle/ref_build.sh (Parameters.h macros on the command line), then
drives them in the order of Propagator::propagate
(Propagator_without_cutoff.cu:406-442) with an injected unit-normal noise
buffer, and the observable kernels in the order of Observables::evaluate
(Observables_without_cutoff.cu:1155-1382).  cuFFT (cufftExecZ2Z over rank
1/2/3 spatial axes, batch C*T, Lattice.cu:135-180) is not available on the host;
it is restated with numpy's unnormalised DFT in the same direction convention:
CUFFT_FORWARD = exp(-2 pi i jk/N), CUFFT_INVERSE = exp(+2 pi i jk/N), no scaling.
cuRAND's curandGenerateNormalDouble(gen, buf, n, 0, sqrt(dt)) is replaced by
sqrt(dt) * z with z the injected standard normals.

Outputs tests/golden/ref4_<name>.npz (inputs, per-step dt/max/mean, fields after
each step, step-0 kinetic term and drift, observables) and ref4_dt_table.npz.
The larger lattices (the reference's shipped 256 x 32 and a 64 x 64 line) go to
tests/golden/ref4l_<name>.npz: their inputs come from tests/golden/detinputs.py
(reproducible anywhere, so not stored) and only the outputs at 4096 sampled
sites per array are kept.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_DIR = os.environ.get("CLV_REFERENCE_DIR", os.path.join(os.path.dirname(REPO), "reference"))
OUT_REF = os.path.join(REPO, "oracle", "_ref")

BASE_MACROS = dict(
    COMPONENTS=4, a_x=1.0, G=0.1, M=0.0, SIGMA=0.0, D=0.27735, OMEGAX=0.0, OMEGAY=0.0,
    OMEGAZ=0.0, Q=0.0, STEPS=10, DT=0.002, SNAPSHOT_TRIGGER=5, EVALUATE_TRIGGER=1,
    BLOCKSIZE=64, BLOCKSIZEX=16, BLOCKSIZEY=1, BLOCKSIZEZ=1, BLOCKSIZETAU=16,
    TERM_EXP=0.0, PREFACTOR=0.0, TERM1=0.0, SIN2=0.0, COS2=1.0, G_2D=0.0, EPS=0.01,
)

# name -> (macros, P, MU, init kind, steps)
CONFIGS = {
    # 1D, the reference's own couplings (Parameters.h, params.txt mu/P)
    "1d_x16_t16": (dict(XSIZE=16, YSIZE=1, ZSIZE=1, TAUSIZE=16), 0.0, -1.5, "random", 4),
    # 1D with Zeeman-like P and Q != 0, EPS and G changed
    "1d_x32_t8_pq": (dict(XSIZE=32, YSIZE=1, ZSIZE=1, TAUSIZE=8, BLOCKSIZETAU=8, EPS=0.025, G=0.3,
                          Q=0.05, DT=0.004),
                     0.2, 0.4, "random", 3),
    # 2D (cuFFT rank 2), a_x != 1
    "2d_x16_y4_t8": (dict(XSIZE=16, YSIZE=4, ZSIZE=1, TAUSIZE=8, BLOCKSIZETAU=8, EPS=0.02, G=0.2, Q=0.01,
                          a_x=0.5),
                     0.1, 0.3, "random", 3),
    # 3D (cuFFT rank 3), odd-ish factorisations; 8-wide x blocks
    "3d_x8_y4_z2_t8": (dict(XSIZE=8, YSIZE=4, ZSIZE=2, TAUSIZE=8, BLOCKSIZEX=8, EPS=0.02, G=0.15),
                       -0.1, 0.5, "random", 2),
    # main.cu's start: fields exactly zero (set_mean_field(0, 0)); max|K| = 0 branch
    "1d_x16_t16_zero": (dict(XSIZE=16, YSIZE=1, ZSIZE=1, TAUSIZE=16), 0.0, -1.5, "zero", 3),
    # a longer 1D line (the reference ships XSIZE=256, TAUSIZE=32), one step
    "1d_x64_t32": (dict(XSIZE=64, YSIZE=1, ZSIZE=1, TAUSIZE=32), 0.0, -1.5, "random", 1),
}


def build_ref(name: str, macros: dict) -> C.CDLL:
    m = dict(BASE_MACROS)
    m.update(macros)
    out = os.path.join(OUT_REF, f"libref_{name}.so")
    args = [os.path.join(REPO, "oracle", "ref_build.sh"), out] + [f"{k}={v}" for k, v in m.items()]
    subprocess.run(args, check=True)
    L = C.CDLL(out)
    cp = np.ctypeslib.ndpointer(dtype=np.complex128, flags="C_CONTIGUOUS")
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    L.ref_config.argtypes = [C.POINTER(C.c_int * 5)]
    L.ref_compute_kinetic_part.argtypes = [cp, cp, cp, cp]
    L.ref_normalization.argtypes = [cp, C.c_double]
    L.ref_drift.argtypes = [cp, cp, cp, cp, cp, cp, C.c_double, C.c_double, C.c_double]
    L.ref_max_and_mean_drift.argtypes = [cp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.ref_compute_new_dt.argtypes = [C.c_double, C.c_double]
    L.ref_compute_new_dt.restype = C.c_double
    L.ref_multiply_by_timestep.argtypes = [cp, cp, C.c_double]
    L.ref_add_noise.argtypes = [cp, cp, dp]
    L.ref_summation.argtypes = [cp, cp]
    L.ref_set_value.argtypes = [cp, C.c_double, C.c_double, C.c_int, C.c_double, C.c_double]
    L.ref_spin_density.argtypes = [cp, cp, dp, C.c_int]
    L.ref_n_kernel.argtypes = [cp, cp, dp, C.c_int]
    L.macros = m
    return L


def cufft(a: np.ndarray, direction: int) -> np.ndarray:
    """cufftExecZ2Z over the spatial axes of (C, T, X, Y, Z); direction -1/+1."""
    _, _, X, Y, Z = a.shape
    rank = 3 if Z > 1 else (2 if Y > 1 else (1 if X > 1 else 0))
    axes = (2, 3, 4)[:rank]
    if direction < 0:
        return np.ascontiguousarray(np.fft.fftn(a, axes=axes))
    return np.ascontiguousarray(np.fft.ifftn(a, axes=axes, norm="forward"))


def ref_propagate(L, psi, psic, z, P, MU):
    """Propagator::propagate with injected noise; returns intermediates."""
    m = L.macros
    kin = cufft(psi.copy(), +1)          # kin->fft(): CUFFT_INVERSE for psi
    kinc = cufft(psic.copy(), -1)        # kin_conjug->fft(): CUFFT_FORWARD
    L.ref_compute_kinetic_part(kin, kinc, kin, kinc)
    kin = cufft(kin, -1)                 # fft_inv(): CUFFT_FORWARD for psi
    kinc = cufft(kinc, +1)
    f = 1.0 / float(m["a_x"] * m["XSIZE"] * m["YSIZE"] * m["ZSIZE"])
    L.ref_normalization(kin, f)
    L.ref_normalization(kinc, f)
    drift = np.zeros_like(psi)
    driftc = np.zeros_like(psi)
    L.ref_drift(psi, psic, kin, kinc, drift, driftc, 1.0, P, MU)
    d0, dc0 = drift.copy(), driftc.copy()
    mx, mean = C.c_double(), C.c_double()
    L.ref_max_and_mean_drift(drift, C.byref(mx), C.byref(mean))
    dt = L.ref_compute_new_dt(mean.value, mx.value)
    random = np.ascontiguousarray(np.sqrt(dt) * z)
    L.ref_multiply_by_timestep(drift, driftc, dt)
    L.ref_add_noise(drift, driftc, random)
    L.ref_summation(psi, drift)
    L.ref_summation(psic, driftc)
    return dict(kin=kin, kinc=kinc, drift=d0, driftc=dc0, dt=dt, max=mx.value, mean=mean.value)


def ref_evaluate(L, psi, psic):
    """Per-call sums of Observables::evaluate for n_tot, n_11..n_22, F_x/F_y/F_z."""
    _, T, X, Y, Z = psi.shape
    V = X * Y * Z
    F = np.zeros((3, V))
    for i in range(3):
        b = np.zeros(V)
        L.ref_spin_density(psic.copy(), psi.copy(), b, i)
        F[i] = b
    pc = cufft(psic.copy(), -1)   # psi_conjugate->fft()
    pk = cufft(psi.copy(), +1)    # psi->fft()
    n = np.zeros(5)
    for w in range(5):
        avg = np.zeros(V * T)
        L.ref_n_kernel(pc, pk, avg, w)
        n[w] = avg.sum()
    return F, n


def make_config(name, macros, P, MU, init, nsteps, rng):
    L = build_ref(name, macros)
    cfg = (C.c_int * 5)()
    L.ref_config(C.byref(cfg))
    X, Y, Z, T, Cn = list(cfg)
    m = L.macros
    # the reference's launch geometry must cover the lattice exactly
    # (Propagator_without_cutoff.cu:325-331 warns otherwise)
    assert X % m["BLOCKSIZEX"] == 0 and Y % m["BLOCKSIZEY"] == 0
    assert (Z * T) % (m["BLOCKSIZEZ"] * m["BLOCKSIZETAU"]) == 0 and Z * T >= m["BLOCKSIZEZ"] * m["BLOCKSIZETAU"]
    assert (Cn * X * Y * Z * T) % m["BLOCKSIZE"] == 0
    shape = (Cn, T, X, Y, Z)
    if init == "zero":
        psi = np.zeros(shape, np.complex128)
        psic = np.zeros(shape, np.complex128)
        L.ref_set_value(psi, 0.0, 0.0, 0, P, MU)
        L.ref_set_value(psic, 0.0, 0.0, 1, P, MU)
    else:
        amp = 0.8
        psi = amp * (1 + 0.3 * rng.standard_normal(shape)) + 0.3j * rng.standard_normal(shape)
        psic = np.conj(psi) + 0.05 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
        psi = np.ascontiguousarray(psi)
        psic = np.ascontiguousarray(psic)
    psi0, psic0 = psi.copy(), psic.copy()
    F0, n0 = ref_evaluate(L, psi, psic)
    noises, dts, maxs, means, psis, psics = [], [], [], [], [], []
    first = None
    for s in range(nsteps):
        z = np.ascontiguousarray(rng.standard_normal((Cn, X, Y, Z, T, 2)))
        r = ref_propagate(L, psi, psic, z, P, MU)
        if first is None:
            first = r
        noises.append(z)
        dts.append(r["dt"]); maxs.append(r["max"]); means.append(r["mean"])
        psis.append(psi.copy()); psics.append(psic.copy())
    F1, n1 = ref_evaluate(L, psi, psic)
    np.savez_compressed(
        os.path.join(HERE, f"ref4_{name}.npz"),
        dims=np.array([X, Y, Z, T, Cn]),
        eps=m["EPS"], a_x=m["a_x"], G=m["G"], Q=m["Q"], DT=m["DT"], P=P, MU=MU,
        psi0=psi0, psic0=psic0, noise=np.stack(noises),
        dt=np.array(dts), max=np.array(maxs), mean=np.array(means),
        psi=np.stack(psis), psic=np.stack(psics),
        kin0=first["kin"], kinc0=first["kinc"], drift0=first["drift"], driftc0=first["driftc"],
        F0=F0, n0=n0, F1=F1, n1=n1,
    )
    print(f"{name}: dims={X}x{Y}x{Z}x{T} C={Cn} dt={dts}")


def make_dt_table(rng):
    L = build_ref("1d_x16_t16", CONFIGS["1d_x16_t16"][0])
    pairs = [(0.0, 0.0), (0.1, 0.0), (0.2, 1.0), (1e-9, 1.0), (5e-6, 1.0), (1.0, 0.1),
             (0.3, 0.9), (1.0, 1.0)] + [(float(a), float(b)) for a, b in rng.uniform(0, 2, (16, 2))]
    out = np.array([[mean, mx, L.ref_compute_new_dt(mean, mx)] for mean, mx in pairs])
    np.savez_compressed(os.path.join(HERE, "ref4_dt_table.npz"), table=out,
                        DT=L.macros["DT"])


# Output-layout cases: Parameters.h macros, mu, P, seed.  The reference's own
# SaveResults.cu (host build, oracle/ref_save_build.sh) writes the files for the
# fake observable values of oracle/ref_save_fake.hpp.
SAVE_CASES = {
    "ref_params": (dict(XSIZE=8, YSIZE=2, ZSIZE=1, TAUSIZE=4, EPS=0.025, G=0.3, Q=0.05, STEPS=1000,
                        SNAPSHOT_TRIGGER=500, EVALUATE_TRIGGER=100, BLOCKSIZEX=8, BLOCKSIZETAU=4),
                   -1.5, 0.0, 7342951900870119),
    "mu_p_fractions": (dict(XSIZE=16, YSIZE=1, ZSIZE=1, TAUSIZE=16, EPS=0.01, G=0.1, DT=0.0015),
                       0.3333, 0.125, 42),
}


def parameters_h(macros: dict) -> str:
    return "".join(f"#define {k} {v}\n" for k, v in macros.items())


def make_saveresults_golden():
    import shutil
    import tempfile
    root = os.path.join(HERE, "saveresults")
    shutil.rmtree(root, ignore_errors=True)
    for name, (macros, MU, P, seed) in SAVE_CASES.items():
        m = dict(BASE_MACROS)
        m.update(macros)
        exe = os.path.join(OUT_REF, f"ref_save_{name}")
        subprocess.run([os.path.join(REPO, "oracle", "ref_save_build.sh"), exe]
                       + [f"{k}={v}" for k, v in m.items()], check=True)
        case = os.path.join(root, name)
        os.makedirs(case)
        with open(os.path.join(case, "Parameters.h"), "w") as f:
            f.write(parameters_h(m))
        with open(os.path.join(case, "args.txt"), "w") as f:
            f.write(f"{MU} {P} {seed}\n")
        with tempfile.TemporaryDirectory() as tmp:
            subprocess.run([exe, tmp, str(MU), str(P), str(seed)], check=True, capture_output=True)
            shutil.copytree(os.path.join(tmp, "DATA"), os.path.join(case, "DATA"))


# Larger lattices: name -> (macros, P, MU, input seed).  The reference's shipped
# Parameters.h / params.txt lattice, and a line of the single-chain benchmark shape.
LARGE_CONFIGS = {
    "1d_x256_t32": (dict(XSIZE=256, YSIZE=1, ZSIZE=1, TAUSIZE=32), 0.0, -1.5, 101),
    "1d_x64_t64": (dict(XSIZE=64, YSIZE=1, ZSIZE=1, TAUSIZE=64, EPS=0.0625), 0.0, -1.5, 202),
}
N_SAMPLES = 4096


def make_large(name, macros, P, MU, seed):
    sys.path.insert(0, HERE)
    import detinputs
    L = build_ref(name, macros)
    cfg = (C.c_int * 5)()
    L.ref_config(C.byref(cfg))
    X, Y, Z, T, Cn = list(cfg)
    shape = (Cn, T, X, Y, Z)
    psi, psic = detinputs.ref4_inputs(shape, seed)
    F0, n0 = ref_evaluate(L, psi, psic)
    z = detinputs.noise((Cn, X, Y, Z, T, 2), seed + 10)
    r = ref_propagate(L, psi, psic, z, P, MU)
    m = L.macros
    idx = np.sort(np.random.default_rng(seed).choice(psi.size, N_SAMPLES, replace=False))
    np.savez_compressed(
        os.path.join(HERE, f"ref4l_{name}.npz"),
        dims=np.array([X, Y, Z, T, Cn]), seed=seed,
        eps=m["EPS"], a_x=m["a_x"], G=m["G"], Q=m["Q"], DT=m["DT"], P=P, MU=MU,
        idx=idx, psi=psi.reshape(-1)[idx], psic=psic.reshape(-1)[idx],
        kin0=r["kin"].reshape(-1)[idx], kinc0=r["kinc"].reshape(-1)[idx],
        drift0=r["drift"].reshape(-1)[idx], driftc0=r["driftc"].reshape(-1)[idx],
        dt=np.array([r["dt"]]), max=np.array([r["max"]]), mean=np.array([r["mean"]]), F0=F0, n0=n0,
    )
    print(f"{name}: dims={X}x{Y}x{Z}x{T} C={Cn} dt={r['dt']}")


def main():
    if not os.path.isdir(REF_DIR):
        sys.exit(f"reference sources not found at {REF_DIR}")
    rng = np.random.default_rng(20261203)
    for name, (macros, P, MU, init, nsteps) in CONFIGS.items():
        make_config(name, macros, P, MU, init, nsteps, rng)
    make_dt_table(rng)
    make_saveresults_golden()
    for name, (macros, P, MU, seed) in LARGE_CONFIGS.items():
        make_large(name, macros, P, MU, seed)


if __name__ == "__main__":
    main()

"""ctypes binding of the FP64 CPU oracle (oracle/clv_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by bench.py's CPU-baseline leg, always as the checker or the timed CPU
baseline, never as part of the product path.

Arrays follow the reference layout ``(C, T, X, Y, Z)`` complex128 (Lattice.cu:2-5);
noise buffers follow ``ind_rand`` (Lattice.cu:7-11): float64 of shape
``(C, X, Y, Z, T, 2)``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field, asdict

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

MODEL_REF4, MODEL_SPIN1 = 0, 1
KIN_REF_LINEAR_PX, KIN_EXP = 0, 1
DT_REF_MEANMAX, DT_K_OVER_MAX = 0, 1


class OrcParams(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nx", "ny", "nz", "nt", "ncomp", "model", "kinetic", "dt_rule")] + [
        (n, C.c_double)
        for n in ("eps", "a_x", "G", "Q", "P", "mu", "DT", "dt_min", "dt_max_clamp", "alpha",
                  "c0", "c1", "q", "Kc", "dt_max")
    ]


@dataclass
class Params:
    """Lattice + model parameters shared by the oracle and the tests."""
    nx: int = 16
    ny: int = 1
    nz: int = 1
    nt: int = 16
    ncomp: int = 4
    model: int = MODEL_REF4
    kinetic: int = KIN_REF_LINEAR_PX
    dt_rule: int = DT_REF_MEANMAX
    eps: float = 0.01
    a_x: float = 1.0
    G: float = 0.1
    Q: float = 0.0
    P: float = 0.0
    mu: float = -1.5
    DT: float = 0.002
    dt_min: float = 1e-8
    dt_max_clamp: float = 0.01
    alpha: float = 0.9
    c0: float = 0.5
    c1: float = -0.1
    q: float = 0.05
    Kc: float = 0.05
    dt_max: float = 1e-3

    def c(self) -> OrcParams:
        return OrcParams(**asdict(self))

    @property
    def shape(self):
        return (self.ncomp, self.nt, self.nx, self.ny, self.nz)

    @property
    def vol(self):
        return self.nx * self.ny * self.nz


def spin1_params(**kw) -> Params:
    base = dict(ncomp=3, model=MODEL_SPIN1, kinetic=KIN_EXP, dt_rule=DT_K_OVER_MAX)
    base.update(kw)
    return Params(**base)


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        cp = np.ctypeslib.ndpointer(dtype=np.complex128, flags="C_CONTIGUOUS")
        P = C.POINTER(OrcParams)
        L.orc_fft_line.argtypes = [cp, C.c_int, C.c_long, C.c_int]
        L.orc_kinetic.argtypes = [P, cp, cp, cp, cp]
        L.orc_drift.argtypes = [P, cp, cp, cp, cp, cp, cp, C.c_double]
        L.orc_max_mean.argtypes = [P, cp, cp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_new_dt.argtypes = [P, C.c_double, C.c_double, C.POINTER(C.c_int)]
        L.orc_new_dt.restype = C.c_double
        L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32 * 4), C.POINTER(C.c_uint32 * 2),
                                        C.POINTER(C.c_uint32 * 4)]
        L.orc_philox_normal.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_int, C.c_uint32,
                                        C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_philox_noise_buffer.argtypes = [P, C.c_uint64, C.c_uint32, C.c_uint64, dp]
        L.orc_update.argtypes = [P, cp, cp, cp, cp, dp, C.c_double]
        L.orc_step.argtypes = [P, cp, cp, C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint64,
                               C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_step.restype = C.c_double
        L.orc_ref_observables.argtypes = [P, cp, cp, dp, dp]
        L.orc_spin1_observables.argtypes = [P, cp, cp, dp]
        L.orc_set_mean_field.argtypes = [P, cp, C.c_double, C.c_double, C.c_int]
        L.orc_spin1_init.argtypes = [P, C.c_uint64, C.c_uint32, C.c_double, C.c_double, cp, cp]
        L.orc_num_threads.restype = C.c_int
        L.orc_set_num_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def fft_line(x: np.ndarray, sign: int) -> np.ndarray:
    y = _c(x, np.complex128).copy()
    lib().orc_fft_line(y, y.size, 1, sign)
    return y


def kinetic(p: Params, psi, psic):
    psi, psic = _c(psi, np.complex128), _c(psic, np.complex128)
    kin, kinc = np.empty_like(psi), np.empty_like(psic)
    lib().orc_kinetic(C.byref(p.c()), psi, psic, kin, kinc)
    return kin, kinc


def drift(p: Params, psi, psic, kin, kinc, factor=1.0):
    args = [_c(a, np.complex128) for a in (psi, psic, kin, kinc)]
    d, dc = np.empty_like(args[0]), np.empty_like(args[0])
    lib().orc_drift(C.byref(p.c()), *args, d, dc, factor)
    return d, dc


def max_mean(p: Params, d, dc):
    mx, mean = C.c_double(), C.c_double()
    lib().orc_max_mean(C.byref(p.c()), _c(d, np.complex128), _c(dc, np.complex128),
                       C.byref(mx), C.byref(mean))
    return mx.value, mean.value


def new_dt(p: Params, mean, mx):
    cl = C.c_int()
    dt = lib().orc_new_dt(C.byref(p.c()), mean, mx, C.byref(cl))
    return dt, cl.value


def philox4x32_10(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(C.byref(c), C.byref(k), C.byref(o))
    return list(o)


def philox_noise(p: Params, seed: int, chain: int, step: int) -> np.ndarray:
    out = np.empty((p.ncomp, p.nx, p.ny, p.nz, p.nt, 2), np.float64)
    lib().orc_philox_noise_buffer(C.byref(p.c()), seed, chain, step, out)
    return out


def step(p: Params, psi, psic, noise=None, seed=0, chain=0, step_index=0):
    """One step in place on copies; returns (psi, psic, dt, max, mean)."""
    psi = _c(psi, np.complex128).copy()
    psic = _c(psic, np.complex128).copy()
    nz = None if noise is None else _c(noise, np.float64)
    mx, mean = C.c_double(), C.c_double()
    dt = lib().orc_step(C.byref(p.c()), psi, psic,
                        None if nz is None else nz.ctypes.data_as(C.c_void_p),
                        seed, chain, step_index, C.byref(mx), C.byref(mean))
    return psi, psic, dt, mx.value, mean.value


def ref_observables(p: Params, psi, psic):
    F = np.empty((3, p.vol), np.float64)
    n = np.empty(5, np.float64)
    lib().orc_ref_observables(C.byref(p.c()), _c(psi, np.complex128), _c(psic, np.complex128), F, n)
    return F, n


def spin1_observables(p: Params, psi, psic) -> np.ndarray:
    out = np.empty(8, np.float64)
    lib().orc_spin1_observables(C.byref(p.c()), _c(psi, np.complex128), _c(psic, np.complex128), out)
    return out


def set_mean_field(p: Params, re, im, conjugated):
    f = np.zeros(p.shape, np.complex128)
    lib().orc_set_mean_field(C.byref(p.c()), f, re, im, int(conjugated))
    return f


def spin1_init(p: Params, seed: int, chain: int, amp=np.sqrt(1 / 3), sigma=0.01):
    psi = np.zeros(p.shape, np.complex128)
    psic = np.zeros(p.shape, np.complex128)
    lib().orc_spin1_init(C.byref(p.c()), seed, chain, amp, sigma, psi, psic)
    return psi, psic


def num_threads() -> int:
    return lib().orc_num_threads()


def set_num_threads(n: int) -> None:
    lib().orc_set_num_threads(n)

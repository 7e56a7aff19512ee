"""ctypes binding of libclv.so (the C ABI in include/clv.h).

The library is built in-tree by ``cl_var_dt_gb300._build.build()``.  Loading
fails loudly when it is missing: there is no CPU fallback in the product path.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, fields as dc_fields

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libclv.so")

OK, ERR_ARG, ERR_CUDA, ERR_NONFINITE, ERR_TIMEOUT, ERR_STATE, ERR_NOMEM, ERR_IO = range(8)
MODEL_REF4, MODEL_SPIN1 = 0, 1
KIN_REF_LINEAR_PX, KIN_EXP = 0, 1
DT_REF_MEANMAX, DT_K_OVER_MAX = 0, 1
NOISE_EXTERNAL, NOISE_PHILOX = 0, 1
PREC_F64, PREC_F32 = 0, 1
HOST, DEVICE, C64, ASYNC = 0, 1, 2, 4
FLAG_NONFINITE, FLAG_DT_CLAMPED_LOW, FLAG_DT_CLAMPED_HIGH, FLAG_TIMEOUT = 1, 2, 4, 8

# Every symbol include/clv.h declares (checked by the CPU test suite).
EXPORTED = (
    "clv_default_chain_params", "clv_create", "clv_destroy", "clv_last_error", "clv_status_string",
    "clv_version", "clv_set_stream", "clv_synchronize", "clv_set_fields", "clv_get_fields",
    "clv_set_mean_field", "clv_set_chemical_potential", "clv_init_spin1", "clv_step", "clv_step_timed", "clv_step_with_noise",
    "clv_get_step_info",
    "clv_get_chain_flags", "clv_evaluate", "clv_get_counter", "clv_read_ref_observables",
    "clv_read_spin1_samples", "clv_save_checkpoint", "clv_load_checkpoint", "clv_device_bytes",
    "clv_ref_observables_noalloc", "clv_get_plan", "clv_autotune", "clv_measure_peaks",
)


class ChainParamsC(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("nt", C.c_int)] + [
        (n, C.c_double)
        for n in ("eps", "a_x", "mu", "P", "Q", "G", "DT", "dt_min", "dt_max_clamp", "alpha",
                  "c0", "c1", "q", "K", "dt_max")
    ] + [("seed", C.c_uint64)]


class ConfigC(C.Structure):
    _fields_ = [("model", C.c_int), ("kinetic", C.c_int), ("dt_rule", C.c_int), ("noise", C.c_int),
                ("precision", C.c_int), ("device", C.c_int), ("nchains", C.c_int),
                ("chains", C.POINTER(ChainParamsC))]


@dataclass
class ChainParams:
    """Per-chain parameters; defaults are the reference's (Parameters.h, params.txt)."""
    nx: int = 256
    ny: int = 1
    nz: int = 1
    nt: int = 32
    eps: float = 0.01
    a_x: float = 1.0
    mu: float = -1.5
    P: float = 0.0
    Q: float = 0.0
    G: float = 0.1
    DT: float = 0.002
    dt_min: float = 1e-8
    dt_max_clamp: float = 0.01
    alpha: float = 0.9
    c0: float = 0.5
    c1: float = -0.1
    q: float = 0.05
    K: float = 0.05
    dt_max: float = 1e-3
    seed: int = 7342951900870119

    def to_c(self) -> ChainParamsC:
        return ChainParamsC(**{f.name: getattr(self, f.name) for f in dc_fields(self)})

    @property
    def vol(self) -> int:
        return self.nx * self.ny * self.nz


class ClvError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"clv status {status}: {msg}")
        self.status = status


_lib = None


def lib() -> C.CDLL:
    """Load libclv.so; raise if the CUDA extension has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build the CUDA extension first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    L.clv_default_chain_params.argtypes = [C.POINTER(ChainParamsC)]
    L.clv_default_chain_params.restype = None
    L.clv_create.argtypes = [C.POINTER(ConfigC), C.POINTER(vp)]
    L.clv_destroy.argtypes = [vp]
    L.clv_last_error.restype = C.c_char_p
    L.clv_status_string.argtypes = [C.c_int]
    L.clv_status_string.restype = C.c_char_p
    L.clv_set_stream.argtypes = [vp, vp]
    L.clv_synchronize.argtypes = [vp]
    L.clv_set_fields.argtypes = [vp, C.c_int, vp, vp, C.c_int]
    L.clv_get_fields.argtypes = [vp, C.c_int, vp, vp, C.c_int]
    L.clv_set_mean_field.argtypes = [vp, C.c_int, C.c_double, C.c_double]
    L.clv_init_spin1.argtypes = [vp, C.c_double, C.c_double]
    L.clv_set_chemical_potential.argtypes = [vp, C.c_int, C.c_double, C.c_double]
    L.clv_step.argtypes = [vp, C.c_int]
    L.clv_step_timed.argtypes = [vp, C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_int)]
    L.clv_step_with_noise.argtypes = [vp, vp, C.c_int]
    L.clv_get_step_info.argtypes = [vp, dp, dp, dp, dp, C.POINTER(C.c_uint64)]
    L.clv_get_chain_flags.argtypes = [vp, C.POINTER(C.c_int)]
    L.clv_evaluate.argtypes = [vp]
    L.clv_get_counter.argtypes = [vp]
    L.clv_read_ref_observables.argtypes = [vp, C.c_int, dp, dp, dp, dp]
    L.clv_read_spin1_samples.argtypes = [vp, C.c_int, dp, C.c_int, C.POINTER(C.c_int)]
    L.clv_save_checkpoint.argtypes = [vp, C.c_char_p]
    L.clv_load_checkpoint.argtypes = [vp, C.c_char_p]
    L.clv_device_bytes.argtypes = [vp, C.POINTER(C.c_size_t)]
    L.clv_get_plan.argtypes = [vp, C.c_char_p, C.c_int]
    L.clv_autotune.argtypes = [vp, C.c_int, C.c_char_p, C.c_int]
    L.clv_ref_observables_noalloc.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                              vp, vp, vp]
    L.clv_measure_peaks.argtypes = [C.c_int, dp, dp]
    _lib = L
    return L


def check(rc: int):
    if rc != OK:
        raise ClvError(rc, lib().clv_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(C.c_void_p)


def measure_peaks(device=0):
    """(FP64, FP32) FMA throughput of the device in TFLOP/s (clv_measure_peaks)."""
    f64, f32 = C.c_double(), C.c_double()
    check(lib().clv_measure_peaks(device, C.byref(f64), C.byref(f32)))
    return f64.value, f32.value


class Engine:
    """A batch of chains on one GPU (owns a clv_engine handle)."""

    def __init__(self, chains, model=MODEL_REF4, kinetic=None, dt_rule=None, noise=NOISE_PHILOX,
                 precision=PREC_F64, device=0):
        if isinstance(chains, ChainParams):
            chains = [chains]
        self.chains = list(chains)
        self.model = model
        self.kinetic = kinetic if kinetic is not None else (
            KIN_REF_LINEAR_PX if model == MODEL_REF4 else KIN_EXP)
        self.dt_rule = dt_rule if dt_rule is not None else (
            DT_REF_MEANMAX if model == MODEL_REF4 else DT_K_OVER_MAX)
        self.noise = noise
        self.precision = precision
        self.ncomp = 4 if model == MODEL_REF4 else 3
        arr = (ChainParamsC * len(self.chains))(*[c.to_c() for c in self.chains])
        self._arr = arr
        cfg = ConfigC(model, self.kinetic, self.dt_rule, noise, precision, device, len(self.chains), arr)
        h = C.c_void_p()
        check(lib().clv_create(C.byref(cfg), C.byref(h)))
        self.h = h

    # -- lifetime
    def close(self):
        if getattr(self, "h", None):
            lib().clv_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- layout helpers
    def shape(self, chain=0):
        c = self.chains[chain]
        return (self.ncomp, c.nt, c.nx, c.ny, c.nz)

    def noise_shape(self, chain=0):
        c = self.chains[chain]
        return (self.ncomp, c.nx, c.ny, c.nz, c.nt, 2)

    # -- fields
    def set_fields(self, chain, psi, psic):
        """Fields of one chain from host arrays; complex64 arrays cross as complex64."""
        dt = np.complex64 if (np.asarray(psi).dtype == np.complex64 and
                              np.asarray(psic).dtype == np.complex64) else np.complex128
        psi = np.ascontiguousarray(psi, dtype=dt)
        psic = np.ascontiguousarray(psic, dtype=dt)
        assert psi.shape == self.shape(chain) and psic.shape == self.shape(chain)
        where = HOST | (C64 if dt == np.complex64 else 0)
        check(lib().clv_set_fields(self.h, chain, _ptr(psi), _ptr(psic), where))

    def get_fields(self, chain=0, dtype=np.complex128):
        dtype = np.dtype(dtype)
        assert dtype in (np.complex64, np.complex128)
        psi = np.empty(self.shape(chain), dtype)
        psic = np.empty(self.shape(chain), dtype)
        where = HOST | (C64 if dtype == np.complex64 else 0)
        check(lib().clv_get_fields(self.h, chain, _ptr(psi), _ptr(psic), where))
        return psi, psic

    def set_fields_device(self, chain, psi_ptr: int, psic_ptr: int):
        check(lib().clv_set_fields(self.h, chain, C.c_void_p(psi_ptr), C.c_void_p(psic_ptr), DEVICE))

    def get_fields_device(self, chain, psi_ptr: int, psic_ptr: int):
        check(lib().clv_get_fields(self.h, chain, C.c_void_p(psi_ptr), C.c_void_p(psic_ptr), DEVICE))

    def set_mean_field(self, field, re, im):
        check(lib().clv_set_mean_field(self.h, field, re, im))

    def set_chemical_potential(self, chain, mu, P=0.0):
        check(lib().clv_set_chemical_potential(self.h, chain, mu, P))
        for i in (range(len(self.chains)) if chain == -1 else [chain]):
            self.chains[i].mu = mu
            self.chains[i].P = P

    def init_spin1(self, amp=np.sqrt(1 / 3), sigma=0.01):
        check(lib().clv_init_spin1(self.h, amp, sigma))

    # -- stepping
    def step(self, n=1):
        check(lib().clv_step(self.h, n))

    def step_timed(self):
        """One Philox step; returns the device ms of each launch (kinetic passes, drift, update)."""
        buf = (C.c_float * 16)()
        n = C.c_int()
        check(lib().clv_step_timed(self.h, buf, 16, C.byref(n)))
        return [float(buf[i]) for i in range(n.value)]

    def step_with_noise(self, noise):
        noise = np.ascontiguousarray(noise, dtype=np.float64)
        check(lib().clv_step_with_noise(self.h, _ptr(noise), HOST))

    def step_with_noise_device(self, ptr: int):
        check(lib().clv_step_with_noise(self.h, C.c_void_p(ptr), DEVICE))

    def synchronize(self):
        check(lib().clv_synchronize(self.h))

    def set_stream(self, stream_ptr: int):
        check(lib().clv_set_stream(self.h, C.c_void_p(stream_ptr)))

    def step_info(self):
        n = len(self.chains)
        dt, mx, mean, t = (np.zeros(n) for _ in range(4))
        steps = np.zeros(n, np.uint64)
        dp = C.POINTER(C.c_double)
        check(lib().clv_get_step_info(self.h, dt.ctypes.data_as(dp), mx.ctypes.data_as(dp),
                                      mean.ctypes.data_as(dp), t.ctypes.data_as(dp),
                                      steps.ctypes.data_as(C.POINTER(C.c_uint64))))
        return dict(dt=dt, max=mx, mean=mean, t=t, steps=steps)

    def chain_flags(self, raise_on_nonfinite=False):
        f = np.zeros(len(self.chains), np.int32)
        rc = lib().clv_get_chain_flags(self.h, f.ctypes.data_as(C.POINTER(C.c_int)))
        if rc not in (OK, ERR_NONFINITE, ERR_TIMEOUT) or (raise_on_nonfinite and rc != OK):
            check(rc)
        return f

    # -- observables
    def evaluate(self):
        check(lib().clv_evaluate(self.h))

    @property
    def counter(self):
        return lib().clv_get_counter(self.h)

    def ref_observables(self, chain=0):
        V = self.chains[chain].vol
        n = np.zeros(5)
        F = np.zeros((3, V))
        dp = C.POINTER(C.c_double)
        check(lib().clv_read_ref_observables(self.h, chain, n.ctypes.data_as(dp),
                                             F[0].ctypes.data_as(dp), F[1].ctypes.data_as(dp),
                                             F[2].ctypes.data_as(dp)))
        return n, F

    def spin1_samples(self, chain=0):
        cnt = C.c_int()
        check(lib().clv_read_spin1_samples(self.h, chain, None, 0, C.byref(cnt)))
        out = np.zeros((max(cnt.value, 1), 8))
        check(lib().clv_read_spin1_samples(self.h, chain, out.ctypes.data_as(C.POINTER(C.c_double)),
                                           cnt.value, C.byref(cnt)))
        return out[: cnt.value]

    # -- checkpoint
    def save_checkpoint(self, path):
        check(lib().clv_save_checkpoint(self.h, os.fsencode(path)))

    def load_checkpoint(self, path):
        check(lib().clv_load_checkpoint(self.h, os.fsencode(path)))

    def plan(self):
        """(path, [phase names]) of the engine's step, e.g. ("tiled", ["axis0_n128", ...])."""
        buf = C.create_string_buffer(512)
        check(lib().clv_get_plan(self.h, buf, 512))
        path, phases = buf.value.decode().split(":", 1)
        return path, phases.split(",")

    def autotune(self, trial_steps=10):
        """Time the candidate plans and keep the fastest; returns the report text."""
        buf = C.create_string_buffer(4096)
        check(lib().clv_autotune(self.h, trial_steps, buf, 4096))
        return buf.value.decode()

    def device_bytes(self):
        b = C.c_size_t()
        check(lib().clv_device_bytes(self.h, C.byref(b)))
        return b.value

"""The reference's own GPU build, for parity and timing on the GPU.

TEST INFRASTRUCTURE ONLY: imported by tests/ and by bench.py's reference-GPU leg,
always as the checker or as the timed reference, never by the product.

Each configuration below is a set of Parameters.h macros.  ``build_cubins``
compiles the reference's kernels for every configuration into
``oracle/_ref/refgpu_<name>.cubin`` with ``oracle/ref_gpu_build.sh`` -- only
where the reference sources are (``CLV_REFERENCE_DIR``, default
``../reference`` beside the repository); the cubins then travel with the
repository.  ``oracle/libref_gpu.so`` (``oracle/ref_gpu_runner.cpp``, built by
``make -C oracle libref_gpu.so`` on the machine that runs it) drives them with
cuFFT and cuRAND in the order of Propagator::propagate
(Propagator_without_cutoff.cu:406-442).
"""
from __future__ import annotations

import concurrent.futures as cf
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref")
LIB_PATH = os.path.join(HERE, "libref_gpu.so")

# Parameters.h of the reference (Parameters.h:6-50) with the lattice left out
BASE_MACROS = dict(
    COMPONENTS=4, a_x=1.0, G=0.1, M=0.0, SIGMA=0.0, D=0.27735, OMEGAX=0.0, OMEGAY=0.0,
    OMEGAZ=0.0, Q=0.0, STEPS=10, DT=0.002, SNAPSHOT_TRIGGER=5, EVALUATE_TRIGGER=1,
    BLOCKSIZE=64, BLOCKSIZEX=16, BLOCKSIZEY=1, BLOCKSIZEZ=1, BLOCKSIZETAU=16,
    TERM_EXP=0.0, PREFACTOR=0.0, TERM1=0.0, SIN2=0.0, COS2=1.0, G_2D=0.0, EPS=0.01,
)

# name -> (macros over BASE_MACROS, P, MU).  The first six are the golden-vector
# configurations (tests/golden/make_golden.py); then the reference's shipped
# Parameters.h lattice (256 x 1 x 1, N_tau 32, params.txt mu = -1.5), a lattice of
# the single-chain benchmark shape (64 sites, N_tau 64, beta 4), one of the
# batched benchmark shape (256 sites, N_tau 128, beta 6), the 2D and 3D benchmark
# lattices and the ensemble line.
CONFIGS = {
    "1d_x16_t16": (dict(XSIZE=16, YSIZE=1, ZSIZE=1, TAUSIZE=16), 0.0, -1.5),
    "1d_x32_t8_pq": (dict(XSIZE=32, YSIZE=1, ZSIZE=1, TAUSIZE=8, BLOCKSIZETAU=8, EPS=0.025, G=0.3,
                          Q=0.05, DT=0.004), 0.2, 0.4),
    "2d_x16_y4_t8": (dict(XSIZE=16, YSIZE=4, ZSIZE=1, TAUSIZE=8, BLOCKSIZETAU=8, EPS=0.02, G=0.2, Q=0.01,
                          a_x=0.5), 0.1, 0.3),
    "3d_x8_y4_z2_t8": (dict(XSIZE=8, YSIZE=4, ZSIZE=2, TAUSIZE=8, BLOCKSIZEX=8, EPS=0.02, G=0.15), -0.1, 0.5),
    "1d_x16_t16_zero": (dict(XSIZE=16, YSIZE=1, ZSIZE=1, TAUSIZE=16), 0.0, -1.5),
    "1d_x64_t32": (dict(XSIZE=64, YSIZE=1, ZSIZE=1, TAUSIZE=32), 0.0, -1.5),
    "1d_x256_t32": (dict(XSIZE=256, YSIZE=1, ZSIZE=1, TAUSIZE=32, STEPS=8000000, SNAPSHOT_TRIGGER=500000,
                         EVALUATE_TRIGGER=100), 0.0, -1.5),
    "1d_x64_t64": (dict(XSIZE=64, YSIZE=1, ZSIZE=1, TAUSIZE=64, EPS=0.0625), 0.0, -1.5),
    "1d_x256_t128": (dict(XSIZE=256, YSIZE=1, ZSIZE=1, TAUSIZE=128, EPS=0.046875), 0.0, -1.5),
    # the lattices of the 2D precision configuration (128 x 128, N_tau 128, beta 8) and of
    # the large 3D configuration (64^3, N_tau 64, beta 4), for timing beside the engine
    "2d_x128_y128_t128": (dict(XSIZE=128, YSIZE=128, ZSIZE=1, TAUSIZE=128, EPS=0.0625), 0.0, -1.5),
    "3d_x64_y64_z64_t64": (dict(XSIZE=64, YSIZE=64, ZSIZE=64, TAUSIZE=64, EPS=0.0625), 0.0, -1.5),
    # ensemble runs: a line whose max/mean reduction has two blocks, so the reference's
    # atomicAdd of the block sums (Propagator_without_cutoff.cu:262-263) is order-free
    # and its trajectories are reproducible run to run
    "1d_x32_t16_ens": (dict(XSIZE=32, YSIZE=1, ZSIZE=1, TAUSIZE=16, BLOCKSIZEX=32, BLOCKSIZETAU=8, EPS=0.05),
                       0.0, -1.5),
}


def macros(name: str) -> dict:
    m = dict(BASE_MACROS)
    m.update(CONFIGS[name][0])
    return m


def reference_dir() -> str:
    return os.environ.get("CLV_REFERENCE_DIR", os.path.join(os.path.dirname(REPO), "reference"))


def cubin_path(name: str) -> str:
    return os.path.join(OUT, f"refgpu_{name}.cubin")


def have_cubin(name: str) -> bool:
    return os.path.exists(cubin_path(name))


def build_cubins(force: bool = False) -> list[str]:
    """Compile the cubins that are missing (needs the reference sources)."""
    ref = reference_dir()
    if not os.path.isdir(ref):
        return []
    env = dict(os.environ, CLV_REFERENCE_DIR=ref)
    script = os.path.join(HERE, "ref_gpu_build.sh")
    kernels = os.path.join(HERE, "ref_gpu_kernels.cu")
    todo = [n for n in CONFIGS
            if force or not have_cubin(n) or os.path.getmtime(cubin_path(n)) < os.path.getmtime(kernels)]

    def one(n):
        subprocess.run([script, cubin_path(n)] + [f"{k}={v}" for k, v in macros(n).items()],
                       check=True, env=env)
        return n

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(todo), os.cpu_count() or 4))) as ex:
        return list(ex.map(one, todo))


def build_runner() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "libref_gpu.so"], check=True)
    return LIB_PATH


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        cp = np.ctypeslib.ndpointer(dtype=np.complex128, flags="C_CONTIGUOUS")
        L.refgpu_last_error.restype = C.c_char_p
        L.refgpu_create.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double),
                                    C.c_ulonglong, C.c_int, C.POINTER(vp)]
        L.refgpu_destroy.argtypes = [vp]
        L.refgpu_set_fields.argtypes = [vp, cp, cp]
        L.refgpu_get_fields.argtypes = [vp, cp, cp]
        L.refgpu_set_mean_field.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double]
        L.refgpu_propagate.argtypes = [vp, C.c_double, C.c_double, vp, C.POINTER(C.c_double)]
        L.refgpu_time.argtypes = [vp, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_float),
                                  C.POINTER(C.c_double)]
        L.refgpu_observables.argtypes = [vp, dp, dp]
        _lib = L
    return _lib


class RefGpuError(RuntimeError):
    pass


class RefGpu:
    """One reference chain on the GPU: its fields, scratch lattices, cuFFT plan and
    cuRAND generator (seeded like Propagator's constructor)."""

    def __init__(self, name: str, seed: int = 7342951900870119, device: int = 0):
        m = macros(name)
        self.name = name
        self.P, self.MU = CONFIGS[name][1], CONFIGS[name][2]
        self.dims = (int(m["XSIZE"]), int(m["YSIZE"]), int(m["ZSIZE"]), int(m["TAUSIZE"]), int(m["COMPONENTS"]))
        X, Y, Z, T, Cn = self.dims
        self.shape = (Cn, T, X, Y, Z)
        self.noise_shape = (Cn, X, Y, Z, T, 2)
        self.macros = m
        L = lib()
        dims = (C.c_int * 5)(*self.dims)
        blocks = (C.c_int * 5)(*(int(m[k]) for k in ("BLOCKSIZE", "BLOCKSIZEX", "BLOCKSIZEY", "BLOCKSIZEZ",
                                                       "BLOCKSIZETAU")))
        consts = (C.c_double * 3)(float(m["EPS"]), float(m["a_x"]), float(m["DT"]))
        h = C.c_void_p()
        if not have_cubin(name):
            raise RefGpuError(f"no cubin for {name}: build it with oracle/refgpu.py where the reference sources are")
        self._check(L.refgpu_create(cubin_path(name).encode(), dims, blocks, consts, seed, device, C.byref(h)))
        self.h = h

    @staticmethod
    def _check(rc):
        if rc != 0:
            raise RefGpuError(lib().refgpu_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            lib().refgpu_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_fields(self, psi, psic):
        psi = np.ascontiguousarray(np.asarray(psi, np.complex128).reshape(self.shape))
        psic = np.ascontiguousarray(np.asarray(psic, np.complex128).reshape(self.shape))
        self._check(lib().refgpu_set_fields(self.h, psi, psic))

    def get_fields(self):
        psi = np.empty(self.shape, np.complex128)
        psic = np.empty(self.shape, np.complex128)
        self._check(lib().refgpu_get_fields(self.h, psi, psic))
        return psi, psic

    def set_mean_field(self, re=0.0, im=0.0):
        self._check(lib().refgpu_set_mean_field(self.h, re, im, self.P, self.MU))

    def propagate(self, normals=None):
        """One step; normals: unit normals of shape (C, X, Y, Z, T, 2) or None for cuRAND.
        Returns (dt, max, mean) of the step."""
        out = (C.c_double * 3)()
        if normals is None:
            ptr = None
        else:
            buf = np.ascontiguousarray(np.asarray(normals, np.float64).reshape(self.noise_shape))
            ptr = buf.ctypes.data_as(C.c_void_p)
        self._check(lib().refgpu_propagate(self.h, self.P, self.MU, ptr, out))
        return out[0], out[1], out[2]

    def time(self, nsteps: int):
        """(CUDA-event ms, wall ms) of nsteps propagate calls with cuRAND noise."""
        ms = C.c_float()
        wall = C.c_double()
        self._check(lib().refgpu_time(self.h, nsteps, self.P, self.MU, C.byref(ms), C.byref(wall)))
        return float(ms.value), float(wall.value)

    def observables(self):
        """(n[5], F[3, V]) of Observables::evaluate for the current fields (per call sums)."""
        X, Y, Z, T, _ = self.dims
        n = np.zeros(5)
        F = np.zeros(3 * X * Y * Z)
        self._check(lib().refgpu_observables(self.h, n, F))
        return n, F.reshape(3, X * Y * Z)


if __name__ == "__main__":
    print(build_cubins(force="--force" in sys.argv))

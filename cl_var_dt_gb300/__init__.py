"""cl_var_dt_gb300 -- GB300-native (sm_103a) complex-Langevin lattice engine.

The engine is a CUDA library (``libclv.so``) behind the C ABI of
``include/clv.h``; this package holds its sources (``csrc/``), the in-tree
build, a ctypes binding (``Engine``), the secant mu-tuning driver (``secant``)
and the rank sharding helpers (``dist``).  The host-side mirror of the
reference's ComplexLattice / Propagator / Observables / SaveResults interface is
the C++ header ``include/clv_compat.hpp``.
"""
from ._native import (  # noqa: F401
    ChainParams, ClvError, Engine, lib, measure_peaks,
    MODEL_REF4, MODEL_SPIN1, KIN_REF_LINEAR_PX, KIN_EXP, DT_REF_MEANMAX, DT_K_OVER_MAX,
    NOISE_EXTERNAL, NOISE_PHILOX, PREC_F64, PREC_F32, HOST, DEVICE, C64, ASYNC,
    FLAG_NONFINITE, FLAG_DT_CLAMPED_LOW, FLAG_DT_CLAMPED_HIGH,
)
from ._build import build  # noqa: F401

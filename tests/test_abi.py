"""The C ABI library builds, loads without a GPU, and exports every entry point
include/clv.h declares; the drop-in main program is built beside it."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import REPO


@pytest.fixture(scope="module")
def built():
    import cl_var_dt_gb300 as clv
    clv.build()
    return clv


def declared():
    src = open(os.path.join(REPO, "include", "clv.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(clv_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_binding_list(built):
    assert declared() == sorted(built._native.EXPORTED)


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(built._native.LIB_PATH)
    for name in declared():
        assert hasattr(lib, name), name
    nm = subprocess.run(["nm", "-D", "--defined-only", built._native.LIB_PATH], capture_output=True,
                        text=True).stdout
    exported = set(re.findall(r" T (clv_[a-z0-9_]+)", nm))
    assert set(declared()) <= exported


def test_host_only_entry_points_work_without_a_gpu(built):
    lib = built.lib()
    assert lib.clv_version() == 1
    assert lib.clv_status_string(3).decode() == "non-finite drift"
    c = built._native.ChainParamsC()
    lib.clv_default_chain_params(ctypes.byref(c))
    assert (c.nx, c.nt, c.eps, c.DT, c.G) == (256, 32, 0.01, 0.002, 0.1)


def test_invalid_config_is_rejected_before_touching_the_device(built):
    # nx = 1 is rejected by the argument checks, which run before any CUDA call
    with pytest.raises(built.ClvError) as e:
        built.Engine(built.ChainParams(nx=1, nt=4), model=built.MODEL_SPIN1)
    assert e.value.status == built._native.ERR_ARG


def test_drop_in_main_is_built(built):
    assert os.access(os.path.join(REPO, "cl_var_dt_gb300", "clv_main"), os.X_OK)

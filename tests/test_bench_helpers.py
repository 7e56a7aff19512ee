"""The benchmark's workload definitions and helpers on the CPU: shapes and
couplings of each configuration, the imaginary-time override, the CPU model
string, and the peak file reader."""
import json
import os
import sys

import pytest

from conftest import REPO

sys.path.insert(0, REPO)
import bench  # noqa: E402


def test_batched_workload_shapes():
    W = bench.workload("batched")
    assert len(W["chains"]) == 256
    c0, c255 = W["chains"][0], W["chains"][-1]
    assert (c0["nx"], c0["ny"], c0["nz"], c0["nt"]) == (256, 1, 1, 128)
    assert c0["eps"] * c0["nt"] == pytest.approx(6.0)
    assert c0["mu"] == pytest.approx(0.2) and c255["mu"] == pytest.approx(2.0)
    assert all(-0.2 <= c["c1"] <= 0.2 for c in W["chains"])
    assert bench.workload("batched", 8)["chains"].__len__() == 8


def test_other_workloads():
    d2 = bench.workload("2d")["chains"][0]
    assert (d2["nx"], d2["ny"], d2["nt"]) == (128, 128, 128) and d2["eps"] * d2["nt"] == pytest.approx(8)
    d3 = bench.workload("3d")["chains"][0]
    assert (d3["nx"], d3["ny"], d3["nz"], d3["nt"]) == (64, 64, 64, 64)
    U = bench.workload("uneven", 16)
    assert len(U["chains"]) == len(U["targets"]) == 16
    for c, t in zip(U["chains"], U["targets"]):
        assert c["nx"] == c["ny"] and c["nx"] in (32, 64, 96, 128) and c["nt"] in (32, 64, 128, 256)
        assert 0.5 <= t <= 2.0 and c["mu"] == pytest.approx(c["c0"] * t)


def test_n_tau_override_keeps_beta():
    W = bench.with_n_tau(bench.workload("3d"), 32)
    c = W["chains"][0]
    assert c["nt"] == 32 and c["eps"] * c["nt"] == pytest.approx(4.0)
    assert W["name"].endswith("-ntau32")
    assert bench.with_n_tau(bench.workload("2d"), None)["chains"][0]["nt"] == 128


def test_cpu_model_and_peaks():
    assert isinstance(bench.cpu_model(), str) and bench.cpu_model()
    peak, kind = bench.peaks()
    if os.path.exists(os.path.join(REPO, "MEASURED_PEAKS.json")):
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            assert peak == float(json.load(f)["hbm_gbs"]) and kind == "measured"
    else:
        assert kind == "fallback"


def test_roofline_credits_algorithmic_bytes_to_the_dominant_kernel():
    """frac uses the 96 B of a spin-1 site-update over the dominant kernel's time;
    kernel_frac the bytes that kernel itself moves (a tiled step: 144 B)."""
    names = ["plane01_n128", "tiled_step", "tiled_redo"]
    r = bench.roofline(names, [0.1, 0.2, 0.01], sites=1_000_000, step_ms=0.31, ncomp=3, peak_gbs=1000.0)
    assert r["kernel"] == "tiled_step"
    assert r["algorithmic_bytes_per_site_update"] == 96 and r["kernel_bytes_per_site_update"] == 144
    assert abs(r["achieved"] - 96 * 1e6 / 0.2e-3 / 1e9) < 1e-9
    assert abs(r["kernel_frac"] / r["frac"] - 1.5) < 1e-12
    assert abs(r["step_frac"] - 96 * 1e6 / 0.31e-3 / 1e9 / 1000.0) < 1e-12

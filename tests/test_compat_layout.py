"""The engine's output writer (include/clv_compat.hpp, SaveResultsT) against
the files the reference's own SaveResults.cu writes for the same observable
values (tests/golden/saveresults, made by tests/golden/make_golden.py), byte
for byte: directory names, Parameters.txt, the shared Skalars.txt and the
F_x/F_y/F_z profiles.  Also the Parameters.h and params.txt readers."""
import os
import shutil
import subprocess

import pytest

from conftest import REPO

GOLD = os.path.join(REPO, "tests", "golden", "saveresults")
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("bin") / "save_harness")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(REPO, "include"), "-I", CUDA_INC,
                    os.path.join(REPO, "tests", "compat_save_harness.cpp"), "-o", exe], check=True)
    return exe


def tree(root):
    out = {}
    for d, _, files in os.walk(root):
        for f in files:
            p = os.path.join(d, f)
            with open(p, "rb") as fh:
                out[os.path.relpath(p, root)] = fh.read()
    return out


@pytest.mark.parametrize("case", sorted(os.listdir(GOLD)))
def test_writer_matches_reference_files(harness, tmp_path, case):
    gdir = os.path.join(GOLD, case)
    mu, P, seed = open(os.path.join(gdir, "args.txt")).read().split()
    r = subprocess.run([harness, str(tmp_path), os.path.join(gdir, "Parameters.h"), mu, P, seed],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = tree(os.path.join(tmp_path, "DATA"))
    want = tree(os.path.join(gdir, "DATA"))
    assert sorted(got) == sorted(want)
    for k in want:
        assert got[k] == want[k], k
    runs = [d for d in os.listdir(os.path.join(tmp_path, "DATA", os.listdir(os.path.join(tmp_path, "DATA"))[0]))
            if d.startswith("Run")]
    assert runs == ["Run1"]


def test_second_run_gets_next_directory(harness, tmp_path):
    gdir = os.path.join(GOLD, "ref_params")
    mu, P, seed = open(os.path.join(gdir, "args.txt")).read().split()
    for _ in range(2):
        r = subprocess.run([harness, str(tmp_path), os.path.join(gdir, "Parameters.h"), mu, P, seed],
                           capture_output=True, text=True)
        assert r.returncode == 0
    base = os.path.join(tmp_path, "DATA", "BoseCL_Sim_mu_-1.5_P_0")
    assert sorted(d for d in os.listdir(base) if d.startswith("Run")) == ["Run1", "Run2"]
    assert os.path.isdir(os.path.join(base, "Run2", "rawdata"))
    # Skalars.txt is shared by the runs of one (mu, P): 2 snapshots per run appended
    with open(os.path.join(base, "Skalars.txt")) as f:
        assert len(f.read().splitlines()) == 4

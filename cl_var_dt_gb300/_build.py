"""In-tree build of the native engine (libclv.so) for sm_103a.

Each CUDA translation unit is compiled in parallel with one -gencode, then
linked into ``cl_var_dt_gb300/libclv.so``.  No cmake, no torch extension
machinery: the library exposes only the C ABI of ``include/clv.h``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libclv.so")
SOURCES = ["clv_engine.cu", "k_kinetic.cu", "k_step.cu", "k_obs.cu", "k_obs_noalloc.cu", "k_peaks.cu", "k_fused.cu",
           "k_axis.cu", "k_plane.cu", "k_tiled.cu", "k_loop.cu",
           "k_fused_f32_ref4.cu", "k_fused_f32_spin1.cu", "k_fused_f64_ref4.cu", "k_fused_f64_spin1.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = os.path.join(cuda, "bin", "nvcc")
    return exe if os.path.exists(exe) else (shutil.which("nvcc") or "nvcc")


def _flags(verbose_ptxas: bool) -> list[str]:
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(REPO, "include")]
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    deps.append(os.path.join(REPO, "include", "clv.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose_ptxas: bool = False, quiet: bool = True) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    jobs = []
    objs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, src):
            jobs.append([cc, *_flags(verbose_ptxas), "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for log in ex.map(run, jobs):
            if log and (verbose_ptxas or not quiet):
                sys.stderr.write(log)
    if jobs or not os.path.exists(LIB):
        link = [cc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(link)}\n{r.stdout}\n{r.stderr}")
    build_main()
    return LIB


MAIN = os.path.join(PKG, "clv_main")


def build_main() -> str:
    """The drop-in replacement of the reference's main program (csrc/clv_main.cpp)."""
    src = os.path.join(CSRC, "clv_main.cpp")
    hdr = os.path.join(REPO, "include", "clv_compat.hpp")
    if os.path.exists(MAIN) and os.path.getmtime(MAIN) > max(os.path.getmtime(src), os.path.getmtime(hdr),
                                                             os.path.getmtime(LIB)):
        return MAIN
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"), "-I", os.path.join(cuda, "include"),
           src, "-o", MAIN, "-L", PKG, "-lclv", "-L", os.path.join(cuda, "lib64"), "-lcudart",
           "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build of clv_main failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return MAIN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv, quiet=False))

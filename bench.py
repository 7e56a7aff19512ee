"""Throughput benchmark: site-updates/s (chains x sites x steps per second).

Default workload (N=1): one chain of the spin-1 model on a 2D 128x128 lattice
with N_tau = 128, beta = 8, c0 = 0.3, c1 = -0.05, q = 0.02, mu = 0.8, step rule
dt = min(1e-3, 0.05 / max|drift|), in-register Philox noise, FP32-mixed
precision (FP32 fields and FFTs; FP64 step-rule reduction, Langevin time and
observable sums).  The same workload in plain FP64 is timed beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one Langevin step of the whole batch.  Timing: per-step CUDA events
on the engine's stream, an L2 flush (a 256 MB write) between timed steps,
max over ranks.  Under torchrun each rank runs an independent replica
(chains do not interact), so scaling is weak.

--impl reference times the CPU restatement of the same update (the reference
has no CPU path of its own; its GPU build is not shipped to the benchmark host)
on all host threads, each step a bounded sample of the workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

WORKLOAD = dict(nx=128, ny=128, nz=1, nt=128, beta=8.0, c0=0.3, c1=-0.05, q=0.02, mu=0.8,
                K=0.05, dt_max=1e-3, seed=20261203)
WORKLOAD_NAME = "spin1-2d-128x128-ntau128-beta8"
OBS_EVERY = 20          # observable cadence of the workload
METRIC = "site-updates/s"


def peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(
        os.environ.get("LOCAL_RANK", 0))


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def chain_params(clv, rank):
    w = WORKLOAD
    return clv.ChainParams(nx=w["nx"], ny=w["ny"], nz=w["nz"], nt=w["nt"], eps=w["beta"] / w["nt"],
                           mu=w["mu"], c0=w["c0"], c1=w["c1"], q=w["q"], K=w["K"], dt_max=w["dt_max"],
                           seed=w["seed"] + rank)


def time_steps(torch, eng, flush, steps, warmup):
    """Per-step device time (ms) with an L2 flush before every timed step."""
    for _ in range(warmup):
        flush.zero_()
        eng.step(1)
    torch.cuda.synchronize()
    evs = []
    for _ in range(steps):
        flush.zero_()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        eng.step(1)
        b.record()
        evs.append((a, b))
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in evs]


def phase_times(torch, eng, flush, reps=5):
    """Device ms of each launch of a step, averaged over reps (flushed L2)."""
    acc = None
    for _ in range(reps):
        flush.zero_()
        torch.cuda.synchronize()
        ph = eng.step_timed()
        acc = ph if acc is None else [x + y for x, y in zip(acc, ph)]
    return [x / reps for x in acc]


def run_ours(args):
    import numpy as np
    import torch
    import cl_var_dt_gb300 as clv

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    clv.build()
    sites = WORKLOAD["nx"] * WORKLOAD["ny"] * WORKLOAD["nz"] * WORKLOAD["nt"]
    ncomp = 3
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)  # flushes, events and the engine share one stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    peak_gbs, peak_kind = peaks()

    def make(prec):
        e = clv.Engine(chain_params(clv, rank), model=clv.MODEL_SPIN1, precision=prec, device=local)
        e.set_stream(stream.cuda_stream)
        e.init_spin1(np.sqrt(1 / 3), 0.01)
        return e

    results = {}
    clocks = Clocks(local)
    for prec, name, steps in ((clv.PREC_F32, "f32", args.steps),
                              (clv.PREC_F64, "f64", max(3, args.steps // 4))):
        eng = make(prec)
        if name == "f32":
            clocks.start()
        if world > 1:
            torch.distributed.barrier()
        ms = time_steps(torch, eng, flush, steps, args.warmup)
        if name == "f32":
            clk = clocks.stop()
        tot = sum(ms)
        if world > 1:
            t = torch.tensor([tot], device="cuda", dtype=torch.float64)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            tot = float(t.item())
        ph = phase_times(torch, eng, flush)
        info = eng.step_info()
        results[name] = dict(ms=tot, steps=steps, phases=ph, launches=len(ph),
                             dt=float(info["dt"][0]), max=float(info["max"][0]),
                             flags=int(eng.chain_flags()[0]))
        if name == "f32":
            results["f32"]["engine"] = eng
        else:
            eng.close()

    # end-to-end through the C ABI with pinned host buffers: fields in, a block of
    # OBS_EVERY steps, one observable evaluation, fields and the sample out.
    eng = results["f32"].pop("engine")
    shape = eng.shape(0)
    hp = torch.empty(shape + (2,), dtype=torch.float64, pin_memory=True)
    hc = torch.empty(shape + (2,), dtype=torch.float64, pin_memory=True)
    psi_h = hp.numpy().view(np.complex128).reshape(shape)
    psic_h = hc.numpy().view(np.complex128).reshape(shape)
    a, b = eng.get_fields(0)
    psi_h[...] = a
    psic_h[...] = b
    import ctypes as C
    L = clv.lib()
    e2e_blocks = max(2, args.steps // OBS_EVERY)

    def e2e_block():
        clv._native.check(L.clv_set_fields(eng.h, 0, C.c_void_p(hp.data_ptr()), C.c_void_p(hc.data_ptr()), clv.HOST))
        clv._native.check(L.clv_step(eng.h, OBS_EVERY))
        clv._native.check(L.clv_evaluate(eng.h))
        clv._native.check(L.clv_get_fields(eng.h, 0, C.c_void_p(hp.data_ptr()), C.c_void_p(hc.data_ptr()), clv.HOST))
        eng.spin1_samples(0)

    for _ in range(max(1, args.warmup // 2)):
        e2e_block()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_blocks):
        e2e_block()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    eng.close()

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(budget_s=args.cpu_seconds)

    if rank == 0:
        f32, f64 = results["f32"], results["f64"]
        value = world * sites * f32["steps"] / (f32["ms"] / 1e3)
        v64 = world * sites * f64["steps"] / (f64["ms"] / 1e3)
        # dominant launch and its algorithmic bytes: a line-filter pass reads and
        # writes both fields once (4 C complex64 per site); the drift reads psi,
        # psibar, kin, kinbar and writes two drifts (6 C); the update reads psi,
        # psibar and both drifts and writes psi, psibar (6 C).
        names = [f"kinetic_axis{i}" for i in range(f32["launches"] - 2)] + ["drift", "update"]
        bytes_per_site = {n: (4 if n.startswith("kinetic") else 6) * ncomp * 8 for n in names}
        i_dom = max(range(len(names)), key=lambda i: f32["phases"][i])
        dom = names[i_dom]
        achieved = bytes_per_site[dom] * sites / (f32["phases"][i_dom] / 1e3) / 1e9
        step_bytes = 4 * ncomp * 8 * sites  # B_alg of a whole step (96 B per site-update)
        step_gbs = step_bytes / (f32["ms"] / f32["steps"] / 1e3) / 1e9
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "site-updates/s",
            "n_gpus": world,
            "steps": f32["steps"],
            "warmup": args.warmup,
            "ms_per_step": f32["ms"] / f32["steps"],
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic (spin-1 start sqrt(1/3) + N(0, 0.01) from Philox seed 20261203)",
            "config": {"workload": WORKLOAD_NAME, "chains": world, "lattice": "128x128", "n_tau": 128,
                       "components": ncomp, "precision": "FP32 fields/FFT, FP64 reductions",
                       "noise": "philox4x32-10 in-register", "l2": "flushed (256 MB write) before every timed step",
                       "parallelism": f"replicas x{world}"},
            "fp64_plain": {"value": v64, "unit": "site-updates/s", "steps": f64["steps"],
                           "ms_per_step": f64["ms"] / f64["steps"],
                           "f32_over_f64": value / v64},
            "step_hbm_gbs": step_gbs,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak_gbs,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak_gbs,
                         "traffic": None,
                         "step_frac": step_gbs / peak_gbs,
                         "phases_ms": dict(zip(names, [round(x, 5) for x in f32["phases"]]))},
            "e2e": {"value": world * sites * OBS_EVERY * e2e_blocks / e2e_s, "unit": "site-updates/s",
                    "h2d_bytes_per_step": 2 * int(np.prod(shape)) * 16,
                    "d2h_bytes_per_step": 2 * int(np.prod(shape)) * 16 + 8 * 8,
                    "inner_steps": OBS_EVERY,
                    "call": "clv_set_fields(host) + clv_step(20) + clv_evaluate + clv_get_fields(host) + samples"},
            "gpu_launches": f32["launches"] * f32["steps"],
            "clocks": clk,
            "dt": f32["dt"], "max_drift": f32["max"], "flags": f32["flags"],
        }
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def cpu_baseline(budget_s=15.0, nt_sample=32):
    """The oracle (FP64 C/OpenMP restatement) on the host cores, bounded sample."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle
    pyoracle.build()
    w = WORKLOAD
    p = pyoracle.spin1_params(nx=w["nx"], ny=w["ny"], nz=w["nz"], nt=nt_sample, eps=w["beta"] / w["nt"],
                              mu=w["mu"], c0=w["c0"], c1=w["c1"], q=w["q"], Kc=w["K"], dt_max=w["dt_max"])
    psi, psic = pyoracle.spin1_init(p, w["seed"], 0)
    psi, psic, *_ = pyoracle.step(p, psi, psic, seed=w["seed"])  # warm
    n, t0 = 0, time.perf_counter()
    while True:
        psi, psic, *_ = pyoracle.step(p, psi, psic, seed=w["seed"], step_index=n + 1)
        n += 1
        el = time.perf_counter() - t0
        if el >= budget_s or n >= 200:
            break
    sites = w["nx"] * w["ny"] * w["nz"] * nt_sample
    return {"value": sites * n / el, "unit": "site-updates/s", "cores": pyoracle.num_threads(),
            "kind": "port", "sample": f"{n} FP64 steps of 128x128 sites x {nt_sample} tau-slices "
                                      f"(per-site work as the full 128-slice lattice), {el:.1f} s"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle
    pyoracle.build()
    w = WORKLOAD
    nt_sample = 16
    p = pyoracle.spin1_params(nx=w["nx"], ny=w["ny"], nz=w["nz"], nt=nt_sample, eps=w["beta"] / w["nt"],
                              mu=w["mu"], c0=w["c0"], c1=w["c1"], q=w["q"], Kc=w["K"], dt_max=w["dt_max"])
    psi, psic = pyoracle.spin1_init(p, w["seed"], 0)
    for k in range(args.warmup):
        psi, psic, *_ = pyoracle.step(p, psi, psic, seed=w["seed"], step_index=k)
    t0 = time.perf_counter()
    for k in range(args.steps):
        psi, psic, *_ = pyoracle.step(p, psi, psic, seed=w["seed"], step_index=args.warmup + k)
    el = time.perf_counter() - t0
    sites = w["nx"] * w["ny"] * w["nz"] * nt_sample
    value = sites * args.steps / el
    sample = (f"each step: FP64 CPU restatement on 128x128 sites x {nt_sample} of the 128 tau-slices "
              "(per-site work of the full workload)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "site-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": WORKLOAD_NAME, "chains": 1, "lattice": "128x128",
                                        "n_tau": 128, "components": 3},
        "cpu_baseline": {"value": value, "unit": "site-updates/s", "cores": pyoracle.num_threads(),
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "site-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

"""Throughput benchmark: site-updates/s (chains x sites x steps per second).

Default workload (N=1), "batched": 256 independent chains of the spin-1 model,
each a 1D lattice Nx = 256 with N_tau = 128 and beta = 6; mu linearly spaced on
[0.2, 2.0], c0 = 0.5, c1 uniform on [-0.2, 0.2] per chain (drawn from seed
20261203), q = 0.05; step rule dt = min(1e-3, 0.05 / max|drift|) per chain;
in-register Philox noise; FP32-mixed precision (FP32 fields and FFTs; FP64
step-rule reduction, Langevin time and observable sums); steps replayed from a
captured CUDA graph.  The same batch in plain FP64 is timed beside it.
"--workload 2d" selects one 2D 128x128 chain with N_tau = 128, beta = 8.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one Langevin step of the whole batch.  Timing: per-step CUDA events
on the engine's stream, an L2 flush (a 256 MB write) before every timed step,
max over ranks.  Under torchrun each rank runs an independent replica batch
(chains do not interact), so scaling is weak.

--impl reference times the CPU restatement of the same update (the reference
has no CPU path of its own; its GPU program cannot be shipped to the benchmark
host) on all host threads, each step a bounded sample of the workload.
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

SEED = 20261203
METRIC = "site-updates/s"
# FP64 flops of one site-update of the batched workload's FP64 step (2 DFMA + DADD + DMUL,
# ncu counters of fused_step_kernel<double, SPIN1, 1, 256, FAST> on 16 chains:
# profiles/fp64_step_spin1_batched_1d256.md)
FP64_FLOPS_PER_SITE_UPDATE = 1024.6


def workload(name, nchains=None):
    """Chains of a workload as dicts of ChainParams fields (nchains: smaller batch for profiling)."""
    import numpy as np
    if name == "batched":
        n = nchains or 256
        rng = np.random.default_rng(SEED)
        c1 = rng.uniform(-0.2, 0.2, n)
        mu = np.linspace(0.2, 2.0, n)
        chains = [dict(nx=256, ny=1, nz=1, nt=128, eps=6.0 / 128, mu=float(mu[i]), c0=0.5,
                       c1=float(c1[i]), q=0.05, K=0.05, dt_max=1e-3, seed=SEED) for i in range(n)]
        return dict(name=f"spin1-batched-{n}x(1d-256)-ntau128-beta6", chains=chains, obs_every=10,
                    lattice=f"{n} chains x 1D 256", n_tau=128)
    if name == "2d":
        chains = [dict(nx=128, ny=128, nz=1, nt=128, eps=8.0 / 128, mu=0.8, c0=0.3, c1=-0.05,
                       q=0.02, K=0.05, dt_max=1e-3, seed=SEED)]
        return dict(name="spin1-2d-128x128-ntau128-beta8", chains=chains, obs_every=20,
                    lattice="1 chain x 2D 128x128", n_tau=128)
    if name == "3d":
        chains = [dict(nx=64, ny=64, nz=64, nt=64, eps=4.0 / 64, mu=0.5, c0=0.2, c1=-0.02,
                       q=0.01, K=0.05, dt_max=1e-3, seed=SEED)]
        return dict(name="spin1-3d-64x64x64-ntau64-beta4", chains=chains, obs_every=20,
                    lattice="1 chain x 3D 64x64x64", n_tau=64)
    if name == "uneven":
        # 2D chains of uneven sides and imaginary-time extents drawn from the seed;
        # mu starts at c0 * n for a target density n (a secant driver would refine it)
        n = nchains or 64
        rng = np.random.default_rng(SEED)
        side = rng.choice([32, 64, 96, 128], n)
        nt = rng.choice([32, 64, 128, 256], n)
        c0 = rng.uniform(0.1, 0.6, n)
        c1 = rng.uniform(-0.2, 0.1, n)
        q = rng.uniform(0.0, 0.1, n)
        target = rng.uniform(0.5, 2.0, n)
        chains = [dict(nx=int(side[i]), ny=int(side[i]), nz=1, nt=int(nt[i]), eps=0.05,
                       mu=float(c0[i] * target[i]), c0=float(c0[i]), c1=float(c1[i]), q=float(q[i]),
                       K=0.05, dt_max=1e-3, seed=SEED) for i in range(n)]
        return dict(name=f"spin1-uneven-{n}x(2d-32..128)-ntau32..256-eps0.05", chains=chains,
                    obs_every=10, lattice=f"{n} chains x 2D, side in {{32,64,96,128}}",
                    n_tau="32..256", targets=[float(t) for t in target])
    raise SystemExit(f"unknown workload {name}")


def with_n_tau(W, n_tau):
    """The workload with every chain's imaginary-time extent set to n_tau (beta kept)."""
    if not n_tau:
        return W
    for c in W["chains"]:
        c["eps"] = c["eps"] * c["nt"] / n_tau
        c["nt"] = n_tau
    W["name"] += f"-ntau{n_tau}"
    W["n_tau"] = n_tau
    return W


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.proc, self.f = index, None, None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.5)  # the sampler is running when the timed region begins
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


def time_steps(torch, eng, flush, steps, warmup):
    """Per-step device time (ms); an L2 flush precedes every timed step."""
    eng.step(max(2, warmup))  # also captures the step graphs of both buffer parities
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


def roofline(names, phases, sites, step_ms, ncomp, peak_gbs):
    """Roofline of a step's dominant kernel.  achieved/frac: the algorithmic bytes of
    a site-update (read psi, psibar once, write them once: 4 C sizeof(complex64) =
    96 B for spin-1) over the dominant kernel's time -- what the step must move per
    unit of that kernel's time.  kernel_*: the bytes that kernel itself must move
    (filters: both fields in and out; tiled step: psi, psibar, kin, kinbar in, psi,
    psibar out), which credits its own traffic."""
    alg = 4 * ncomp * 8
    own = {}
    for n in names:
        if n.endswith("_redo"):
            own[n] = 0
        elif (n in ("fused_step", "fused_reduce", "fused_apply") or n.startswith("axis") or n.startswith("plane")
              or n.startswith("kinetic")):
            own[n] = alg  # (the reduce pass reads only: a bound, not a count)
        else:
            own[n] = 6 * ncomp * 8
    i = max(range(len(names)), key=lambda k: phases[k])
    t = phases[i] / 1e3
    achieved = alg * sites / t / 1e9
    kernel = own[names[i]] * sites / t / 1e9
    step = alg * sites / (step_ms / 1e3) / 1e9
    return {"bound": "hbm", "kernel": names[i], "achieved": achieved, "peak": peak_gbs, "unit": "GB/s",
            "frac": achieved / peak_gbs, "algorithmic_bytes_per_site_update": alg,
            "kernel_bytes_per_site_update": own[names[i]], "kernel_achieved": kernel,
            "kernel_frac": kernel / peak_gbs, "step_achieved": step, "step_frac": step / peak_gbs,
            "phases_ms": dict(zip(names, [round(x, 5) for x in phases]))}


def extra_workload(torch, clv, name, args, stream, flush, peak_gbs, local):
    """FP32-mixed throughput of another configuration's workload (after autotune),
    with its roofline: the 2D 128^2 precision-comparison shape, the 3D 64^3 lattice
    and the uneven 2D batch."""
    import numpy as np
    W = workload(name)
    chains = [clv.ChainParams(**c) for c in W["chains"]]
    sites = sum(c.nx * c.ny * c.nz * c.nt for c in chains)
    with clv.Engine(chains, model=clv.MODEL_SPIN1, precision=clv.PREC_F32, device=local) as e:
        e.set_stream(stream.cuda_stream)
        e.init_spin1(np.sqrt(1 / 3), 0.01)
        tuned = e.autotune(3).splitlines()[-1] if not args.no_autotune else "off"
        steps = max(10, args.steps // 2)
        ms = time_steps(torch, e, flush, steps, args.warmup)
        ph = phase_times(torch, e, flush)
        path, names = e.plan()
        flags = int(np.bitwise_or.reduce(e.chain_flags()))
    step_ms = sum(ms) / steps
    return {"workload": W["name"], "value": sites / (step_ms / 1e3), "unit": "site-updates/s",
            "ms_per_step": step_ms, "steps": steps, "plan": f"{path}; autotune {tuned}", "flags": flags,
            "roofline": roofline(names, ph, sites, step_ms, 3, peak_gbs)}


def run_ours(args):
    import ctypes as C
    import numpy as np
    import torch
    import cl_var_dt_gb300 as clv

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    clv.build()
    W = with_n_tau(workload(args.workload, args.chains), args.n_tau)
    chains = [clv.ChainParams(**{**c, "seed": c["seed"] + 7919 * rank}) for c in W["chains"]]
    sites = sum(c.nx * c.ny * c.nz * c.nt for c in chains)
    ncomp = 3
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)  # flushes, events and the engine share one stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    peak_gbs, peak_kind = peaks()

    tune_reports = {}

    def make(prec):
        e = clv.Engine(chains, model=clv.MODEL_SPIN1, precision=prec, device=local)
        e.set_stream(stream.cuda_stream)
        e.init_spin1(np.sqrt(1 / 3), 0.01)
        if not args.no_autotune and prec == clv.PREC_F32:
            # setup, outside the timed region; the state is restored after the trials
            tune_reports[prec] = e.autotune(5).splitlines()[-1]
        return e

    res = {}
    clocks = Clocks(local)
    clk = None
    runs = [(clv.PREC_F32, "f32", args.steps)]
    if not args.skip_fp64:
        runs.append((clv.PREC_F64, "f64", max(3, args.steps // 4)))
    for prec, name, steps in runs:
        eng = make(prec)
        if world > 1:
            torch.distributed.barrier()
        if name == "f32":
            clocks.start()
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
        res[name] = dict(ms=tot, steps=steps, phases=ph, launches=len(ph), plan=eng.plan(),
                         dt_min=float(info["dt"].min()), max=float(info["max"].max()),
                         flags=int(np.bitwise_or.reduce(eng.chain_flags())))
        if name == "f32":
            res["f32"]["engine"] = eng
        else:
            eng.close()

    # the plain FP64 drop-in as main.cu runs it: one chain of the workload at a time
    single64 = None
    if not args.skip_fp64:
        e1 = clv.Engine(chains[:1], model=clv.MODEL_SPIN1, precision=clv.PREC_F64, device=local)
        e1.set_stream(stream.cuda_stream)
        e1.init_spin1(np.sqrt(1 / 3), 0.01)
        n1 = max(20, args.steps // 4)
        e1.step(3)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        e1.step(n1)
        b.record()
        torch.cuda.synchronize()
        ms1 = a.elapsed_time(b) / n1
        c0 = chains[0]
        single64 = {"value": c0.nx * c0.ny * c0.nz * c0.nt / (ms1 / 1e3), "unit": "site-updates/s",
                    "ms_per_step": ms1, "steps": n1, "chain": "the workload's first chain, FP64, graph replay"}
        e1.close()

    # end to end through the C ABI with pinned host buffers: every chain's fields in,
    # a block of obs_every steps, one observable evaluation, fields and samples out.
    # Headline: complex64 host buffers (CLV_C64, the FP32 engine's own element type);
    # also measured with the reference's complex128 buffers.
    eng = res["f32"].pop("engine")
    total = sum(int(np.prod(eng.shape(i))) for i in range(len(chains)))
    L = clv.lib()
    chk = clv._native.check
    blocks = max(2, args.steps // W["obs_every"])

    def e2e_run(c64):
        dt = torch.float32 if c64 else torch.float64
        where = clv.HOST | (clv.C64 if c64 else 0)
        hp = torch.empty((total, 2), dtype=dt, pin_memory=True)
        hc = torch.empty((total, 2), dtype=dt, pin_memory=True)
        chk(L.clv_get_fields(eng.h, -1, C.c_void_p(hp.data_ptr()), C.c_void_p(hc.data_ptr()), where))

        def e2e_block():
            chk(L.clv_set_fields(eng.h, -1, C.c_void_p(hp.data_ptr()), C.c_void_p(hc.data_ptr()), where))
            chk(L.clv_step(eng.h, W["obs_every"]))
            chk(L.clv_evaluate(eng.h))
            chk(L.clv_get_fields(eng.h, -1, C.c_void_p(hp.data_ptr()), C.c_void_p(hc.data_ptr()), where))
            eng.spin1_samples(0)

        e2e_block()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(blocks):
            e2e_block()
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        if world > 1:
            t = torch.tensor([el], device="cuda", dtype=torch.float64)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            el = float(t.item())
        return el, (8 if c64 else 16) * 2 * total

    e2e_s, xfer = e2e_run(True)
    e2e128_s, xfer128 = e2e_run(False)
    eng.close()

    # pipelined end to end: the batch split over G engines on their own streams;
    # each block enqueues, per engine, asynchronous complex64 fields in, obs_every
    # steps, one evaluation and asynchronous fields out, then collects the samples,
    # so one group's host transfers overlap the other groups' kernels
    G = int(os.environ.get("CLV_BENCH_GROUPS", "8")) if len(chains) >= 16 else 1
    from cl_var_dt_gb300 import dist as cdist
    groups = [cdist.shard(chains, g, G) for g in range(G)]
    streams = [torch.cuda.Stream() for _ in range(G)]
    engs = []
    for g in range(G):
        eg = clv.Engine(groups[g], model=clv.MODEL_SPIN1, precision=clv.PREC_F32, device=local)
        eg.set_stream(streams[g].cuda_stream)
        eg.init_spin1(np.sqrt(1 / 3), 0.01)
        if not args.no_autotune:
            eg.autotune(3)
        engs.append(eg)

    def group_bufs(c64):
        # pinned host buffers of every group's fields: complex64 (the FP32 engine's own
        # element type) or complex128 (the reference's)
        out = []
        for g, eg in enumerate(engs):
            n_g = sum(int(np.prod(eg.shape(i))) for i in range(len(groups[g])))
            dtp = torch.float32 if c64 else torch.float64
            hp = torch.empty((n_g, 2), dtype=dtp, pin_memory=True)
            hc = torch.empty((n_g, 2), dtype=dtp, pin_memory=True)
            chk(L.clv_get_fields(eg.h, -1, C.c_void_p(hp.data_ptr()), C.c_void_p(hc.data_ptr()),
                                 clv.HOST | (clv.C64 if c64 else 0)))
            out.append((hp, hc))
        return out

    def enqueue(g, bufs, wa):
        eg, (hp, hc) = engs[g], bufs[g]
        chk(L.clv_set_fields(eg.h, -1, C.c_void_p(hp.data_ptr()), C.c_void_p(hc.data_ptr()), wa))
        chk(L.clv_step(eg.h, W["obs_every"]))
        chk(L.clv_evaluate(eg.h))
        chk(L.clv_get_fields(eg.h, -1, C.c_void_p(hp.data_ptr()), C.c_void_p(hc.data_ptr()), wa))

    def collect(g):
        chk(L.clv_synchronize(engs[g].h))
        engs[g].spin1_samples(0)

    def pipe_run(nblocks, bufs, wa):
        # each group runs its blocks back to back; the host collects a group's
        # result and enqueues its next block in turn, so the groups stay staggered
        for g in range(G):
            enqueue(g, bufs, wa)
        for b in range(nblocks):
            for g in range(G):
                collect(g)
                if b + 1 < nblocks:
                    enqueue(g, bufs, wa)

    def pipe_timed(c64):
        bufs = group_bufs(c64)
        wa = clv.HOST | clv.ASYNC | (clv.C64 if c64 else 0)
        pipe_run(1, bufs, wa)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pipe_run(blocks, bufs, wa)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        if world > 1:
            t = torch.tensor([el], device="cuda", dtype=torch.float64)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            el = float(t.item())
        return el

    pipe_s = pipe_timed(True)
    pipe128_s = pipe_timed(False)
    for eg in engs:
        eg.close()

    extras = {}
    if world == 1 and args.workload == "batched" and not args.no_extra_workloads:
        for name in ("2d", "3d", "uneven"):
            extras[name] = extra_workload(torch, clv, name, args, stream, flush, peak_gbs, local)
    single = None
    if world == 1 and args.workload == "batched" and not args.no_extra_workloads:
        single = single_chain_fp64_leg(torch, clv, local, stream)
    ref_gpu = None
    if rank == 0 and not args.no_reference_gpu:
        ref_gpu = reference_gpu_leg(torch, clv, local, stream)
    cpu = cpu_baseline(W, budget_s=args.cpu_seconds) if (rank == 0 and not args.no_cpu_baseline) else None
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    f32, f64 = res["f32"], res.get("f64")
    value = world * sites * f32["steps"] / (f32["ms"] / 1e3)
    v64 = world * sites * f64["steps"] / (f64["ms"] / 1e3) if f64 else None
    fp64_roof = None
    if f64:
        # the FP64 step is bound by the FP64 pipe: flops per site-update (ncu count) over the
        # device's DFMA rate measured here (clv_measure_peaks)
        fp64_peak, fp32_peak = clv.measure_peaks(local)
        ach = FP64_FLOPS_PER_SITE_UPDATE * v64 / world / 1e12
        fp64_roof = {"bound": "fp64", "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                     "frac": ach / fp64_peak, "flops_per_site_update": FP64_FLOPS_PER_SITE_UPDATE,
                     "peak_source": "measured (clv_measure_peaks: DFMA rate of this GPU)",
                     "fp32_fma_tflops": fp32_peak}
    nph = f32["launches"]
    path, names = f32["plan"]
    assert len(names) == nph, (names, nph)
    roof = roofline(names, f32["phases"], sites, f32["ms"] / f32["steps"], ncomp, peak_gbs)
    dom = roof["kernel"]
    prof = os.path.join(REPO, "profiles", "traffic.json")
    traffic = None
    try:
        with open(prof) as f:
            traffic = json.load(f).get(f"{args.workload}:{dom}")
    except Exception:
        pass
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
        "data": f"synthetic (spin-1 start sqrt(1/3) + N(0, 0.01) per field from Philox seed {SEED})",
        "config": {"workload": W["name"], "chains": len(chains) * world, "lattice": W["lattice"],
                   "n_tau": W["n_tau"], "components": ncomp,
                   "precision": "FP32 fields/FFT/drift, FP64 step rule, time and observable sums",
                   "noise": "philox4x32-10 in-register", "dt": "per chain, min(1e-3, 0.05/max|drift|)",
                   "l2": "flushed (256 MB write) before every timed step; state larger than L2",
                   "parallelism": f"replicas x{world}",
                   "plan": f"{path}; autotune {tune_reports.get(clv.PREC_F32, 'off')}"},
        "fp64_plain": ({"value": v64, "unit": "site-updates/s", "steps": f64["steps"],
                        "ms_per_step": f64["ms"] / f64["steps"], "f32_over_f64": value / v64,
                        "single_chain": single64, "f32_over_single_chain_f64":
                            (value / single64["value"]) if single64 else None,
                        "roofline": fp64_roof}
                       if f64 else None),
        "roofline": {**roof, "traffic": traffic,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind},
        "e2e": {"value": world * sites * W["obs_every"] * blocks / pipe_s, "unit": "site-updates/s",
                "h2d_bytes_per_step": xfer / W["obs_every"],
                "d2h_bytes_per_step": (xfer + 8 * 8 * G) / W["obs_every"],
                "inner_steps": W["obs_every"], "h2d_bytes_per_block": xfer,
                "call": f"{G} engines (chain groups) on their own streams, staggered; each block of each "
                        f"group: clv_set_fields(all, host complex64, async) + clv_step({W['obs_every']}) + "
                        "clv_evaluate + clv_get_fields(all, host complex64, async), then clv_synchronize + "
                        "samples before the group's next block",
                "sequential": {"value": world * sites * W["obs_every"] * blocks / e2e_s,
                               "call": "one engine, synchronous complex64 transfers"},
                "complex128": {"value": world * sites * W["obs_every"] * blocks / e2e128_s,
                               "h2d_bytes_per_step": xfer128 / W["obs_every"],
                               "d2h_bytes_per_step": (xfer128 + 8 * 8) / W["obs_every"],
                               "call": "one engine, synchronous complex128 transfers"},
                "complex128_pipelined": {"value": world * sites * W["obs_every"] * blocks / pipe128_s,
                                         "h2d_bytes_per_step": xfer128 / W["obs_every"],
                                         "d2h_bytes_per_step": (xfer128 + 8 * 8 * G) / W["obs_every"],
                                         "call": f"as the headline, with the reference's complex128 host "
                                                 f"buffers (the engine converts on the device)"}},
        "gpu_launches": nph * f32["steps"],
        "clocks": clk,
        "min_dt": f32["dt_min"], "max_drift": f32["max"], "flags": f32["flags"],
    }
    if extras:
        line["workloads"] = extras
    if single:
        line["fp64_single_chain"] = single
    if ref_gpu:
        bs = ref_gpu.get("benchmark_shape", {})
        if "value" in bs:
            # the batched FP32-mixed engine against the reference's own GPU step (one chain
            # per process, the reference's form), both in site-updates/s
            ref_gpu["batched_f32_over_reference"] = value / bs["value"]
        line["reference_gpu"] = ref_gpu
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def single_chain_fp64_leg(torch, clv, local, stream, steps=2000):
    """The plain-FP64 single-chain workload (spin-1, 1D Nx = 64, N_tau = 64, beta = 4, c0 = 0.5,
    c1 = -0.1, q = 0.05, mu = 1.0, the spin-1 start; K/max rule with the batched workload's
    K = 0.05 and dt_max = 1e-3): clv_step(n) with CUDA events on the engine's stream, by the
    step loop (the engine's choice for this size) and by the two-kernel form beside it."""
    c = clv.ChainParams(nx=64, ny=1, nz=1, nt=64, eps=4.0 / 64, mu=1.0, c0=0.5, c1=-0.1, q=0.05, K=0.05,
                        dt_max=1e-3, seed=20261203)
    out = {"workload": "spin1-1d-64-ntau64-beta4 (one chain, FP64)", "unit": "site-updates/s"}
    for key, no_loop in (("loop", False), ("two_kernel", True)):
        if no_loop:
            os.environ["CLV_NO_LOOP"] = "1"
        try:
            with clv.Engine(c, model=clv.MODEL_SPIN1, precision=clv.PREC_F64, device=local) as e:
                e.set_stream(stream.cuda_stream)
                e.init_spin1()
                e.step(50)
                torch.cuda.synchronize()
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                e.step(steps)
                b.record(stream)
                torch.cuda.synchronize()
                ms = a.elapsed_time(b) / steps
                plan = ":".join([e.plan()[0], ",".join(e.plan()[1])])
        finally:
            if no_loop:
                os.environ.pop("CLV_NO_LOOP", None)
        r = {"value": c.nx * c.nt / (ms / 1e3), "ms_per_step": ms, "plan": plan}
        if key == "loop":
            out.update(r)
        else:
            out["two_kernel"] = r
    out["steps"] = steps
    return out


def reference_gpu_leg(torch, clv, local, stream, steps=200):
    """The reference's own GPU build on this GPU: its kernels compiled unchanged from
    its sources (sm_103a cubins, oracle/ref_gpu_build.sh), cuFFT Z2Z and cuRAND XORWOW,
    driven in the order of Propagator::propagate (Propagator_without_cutoff.cu:406-442)
    by oracle/ref_gpu_runner.cpp, timed with CUDA events over `steps` propagate calls
    from main.cu's zero start (one chain: the reference steps one chain per process).
    Beside it, this engine's plain FP64 drop-in of the same model, lattice and step rule
    (one chain, clv_step(n)), on the batched benchmark's shape, the reference's shipped
    lattice and the lattices of the single-chain, 2D and 3D configurations.  Returns the
    report, or {"unavailable": why}."""
    import numpy as np
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    try:
        import refgpu
        refgpu.build_runner()
    except Exception as e:  # the host driver needs cuFFT/cuRAND/libcuda of the toolkit
        return {"unavailable": f"reference GPU driver not built: {type(e).__name__}: {e}"}
    out = {}
    # the batched benchmark's shape, the reference's shipped lattice, and the lattices of
    # the single-chain (64 x 64), 2D (128^2 x 128) and 3D (64^3 x 64) configurations
    legs = (("1d_x256_t128", "benchmark_shape", steps), ("1d_x256_t32", "reference_default_lattice", steps),
            ("1d_x64_t64", "single_chain_lattice", steps), ("2d_x128_y128_t128", "lattice_2d", 30),
            ("3d_x64_y64_z64_t64", "lattice_3d", 10))
    for name, key, steps in legs:
        if not refgpu.have_cubin(name):
            out[key] = {"unavailable": "reference cubins not built (built where the reference sources are)"}
            continue
        m = refgpu.macros(name)
        X, Y, Z, T = (int(m[k]) for k in ("XSIZE", "YSIZE", "ZSIZE", "TAUSIZE"))
        with refgpu.RefGpu(name, device=local) as r:
            r.set_mean_field(0.0, 0.0)
            r.time(max(3, steps // 10))
            ms, wall = r.time(steps)
        ref_v = X * Y * Z * T * steps / (ms / 1e3)
        P, MU = refgpu.CONFIGS[name][1], refgpu.CONFIGS[name][2]
        c = clv.ChainParams(nx=X, ny=Y, nz=Z, nt=T, eps=float(m["EPS"]), a_x=float(m["a_x"]), G=float(m["G"]),
                            Q=float(m["Q"]), P=P, mu=MU, DT=float(m["DT"]))
        with clv.Engine(c, model=clv.MODEL_REF4, precision=clv.PREC_F64, device=local) as e:
            e.set_stream(stream.cuda_stream)
            e.set_mean_field(0, 0.0, 0.0)
            e.set_mean_field(1, 0.0, 0.0)
            e.step(max(3, steps // 10))
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            e.step(steps)
            b.record()
            torch.cuda.synchronize()
            ours_ms = a.elapsed_time(b)
            ph = [e.step_timed() for _ in range(3)]
            phases = dict(zip(e.plan()[1], [round(sum(x) / len(x), 5) for x in zip(*ph)]))
            e_plan = ":".join([e.plan()[0], ",".join(e.plan()[1])])
        ours_v = X * Y * Z * T * steps / (ours_ms / 1e3)
        out[key] = {"value": ref_v, "unit": "site-updates/s", "ms_per_step": ms / steps,
                    "wall_ms_per_step": wall / steps, "steps": steps,
                    "lattice": f"1 chain x {X} x {Y} x {Z}, N_tau {T}, 4 components, FP64 (Parameters.h macros "
                               f"EPS={m['EPS']}, G={m['G']}, DT={m['DT']}; mu={MU}, P={P})",
                    "ours_fp64_dropin": {"value": ours_v, "ms_per_step": ours_ms / steps, "phases_ms": phases,
                                         "plan": e_plan,
                                         "call": "clv_step(n), same model, lattice and dt rule (the step loop's "
                                                 "cooperative launch where the problem fits it, else graph replay)"},
                    "dropin_over_reference": ours_v / ref_v}
    out["build"] = ("the reference's own kernels compiled unchanged for sm_103a (cubins), cuFFT Z2Z plans "
                    "and cuRAND XORWOW normals, propagate() order with its per-step allocations and "
                    "synchronisations; CUDA events on the default stream")
    return out


def _oracle_params(pyoracle, c, nt=None):
    return pyoracle.spin1_params(nx=c["nx"], ny=c["ny"], nz=c["nz"], nt=nt or c["nt"], eps=c["eps"],
                                 mu=c["mu"], c0=c["c0"], c1=c["c1"], q=c["q"], Kc=c["K"],
                                 dt_max=c["dt_max"])


def cpu_steps(W, budget_s, max_steps=None, warm=1):
    """Oracle steps over the workload's chains in turn until the budget is used."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle
    pyoracle.build()
    chains = W["chains"]
    # a 2D (3D) lattice is sampled over 32 (8) of its imaginary-time slices (same per-site work)
    nt_s = None
    if chains[0]["ny"] > 1:
        nt_s = min(8 if chains[0]["nz"] > 1 else 32, chains[0]["nt"])
    states = {}
    n = sites = 0
    t0 = None
    k = 0
    while True:
        i = k % len(chains)
        c = chains[i]
        p = _oracle_params(pyoracle, c, nt_s)
        if i not in states:
            states[i] = pyoracle.spin1_init(p, c["seed"], i)
        psi, psic = states[i]
        psi, psic, *_ = pyoracle.step(p, psi, psic, seed=c["seed"], chain=i, step_index=k)
        states[i] = (psi, psic)
        k += 1
        if k == warm:
            t0 = time.perf_counter()
            continue
        if t0 is None:
            continue
        n += 1
        sites += p.nx * p.ny * p.nz * p.nt
        el = time.perf_counter() - t0
        if (max_steps and n >= max_steps) or (not max_steps and el >= budget_s):
            return sites / el, n, el, pyoracle.num_threads(), nt_s


def cpu_model():
    """Host CPU description from /proc/cpuinfo (x86 model name or Arm implementer/part)."""
    try:
        info = open("/proc/cpuinfo").read().splitlines()
    except OSError:
        return "unknown"
    for key in ("model name", "Model"):
        for line in info:
            if line.startswith(key) and ":" in line:
                return line.split(":", 1)[1].strip()
    parts = {l.split(":", 1)[0].strip(): l.split(":", 1)[1].strip() for l in info if ":" in l}
    if "CPU implementer" in parts:
        return f"Arm implementer {parts['CPU implementer']} part {parts.get('CPU part', '?')}"
    return "unknown"


def cpu_baseline(W, budget_s=12.0):
    v, n, el, cores, nt_s = cpu_steps(W, budget_s)
    what = "chain-steps" if nt_s is None else f"chain-steps on {nt_s} of the tau-slices"
    # the same restatement on one thread (a shorter sample)
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle
    pyoracle.set_num_threads(1)
    v1, n1, el1, _, _ = cpu_steps(W, max(2.0, budget_s / 4))
    pyoracle.set_num_threads(cores)
    return {"value": v, "unit": "site-updates/s", "cores": cores, "kind": "port",
            "sample": f"{n} FP64 {what} of the workload's chains in turn, {el:.1f} s",
            "single_thread_value": v1, "single_thread_sample": f"{n1} chain-steps, {el1:.1f} s",
            "cpu_model": cpu_model(), "nproc": os.cpu_count()}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    W = workload(args.workload, args.chains)
    v, n, el, cores, nt_s = cpu_steps(W, 0, max_steps=args.steps * 4, warm=args.warmup)
    sample = ("each step: 4 FP64 chain-steps of the batch's chains in turn (CPU restatement of the "
              "same update on all host threads)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "site-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": W["name"], "chains": len(W["chains"]),
                                        "lattice": W["lattice"], "n_tau": W["n_tau"], "components": 3},
        "cpu_baseline": {"value": v, "unit": "site-updates/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": "site-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def compare_precision(args):
    """The precision comparison: the workload's chains run from the same Philox seed
    in FP64 and in FP32-mixed for --steps steps (observables every obs_every steps
    after --warmup thermalisation steps); for density, F_z, <F^2> and energy the
    report gives each precision's mean with its block error (autocorrelated
    series, 16 blocks per chain) and the deviation in units of the combined error.
    Prints one JSON report (not a benchmark line)."""
    import numpy as np
    import torch
    import cl_var_dt_gb300 as clv
    from cl_var_dt_gb300.secant import block_error
    W = workload(args.workload, args.chains)
    chains = [clv.ChainParams(**c) for c in W["chains"]]
    names = ("density", "F_z", "F2", "energy")
    out, wall = {}, {}
    for prec, tag in ((clv.PREC_F64, "fp64"), (clv.PREC_F32, "fp32")):
        t0 = time.perf_counter()
        with clv.Engine(chains, model=clv.MODEL_SPIN1, precision=prec) as e:
            e.init_spin1(np.sqrt(1 / 3), 0.01)
            e.step(args.warmup)
            for _ in range(args.steps // W["obs_every"]):
                e.step(W["obs_every"])
                e.evaluate()
            out[tag] = np.stack([e.spin1_samples(i) for i in range(len(chains))])  # chain, k, 8
            flags = int(np.bitwise_or.reduce(e.chain_flags()))
            t_lang = float(e.step_info()["t"].mean())
        torch.cuda.synchronize()
        wall[tag] = dict(seconds=time.perf_counter() - t0, flags=flags, langevin_time=t_lang)
    report = {}
    for j, name in enumerate(names):
        row = {}
        for tag in ("fp64", "fp32"):
            x = out[tag][:, :, 2 * j]  # real parts
            means = x.mean(axis=1)
            errs = np.array([block_error(c, 16) for c in x])
            # chains combined by inverse-variance weighting
            wts = 1 / np.maximum(errs, 1e-300) ** 2
            row[tag] = float((means * wts).sum() / wts.sum())
            row[tag + "_err"] = float(1 / np.sqrt(wts.sum()))
        row["deviation_sigma"] = abs(row["fp32"] - row["fp64"]) / float(np.hypot(row["fp64_err"], row["fp32_err"]))
        report[name] = row
    print(json.dumps({"workload": W["name"], "steps": args.steps, "thermalisation": args.warmup,
                      "obs_every": W["obs_every"], "samples_per_chain": int(out["fp64"].shape[1]),
                      "chains": len(chains), "same_seed": True, "observables": report, "runs": wall}),
          flush=True)


def tune_demo(args):
    """The uneven batch's caller (configuration 5): every chain's mu tuned by the
    driver (damped Newton steps with the mean-field slope 1 / c0 on each round's
    equilibrium estimate) to the target density its configuration drew,
    |n - target| < 0.05 on a settled round, all chains of the batch on one engine reused across
    rounds (mu set in place; the engine re-batched when fewer than half of its
    chains are still tuning), each chain started at its target density.  Prints one
    JSON report (not a benchmark line)."""
    import cl_var_dt_gb300 as clv
    from cl_var_dt_gb300 import secant
    W = with_n_tau(workload("uneven", args.chains or 64), args.n_tau)
    n = len(W["chains"])
    targets = W["targets"]
    chains = [clv.ChainParams(**c) for c in W["chains"]]
    therm, meas, every = args.warmup * 100, args.steps, W["obs_every"]
    active = args.max_active or n
    # every chain starts (and restarts) at its target density: the density mode relaxes
    # over tens of Langevin-time units at the small couplings of the batch
    sampler = secant.EngineBatchSampler(therm_steps=therm, meas_steps=meas, obs_every=every,
                                        start_density={i: float(t) for i, t in enumerate(targets)})
    log = []
    # steps of at most 0.5 in mu: a chain pushed far above its target density relaxes back
    # slowly, so the driver avoids overshooting
    # damped Newton steps with the mean-field slope dn/dmu = 1 / c0 (n = mu / c0): at the
    # batch's small c0 the density moves by several units per unit of mu
    tt = [secant.TuneTarget(c, target=float(t), mu_step=0.2, tol=0.05, max_jump=0.5, slope=1.0 / c.c0)
          for c, t in zip(chains, targets)]
    t0 = time.perf_counter()
    try:
        states = secant.tune(tt, sampler, max_active=active, max_rounds=args.rounds, log=log.append)
    finally:
        sampler.close()
    wall = time.perf_counter() - t0
    print(json.dumps({
        "workload": W["name"], "chains": n, "max_active": active, "rounds_max": args.rounds,
        "rounds_run": max(len(s.mus) for s in states), "steps_per_round": therm + meas,
        "tolerance": 0.05, "converged": int(sum(s.converged for s in states)),
        "engine_builds": sampler.builds, "restarts": sampler.restarts, "site_updates": sampler.site_updates,
        "site_updates_per_s_incl_tuning": sampler.site_updates / wall, "seconds": wall, "log": log,
        "chains_report": [{"side": c.nx, "n_tau": c.nt, "c0": c.c0, "target": s.target.target,
                           "mu": s.mus, "density": s.dens, "err": s.errs, "settled": s.settled,
                           "rounds": len(s.mus),
                           "dt": sampler.last_dt.get(i), "converged": s.converged}
                          for i, (c, s) in enumerate(zip(chains, states))]}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched", choices=["batched", "2d", "3d", "uneven"])
    ap.add_argument("--chains", type=int, default=None, help="batch size of the batched workload")
    ap.add_argument("--n-tau", type=int, default=None,
                    help="override the imaginary-time extent (smaller cases of a workload for profiling)")
    ap.add_argument("--skip-fp64", action="store_true", help="time the FP32-mixed engine only")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra-workloads", action="store_true",
                    help="skip the 2D, 3D and uneven workloads beside the batched one")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip timing the reference's own GPU build beside the engine")
    ap.add_argument("--no-autotune", action="store_true", help="keep the engine's heuristic plan")
    ap.add_argument("--compare-precision", action="store_true",
                    help="FP64 vs FP32-mixed observables from the same seed (report, not a benchmark line)")
    ap.add_argument("--tune-demo", action="store_true",
                    help="secant mu-tuning of the uneven batch to its target densities (report)")
    ap.add_argument("--rounds", type=int, default=8, help="secant rounds of --tune-demo")
    ap.add_argument("--max-active", type=int, default=None, help="chains tuned at once by --tune-demo (default all)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.compare_precision:
        compare_precision(args)
    elif args.tune_demo:
        tune_demo(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

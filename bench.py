#!/usr/bin/env python
"""Benchmark of the TeaLeaf implicit solve on GB300.

Workload (default): the standard five-state deck (10 x 10 domain,
dt 0.004) at 8192 x 8192 cells solved to tl_eps 1e-15, timesteps 1..K of a
fresh run, by two methods on the same GPU:
  headline  PPCG with the 4-row block-Jacobi preconditioner and 10 inner
            Chebyshev steps, FP32 inner steps inside the FP64 outer solve,
            started by the learned warm start (network + previous step,
            Galerkin-combined);
  plain     FP64 CG with the diagonal Jacobi preconditioner from u = u^n
            (the reference's method; its iteration counts define the work).
A step is one timestep: one complete implicit solve (tea_leaf(),
tea_solve.f90:37), with every field resident in HBM.  The metric is
plain-CG cell-iterations per second: cells x (iterations the plain FP64 CG
takes for those timesteps) / time, so a method that reaches tl_eps in less
time scores higher in proportion; the time to solution per step of both
methods and the field_summary difference between them are reported beside
it.  --solver/--precond/--precision/--warm select another headline method.

Legs (one JSON line):
  value      K device-resident solves of the headline method (CUDA graphs),
             timed with CUDA events on the library's stream.  Every field is
             larger than L2 (537 MB each at 8192^2), so no flush is needed
             between steps.
  plain      K solves of FP64 CG + jac_diag from a fresh start (timed the
             same way; gives the work count and the baseline time).
Each timed step is a solve plus its field summary, and the summaries of the
two methods are compared timestep by timestep.
  roofline   K more headline solves with per-kernel CUDA events (eager
             launches); the dominant kernel's algorithmic bytes per launch /
             its mean launch time, against the measured HBM copy bandwidth;
             and the three largest kernels each against its own bound (HBM,
             or the FP64 pipe at a measured DGEMM FMA rate).
  prev       (learned warm start only) K solves of the same method started
             from the increment history alone, to show the network's gain.
  e2e        K more headline solves through the C-ABI with host buffers:
             density and energy copied host->device before and energy copied
             back after every solve, inside the timed region.
  cpu_baseline  the CPU oracle (oracle/) on the host cores: one timestep of
             the same deck by CG + jac_diag, capped at --cpu-iters iterations.

--impl reference runs the reference algorithm on the host CPU instead (the
reference has no CPU implementation of this path, so the oracle's
restatement of it is timed, all host threads): FP64 CG + jac_diag on the same
deck, each step a timestep capped at --ref-iters iterations.

Multi-GPU: one process per GPU (torchrun); each rank solves its own replica
(the single-chunk solve has no data-parallel split), value = all ranks'
cell-iterations / the slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time-to-solution & cell-iters/s at tl_eps: mixed+learned vs plain FP64 CG, 1 GB300"
DEFAULT_MODEL = os.path.join(ROOT, "tealeaf_cuda_gb300", "warm_start.tlws")

STATES = """state 1 density=100.0 energy=0.0001
state 2 density=0.1 energy=25.0 geometry=rectangle xmin=0.0 xmax=1.0 ymin=1.0 ymax=2.0
state 3 density=0.1 energy=0.1 geometry=rectangle xmin=1.0 xmax=6.0 ymin=1.0 ymax=2.0
state 4 density=0.1 energy=0.1 geometry=rectangle xmin=5.0 xmax=6.0 ymin=1.0 ymax=8.0
state 5 density=0.1 energy=0.1 geometry=rectangle xmin=5.0 xmax=10.0 ymin=7.0 ymax=8.0
"""

# algorithmic bytes per interior cell of each kernel: every array the kernel
# must read or write, counted once (halos ignored); FP64 arrays 8 bytes, FP32
# arrays 4
BYTES_PER_CELL = {
    "cg_w": 32,          # read p, Kx, Ky; write w
    "cg_ur": 64,         # jac_diag: read u, p, r, w, Mi; write u, r, z
    "cg_p": 24,          # read z, p; write p
    "residual": 40,      # read u, u0, Kx, Ky; write r
    "cg_init": 48,       # read r, Kx, Ky; write Mi, z, p
    "common_init": 56,   # read density, energy; write Kx, Ky, u, u0
    "diag": 24,          # read Kx, Ky; write diag
    "field_summary": 32,
    "finalise": 24,
    "ppcg_p": 24,        # read z, p; write p
    "ppcg_up": 40,       # read p, u, z; write u, p (mixed PPCG with fused inner passes)
    "ppcg_update_r": 48,  # read sd, Kx, Ky, diag, rtemp; write rtemp
    "cheby_calc_u": 24,  # read u, p; write u
    "copy": 16,          # read src; write dst
    "ppcg_w_zr": 64,     # read p, Kx, Ky, diag, r, z; write w, r_store
    "ppcg_rrn": 24,      # read r, r_store, z
    # mixed precision: FP32 inner iteration (4-byte elements)
    "mixed_w": 16,       # read p, Kx, Ky; write w
    "mixed_ur": 32,      # jac_diag: read d, p, r, w, Mi; write d, r, z
    "mixed_p": 12,       # read z, p; write p
    "mixed_init": 28,    # read r (FP64), Mi; write r, z, p, d
    "mixed_update_u": 20,  # read u (FP64), d; write u (FP64)
    "mixed_convert": 40,   # read Kx, Ky (FP64); write Kx, Ky, Mi (FP32)
    "mixed_pp_init": 28,   # read r, z (FP64); write sd, rtemp, utemp
}


# DRAM bytes per cell measured by ncu (dram__bytes_read.sum + write.sum of one
# launch / cells), for the kernels that can dominate the default workload
# (mixed_pp_fused measured at the workload's own 8192^2, cg_w at 4096^2);
# scaled to a launch by the cells it processes
TRAFFIC_PER_CELL = {
    "mixed_pp_fused": 42.98,  # k_pp_fused<5, jac_block> first + last pass at 8192^2: mean 2884.2 MB a launch
    "cg_w": 39.6,             # BodyCgW at 4096^2: 545.5 + 119.4 MB
}


# FP64 instructions per interior cell of the kernels whose bound is GB300's
# FP64 pipe rather than HBM (DFMA, DMUL and DADD each take one issue of the
# pipe): the operator of tea_leaf_common.cuknl:28-34 as 6 instructions
# (DMUL, DFMA, DMUL, DFMA, DFMA, DADD), or 5 in the mixed-precision outer
# pass (DMUL + 4 DFMA), plus one DFMA per dot product
FP64_INSTR_PER_CELL = {
    "ppcg_w_zr": 7,   # 5-instruction operator, p.w, r.z
    "cg_w": 7,        # 6-instruction operator, p.w
    "residual": 8,    # 6-instruction operator, u0 - Au, r.r
}

INNER_STEPS = 10  # tl_ppcg_inner_steps of the workload's deck
FUSED_STEPS = 5   # FP32 inner steps per fused pass (the library's default)


def bytes_per_cell(kernel, precond):
    """algorithmic bytes per cell of `kernel` under preconditioner `precond`"""
    if kernel == "mixed_pp_step":
        # read sd, Kx, Ky, rtemp, utemp + the preconditioner (Mi; or cp and
        # 1/b of the strip solve); write sd', rtemp, utemp (an inner step
        # before the last)
        return {"none": 32, "jac_diag": 36, "jac_block": 40}[precond]
    if kernel == "cheby_p":
        # read u, Kx, Ky, diag, u0, p + the preconditioner (Mi; or cp, bfp);
        # write w, r, p
        return {"none": 72, "jac_diag": 80, "jac_block": 88}[precond]
    if kernel == "ppcg_sd":
        # read rtemp, sd, utemp + the preconditioner (Mi; or diag, Ky, cp,
        # bfp); write sd, utemp
        return {"none": 40, "jac_diag": 48, "jac_block": 72}[precond]
    if kernel == "mixed_ur":
        # read d, p, r, w + the preconditioner (Mi; or Ky, cp, bfp); write d, r, z
        return {"none": 28, "jac_diag": 32, "jac_block": 40}[precond]
    if kernel == "mixed_init":
        # read r (FP64) + the preconditioner; write r, z, p, d
        return {"none": 24, "jac_diag": 28, "jac_block": 36}[precond]
    if kernel == "mixed_pp_ur":
        if FUSED_STEPS > 1:
            # read w, r; write r (FP64): the first fused pass starts the inner
            # steps from r itself and u += alpha p runs in ppcg_up
            return 24
        # + the FP32 preconditioner (Mi; or Ky, cp, bfp); write rtemp, sd,
        # utemp (FP32)
        return {"none": 60, "jac_diag": 64, "jac_block": 72}[precond]
    if kernel == "mixed_pp_fused":
        # the same arrays once per pass of several inner steps; the first
        # pass of a solve reads r (FP64) instead of sd, rtemp and utemp and
        # the last one writes z (FP64) instead of sd, rtemp and utemp (FP32):
        # the mean over the INNER_STEPS / FUSED_STEPS passes of one solve
        passes = -(-INNER_STEPS // FUSED_STEPS)
        full = {"none": 32, "jac_diag": 36, "jac_block": 40}[precond]
        return full - 8.0 / passes
    return BYTES_PER_CELL.get(kernel)


def make_deck(n, solver="cg", precond="jac_diag", max_iters=10000, end_step=100000, precision="fp64",
              warm="none"):
    return ("*tea\n" + STATES +
            f"x_cells={n}\ny_cells={n}\nxmin=0.0\nymin=0.0\nxmax=10.0\nymax=10.0\n"
            f"initial_timestep=0.004\nend_step={end_step}\ntl_max_iters={max_iters}\n"
            f"tl_use_{solver}\ntl_preconditioner_type {precond}\ntl_eps 1.0e-15\n"
            f"tl_ppcg_inner_steps {INNER_STEPS}\ntl_precision {precision}\ntl_warm_start {warm}\n"
            f"summary_frequency 0\n*endtea\n")


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ distributed
def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    dist.init_process_group("nccl" if os.environ.get("TL_BENCH_GLOO") is None else "gloo")
    return rank, ws, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, ws, local):
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=f"cuda:{local}" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(x, ws, local):
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=f"cuda:{local}" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------- oracle
def oracle_sample(n, iters, steps, threads=None):
    """Run the CPU oracle on the deck capped at `iters` iterations per step;
    returns per-step (iterations, wall seconds)."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    exe = os.path.join(ROOT, "oracle", "_build", "tea_oracle")
    with tempfile.NamedTemporaryFile("w", suffix=".in", delete=False) as f:
        f.write(make_deck(n, max_iters=iters, end_step=steps))
        path = f.name
    env = dict(os.environ)
    env["OMP_NUM_THREADS"] = str(threads or os.cpu_count())
    env.setdefault("OMP_PROC_BIND", "close")
    try:
        out = subprocess.run([exe, path], check=True, capture_output=True, text=True, env=env).stdout
    finally:
        os.unlink(path)
    recs = [json.loads(l) for l in out.splitlines() if l.strip()]
    steps_r = [r for r in recs if r["kind"] == "step" and r["step"] > 0]
    walls, prev = [], 0.0
    for r in steps_r:
        walls.append(r["wall"] - prev)
        prev = r["wall"]
    return [(r["iterations"], w) for r, w in zip(steps_r, walls)], recs[-1]["threads"]


def run_reference(args):
    # the CPU oracle runs on rank 0 alone and needs no collective: the rank
    # comes from the launcher's environment, with no process group
    if int(os.environ.get("RANK", "0")) != 0:
        return
    n = args.n
    per, threads = oracle_sample(n, args.ref_iters, args.warmup + args.steps)
    timed = per[args.warmup:]
    its = sum(i for i, _ in timed)
    secs = sum(w for _, w in timed)
    value = n * n * its / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "plain-CG cell-iters/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * secs / len(timed), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (standard five-state deck)",
        "config": {"workload": f"standard deck {n}x{n}, tl_eps 1e-15, timesteps 1..{args.steps} "
                               "after the warm-up timesteps",
                   "method": f"CG + jac_diag, fp64 (the reference's method), each timestep capped at "
                             f"{args.ref_iters} iterations",
                   "parallelism": "cpu", "cells": n * n},
        "cpu_baseline": {"value": value, "unit": "plain-CG cell-iters/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} timesteps of the {n}^2 deck, {args.ref_iters} "
                                   "CG iterations each, CPU oracle (C, OpenMP)"},
        "e2e": {"value": value, "unit": "plain-CG cell-iters/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------- ours
def timed_solves(ch, stream, steps, torch):
    """`steps` timesteps (solve + field summary, the loop body of
    diffuse.f90:43-101) timed with CUDA events on the library stream;
    returns (total ms, per-step ms, per-step solve infos, per-step field
    summaries)"""
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    infos, sums = [], []
    evs[0].record(stream)
    for k in range(steps):
        infos.append(ch.timestep())
        sums.append(ch.field_summary())
        evs[k + 1].record(stream)
    evs[-1].synchronize()
    per = [evs[k].elapsed_time(evs[k + 1]) for k in range(steps)]
    return evs[0].elapsed_time(evs[-1]), per, infos, sums


def fp64_fma_peak(torch, device):
    """measured FP64 FMA rate of this GPU (FMA/s): a cuBLAS DGEMM of
    4096^3 (2 n^3 flops = n^3 FMAs), best of 5 after a warm-up"""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=device)
    b = torch.randn(n, n, dtype=torch.float64, device=device)
    torch.matmul(a, b)
    best = None
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    del a, b
    return n ** 3 / (best * 1e-3)


def kernel_roofline(name, st, cells, precond, hbm_peak, fp64_peak):
    """one kernel's roofline entry from its launch count and total ms: the
    HBM fraction (algorithmic bytes / mean launch time) and, for the
    FP64-pipe kernels, the FP64 instruction fraction; `bound` is the larger"""
    launch_ms = st["ms"] / st["launches"]
    out = {"kernel": name, "launches": st["launches"], "launch_ms": launch_ms}
    bpc = bytes_per_cell(name, precond)
    if bpc:
        gbs = bpc * cells / (launch_ms * 1e-3) / 1e9
        out.update({"bytes_per_cell": bpc, "hbm_gbs": gbs, "hbm_frac": gbs / hbm_peak})
    ipc = FP64_INSTR_PER_CELL.get(name)
    if ipc and fp64_peak:
        rate = ipc * cells / (launch_ms * 1e-3)
        out.update({"fp64_instr_per_cell": ipc, "fp64_instr_per_s": rate, "fp64_frac": rate / fp64_peak})
    out["bound"] = "fp64" if out.get("fp64_frac", 0.0) > out.get("hbm_frac", 0.0) else "hbm"
    return out


def load_model(ch, lib, path):
    import ctypes as C

    import numpy as np
    from tealeaf_cuda_gb300 import learned
    if not os.path.exists(path):
        raise SystemExit(f"bench: warm start model {path} not found (train one with "
                         "python -m tealeaf_cuda_gb300.learned train)")
    p = np.ascontiguousarray(learned.load_model(path), dtype=np.float32)
    if lib.tl_set_warm_start_model(ch._h, C.c_void_p(p.ctypes.data), p.size) != 0:
        raise SystemExit("bench: tl_set_warm_start_model failed")


def run_ours(args):
    import ctypes as C

    import torch

    import tealeaf_cuda_gb300 as tl

    rank, ws, local = dist_init()
    torch.cuda.set_device(local)
    lib = tl.load()
    n, K = args.n, args.steps
    cells = n * n

    # ---------------- headline method
    cfg = tl.parse_deck(make_deck(n, solver=args.solver, precond=args.precond, precision=args.precision,
                                  warm=args.warm))
    cfg.cuda_device = local
    ch = tl.Chunk(cfg)
    if args.warm == "learned":
        load_model(ch, lib, args.model)
    stream = torch.cuda.ExternalStream(lib.tl_chunk_stream(ch._h), device=local)
    ch.start()
    for _ in range(args.warmup):
        ch.timestep()

    # ---- value: timesteps 1..K of a fresh run, device-resident
    ch.start()
    barrier(ws)
    torch.cuda.synchronize()
    launches0 = ch.kernel_launches
    with ClockSampler(local) as clk:
        ms, per_ms, infos, sums_h = timed_solves(ch, stream, K, torch)
    torch.cuda.synchronize()
    barrier(ws)
    launches = ch.kernel_launches - launches0
    clocks = clk.summary()
    summary_h = sums_h[-1]
    its_h = [i["iterations"] for i in infos]

    # ---- roofline: per-kernel CUDA events over the same K timesteps
    ch.start()
    lib.tl_set_profiling(ch._h, 1)
    lib.tl_profile_reset(ch._h)
    for _ in range(K):
        ch.timestep()
    kernels = {}
    k = 0
    while True:
        name, cnt, kms = C.c_char_p(), C.c_longlong(), C.c_double()
        if lib.tl_profile_read(ch._h, k, C.byref(name), C.byref(cnt), C.byref(kms)) != 0:
            break
        if cnt.value:
            kernels[name.value.decode()] = {"launches": cnt.value, "ms": kms.value}
        k += 1
    lib.tl_set_profiling(ch._h, 0)
    fp64_peak = fp64_fma_peak(torch, f"cuda:{local}")
    total_kms = sum(v["ms"] for v in kernels.values()) or 1.0
    dom = max(kernels, key=lambda x: kernels[x]["ms"])
    dom_launch_ms = kernels[dom]["ms"] / kernels[dom]["launches"]
    bpc = bytes_per_cell(dom, args.precond)
    achieved = (bpc or 0) * cells / (dom_launch_ms * 1e-3) / 1e9
    peaks = {}
    pk_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk_path):
        peaks = json.load(open(pk_path))
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    peak = peak or 6800.0
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_src,
                "traffic": (args.traffic_per_launch if args.traffic_per_launch is not None else
                            (TRAFFIC_PER_CELL[dom] * cells if dom in TRAFFIC_PER_CELL and
                             (dom != "mixed_pp_fused" or args.precond == "jac_block") else None)),
                "bytes_per_cell": bpc, "launch_ms": dom_launch_ms,
                "kernel_share": {k2: round(v["ms"] / total_kms, 4) for k2, v in
                                 sorted(kernels.items(), key=lambda kv: -kv[1]["ms"])},
                "measured_over": f"timesteps 1..{K}, eager launches with per-kernel CUDA events",
                # the three kernels with the largest share, each against its own bound:
                # HBM (measured copy rate) or the FP64 pipe (measured DGEMM FMA rate)
                "top_kernels": [kernel_roofline(k2, kernels[k2], cells, args.precond, peak, fp64_peak)
                                for k2 in sorted(kernels, key=lambda x: -kernels[x]["ms"])[:3]],
                "fp64_peak": {"value": fp64_peak, "unit": "FP64 FMA/s",
                              "how": "torch.matmul float64 4096^3 (cuBLAS DGEMM), best of 5, n^3 FMAs"}}

    # ---- e2e: the state lives on the host; every timestep uploads density
    # and energy from pinned buffers, solves and reads energy back
    ch.start()
    pin = dict(dtype=torch.float64, pin_memory=True)
    host_rho = torch.empty(ch.shape, **pin).numpy()
    host_e = torch.empty(ch.shape, **pin).numpy()
    ch.get_field("density", out=host_rho)
    ch.get_field("energy1", out=host_e)
    h2d = host_rho.nbytes + host_e.nbytes
    d2h = host_e.nbytes
    barrier(ws)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_its = []
    t_in = t_solve = t_out = 0.0  # host wall time of the copies in, the solves, the copy out
    for _ in range(K):
        ta = time.perf_counter()
        ch.set_field("density", host_rho)
        ch.set_field("energy1", host_e)
        tb = time.perf_counter()
        e2e_its.append(ch.timestep()["iterations"])
        tc = time.perf_counter()
        ch.get_field("energy1", out=host_e)
        td = time.perf_counter()
        t_in, t_solve, t_out = t_in + (tb - ta), t_solve + (tc - tb), t_out + (td - tc)
    torch.cuda.synchronize()
    e2e_s = allreduce_max(time.perf_counter() - t0, ws, local)
    ch.close()

    # ---- the same method started from the increment history alone (no
    # network), for the network's gain over the method without it
    prev_ms = prev_per_ms = prev_its = None
    if args.warm == "learned":
        qcfg = tl.parse_deck(make_deck(n, solver=args.solver, precond=args.precond, precision=args.precision,
                                       warm="prev"))
        qcfg.cuda_device = local
        qch = tl.Chunk(qcfg)
        qstream = torch.cuda.ExternalStream(lib.tl_chunk_stream(qch._h), device=local)
        qch.start()
        torch.cuda.synchronize()
        prev_ms, prev_per_ms, qinfos, _ = timed_solves(qch, qstream, K, torch)
        prev_its = [i["iterations"] for i in qinfos]
        qch.close()

    # ---------------- plain FP64 CG + jac_diag on the same timesteps
    pcfg = tl.parse_deck(make_deck(n))
    pcfg.cuda_device = local
    pch = tl.Chunk(pcfg)
    pstream = torch.cuda.ExternalStream(lib.tl_chunk_stream(pch._h), device=local)
    pch.start()
    barrier(ws)
    torch.cuda.synchronize()
    pms, pper_ms, pinfos, sums_p = timed_solves(pch, pstream, K, torch)
    summary_p = sums_p[-1]
    pch.close()
    its_p = [i["iterations"] for i in pinfos]

    ms_max = allreduce_max(ms, ws, local)
    work = allreduce_sum(float(cells * sum(its_p)), ws, local)
    value = work / (ms_max * 1e-3)
    e2e = {"value": work / e2e_s, "unit": "plain-CG cell-iters/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * e2e_s / K, "iterations_per_step": e2e_its,
           "ms_per_step_h2d_solve_d2h": [1e3 * t_in / K, 1e3 * t_solve / K, 1e3 * t_out / K]}
    rel = [abs(a - b) / abs(b) if b else abs(a) for a, b in zip(summary_h, summary_p)]
    rel_steps = [max(abs(a - b) / abs(b) if b else abs(a) for a, b in zip(x, y)) for x, y in zip(sums_h, sums_p)]

    # ---- CPU baseline (rank 0, N = 1 only)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cap = args.cpu_iters or max(50, min(3000, int(4e10 / cells)))
        per, threads = oracle_sample(n, cap, 1)
        it0, w0 = per[0]
        cpu = {"value": cells * it0 / w0, "unit": "plain-CG cell-iters/s", "cores": threads, "kind": "port",
               "sample": f"timestep 1 of the {n}^2 deck by CG + jac_diag capped at {cap} iterations "
                         f"({it0} run, {w0:.1f} s), CPU oracle (C, OpenMP)"}

    if rank == 0:
        method = (f"{args.solver.upper()} + {args.precond}"
                  + (" (10 inner steps)" if args.solver == "ppcg" else "")
                  + f", {args.precision}, warm start {args.warm}")
        line = {
            "metric": METRIC, "value": value, "unit": "plain-CG cell-iters/s", "n_gpus": ws,
            "steps": K, "warmup": args.warmup, "ms_per_step": ms_max / K,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "data": "synthetic (standard five-state deck of the reference benchmarks)",
            "config": {"workload": f"standard deck {n}x{n}, tl_eps 1e-15, timesteps 1..{K} of a fresh run",
                       "method": method, "cells": cells,
                       "iterations_per_step": its_h,
                       "time_to_solution_ms": per_ms,
                       "plain_method": "CG + jac_diag, fp64, u = u^n start",
                       "plain_iterations_per_step": its_p,
                       "plain_time_to_solution_ms": pper_ms,
                       "time_to_solution_speedup_vs_plain": pms / ms,
                       "field_summary_rel_diff_vs_plain": max(rel),
                       "field_summary_rel_diff_vs_plain_per_step": rel_steps,
                       "prev_start_time_to_solution_ms": prev_per_ms,
                       "prev_start_iterations_per_step": prev_its,
                       "learned_over_prev_speedup": (prev_ms / ms) if prev_ms else None,
                       "warm_used": [i.get("warm_used") for i in infos],
                       "warm_net_share": [i.get("warm_net_share") for i in infos],
                       "warm_ratio": [i.get("warm_ratio") for i in infos],
                       "l2": "fields larger than L2, no flush",
                       "parallelism": "replicas" if ws > 1 else "single GPU"},
            # the speed-up over the reference arm is the product of the
            # method's gain (same GPU) and the GPU's over the CPU (same method)
            "ratio_split": {
                "method_speedup_vs_plain_gpu": pms / ms,
                "plain_gpu_cell_iters_per_s": work / (pms * 1e-3),
                "plain_gpu_over_cpu": (work / (pms * 1e-3)) / cpu["value"] if cpu else None},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
            "gpu_launches": launches,
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--solver", default="ppcg", choices=["cg", "ppcg", "chebyshev"])
    ap.add_argument("--precond", default="jac_block", choices=["none", "jac_diag", "jac_block"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--warm", default="learned", choices=["none", "prev", "learned"])
    ap.add_argument("--model", default=DEFAULT_MODEL)
    ap.add_argument("--ref-iters", type=int, default=100)
    ap.add_argument("--cpu-iters", type=int, default=None)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--traffic-per-launch", type=float, default=None,
                    help="dram bytes per launch of the dominant kernel from an ncu capture")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

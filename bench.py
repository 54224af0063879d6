"""Benchmark: RK4 grid-point-steps/s of the NLSE step loop on GB300.

Workload (one bench step = one whole job): the 3D vortex-ring solve, 320^3
grid, h = 0.3, a = 1, s = -1, harmonic trap (w = 0.02), MSD boundary,
2SHOC, k = 0.8 x the linear stability limit, 500 RK4 steps, mixed precision
(FP32 stages, compensated FP32 hi/lo state).  Inputs are seeded synthetic
data (nlsemagic_gb300.workloads.vortex_rings_3d).  The working set (about
1.9 GB) is far larger than L2, so no L2 flush is needed between steps.

  value  device-resident throughput: job = re-ingest the initial state from
         device planar arrays + 500 RK4 steps (CUDA graphs), timed with CUDA
         events on the solver stream.
  e2e    the same job through the C ABI one-shot entry point
         NLSE3D_TAKE_STEPS_CUDA_MIXED with pinned host planar buffers
         (host->device copies, 500 steps, device->host copies inside).

--impl reference times the reference CPU integrator (the C oracle port of
NLSE3D_TAKE_STEPS_2SHOC.c) on the host cores: one independent solve per
thread, each bench step one bounded sample (RK4 steps on the full grid).

Multi-GPU: replicas only (each rank runs its own independent solve; no
collective on the data path), weak scaling.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RK4 Gpt-steps/s & %HBM roofline at stated FP64 error; served p50/p99 latency"
UNIT = "Gpt-steps/s"
# Algorithmic HBM bytes per grid-point-step.  The per-stage model of the
# path (one HBM pass per RK4 stage, D kept on chip; psi and K at 16 B, the
# stage input at 8 B, V at 4 B) gives 240 B for FP32-stage / wide-accumulate
# and 304 B for FP64: these are the roofline figures.  This implementation's
# mixed path stores less (E in place of Y, K1 + 2 K2 only: 28 + 44 + 36 + 52
# = 160 B), reported beside it.
BYTES_MODEL_MIXED = 240.0
BYTES_DESIGN_MIXED = 160.0
BYTES_FP64 = 304.0
# FP64 instructions per interior grid-point-step of the exact FP64 class,
# counted from the reference expressions (each +, -, x one instruction; the
# reference operation order forbids contraction): 3D 2SHOC per stage D 16,
# F 57 (the |U|^2 term shared by both components), update 7 -> 80 x 4; 2D
# 2SHOC D 12, F 35, update 7 -> 54 x 4 (src/NLSEmagic3D/NLSE3D_TAKE_STEPS_2SHOC.c:
# 56-72, 233-262; src_old/NLSE2D_v1/NLSE2D_TAKE_STEPS_2SHOC.c:59-67, 169-187).
FP64_OPS = {(3, 2): 320.0, (2, 2): 216.0}
# The timed CPU arm is the C restatement of the reference integrator (the
# reference's own build cannot travel to an aarch64 host).  Both were timed
# side by side on one x86-64 core (320^3, one RK4 step of FP64 2SHOC MSD, the
# reference built with its own -O3 -funroll-loops through the mex shim): the
# restatement took 9.2-11.0 s, the reference 12.0-15.3 s, with identical
# bits.  The restatement is the faster of the two, so the CPU figure is not
# understated by the substitution.
PORT_VS_REFERENCE = {"grid": "320^3", "rk4_steps": 1, "threads": 1, "host": "x86-64 Xeon 2.7 GHz",
                     "port_s": [9.2, 11.0], "reference_s": [12.0, 15.3],
                     "same_bits": True}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


def max_over_ranks(x, world):
    """Max of a host scalar over ranks (the slowest rank's time); tensors live
    on the GPU under NCCL and on the CPU under gloo."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def read_traffic():
    """DRAM bytes per point-step of the stage kernels from the committed ncu
    summary (profiles/stage_kernels_3d2shoc_mixed.md), or None."""
    p = os.path.join(ROOT, "profiles", "stage_kernels_3d2shoc_mixed.md")
    if not os.path.exists(p):
        return None
    for ln in open(p):
        if ln.startswith("dram_bytes_per_point_step:"):
            try:
                return float(ln.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


# ---------------------------------------------------------------------------
# CPU baseline: the C oracle port of the reference integrator, one
# independent solve per thread (the reference is serial; aggregate host
# throughput is P independent solves).
# ---------------------------------------------------------------------------
def cpu_sample(w, steps, threads, precision=2):
    import oracle
    oracle._load_port()
    results = [None] * threads

    def one(t):
        t0 = time.perf_counter()
        oracle.take_steps(w.U, w.V, w.s, w.a, w.h2, w.BC, steps, w.k, method=w.method,
                          precision=precision, flags=oracle.MSD_GUARD)
        results[t] = time.perf_counter() - t0

    th = [threading.Thread(target=one, args=(t,)) for t in range(threads)]
    t0 = time.perf_counter()
    for x in th:
        x.start()
    for x in th:
        x.join()
    wall = time.perf_counter() - t0
    pts = float(w.points) * steps * threads
    return pts / wall / 1e9, wall


def host_cpu():
    """Model and core count of the host, from lscpu (else /proc/cpuinfo and
    os.cpu_count())."""
    info = {"cores": os.cpu_count(), "model": None, "arch": None}
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        kv = {}
        for ln in out.splitlines():
            if ":" in ln:
                k, v = ln.split(":", 1)
                kv[k.strip()] = v.strip()
        info["model"] = kv.get("Model name") or kv.get("Vendor ID")
        info["arch"] = kv.get("Architecture")
        if kv.get("CPU(s)", "").isdigit():
            info["cores"] = int(kv["CPU(s)"])
        if kv.get("Socket(s)", "").isdigit() and kv.get("Core(s) per socket", "").isdigit():
            info["physical_cores"] = int(kv["Socket(s)"]) * int(kv["Core(s) per socket"])
    except Exception:
        pass
    return info


def cpu_threads_for(w):
    n = os.cpu_count() or 1
    try:
        import psutil
        avail = psutil.virtual_memory().available
    except Exception:
        avail = None
    per = w.points * 8 * 13  # oracle scratch (8 planes) + in/out planes
    if avail:
        n = max(1, min(n, int(0.6 * avail // per)))
    return min(n, 64)


def tune_for(args, shape, method, precision, BC):
    """Launch knobs for this problem class from the autotuner
    (nlsemagic_gb300/autotune.py: tuned once per device and class, cached),
    applied before the solvers are created; returns the knobs in force."""
    from nlsemagic_gb300 import autotune
    entry = None
    if args.tune:
        t0 = time.perf_counter()
        entry = autotune.tune(shape, method=method, precision=precision, BC=BC, steps=20)
        autotune.apply(shape, method=method, precision=precision, BC=BC)
        log("autotune %s: %s (%.1f s)" % (list(shape), json.dumps(entry),
                                          time.perf_counter() - t0))
    knobs = {k: autotune.get_knob(k) for k in autotune.KNOBS + ("wide.pdl",)}
    knobs["source"] = "autotuner" if entry else "library defaults"
    return knobs


def run_reference(args, w):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = cpu_threads_for(w)
    steps_per_sample = args.cpu_sample_steps
    for _ in range(args.warmup):
        cpu_sample(w, 1, 1)  # touch pages / load library; short
    vals = []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        v, wall = cpu_sample(w, steps_per_sample, threads)
        vals.append(v)
    elapsed = time.perf_counter() - t_all
    value = float(np.mean(vals))
    sample = ("%d RK4 step(s) of the %s solve per thread, %d threads, FP64 C oracle port "
              "(oracle/nlse_oracle.c) of the reference CPU integrator" % (
                  steps_per_sample, w.name, threads))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * elapsed / max(1, args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": w.name, "grid": list(w.U.shape), "method": "2SHOC",
                   "bc": "MSD", "rk4_steps_per_sample": steps_per_sample,
                   "precision": "fp64 (reference CPU integrator)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample, "host_cpu": host_cpu(),
                         "port_vs_reference": PORT_VS_REFERENCE},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_gpu(args, w):
    import torch

    import nlsemagic_gb300 as ng
    from nlsemagic_gb300 import workloads as W

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    ng.load()
    n = w.points
    steps = w.steps
    prec = ng.PREC_MIXED

    # device-resident planar inputs
    Ur = torch.from_numpy(np.ascontiguousarray(w.U.real.ravel(order="F"))).cuda()
    Ui = torch.from_numpy(np.ascontiguousarray(w.U.imag.ravel(order="F"))).cuda()
    Vd = torch.from_numpy(np.ascontiguousarray(w.V.ravel(order="F"))).cuda()
    tuned = tune_for(args, w.U.shape, w.method, prec, w.BC)
    solver = ng.Solver(w.U.shape, method=w.method, precision=prec, BC=w.BC, s=w.s, a=w.a,
                       h2=w.h2, k=w.k)
    if args.graph_steps > 0:
        solver.set_graph_steps(args.graph_steps)
    stream = torch.cuda.ExternalStream(solver.stream)

    def job():
        solver.upload_device(Ur.data_ptr(), Ui.data_ptr(), Vd.data_ptr())
        solver.run(steps)

    t0 = time.perf_counter()
    for _ in range(args.warmup):
        job()
    solver.sync()
    torch.cuda.synchronize()
    log("warmup: %d jobs in %.2f s" % (args.warmup, time.perf_counter() - t0))
    barrier(world)

    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        barrier(world)
        start.record(stream)
        for _ in range(args.steps):
            job()
        end.record(stream)
        end.synchronize()
        torch.cuda.synchronize()
        barrier(world)
    t_ms = start.elapsed_time(end)
    log("timed: %d jobs in %.1f ms" % (args.steps, t_ms))
    t_ms = max_over_ranks(t_ms, world)
    clocks = clk.summary()
    pts = float(n) * steps * args.steps * world
    value = pts / (t_ms / 1000.0) / 1e9
    ms_per_step = t_ms / args.steps

    # accuracy + mass diagnostics of the last job
    sum2 = solver.sum_abs2()
    out = solver.download()
    mass0 = float(np.sum(np.abs(w.U) ** 2))
    mass_drift = abs(sum2 - mass0) / mass0

    # ---- end to end through the C ABI one-shot call (pinned host buffers)
    pin = lambda a: torch.from_numpy(a).pin_memory()  # noqa: E731
    hUr = pin(np.ascontiguousarray(w.U.real.ravel(order="F")))
    hUi = pin(np.ascontiguousarray(w.U.imag.ravel(order="F")))
    hV = pin(np.ascontiguousarray(w.V.ravel(order="F")))
    oR = torch.empty(n, dtype=torch.float64).pin_memory()
    oI = torch.empty(n, dtype=torch.float64).pin_memory()
    lib = ng.load()
    import ctypes
    dp = ctypes.POINTER(ctypes.c_double)
    P = lambda t: ctypes.cast(t.data_ptr(), dp)  # noqa: E731
    M_, N_, L_ = w.U.shape

    def e2e_call():
        rc = lib.NLSE3D_TAKE_STEPS_CUDA_MIXED(P(hUr), P(hUi), P(hV), P(oR), P(oI), w.s, w.a,
                                              w.h2, w.BC, steps, w.k, L_, N_, M_, w.method)
        if rc:
            raise RuntimeError(ng._lib.last_error())

    e2e_call()  # warm (workspace cached after this call)
    torch.cuda.synchronize()
    barrier(world)
    ke = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(ke):
        e2e_call()
    t_e2e = time.perf_counter() - t0
    log("e2e: %d calls in %.2f s" % (ke, t_e2e))
    t_e2e = max_over_ranks(t_e2e, world)
    e2e_value = float(n) * steps * ke * world / t_e2e / 1e9
    e2e_out = (oR.numpy() + 1j * oI.numpy()).reshape(w.U.shape, order="F")

    # ---- FP64 plain path on the same workload (for the mixed/FP64 ratio and
    # the error of the mixed path), a shorter run
    fp64 = None
    fp64_steps = steps if args.fp64_steps < 0 else args.fp64_steps
    if fp64_steps > 0 and rank == 0:
        s64 = ng.Solver(w.U.shape, method=w.method, precision=ng.PREC_DOUBLE, BC=w.BC, s=w.s,
                        a=w.a, h2=w.h2, k=w.k)
        if args.graph_steps > 0:
            s64.set_graph_steps(args.graph_steps)
        smx = ng.Solver(w.U.shape, method=w.method, precision=prec, BC=w.BC, s=w.s, a=w.a,
                        h2=w.h2, k=w.k)
        st64 = torch.cuda.ExternalStream(s64.stream)
        s64.upload_device(Ur.data_ptr(), Ui.data_ptr(), Vd.data_ptr())
        s64.run(max(1, args.graph_steps, 8))  # captures the graph outside the timed run
        s64.sync()
        s64.upload_device(Ur.data_ptr(), Ui.data_ptr(), Vd.data_ptr())
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st64)
        s64.run(fp64_steps)
        e1.record(st64)
        e1.synchronize()
        t64 = e0.elapsed_time(e1) / 1000.0
        smx.upload_device(Ur.data_ptr(), Ui.data_ptr(), Vd.data_ptr())
        smx.run(fp64_steps)
        u64 = s64.download()
        umx = smx.download()
        err = float(np.linalg.norm((umx - u64).ravel()) / np.linalg.norm(u64.ravel()))
        m64 = float(np.sum(np.abs(u64) ** 2))
        fp64 = {"value": float(n) * fp64_steps / t64 / 1e9, "unit": UNIT,
                "rk4_steps": fp64_steps,
                "roofline_frac_of_measured_hbm": float(n) * fp64_steps * BYTES_FP64 / t64 /
                1e9 / peaks()[0],
                "mass_rel_drift": abs(m64 - mass0) / mass0,
                "mixed_rel_l2_vs_oracle_fp64": err,
                "mixed_rel_l2_tolerance": 1e-6,
                "fp64_bit_identical_to_oracle": "by test (tests/test_config_parity_gpu.py, "
                                                "this grid, all 500 steps)"}
        vf, uf = fp64_solve(w, fp64_steps, fma=True)
        fp64["contracted"] = {"value": vf, "unit": UNIT, "speedup": vf / fp64["value"],
                              "rel_l2_vs_oracle_fp64": W.rel_l2(uf, u64),
                              "what": "NLSE_FLAG_FMA: the FP64 kernels compiled with "
                                      "multiply-add contraction (tolerance 1e-12)"}
        try:
            rates = fp64_rates()
            ops = FP64_OPS[(3, w.method)]
            fp64["fp64_rates"] = rates
            fp64["fp64_ops_per_point_step"] = ops
            fp64["fp64_issue_frac_of_measured_add_rate"] = fp64["value"] * 1e9 * ops / \
                rates["add_per_s"]
        except Exception as e:  # the probe is a report, not the measurement
            fp64["fp64_rates"] = {"error": str(e)}
        s64.close()
        smx.close()

    peak, peak_kind = peaks()
    achieved = value * BYTES_MODEL_MIXED / world  # GB/s per GPU (Gpt/s * B)
    traffic_ppt = read_traffic()
    # + 2 ingest conversions, + 1 refill of the x-face strips (3D 2SHOC) after
    # each upload
    from nlsemagic_gb300 import autotune as _at
    strips = w.U.ndim == 3 and w.method == 2 and _at.get_knob("wide.strips") == 1
    launches_per_job = steps * solver.launches_per_step + 2 + (1 if strips else 0)
    roof = {
        "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak,
        "traffic": (traffic_ppt * n / 4.0) if traffic_ppt else None,
        "peak_kind": peak_kind,
        "kernel": "RK4 stage (face-ghost, interior wide3d and face kernels; %d launches "
                  "per RK4 step, timed as CUDA graphs); achieved and traffic per average "
                  "stage" % solver.launches_per_step,
        "algorithmic_bytes_per_point_step": BYTES_MODEL_MIXED,
        "algorithmic_bytes_per_stage": BYTES_MODEL_MIXED / 4.0 * n,
        "design_bytes_per_point_step": BYTES_DESIGN_MIXED,
        "design_bytes_frac": value * BYTES_DESIGN_MIXED / world / peak,
        "traffic_bytes_per_point_step": traffic_ppt,
    }
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32-stage/f32x2-accumulate",
        "data": "synthetic (seeded vortex rings in a harmonic trap)",
        "config": {"workload": w.name, "grid": list(w.U.shape), "method": "2SHOC", "bc": "MSD",
                   "launch": "programmatic dependent launch (interior tiles overlap the face "
                   "kernels)" if args.pdl else "stream order",
                   "rk4_steps_per_job": steps, "k": w.k, "h": w.h,
                   "precision": "mixed (FP32 stages, compensated FP32 hi/lo state)",
                   "parallelism": "replicas x%d" % world,
                   "l2": "inputs (~1.9 GB working set) larger than L2; no flush",
                   "launch_knobs": tuned},
        "roofline": roof,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 3 * 8 * n,
                "d2h_bytes_per_step": 2 * 8 * n,
                "path": "C ABI NLSE3D_TAKE_STEPS_CUDA_MIXED, pinned host planar buffers",
                "same_result_as_value_path": bool(np.array_equal(e2e_out, out))},
        "gpu_launches": int(args.steps * launches_per_job),
        "clocks": clocks,
        "accuracy": {"mass_rel_drift_job": mass_drift},
    }
    if fp64:
        result["fp64_path"] = fp64
        result["mixed_over_fp64"] = value / world / fp64["value"]
    if rank == 0 and args.batch_solves > 0:
        result["batched"] = run_batched(args)
    if rank == 0 and args.serve_requests > 0:
        result["serving"] = run_serving(args)
    if rank == 0 and world == 1 and args.cpu_sample_steps > 0:
        threads = cpu_threads_for(w)
        v, wall = cpu_sample(w, args.cpu_sample_steps, threads)
        result["cpu_baseline"] = {
            "value": v, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d RK4 step(s) of the %s solve per thread (FP64 2SHOC), %d threads, C "
                      "oracle port of NLSE3D_TAKE_STEPS_2SHOC.c, %.1f s wall" % (
                          args.cpu_sample_steps, w.name, threads, wall),
            "host_cpu": host_cpu(), "port_vs_reference": PORT_VS_REFERENCE}
    if rank == 0:
        print(json.dumps(result), flush=True)
    solver.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_batched(args):
    """Uneven batch (512 solves: 60% 1D N in [256, 16384], 40% 2D side in
    [64, 512], CD/2SHOC, mixed precision, 1000 steps): one persistent launch
    for all solves vs one solve at a time through resident solvers with
    graph-captured chunks."""
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300 import workloads as W
    insts = W.batch_instances(count=args.batch_solves, steps=args.batch_steps)
    pts = float(sum(i.U.size for i in insts)) * args.batch_steps
    w0 = insts[0]  # warm the persistent kernel on a tiny batch
    b = ng.Batch(1 << 26)
    b.add(w0.U, w0.V, w0.s, w0.a, w0.h * w0.h, w0.BC, 2, w0.k, w0.method, ng.PREC_MIXED)
    b.run(2)
    b.sync()
    b.close()
    b = ng.Batch(sum(ng.Batch.bytes_for(i.U.shape, ng.PREC_MIXED) for i in insts) + (1 << 20),
                 max_solves=len(insts) + 1)
    for i in insts:
        b.add(i.U, i.V, i.s, i.a, i.h * i.h, i.BC, args.batch_steps, i.k, i.method, ng.PREC_MIXED)
    t0 = time.perf_counter()
    b.run(args.batch_steps)
    b.sync()
    t_batch = time.perf_counter() - t0
    launches = b.last_launches
    b.close()
    log("batched: %d solves x %d steps in %.3f s" % (len(insts), args.batch_steps, t_batch))
    # one solve at a time (a subset when large, scaled by its share of work)
    # (solvers created and uploaded beforehand: only their launches are timed)
    sub = insts[:args.batch_seq_sample] if args.batch_seq_sample else insts
    solvers = []
    for i in sub:
        sv = ng.Solver(i.U.shape, method=i.method, precision=ng.PREC_MIXED, BC=i.BC, s=i.s, a=i.a,
                       h2=i.h * i.h, k=i.k)
        sv.upload(i.U, i.V)
        sv.run(sv_warm := 8)  # captures the chunk graph outside the timed loop
        sv.sync()
        solvers.append(sv)
    t0 = time.perf_counter()
    for sv in solvers:
        sv.run(args.batch_steps)
        sv.sync()
    t_seq = time.perf_counter() - t0
    for sv in solvers:
        sv.close()
    del sv_warm
    pts_sub = float(sum(i.U.size for i in sub)) * args.batch_steps
    log("one-at-a-time: %d solves in %.3f s" % (len(sub), t_seq))
    v_batch = pts / t_batch / 1e9
    v_seq = pts_sub / t_seq / 1e9
    return {"workload": "%d uneven 1D/2D solves, %d RK4 steps, mixed precision" % (
                len(insts), args.batch_steps),
            "value": v_batch, "unit": UNIT, "seconds": t_batch, "launches": launches,
            "one_at_a_time": {"value": v_seq, "unit": UNIT, "solves_timed": len(sub),
                              "seconds": t_seq},
            "speedup": v_batch / v_seq}


def oracle_trajectory(w, marks, precision):
    """The C oracle's state after each number of RK4 steps in marks (chained
    calls, same bits as one call), the solve spread over the host's cores."""
    import oracle
    oracle.set_threads(os.cpu_count() or 1)
    out, U, done = {}, w.U, 0
    try:
        for m in marks:
            U = oracle.take_steps(U, w.V, w.s, w.a, w.h2, w.BC, m - done, w.k, method=w.method,
                                  precision=precision, flags=oracle.MSD_GUARD)
            done = m
            out[m] = U
    finally:
        oracle.set_threads(1)
    return out


def fp64_rates():
    """Measured FP64 issue rates of this GPU (nlse_device_fp64_rates)."""
    import ctypes

    import nlsemagic_gb300 as ng
    fma, add = ctypes.c_double(), ctypes.c_double()
    ng._lib.check(ng.load().nlse_device_fp64_rates(ctypes.byref(fma), ctypes.byref(add)))
    return {"fma_per_s": fma.value, "add_per_s": add.value,
            "fma_tflops": 2 * fma.value / 1e12,
            "how": "timed kernel, 8 independent chains per thread, 16 blocks of 256 per SM"}


def fp64_solve(w, steps, graph_steps=10, fma=False):
    """Gpt-steps/s of the FP64 class on workload w (resident solver, graphs,
    CUDA events on the solver stream) and its final state; fma: the
    contracted kernels (NLSE_FLAG_FMA)."""
    import torch

    import nlsemagic_gb300 as ng
    flags = ng.FLAG_MSD_GUARD | (ng.FLAG_FMA if fma else 0)
    with ng.Solver(w.U.shape, method=w.method, precision=ng.PREC_DOUBLE, BC=w.BC, s=w.s, a=w.a,
                   h2=w.h2, k=w.k, flags=flags) as sv:
        sv.set_graph_steps(graph_steps)
        sv.upload(w.U, w.V)
        sv.run(max(1, min(steps, graph_steps)))  # captures the graph
        sv.sync()
        sv.upload(w.U, w.V)
        st = torch.cuda.ExternalStream(sv.stream)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        sv.run(steps)
        e1.record(st)
        e1.synchronize()
        t = e0.elapsed_time(e1) / 1000.0
        return float(w.points) * steps / t / 1e9, sv.download()


def run_fp64(args):
    """The exact FP64 class against its compute bound: the vortex-ring solve
    (--grid, --fp64-steps RK4 steps) and the dark-vortex solve (--grid2d,
    200 steps), Gpt-steps/s and the fraction of the measured FP64 add rate
    their instruction counts imply."""
    from nlsemagic_gb300 import workloads as W
    rates = fp64_rates()
    out = {"fp64_rates": rates}
    steps3 = args.fp64_steps if args.fp64_steps > 0 else 20
    for name, w, steps in (("3d_2shoc", W.vortex_rings_3d(n=args.grid, method=2), steps3),
                           ("2d_2shoc", W.dark_vortices_2d(n=args.grid2d), 200)):
        v, u = fp64_solve(w, steps)
        vf, uf = fp64_solve(w, steps, fma=True)
        ops = FP64_OPS[(w.ndim, w.method)]
        out[name] = {"workload": w.name, "rk4_steps": steps, "value": v, "unit": UNIT,
                     "fp64_ops_per_point_step": ops,
                     "fp64_issue_frac_of_measured_add_rate": v * 1e9 * ops / rates["add_per_s"],
                     "hbm_frac_of_measured": v * BYTES_FP64 / peaks()[0],
                     "contracted": {"value": vf, "unit": UNIT, "speedup": vf / v,
                                    "rel_l2_vs_exact_fp64": W.rel_l2(uf, u)}}
        log("%s: %s" % (name, json.dumps(out[name])))
    return out


def run_configs(args):
    """The reference's CPU-runnable case and its 2D case, through resident
    solvers (graph-captured chunks), in every precision class: configuration
    1 (1D CD grey soliton, 1024 points, 1000 steps) and configuration 2 (2D
    2SHOC dark vortices, 512^2 unless --grid2d, 2000 steps unless
    --config2-steps).  Gpt-steps/s per class, timed after a warm-up run that
    captures the graphs; every class's result against the C oracle (FP64 and
    FP32 bit for bit, relative L2 distance to the FP64 oracle) and the mixed
    class's distance at checkpoints through the run."""
    import nlsemagic_gb300 as ng
    from nlsemagic_gb300 import workloads as W
    w1 = W.grey_soliton_1d()
    w2 = W.dark_vortices_2d(n=args.grid2d, steps=args.config2_steps)
    out = {}
    for name, w, steps in (("config1", w1, w1.steps), ("config2", w2, args.config2_steps)):
        marks = sorted({max(1, steps // 8), max(1, steps // 4), max(1, steps // 2), steps})
        t0 = time.perf_counter()
        ref = oracle_trajectory(w, marks, 2)
        ref32 = oracle_trajectory(w, [steps], 1)[steps]
        t_oracle = time.perf_counter() - t0
        res = {"workload": w.name, "rk4_steps": steps,
               "oracle": "C oracle (FP64 and FP32, bit-identical to the reference C "
                         "integrators), %d host threads, %.1f s" % (os.cpu_count() or 1, t_oracle)}
        mass0 = W.mass(w.U, w.h, w.ndim)
        for prec, label in ((ng.PREC_DOUBLE, "fp64"), (ng.PREC_MIXED, "mixed"),
                            (ng.PREC_SINGLE, "fp32")):
            knobs = tune_for(args, w.U.shape, w.method, prec, w.BC)
            with ng.Solver(w.U.shape, method=w.method, precision=prec, BC=w.BC, s=w.s, a=w.a,
                           h2=w.h2, k=w.k) as sv:
                sv.upload(w.U, w.V)
                sv.run(min(steps, 16))  # captures the chunk graphs
                sv.sync()
                sv.upload(w.U, w.V)
                t0 = time.perf_counter()
                sv.run(steps)
                sv.sync()
                t = time.perf_counter() - t0
                final = sv.download()
                r = {"value": w.U.size * steps / t / 1e9, "unit": UNIT,
                     "launches_per_step": sv.launches_per_step, "launch_knobs": knobs,
                     "rel_l2_vs_oracle_fp64": W.rel_l2(final, ref[steps]),
                     "mass_rel_drift": abs(W.mass(final, w.h, w.ndim) - mass0) / mass0}
                if label == "fp64":
                    r["bit_identical_to_oracle"] = bool(np.array_equal(final, ref[steps]))
                elif label == "fp32":
                    r["bit_identical_to_fp32_oracle"] = bool(np.array_equal(final, ref32))
                else:
                    r["tolerance"] = 1e-6
                    sv.upload(w.U, w.V)
                    done, by_step = 0, {}
                    for m in marks:
                        sv.run(m - done)
                        done = m
                        by_step[str(m)] = W.rel_l2(sv.download(), ref[m])
                    r["rel_l2_vs_oracle_fp64_by_step"] = by_step
                res[label] = r
        out[name] = res
        log("%s: %s" % (name, json.dumps(res)))
    return out


def fifo_latencies(arrivals, service):
    """Latencies of a single first-come-first-served server with the given
    arrival times and per-request service times."""
    clock, lat = 0.0, []
    for a, d in sorted(zip(arrivals, service)):
        clock = max(clock, a) + d
        lat.append(clock - a)
    return lat


def run_serving(args):
    """Continuous-batching request loop on a seeded Poisson stream with the
    serving configuration's distributions (dims 1D:2D:3D = 5:4:1, sizes
    log-uniform 1D 512-65536, 2D 64^2-1024^2, 3D 32^3-256^3, steps 100-5000,
    FP64 or mixed 50/50), scaled down from 20,000 requests to
    --serve-requests.  First every request is queued at t = 0 (saturated:
    the loop's capacity); then the same stream arrives at several offered
    rates (fractions of that capacity, or --serve-rates).  Against: one solve
    at a time, first come first served (each request through its own Solver:
    create, upload, run, download, release), whose latencies at each rate
    follow from the measured service times of a back-to-back pass."""
    from nlsemagic_gb300 import workloads as W
    from nlsemagic_gb300.serve import Server, percentile, serve_sequential
    full = 20000
    reqs = W.serving_requests(count=args.serve_requests, rate=1.0,
                              n1=(512, 65536), n2=(64, 1024), n3=(32, args.serve_max3d),
                              steps=(100, args.serve_max_steps))
    pool = args.serve_pool_gb << 30

    def server(order="srpt"):
        return Server(pool_bytes=pool, chunk_steps=args.serve_chunk, solo_bytes=pool, order=order)

    seq, seq_done = serve_sequential(reqs, time_scale=0.0)
    service = [c.done - c.admitted for c in seq_done]  # in arrival order
    log("one at a time: %s" % json.dumps(seq))
    srv = server()
    sat, _ = srv.serve(reqs, time_scale=0.0)
    srv.close()
    log("served (saturated): %s" % json.dumps(sat))
    srv = Server(pool_bytes=pool, chunk_steps=args.serve_chunk, solo_bytes=pool, per_class=False)
    sat1, _ = srv.serve(reqs, time_scale=0.0)
    srv.close()
    log("served (saturated, one large solve at a time): %s" % json.dumps(sat1))
    if args.serve_rates:
        rates = [float(x) for x in args.serve_rates.split(",")]
    else:
        rates = [f * sat["requests_per_s"] for f in (0.3, 0.6, 0.9)]
    arrivals1 = [r.arrival for r in sorted(reqs, key=lambda r: r.arrival)]
    per_rate = []
    for rate in rates:
        srv = server()
        live, _ = srv.serve(reqs, time_scale=1.0 / rate)
        srv.close()
        lat = fifo_latencies([a / rate for a in arrivals1], service)
        fcfs = {"p50_latency_s": percentile(lat, 50), "p99_latency_s": percentile(lat, 99)}
        row = {"rate_per_s": rate,
               "server": {k: live[k] for k in ("p50_latency_s", "p99_latency_s", "p50_queue_s",
                                               "p99_queue_s", "gpt_steps_per_s", "wall_s")},
               "one_at_a_time_fcfs": fcfs,
               "server_p99_le_fcfs_p99": live["p99_latency_s"] <= fcfs["p99_latency_s"]}
        per_rate.append(row)
        log("rate %.2f/s: %s" % (rate, json.dumps(row)))
    return {"requests": len(reqs), "stream_size": full,
            "scaled_down_by": full / float(len(reqs)),
            "dims_ratio": "5:4:1", "sizes": {"1d": [512, 65536], "2d": [64, 1024],
                                             "3d": [32, args.serve_max3d]},
            "steps": [100, args.serve_max_steps], "precision": "FP64 or mixed, 50/50",
            "chunk_steps": args.serve_chunk,
            "policy": "batched launch for 1D/2D/small 3D plus one large 3D solve of each "
                      "precision class at a time, shortest remaining work first",
            "value": sat["gpt_steps_per_s"], "unit": UNIT,
            "requests_per_s": sat["requests_per_s"],
            "saturated_one_large_solve_at_a_time": {
                "value": sat1["gpt_steps_per_s"], "unit": UNIT,
                "requests_per_s": sat1["requests_per_s"],
                "p99_latency_s": sat1["p99_latency_s"]},
            "rates": per_rate,
            "one_at_a_time": {"value": seq["gpt_steps_per_s"], "unit": UNIT,
                              "requests_per_s": seq["requests_per_s"]},
            "throughput_over_one_at_a_time": sat["gpt_steps_per_s"] / seq["gpt_steps_per_s"]
            if seq["gpt_steps_per_s"] else None,
            "requests_per_s_over_one_at_a_time": sat["requests_per_s"] / seq["requests_per_s"]
            if seq["requests_per_s"] else None}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--grid", type=int, default=320)
    ap.add_argument("--rk4-steps", type=int, default=500)
    ap.add_argument("--graph-steps", type=int, default=0,
                    help="RK4 steps per captured graph (0: the autotuned or default knob)")
    ap.add_argument("--tune", type=int, default=1, choices=[0, 1],
                    help="1: tune the launch knobs of each problem class (cached) and apply them")
    ap.add_argument("--fp64-steps", type=int, default=-1,
                    help="RK4 steps of the FP64 comparison run (-1: the workload's own)")
    ap.add_argument("--cpu-sample-steps", type=int, default=1)
    ap.add_argument("--batch-solves", type=int, default=512)
    ap.add_argument("--batch-steps", type=int, default=1000)
    ap.add_argument("--batch-seq-sample", type=int, default=0,
                    help="time only the first N solves one at a time (0: all)")
    ap.add_argument("--serve-requests", type=int, default=100,
                    help="requests of the serving stream (the configuration names 20,000)")
    ap.add_argument("--serve-rates", default="",
                    help="offered rates, requests/s, comma-separated (default: 0.3, 0.6 and "
                         "0.9 of the saturated rate)")
    ap.add_argument("--serve-chunk", type=int, default=100)
    ap.add_argument("--serve-max3d", type=int, default=256)
    ap.add_argument("--serve-max-steps", type=int, default=5000)
    ap.add_argument("--serve-pool-gb", type=int, default=64)
    ap.add_argument("--pdl", type=int, default=1, choices=[0, 1],
                    help="3D 2SHOC stage kernels: 1 overlap through programmatic dependent "
                         "launch, 0 plain stream order (same bits)")
    ap.add_argument("--only", choices=["batched", "serving", "configs", "fp64"], default=None,
                    help="run one auxiliary section alone and print its JSON (for profiling)")
    ap.add_argument("--grid2d", type=int, default=512, help="side of configuration 2")
    ap.add_argument("--config2-steps", type=int, default=2000)
    args = ap.parse_args()
    if args.impl == "ours":
        from nlsemagic_gb300 import autotune
        autotune.set_knob("wide.pdl", args.pdl)
    if args.only:
        import nlsemagic_gb300 as ng
        ng.load()
        out = {"batched": run_batched, "serving": run_serving, "configs": run_configs,
               "fp64": run_fp64}[args.only](args)
        print(json.dumps({"section": args.only, **out}), flush=True)
        return
    from nlsemagic_gb300 import workloads as W
    rank, world, _ = dist_env()
    w = W.vortex_rings_3d(seed=1002 + rank, n=args.grid, method=2, steps=args.rk4_steps)
    if args.impl == "reference":
        run_reference(args, w)
    else:
        run_gpu(args, w)


if __name__ == "__main__":
    main()

#!/usr/bin/env python3
"""Headline benchmark of tdbem-gb300: DOF*steps/s of a full transient solve.

A bench step is one pass of the hot path over the workload: assembly of every
G^k/H^k level (collocation node x element x level quadrature) followed by the
whole time march (history convolution + H^0 solve for every step).  Default
workload: spherical cavity of radius 1 in a full space, 6x16x16 cubed-sphere
quads (1536 elements, 1538 nodes, 4614 DOF), uniform step pressure, mu = 1,
nu = 0.25, rho = 1, dt = 0.6 h / c_p, 400 steps, alpha = (0.25, 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|mixed]
    python bench.py --workload sphere_6x16x16_batch64   (64 load cases, batched march)
    python bench.py --impl reference ...   (the reference's algorithm on the host cores)

Batched workloads march many load cases on one mesh: a step is the assembly
plus one batched march of every case (seeded Gaussian pulses on random
4-element patches); DOF*steps counts every case.

Multi-GPU runs (torchrun, one process per GPU) are independent replicas of the
workload (the path does not shard): value = total DOF*steps of all ranks / the
slowest rank's time.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "td-bem_gb300"))

import numpy as np  # noqa: E402

ALPHA = (0.25, 0.0)
WORKLOADS = {
    "sphere_6x16x16": dict(kind="sphere", n=16, numstep=400),
    "sphere_6x24x24": dict(kind="sphere", n=24, numstep=500),
    "sphere_6x8x8": dict(kind="sphere", n=8, numstep=200),
    "bar_1x1x4_q2": dict(kind="bar", numstep=200),
    "sphere_6x16x16_batch64": dict(kind="sphere", n=16, numstep=400, cases=64),
    "sphere_6x8x8_batch64": dict(kind="sphere", n=8, numstep=200, cases=64),
    "bars32_group": dict(kind="bars", count=32, numstep=200),
}


def group_models(count, numstep, seed=0):
    """Bars 1 x 1 x L, L ~ U{2..8}, 1..3 quads per unit length (seeded)."""
    from tdbem import meshes
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        L = int(rng.integers(2, 9))
        p = int(rng.integers(1, 4))
        out.append(meshes.bar(1, 1, L, per_unit=p, numstep=numstep))
    return out
METRIC = "DOF*steps/s"


def workload_config(name, model, M, world):
    """The workload's identity, the same in both arms (method details go elsewhere)."""
    cases = WORKLOADS[name].get("cases", 0)
    D = model.ndof
    fp64_gb = 2 * (M + 1) * D * D * 8 / 1e9
    return {"workload": name, "dof": D, "steps": model.numstep, "max_step": M,
            "alpha": list(ALPHA), "load_cases": max(1, cases), "parallelism": f"replicas{world}",
            "l2": f"inputs larger than L2: the FP64 level store is {fp64_gb:.1f} GB "
                  "(the mixed form's FP32 store and merged BF16 planes: 3/4 of it)"}


def make_model(name):
    from tdbem import meshes
    w = WORKLOADS[name]
    if w["kind"] == "sphere":
        return meshes.cubed_sphere(w["n"], numstep=w["numstep"])
    return meshes.bar(1, 1, 4, per_unit=2, numstep=w["numstep"])


# --------------------------------------------------------------------------
# distributed plumbing (replicas only)
# --------------------------------------------------------------------------
class Dist:
    """Replicas of the workload, one process per GPU (torchrun): a barrier around the
    timed region and the slowest rank's time.  NCCL on GPUs, gloo on CPU-only hosts."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        self.device = "cpu"
        if self.world > 1:
            import torch
            import torch.distributed as dist
            if torch.cuda.is_available():
                torch.cuda.set_device(self.local)
                self.device = "cuda"
            dist.init_process_group("nccl" if self.device == "cuda" else "gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device=self.device)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device=self.device)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 9:
                    rows.append(p)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        loaded = [x for x in sm if smax and x > 0.5 * max(smax)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def measure_fp_peaks(torch):
    """FP64 and FP32 (no TF32) GEMM throughput on this GPU, TFLOP/s, via cuBLAS (best of 3)."""
    out = {}
    for name, dt, n in (("fp64_tflops", torch.float64, 4096), ("fp32_tflops", torch.float32, 8192)):
        prev = torch.backends.cuda.matmul.allow_tf32
        torch.backends.cuda.matmul.allow_tf32 = False
        a = torch.randn(n, n, dtype=dt, device="cuda")
        b = torch.randn(n, n, dtype=dt, device="cuda")
        torch.mm(a, b)
        best = 0.0
        for _ in range(3):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.mm(a, b)
            e1.record()
            e1.synchronize()
            best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12)
        torch.backends.cuda.matmul.allow_tf32 = prev
        out[name] = best
        del a, b
    torch.cuda.empty_cache()
    return out


def ncu_traffic():
    """Per-launch DRAM bytes of the dominant kernels from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f)
    except OSError:
        return {}


# --------------------------------------------------------------------------
# CPU baseline: the reference's algorithm (the oracle restatement) on a sample
# --------------------------------------------------------------------------
def cpu_sample(model, M, numstep, a1, a2, nthreads, cases=0):
    """Estimate the reference CPU path's time for the whole workload from a bounded sample.

    assembly: ElastoDynamicsT::G_H_Driver on the first R collocation rows at a mid step
      (its cost does not depend on the step), scaled to all rows and M steps;
    marching: Solve_Averaging steps at full size D on a synthetic level store (dense
      random levels, diagonal level 0/1 so the LHS factorisation is cheap) with 2 and 5
      levels, giving the per-step cost c0 + c1 * (level terms); summed over the
      workload's steps with the reference's level-term count;
    LU: the KSPSolve stand-in's dense LU timed at n = 2000 and scaled by (D/2000)^3,
      once per distinct LHS.
    With cases > 0 (a batch of load cases) the reference runs once per case; the
    estimate keeps its levels and LU from the first case (one assembly, one LU,
    cases x marching), which favours the reference."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    D = model.ndof
    o = oracle.Oracle(model, nthreads=nthreads)
    R = min(model.nnd, 4 * nthreads)
    t0 = time.perf_counter()
    o.gh_driver(max(1, M // 2) * model.dt, model.dt, 0, R - 1)
    t_rows = time.perf_counter() - t0
    t_asm = t_rows * (model.nnd / R) * M

    rng = np.random.default_rng(0)

    def march_cost(m_s, steps):
        G = rng.standard_normal((m_s + 1, D, D)) * 1e-3
        H = rng.standard_normal((m_s + 1, D, D)) * 1e-3
        for k in (0, 1):
            H[k] = np.diag(1.0 + rng.random(D))
        u = np.zeros((steps + 2, D))
        t = np.zeros((steps + 2, D))
        ubc = np.zeros(0, np.int32)
        fbc = np.arange(D, dtype=np.int32)
        fv = np.ones(D)
        t0 = time.perf_counter()
        oracle.march_range(D, m_s, G, H, ubc, np.zeros(0), fbc, fv, a1, a2, 2, steps, u, t,
                           nthreads=nthreads)
        return time.perf_counter() - t0

    def terms(s, m):
        """Level-term pairs of Solve_Averaging at solve step s (SolverStepLinearT.cpp:408-482)."""
        if s < 2:
            return 0
        return 1 + max(0, min(s + 1, m) - 2) + max(0, min(s - 1, m)) + max(0, min(s - 2, m) + 1)

    m_a, m_b, n_a, n_b = 2, 5, 9, 13
    ta = march_cost(m_a, n_a)
    tb = march_cost(m_a, n_b)
    tc = march_cost(m_b, n_a)
    td = march_cost(m_b, n_b)
    per_a = (tb - ta) / (n_b - n_a)  # saturated steps: 3*m term pairs
    per_b = (td - tc) / (n_b - n_a)
    c1 = max(0.0, (per_b - per_a) / (terms(40, m_b) - terms(40, m_a)))
    c0 = max(0.0, per_a - c1 * terms(40, m_a))
    t_march = sum(c0 + c1 * terms(s, M) for s in range(1, numstep))
    n_lu = 2 if a1 != 0 or a2 != 0 else 1
    A = rng.standard_normal((2000, 2000))
    t0 = time.perf_counter()
    oracle.lu_factor(A, nthreads)
    t_lu = (time.perf_counter() - t0) * (D / 2000.0) ** 3 * n_lu
    nc = max(1, cases)
    total = t_asm + nc * t_march + t_lu
    return {"seconds": total, "assembly_s": t_asm, "march_s": nc * t_march, "lu_s": t_lu,
            "value": nc * D * numstep / total,
            "sample_fractions": {"assembly_rows": R / model.nnd, "assembly_levels": 1.0 / M,
                                 "march": "4 short marches on 2- and 5-level stores at full D "
                                          "(per-term cost fitted, not the workload's levels)",
                                 "lu_size": 2000.0 / D},
            "sample": (f"G_H_Driver on {R} of {model.nnd} rows at one step scaled to all rows "
                       f"x {M} steps; Solve_Averaging steps at D={D} on synthetic {m_a}- and "
                       f"{m_b}-level stores fitted to c0+c1*terms and summed over {numstep} "
                       f"steps; dense LU timed at n=2000 scaled by (D/2000)^3 x {n_lu}"
                       + (f"; {nc} load cases: one assembly and LU, {nc} marches" if cases
                          else ""))}


def run_reference(args, dist):
    if dist.rank != 0:
        return 0
    model = make_model(args.workload)
    M = model.max_step()
    nthreads = os.cpu_count() or 1
    cases = WORKLOADS[args.workload].get("cases", 0)
    vals = []
    last = None
    for i in range(args.warmup + args.steps):
        r = cpu_sample(model, M, model.numstep, *ALPHA, nthreads, cases)
        if i >= args.warmup:
            vals.append(r["value"])
            last = r
    value = statistics.median(vals)
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * max(1, cases) * model.ndof * model.numstep / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": workload_config(args.workload, model, M, args.gpus),
            "method": {"precision": "fp64", "solver": "the oracle port of the reference's "
                       "G_H_Driver, Solve_Averaging and dense LU, on the host cores"},
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": nthreads,
                             "kind": "port, extrapolated", "sample": last["sample"],
                             "sample_fractions": last["sample_fractions"]},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "estimate_seconds": {k: last[k] for k in ("assembly_s", "march_s", "lu_s")}}
    print(json.dumps(line))
    return 0


# --------------------------------------------------------------------------
# our arm
# --------------------------------------------------------------------------
def compare_batch(lib, torch, ctx, model, trac, amp, ms_step, check=(0, 1, 2)):
    """Plain FP64 form of a batched workload: one FP64 assembly and one FP64 march
    per case (timed on the first case), and the batch's error on a few cases."""
    from tdbem import loads
    D, n, nc = model.ndof, model.numstep, trac.shape[0]
    ub, tb = ctx.march_batch(trac, amp)
    errs_u, errs_t = [], []
    with lib.Context(model) as c64:
        c64.set_alpha(*ALPHA)
        s64 = torch.cuda.ExternalStream(c64.stream)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record(s64)
        c64.assemble(precision=lib.FP64)
        ev[1].record(s64)
        for i, c in enumerate(check):
            c64.set_bc(*loads.single_case_bc(model, trac[c]))
            c64.set_load_history(amp[c])
            u, t = c64.march()
            if i == 0:
                ev[2].record(s64)
                ev[2].synchronize()
                t_asm = ev[0].elapsed_time(ev[1])
                t_march = ev[1].elapsed_time(ev[2])
            errs_u.append(float(np.linalg.norm(ub[:, c] - u) / np.linalg.norm(u)))
            errs_t.append(float(np.linalg.norm(tb[:, c] - t) / np.linalg.norm(t)))
    ms64 = t_asm + nc * t_march
    return {"plain_fp64_value": nc * D * n / (ms64 / 1e3), "plain_fp64_ms_per_step": ms64,
            "plain_fp64_assembly_ms": t_asm, "plain_fp64_march_ms_per_case": t_march,
            "speedup_vs_plain_fp64": ms64 / ms_step, "cases_checked": list(check),
            "u_rel_l2_err": max(errs_u), "t_rel_l2_err": max(errs_t)}


def compare_fixed_cap(lib, model):
    """The traction-unknown path of the mixed march at the workload's size: the same
    cavity with the displacement of its nodes above z = 0.7 prescribed (zero) and the
    pressure elsewhere, so that the march solves for tractions at the cap's dofs;
    the mixed form's u and t errors against the plain FP64 form."""
    import dataclasses
    cap = np.flatnonzero(model.coords[:, 2] > 0.7)
    udofs = (3 * cap[:, None] + np.arange(3)).reshape(-1).astype(np.int32)
    keep = ~np.isin(model.fbc_dofs, udofs)
    m = dataclasses.replace(model, ubc_dofs=udofs, ubc_vals=np.zeros(len(udofs)),
                            fbc_dofs=np.ascontiguousarray(model.fbc_dofs[keep]),
                            fbc_vals=np.ascontiguousarray(model.fbc_vals[keep]))
    out = {}
    for prec in (lib.FP64, lib.MIXED):
        with lib.Context(m) as c:
            c.set_alpha(*ALPHA)
            c.assemble(precision=prec)
            out[prec] = c.march()
    (u64, t64), (u32, t32) = out[lib.FP64], out[lib.MIXED]
    return {"prescribed_displacement_dofs": int(len(udofs)),
            "u_rel_l2_err": float(np.linalg.norm(u32 - u64) / np.linalg.norm(u64)),
            "t_rel_l2_err": float(np.linalg.norm(t32 - t64) / np.linalg.norm(t64)),
            "t_rel_l2_err_at_cap": float(np.linalg.norm((t32 - t64)[:, udofs]) /
                                         np.linalg.norm(t64[:, udofs]))}


def run_ours(args, dist):
    import torch
    from tdbem import lib

    dev = dist.local if dist.world > 1 else 0
    torch.cuda.set_device(dev)
    torch.cuda.init()
    lib.load()
    prec = lib.FP64 if args.precision == "fp64" else lib.MIXED
    if WORKLOADS[args.workload]["kind"] == "bars":
        return run_group(lib, torch, args, dist)
    model = make_model(args.workload)
    D, nsteps = model.ndof, model.numstep
    cases = WORKLOADS[args.workload].get("cases", 0)
    nc = max(1, cases)
    trac = amp = None
    if cases:
        if prec != lib.MIXED:
            raise SystemExit("batched workloads march FP32 levels: use --precision mixed")
        from tdbem import loads
        trac, amp = loads.gaussian_patch_cases(model, cases, seed=0)
    ctx = lib.Context(model)
    ctx.set_alpha(*ALPHA)
    engine = lib.ENGINE_TCGEN05 if args.engine == "tcgen05" else lib.ENGINE_MMA_SYNC
    refine = args.refine if args.refine is not None else 0
    march_engine = lib.ENGINE_TCGEN05 if args.march_engine == "tcgen05" else lib.ENGINE_FP32
    ctx.set_march_options(args.block, refine)
    ctx.set_march_engine(march_engine)
    ctx.set_batch_options(engine, refine)
    stream = torch.cuda.ExternalStream(ctx.stream)

    def job():
        ctx.assemble(precision=prec)
        if cases:
            ctx.march_batch(trac, amp, to_host=False)
        else:
            ctx.march(to_host=False)

    for _ in range(args.warmup):
        job()
    torch.cuda.synchronize()
    dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    n0 = ctx.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        job()
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    dist.barrier()
    clk = clocks.stop()
    launches = ctx.launch_count() - n0
    ms_total = dist.max(e0.elapsed_time(e1))
    ms_step = ms_total / args.steps
    value = nc * D * nsteps * args.steps * dist.world / (ms_total / 1000.0)

    # untimed profiling pass: per-kernel-class device time and algorithmic units
    ctx.set_profiling(True)
    job()
    stats = ctx.kernel_stats()
    ctx.set_profiling(False)
    phase = ctx.timings()

    # end to end through the C ABI with host buffers (create/copy in, solve, copy out)
    e2e_times = []
    e2e_value = None
    h2d = model.coords.nbytes + model.ien.astype(np.int32).nbytes + \
        model.fbc_dofs.nbytes + model.fbc_vals.nbytes + model.ubc_dofs.nbytes + \
        model.ubc_vals.nbytes
    d2h = 2 * (nsteps + 1) * nc * D * 8
    if cases:
        h2d += trac.nbytes + amp.nbytes
    for _ in range(args.e2e_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with lib.Context(model) as c2:
            c2.set_alpha(*ALPHA)
            c2.set_march_options(args.block, refine)
            c2.set_march_engine(march_engine)
            c2.set_batch_options(engine, refine)
            c2.assemble(precision=prec)
            if cases:
                c2.march_batch(trac, amp)
            else:
                c2.march()
        t1 = time.perf_counter()
        e2e_times.append(t1 - t0)
    if e2e_times:
        e2e_s = dist.max(statistics.median(e2e_times))
        e2e_value = nc * D * nsteps * dist.world / e2e_s
    level_gb = ctx.level_bytes(prec) / 1e9
    M = ctx.M
    # the plain FP64 form on the same workload: its time, and the mixed form's error
    compare = None
    if cases and not args.no_compare:
        compare = compare_batch(lib, torch, ctx, model, trac, amp, ms_step)
    elif prec == lib.MIXED and not args.no_compare:
        u32, t32 = ctx.march()  # histories of the mixed form (levels already assembled)
        ctx.close()  # its level stores make room for the FP64 ones (6x24x24: 125 + 158 GB)
        with lib.Context(model) as c64:
            c64.set_alpha(*ALPHA)
            c64.assemble(precision=lib.FP64)
            c64.march(to_host=False)
            torch.cuda.synchronize()
            s64 = torch.cuda.ExternalStream(c64.stream)
            a0 = torch.cuda.Event(enable_timing=True)
            a1 = torch.cuda.Event(enable_timing=True)
            a0.record(s64)
            c64.assemble(precision=lib.FP64)
            u64, t64 = c64.march()
            a1.record(s64)
            a1.synchronize()
            ms64 = a0.elapsed_time(a1)
        compare = {"plain_fp64_value": D * nsteps / (ms64 / 1e3),
                   "plain_fp64_ms_per_step": ms64,
                   "speedup_vs_plain_fp64": (D * nsteps / (ms_step / 1e3)) / (D * nsteps / (ms64 / 1e3)),
                   "u_rel_l2_err": float(np.linalg.norm(u32 - u64) / np.linalg.norm(u64)),
                   "t_rel_l2_err": float(np.linalg.norm(t32 - t64) / np.linalg.norm(t64))}
    ctx.close()
    if compare is not None and not cases and WORKLOADS[args.workload]["kind"] == "sphere":
        compare["fixed_cap"] = compare_fixed_cap(lib, model)

    if dist.rank != 0:
        return 0
    peaks, peak_kind = measured_peaks()
    peaks.update(measure_fp_peaks(torch))
    traffic = ncu_traffic()
    # the dominant single kernel: "factor" (the inverses, ~440 kernels each, two running
    # side by side next to the assembly) and "aux" are composites, not one kernel
    dom = max((k for k in stats if k not in ("factor", "aux")), key=lambda k: stats[k]["ms"])
    st = stats[dom]
    if dom == "conv_batch":
        # split-BF16 GEMM: 3 BF16 MMA products per useful FP32 product
        kname_b = "k_conv_tc (tcgen05)" if args.engine == "tcgen05" else "k_conv_mma (mma.sync)"
        mma_tf = 3.0 * st["flops"] / (st["ms"] / 1e3) / 1e12
        gbs = st["bytes"] / (st["ms"] / 1e3) / 1e9
        f_t, f_h = mma_tf / peaks["bf16_tflops"], gbs / peaks["hbm_gbs"]
        if f_t >= f_h:
            roof = {"bound": "tensor", "kernel": kname_b, "achieved": mma_tf,
                    "peak": peaks["bf16_tflops"], "unit": "TFLOP/s", "frac": f_t,
                    "peak_source": f"bf16_tflops of {peak_kind} (BF16 MMA flops, 3 per "
                                   "split product)", "hbm_frac": f_h, "hbm_gbs": gbs}
        else:
            roof = {"bound": "hbm", "kernel": kname_b, "achieved": gbs,
                    "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": f_h,
                    "peak_source": f"hbm_gbs of {peak_kind}", "tensor_frac": f_t,
                    "bf16_mma_tflops": mma_tf}
    elif dom in ("conv", "conv_block"):
        achieved = st["bytes"] / (st["ms"] / 1e3) / 1e9
        tc_march = prec != lib.FP64 and args.march_engine == "tcgen05"
        kname = "k_conv" if prec == lib.FP64 else \
            "k_conv_tc (tcgen05, split-BF16)" if tc_march else "k_conv_f32<NB>"
        roof = {"bound": "hbm", "kernel": kname, "achieved": achieved,
                "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                "peak_source": f"hbm_gbs of {peak_kind}"}
    else:
        achieved = st["flops"] / (st["ms"] / 1e3) / 1e12
        key = "fp32_tflops" if dom == "assemble_f32" or prec != lib.FP64 and dom == "factor" \
            else "fp64_tflops"
        fp64 = peaks.get(key)
        roof = {"bound": "fp32" if key == "fp32_tflops" else "fp64",
                "kernel": {"assemble": "k_assemble_items", "assemble_f32": "k_assemble_far_rows",
                           "factor": "blocked Gauss-Jordan", "solve": "solve"}.get(dom, dom),
                "achieved": achieved, "peak": fp64, "unit": "TFLOP/s",
                "frac": (achieved / fp64) if fp64 else None,
                "peak_source": f"{key}: cuBLAS GEMM measured in this run"}
        if dom == "assemble_f32":
            roof["flops_counted"] = (
                "algorithmic: every far (node, element, level) item x its Gauss points x 425 "
                "flops, settled levels included; about half the items are settled levels, "
                "which the kernel produces from one quasi-static pass per pair (201 flops "
                "per point) and one scaled add per level, so it executes fewer flops than "
                "it is credited with")
    roof["launches"] = st["launches"]
    roof["avg_launch_ms"] = st["ms"] / max(1, st["launches"])
    tkey = f"{args.workload}:{args.precision}:{dom}"
    if dom in ("conv", "conv_block") and prec != lib.FP64:
        tkey += f":{args.march_engine}"
    t = traffic.get(tkey)
    if isinstance(t, dict) and "ratio_to_algorithmic" in t:
        roof["traffic"] = t["ratio_to_algorithmic"] * st["bytes"] / max(1, st["launches"])
        roof["traffic_source"] = t["source"]
    else:
        roof["traffic"] = t
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec == lib.FP64 else "f32+f64", "data": "synthetic",
            "config": workload_config(args.workload, model, M, dist.world),
            "method": {"precision": args.precision, "refine_sweeps": refine,
                       "block_steps": args.block or (32 if args.march_engine == "tcgen05" else 8),
                       "march_engine": args.march_engine if prec == lib.MIXED else None,
                       "batch_engine": args.engine if cases else None,
                       "level_store_gb": round(level_gb, 2),
                       "parity": "plain FP64 form: 1e-10 per level and per step against the "
                                 "oracle in exact-zero mode (the step response of a point both "
                                 "wave fronts have passed is exactly 0); against the "
                                 "reference's raw outputs 1e-10 plus twice their round-off "
                                 "floor (up to ~6e-8 of a level's max-norm)"},
            "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches),
            "roofline": roof,
            "phases_ms": phase,
            "kernels": {k: {"launches": v["launches"], "ms": round(v["ms"], 3),
                            "share": v["ms"] / max(1e-9, sum(x["ms"] for x in stats.values())),
                            "GB/s": v["bytes"] / max(1e-9, v["ms"]) / 1e6,
                            "TFLOP/s": v["flops"] / max(1e-9, v["ms"]) / 1e9}
                        for k, v in stats.items() if v["launches"]},
            "clocks": clk,
            "peaks_used": {k: peaks.get(k) for k in ("hbm_gbs", "fp64_tflops", "fp32_tflops")}}
    if compare:
        line["vs_plain_fp64"] = compare
    if dist.world == 1 and not cases and prec == lib.MIXED and not args.no_batched:
        line["batched"] = run_batched(lib, torch, args)
    if dist.world == 1 and not cases and prec == lib.MIXED and not args.no_batched:
        g = group_measure(lib, torch, args, dist, "bars32_group")
        line["grouped"] = {k: g[k] for k in ("value", "unit", "ms_per_step", "config", "e2e",
                                              "autotuned_shape", "vs_plain_fp64") if k in g}
    if dist.world == 1 and not cases and prec == lib.MIXED and not args.no_precision_config:
        line["precision_config"] = run_precision_config(lib, torch, args, peaks, peak_kind)
    if args.serve_requests > 0:
        line["serve"] = run_serve(lib, args, dev)
    if dist.world == 1 and not args.no_cpu_baseline:
        r = cpu_sample(model, M, nsteps, *ALPHA, os.cpu_count() or 1, cases)
        line["cpu_baseline"] = {"value": r["value"], "unit": METRIC, "cores": os.cpu_count(),
                                "kind": "port, extrapolated", "sample": r["sample"],
                                "sample_fractions": r["sample_fractions"]}
    print(json.dumps(line))
    return 0


def run_batched(lib, torch, args, workload="sphere_6x16x16_batch64"):
    """The batched mixed form on the 64-load-case workload, timed like the headline
    (W warm-up and K timed solves between CUDA events on the library's stream), with
    its tensor-core convolution's share and bandwidth and its error against the plain
    FP64 form.  Reported as the "batched" object of the headline line."""
    from tdbem import loads
    model = make_model(workload)
    cases = WORKLOADS[workload]["cases"]
    D, n = model.ndof, model.numstep
    trac, amp = loads.gaussian_patch_cases(model, cases, seed=0)
    ctx = lib.Context(model)
    ctx.set_alpha(*ALPHA)
    ctx.set_batch_options(lib.ENGINE_TCGEN05, 0)
    stream = torch.cuda.ExternalStream(ctx.stream)

    def job():
        ctx.assemble(precision=lib.MIXED)
        ctx.march_batch(trac, amp, to_host=False)

    for _ in range(args.warmup):
        job()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        job()
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    ctx.set_profiling(True)
    job()
    stats = ctx.kernel_stats()
    ctx.set_profiling(False)
    cb = stats["conv_batch"]
    out = {"workload": workload, "load_cases": cases, "dof": D, "steps": n,
           "value": cases * D * n / (ms / 1e3), "unit": METRIC, "ms_per_step": ms,
           "engine": "tcgen05", "refine_sweeps": 0,
           "conv_batch": {"kernel": "k_conv_tc (tcgen05)", "launches": cb["launches"],
                          "share": cb["ms"] / max(1e-9, sum(v["ms"] for v in stats.values())),
                          "GB/s": cb["bytes"] / max(1e-9, cb["ms"]) / 1e6}}
    if not args.no_compare:
        out["vs_plain_fp64"] = compare_batch(lib, torch, ctx, model, trac, amp, ms)
    ctx.close()
    return out


def run_precision_config(lib, torch, args, peaks, peak_kind, workload="sphere_6x24x24"):
    """The precision configuration: the 6x24x24 cubed-sphere cavity (10374 DOF, 500
    steps, 91 levels) in the mixed form, timed like the headline (W warm-up and K
    timed solves between CUDA events), its dominant kernel's roofline, and its error
    against the plain FP64 form of the same solve (the FP64 level store, 157 GB, is
    made after the mixed context is released)."""
    model = make_model(workload)
    D, n = model.ndof, model.numstep
    ctx = lib.Context(model)
    ctx.set_alpha(*ALPHA)
    M = ctx.M
    stream = torch.cuda.ExternalStream(ctx.stream)

    def job():
        ctx.assemble(precision=lib.MIXED)
        ctx.march(to_host=False)

    for _ in range(args.warmup):
        job()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        job()
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    ctx.set_profiling(True)
    job()
    stats = ctx.kernel_stats()
    ctx.set_profiling(False)
    phases = ctx.timings()
    far = stats["assemble_f32"]
    tf = far["flops"] / max(1e-9, far["ms"] / 1e3) / 1e12
    out = {"workload": workload, "value": D * n / (ms / 1e3), "unit": METRIC, "ms_per_step": ms,
           "config": workload_config(workload, model, M, 1), "phases_ms": phases,
           "roofline": {"bound": "fp32", "kernel": "k_assemble_far_rows", "achieved": tf,
                        "peak": peaks.get("fp32_tflops"), "unit": "TFLOP/s",
                        "frac": tf / peaks["fp32_tflops"] if peaks.get("fp32_tflops") else None,
                        "launches": far["launches"],
                        "share": far["ms"] / max(1e-9, sum(v["ms"] for v in stats.values())),
                        "peak_source": "fp32_tflops: cuBLAS GEMM measured in this run"},
           "kernels": {k: {"launches": v["launches"], "ms": round(v["ms"], 3)}
                       for k, v in stats.items() if v["launches"]}}
    if not args.no_compare:
        u32, t32 = ctx.march()
        ctx.close()
        with lib.Context(model) as c64:
            c64.set_alpha(*ALPHA)
            s64 = torch.cuda.ExternalStream(c64.stream)
            a0 = torch.cuda.Event(enable_timing=True)
            a1 = torch.cuda.Event(enable_timing=True)
            a0.record(s64)
            c64.assemble(precision=lib.FP64)
            u64, t64 = c64.march()
            a1.record(s64)
            a1.synchronize()
            ms64 = a0.elapsed_time(a1)
        out["vs_plain_fp64"] = {
            "plain_fp64_value": D * n / (ms64 / 1e3), "plain_fp64_ms_per_step": ms64,
            "speedup_vs_plain_fp64": ms64 / ms,
            "u_rel_l2_err": float(np.linalg.norm(u32 - u64) / np.linalg.norm(u64)),
            "t_rel_l2_err": float(np.linalg.norm(t32 - t64) / max(1e-300, np.linalg.norm(t64))),
            "note": "the cavity's tractions are all prescribed, so t matches exactly"}
    else:
        ctx.close()
    return out


def run_group(lib, torch, args, dist):
    """Many meshes at once (the --workload bars32_group line)."""
    line = group_measure(lib, torch, args, dist, args.workload)
    if dist.rank == 0:
        print(json.dumps(line))
    return 0


def group_measure(lib, torch, args, dist, workload):
    """Many meshes at once: grouped assembly + one persistent launch for every step
    of every mesh, against the same meshes solved one after another (plain FP64
    both ways)."""
    w = WORKLOADS[workload]
    models = group_models(w["count"], w["numstep"])
    dofs = [m.ndof for m in models]
    units = sum(d * m.numstep for d, m in zip(dofs, models))
    prec = lib.FP64 if args.precision == "fp64" else lib.MIXED
    ctxs = [lib.Context(m) for m in models]
    for c in ctxs:
        c.set_alpha(*ALPHA)
    stream = torch.cuda.ExternalStream(ctxs[0].stream)

    def job():
        lib.assemble_group(ctxs, precision=prec)
        lib.march_group(ctxs, to_host=False)

    for _ in range(args.warmup):
        job()
    torch.cuda.synchronize()
    dist.barrier()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    n0 = sum(c.launch_count() for c in ctxs)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        job()
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    dist.barrier()
    clk = clocks.stop()
    launches = sum(c.launch_count() for c in ctxs) - n0
    ms_total = dist.max(e0.elapsed_time(e1))
    ms = ms_total / args.steps
    value = units * args.steps * dist.world / (ms_total / 1e3)
    timing = ctxs[0].timings()
    shape = lib.group_shape()
    # e2e through the C ABI: contexts from host meshes, grouped assembly and march,
    # histories back to the host
    t0 = time.perf_counter()
    c2 = [lib.Context(m) for m in models]
    for c in c2:
        c.set_alpha(*ALPHA)
    lib.assemble_group(c2, precision=prec)
    outs = lib.march_group(c2)
    e2e_s = dist.max(time.perf_counter() - t0)
    for c in c2:
        c.close()
    line_extra = {}
    if not args.no_compare:
        # the meshes one after another in the plain FP64 form, and the group's error
        torch.cuda.synchronize()
        a0 = time.perf_counter()
        err = 0.0
        for c, (u, _) in zip(ctxs, outs):
            c.assemble(precision=lib.FP64)
            ur, _ = c.march()
            err = max(err, float(np.linalg.norm(u - ur) / max(1e-300, np.linalg.norm(ur))))
        seq_s = time.perf_counter() - a0
        line_extra = {"vs_plain_fp64": {
            "plain_fp64_value": units / seq_s, "plain_fp64_seconds": seq_s,
            "form": "each mesh's tdbem_assemble_levels + tdbem_march (FP64), one after another",
            "speedup_vs_plain_fp64": seq_s / (ms / 1e3),
            "u_rel_l2_err_max_over_meshes": err}}
    for c in ctxs:
        c.close()
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec == lib.FP64 else "f32+f64", "data": "synthetic",
            "config": {"workload": workload, "meshes": len(models),
                       "dof_range": [min(dofs), max(dofs)], "dof_total": sum(dofs),
                       "steps": w["numstep"], "alpha": list(ALPHA), "precision": args.precision,
                       "parallelism": f"replicas{dist.world}",
                       "l2": "levels of all meshes together are larger than L2" if
                             sum((m.max_step() + 1) * d * d * 16 for m, d in zip(models, dofs))
                             > 129e6 else "levels fit in L2"},
            "e2e": {"value": units * dist.world / e2e_s, "unit": METRIC,
                    "h2d_bytes_per_step": int(sum(m.coords.nbytes + m.ien.nbytes for m in models)),
                    "d2h_bytes_per_step": int(sum(2 * (m.numstep + 1) * d * 8
                                                  for m, d in zip(models, dofs)))},
            "gpu_launches": int(launches), "phases_ms": timing, "autotuned_shape": shape,
            "clocks": clk}
    line.update(line_extra)
    return line


def run_serve(lib, args, dev):
    """Seeded Poisson streams of mixed transient solves through the server
    (continuous batching: slots assemble, one grouped launch per time block advances
    every resident solve; admission by HBM footprint) at several arrival rates:
    latency percentiles, throughput and how many solves each grouped launch carried.
    Not part of the timed region of the headline number."""
    from tdbem import serve
    rates = [float(x) for x in args.serve_rates.split(",")]
    curves = []
    for i, rate in enumerate(rates):
        reqs = serve.request_mix(args.serve_requests, rate, seed=i)
        with lib.Server(dev, 0, slots=args.serve_slots) as srv:
            res = serve.run_stream(srv, reqs, alpha=ALPHA)
            ms = srv.march_stats()
        mix = {}
        for r in res["records"]:
            k = r["name"].split("_")[0]
            mix[k] = mix.get(k, 0) + 1
        done_hz = len(reqs) / res["wall_s"]
        curves.append({
            "rate_hz": rate, "requests": len(reqs), "p50_s": res["p50_s"],
            "p99_s": res["p99_s"], "mean_queued_s": res["mean_queued_s"],
            "wall_s": res["wall_s"], "completed_per_s": done_hz,
            "saturated": done_hz < 0.9 * rate,
            "dof_steps_per_s": res["dof_steps_per_s"],
            "grouped_launches": ms["launches"], "solve_steps": ms["solve_steps"],
            "mean_resident_per_launch": ms["mean_resident"],
            "launches_per_solve_step": ms["launches"] / max(1, ms["solve_steps"]),
            "mix": mix,
            "dof_range": [min(r["dof"] for r in reqs), max(r["dof"] for r in reqs)],
            "steps_range": [min(r["steps"] for r in reqs), max(r["steps"] for r in reqs)],
            "seed": i})
    return {"slots": args.serve_slots, "precision": "mixed", "curves": curves,
            "note": "each grouped launch advances every resident solve by a 12-step block"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="sphere_6x16x16")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the plain FP64 run that measures the mixed form's error")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--refine", type=int, default=None,
                    help="FP64 refinement sweeps of the mixed-precision solves (0..4; default 0)")
    ap.add_argument("--engine", choices=["tcgen05", "mma_sync"], default="tcgen05",
                    help="tensor-core engine of the batched convolution")
    ap.add_argument("--march-engine", choices=["tcgen05", "fp32"], default="tcgen05",
                    help="old-history pass of the mixed march: split-BF16 products on the "
                         "tensor cores, or FP32 products on the CUDA cores")
    ap.add_argument("--block", type=int, default=0, choices=[0, 1, 4, 6, 8, 12, 16, 24, 32],
                    help="time-block steps of the mixed march (0: the engine's default)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the 64-load-case batched measurement beside the headline")
    ap.add_argument("--serve-requests", type=int, default=200,
                    help="requests of each serving stream reported beside the headline (0: off)")
    ap.add_argument("--serve-rates", default="2,4,8",
                    help="Poisson arrival rates of the serving streams, 1/s, comma-separated")
    ap.add_argument("--serve-slots", type=int, default=8)
    ap.add_argument("--no-precision-config", action="store_true",
                    help="skip the 6x24x24 precision configuration beside the headline")
    args = ap.parse_args()
    dist = Dist()
    try:
        if args.impl == "reference":
            return run_reference(args, dist)
        return run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    sys.exit(main())

#!/usr/bin/env python3
"""Benchmark of the IBIM Poisson-Boltzmann path on GB300: FMM-GMRES solves/sec, p50/p99 latency.

One step = one whole solve of the workload (level set -> tube quadrature -> octree plan ->
GMRES on the fused BIE FMM -> polarization energy) through the C ABI.  The default precision is
the mixed path (FP32 level set, tensor-core M2L on scaled FP16 splits, FP32 near field, FP64-class
iterative refinement); --precision fp64 times the reference-exact FP64 path.

  value   solves/sec with the atoms already in HBM (ibim_solve_dev), device time from CUDA events
          on the library's stream, L2 flushed (256 MB write) between steps
  e2e     the same through ibim_solve with host buffers (host->device copies inside the region)
  roofline  the dominant kernel category of the timed region: algorithmic flops (or bytes) of its
          launches / their CUDA-event time, against the measured peak of its bound
          (rooflines: the same for every category with counted work)
  accuracy  mixed path only: one untimed FP64 solve of the same workload after the timed region;
          the energy's relative error against it (the metric's 1e-4 bound) and the FP64 path's
          own solves/s
  cpu_baseline  the oracle (plain-C restatement of the reference, reference-structured: 16 scalar
          FMMs per matvec with on-the-fly M2L, as electric.cpp/bbfmm.h do) timed on a bounded
          sample of the same workload on the host cores, extrapolated to one solve

--impl reference runs only that CPU path and prints its line.
Multi-GPU: replicas only (independent solves per rank, no collective on the data path).
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "ibim-levelset_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

import workloads  # noqa: E402

METRIC = "FMM-GMRES solves/sec (whole IBIM PB solve) at <=1e-4 rel. energy err vs FP64 path"
UNIT = "solves/s"
# Arnoldi steps + 1 (the reference also applies the operator to x0 = 0) of the FP64 path on
# protein2000, measured on GB300 (25 + 1); the FP64 GPU path reproduces the reference's iteration
# counts on every golden case, so the CPU baseline extrapolates with it when the run itself has no
# FP64 solve to take the count from.
REF_MATVECS = {"synthetic_protein_2000_atoms_h0.5": 26}
FMM_STRIDE = 32
FMM_SAMPLE_NODES = 2048
# one kernel of each family timed by the CPU sample (ids of include/ibim.h), and how many of the
# 16 FMMs of one matvec belong to each family
FMM_FAMILIES = (("K1", 0), ("K2", 3), ("K3", 4), ("K4", 13))
FAMILY_COUNT = {"K1": 3, "K2": 1, "K3": 9, "K4": 3}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    ap.add_argument("--workload", choices=["protein2000", "born", "serve", "batch"], default="protein2000",
                    help="serve: a bounded sample of the Poisson request stream through the request loop; "
                         "batch: many molecules submitted at once (atoms log-uniform, default 50-5000)")
    ap.add_argument("--requests", type=int, default=None, help="serve/batch: number of requests (40 / 256)")
    ap.add_argument("--rate", type=float, default=4.0, help="serve: offered rate, requests/s")
    ap.add_argument("--slots", type=int, default=4, help="serve/batch: solves in flight (request loop)")
    ap.add_argument("--batch-mode", choices=["lockstep", "pool"], default="lockstep",
                    help="batch: lock-step waves on merged plans (ibim_batch_solve) or the request loop's "
                         "concurrent whole solves; serve: the request loop in lock-step or pool mode")
    ap.add_argument("--max-wave", type=int, default=6, help="batch lockstep: molecules per wave")
    ap.add_argument("--workers", type=int, default=4, help="batch lockstep: preparation threads")
    ap.add_argument("--wave-slots", type=int, default=3, help="batch lockstep: waves solved at once")
    ap.add_argument("--atoms", type=str, default=None, help="serve/batch: log-uniform atom-count range")
    ap.add_argument("--accuracy-sample", type=int, default=2,
                    help="serve/batch: requests (smallest first) re-solved alone in FP64 to state the error")
    ap.add_argument("--hs", type=str, default="0.5", help="serve: grid spacings to draw from, e.g. 0.25,0.5")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64-check", action="store_true",
                    help="skip the untimed FP64 solve that states the mixed path's energy error")
    ap.add_argument("--order", type=int, default=None,
                    help="override the workload's Chebyshev order (smaller operator storage for profiler captures)")
    ap.add_argument("--protein-atoms", type=int, default=None,
                    help="protein workload with this many atoms instead of 2,000 (smaller profiler captures)")
    return ap.parse_args()


def get_workload(name, order=None, atoms=None):
    if name == "protein2000":
        W = workloads.protein(atoms, 1_000_000, 0.5, 5) if atoms else workloads.protein2000()
    else:
        W = workloads.born()
    if order is not None:
        W.np_ = order
        W.name = f"{W.name}_p{order}"
    return W


# ---------------------------------------------------------------------------------------------
# CPU baseline: bounded sample of the reference's CPU algorithm (the oracle restatement)
# ---------------------------------------------------------------------------------------------

def cpu_sample(W, grid_reinit=None, tube7=None, matvecs=None, stages=None):
    """Time one bounded sample; return (extrapolated seconds per solve, parts dict).

    Sample: one TVD-RK3 step (3 stages) of the level set on the full grid, the tube extraction,
    the direct right-hand side, and one scalar FMM of each kernel family (K1x, K2, K3xx, K4x; tree
    built per FMM) on the full tube.  A solve = stages/3 level-set steps + tube + RHS + per matvec
    3 K1 + 1 K2 + 9 K3 + 3 K4 FMMs, + 3 K1 + 1 K2 (polarize).
    """
    import oracle as O

    # the -ffast-math build of the port: the reference is built -Ofast, and the exact build
    # (the checker's) measured 1.4-1.6x the reference binary's FMM time on an x86 host
    O.use_timing_build()
    threads = os.cpu_count() or 1
    geo = W.geo
    parts = {}
    if grid_reinit is None or tube7 is None:
        g, steps = O.levelset(W.mol.centers, W.mol.radii, geo.lo, geo.h, geo.n, reinit_t=W.reinit_t,
                              thickness=W.thickness, thres=W.thres, init=W.init)
        if stages is None:
            stages = 3 * (int(1.4 / (0.2 * geo.h)) + 1 + int(steps[0]) + int(steps[1]))
        grid_reinit = g.copy()
        t0 = time.perf_counter()
        tube7, _ = O.surface(g, geo.lo, geo.h, W.thickness)
        parts["surface_s"] = time.perf_counter() - t0
    else:
        g = grid_reinit.copy()
        t0 = time.perf_counter()
        O.surface(g, geo.lo, geo.h, W.thickness)
        parts["surface_s"] = time.perf_counter() - t0
    # one level-set step (3 full-grid stages): evolve with final_t < dt takes exactly one step
    g = grid_reinit.copy()
    t0 = time.perf_counter()
    O.evolve(g, geo.h, 0.5 * 0.2 * geo.h, 1.0, 0.2)
    parts["levelset_step_s"] = time.perf_counter() - t0
    bp = O.bie_params(W.np_, W.maxpoint, W.maxlevel, W.restart, W.maxiter, W.kappa, W.dE, W.dI, W.tau, W.tol, 1)
    t0 = time.perf_counter()
    O.rhs(tube7, W.mol.centers, W.mol.charges, bp)
    parts["rhs_s"] = time.perf_counter() - t0
    N = len(tube7)
    dens = np.sin(0.37 * np.arange(N)) * tube7[:, 3] * tube7[:, 6] * geo.h ** 3
    # one scalar FMM of each kernel family with its own tree, as electric.cpp:333-367 runs each of
    # the 16 kernels: K1 (3 of the 16), K2 (1), K3 (9), K4 (3); the downward pass is sampled on every
    # FMM_STRIDE-th node and scaled back
    t0 = time.perf_counter()
    T = O.Tree(tube7[:, :3], tube7[:, :3], W.maxpoint, W.maxlevel)
    t_tree = time.perf_counter() - t0
    kp = O.KParams(W.kappa, W.dE, W.dI, W.tau * geo.h)
    # every stride-th node's downward pass, at least FMM_SAMPLE_NODES of them: a sparser sample of
    # a small tree overstated the full FMM by 1.5x (100-atom protein)
    stride = max(1, min(FMM_STRIDE, T.nnodes // FMM_SAMPLE_NODES))
    fam_s = {}
    for fam, kid in FMM_FAMILIES:
        t0 = time.perf_counter()
        T.fmm(W.np_, kp, kid, dens, sample_stride=stride)
        t_sampled = time.perf_counter() - t0
        if stride > 1:
            t0 = time.perf_counter()
            T.fmm(W.np_, kp, kid, dens, sample_stride=1 << 30)
            t_up = time.perf_counter() - t0  # upward pass alone (node 0 only downward)
            fam_s[fam] = t_tree + t_up + (t_sampled - t_up) * stride
        else:
            fam_s[fam] = t_tree + t_sampled
        parts[f"fmm_{fam}_s"] = fam_s[fam]
    del T
    if matvecs is None:
        matvecs = REF_MATVECS.get(W.name) or 26
    if stages is None:
        stages = 3 * (int(1.4 / (0.2 * geo.h)) + 1 + 2 * W.reinit_steps)
    matvec_s = sum(FAMILY_COUNT[f] * t for f, t in fam_s.items())
    # polarizeMap: K1x, K1y, K1z and K2 with atom targets (electric.cpp:468-478)
    polarize_s = 3 * fam_s["K1"] + fam_s["K2"]
    parts["matvec_s"] = matvec_s
    solve_s = (parts["levelset_step_s"] * stages / 3.0 + parts["surface_s"] + parts["rhs_s"] +
               matvec_s * matvecs + polarize_s)
    parts.update(threads=threads, matvecs=matvecs, stages=stages, points=N, stride=stride)
    return solve_s, parts


def cpu_baseline_object(solve_s, parts, kind="port"):
    sample = (f"oracle port (reference-structured) on {parts['threads']} host threads: one level-set step "
              f"(3 full-grid stages) x {parts['stages'] // 3}, tube extraction, direct RHS, one scalar FMM "
              f"per kernel family (K1x, K2, K3xx, K4x; own tree each; downward pass timed on every "
              f"{parts['stride']}th node and scaled) weighted 3/1/9/3 per matvec x {parts['matvecs']} matvecs, "
              f"+ 4 polarize FMMs, on {parts['points']} tube points, with the port built -ffast-math as the "
              f"reference is built -Ofast; an extrapolated estimate, not a timed solve")
    return {"value": 1.0 / solve_s, "unit": UNIT, "cores": parts["threads"], "kind": kind, "sample": sample,
            "seconds_per_solve": solve_s, "parts_s": {k: round(v, 4) for k, v in parts.items() if k.endswith("_s")}}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    W = get_workload(args.workload, args.order, args.protein_atoms)
    import oracle as O

    O.build()
    geo = W.geo
    g, steps = O.levelset(W.mol.centers, W.mol.radii, geo.lo, geo.h, geo.n, reinit_t=W.reinit_t,
                          thickness=W.thickness, thres=W.thres, init=W.init)
    stages = 3 * (int(1.4 / (0.2 * geo.h)) + 1 + int(steps[0]) + int(steps[1]))
    gg = g.copy()
    tube7, _ = O.surface(gg, geo.lo, geo.h, W.thickness)
    times, walls, parts = [], [], None
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        s, parts = cpu_sample(W, grid_reinit=g, tube7=tube7, stages=stages)
        if i >= args.warmup:
            times.append(s)
            walls.append(time.perf_counter() - t0)
    solve_s = statistics.mean(times)
    value = 1.0 / solve_s
    cb = cpu_baseline_object(solve_s, parts, kind="port")
    # a step is one bounded sample (its wall time is ms_per_step); value is the solves/s that the
    # sample extrapolates to, not a timed solve
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(walls) * 1e3,
           "extrapolated_ms_per_solve": solve_s * 1e3, "value_is_estimate": True, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
           "config": W.describe(), "cpu_baseline": cb,
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


# ---------------------------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.f = tempfile.NamedTemporaryFile("w+", delete=False, suffix=".csv")
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms",
                                       "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for ln in fh:
                c = [v.strip() for v in ln.split(",")]
                if len(c) >= 9:
                    rows.append(c)
        os.unlink(self.f.name)
        dev = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]
        mine = [r for r in rows if r[0] == dev] or rows
        sm = [float(r[1]) for r in mine if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in mine if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in mine for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(mine)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def committed_traffic(kernel, workload):
    """DRAM bytes per launch from the committed ncu summary (profiles/traffic_per_launch.txt)."""
    path = os.path.join(ROOT, "profiles", "traffic_per_launch.txt")
    try:
        with open(path) as f:
            for ln in f:
                t = ln.split()
                if len(t) >= 3 and t[0] == kernel and t[1] == workload:
                    return float(t[2])
    except OSError:
        pass
    return None


def max_over_ranks(x: float, device=None) -> float:
    """The maximum of x over the ranks of the default process group (x itself without one):
    the whole job's time is its slowest replica's."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world: int, steps: int, total_ms: float) -> float:
    """Whole-job solves/s of `world` independent replicas that each ran `steps` solves in at most
    total_ms (weak scaling: per-GPU work fixed)."""
    return world * steps / (total_ms / 1e3)


def run_ours(args):
    import torch

    import ibim

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    W = get_workload(args.workload, args.order, args.protein_atoms)
    precision = ibim.PRECISION_FP64 if args.precision == "fp64" else ibim.PRECISION_MIXED
    cfg = W.config(precision)
    ctx = ibim.Context(local)
    ext = torch.cuda.ExternalStream(ctx.stream)
    dev = torch.device("cuda", local)
    centers = torch.tensor(W.mol.centers, dtype=torch.float64, device=dev).contiguous()
    charges = torch.tensor(W.mol.charges, dtype=torch.float64, device=dev).contiguous()
    radii = torch.tensor(W.mol.radii, dtype=torch.float64, device=dev).contiguous()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step_dev():
        return ctx.solve_dev(centers.data_ptr(), charges.data_ptr(), radii.data_ptr(), W.mol.n, cfg)

    def timed(fn, n):
        out, ms = [], []
        for _ in range(n):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(ext)
            r = fn()
            b.record(ext)
            b.synchronize()
            ms.append(a.elapsed_time(b))
            out.append(r)
        return out, ms

    for _ in range(args.warmup):
        step_dev()
    # timed region: no per-kernel events (the library's profiling is off)
    ctx.profile([])
    sampler = ClockSampler()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler.start()
    l0 = ibim.launch_count()
    results, step_ms = timed(step_dev, args.steps)
    launches = ibim.launch_count() - l0
    torch.cuda.synchronize()
    clocks = sampler.stop()
    total_ms = max_over_ranks(sum(step_ms), dev)
    value = replica_rate(world, args.steps, total_ms)
    r0 = results[-1]

    # end to end through the host-buffer entry point
    e2e = None
    if not args.no_e2e:
        _, e2e_ms = timed(lambda: ctx.solve(W.mol.centers, W.mol.charges, W.mol.radii, cfg), args.steps)
        e2e = {"value": replica_rate(world, args.steps, max_over_ranks(sum(e2e_ms), dev)), "unit": UNIT,
               "h2d_bytes_per_step": int(W.mol.n * 5 * 8), "d2h_bytes_per_step": int(ctypes.sizeof(ibim.Result)),
               "ms_per_step": statistics.mean(e2e_ms)}

    # profiled pass, after the timed regions: the same steps again with CUDA events recorded around
    # every launch of each kernel category on the stream it runs on (per-launch durations for the
    # rooflines and the per-category breakdown)
    ctx.profile(ibim.PROFILE_CATEGORIES)
    ctx.profile_read()
    _, prof_ms = timed(step_dev, args.steps)
    prof = ctx.profile_read()
    ctx.profile([])

    # roofline of every kernel category with counted work; the headline one is the dominant
    peaks = measured_peaks()
    fp64_peak = ctx.measure_peak("fp64")
    fp32_peak = ctx.measure_peak("fp32")
    mixed = precision == ibim.PRECISION_MIXED
    # operand form of the mixed path's tensor-core M2L (the library's default: scaled FP16 splits)
    tc_form = ("tf32x3 tensor" if os.environ.get("IBIM_TC_FP16") == "0" or os.environ.get("IBIM_TC_PAIR") == "1"
               else "fp16x3 tensor")
    # digit-pair MMAs per multiply-add of the sliced FP64-class M2L: 6 digits of 7 bits (21 pairs)
    # while K = 4 p^3 padded to 16 is at most 800, else 7 digits of 6 bits (28 pairs)
    oz_digits = 6 if (4 * W.np_ ** 3 + 15) // 16 * 16 <= 800 else 7
    oz_mmas = oz_digits * (oz_digits + 1) // 2
    fp_bound = {"m2l_v_fp64": "fp64", "m2l_x_fp64": "fp64", "near_l2p_fp64": "fp64", "near_l2p": "fp32",
                "m2l_x": "fp32", "m2l_v": tc_form if mixed else "fp64", "rhs": "fp32" if mixed else "fp64",
                "weno_stage": "fp32" if mixed else "fp64", "p2m": "fp32" if mixed else "fp64",
                "count_gradient": "hbm", "gmres_vectors": "hbm", "m2l_v_sliced": f"bf16x{oz_mmas} tensor",
                "near_ff": "fp32", "l2p": "fp32", "l2p_fp64": "fp64"}

    def roofline_of(name, d):
        bound = fp_bound.get(name, "hbm")
        extra = {}
        per_launch_ms = d["ms"] / d["launches"]
        if bound == "hbm":
            if d["bytes"] <= 0:
                return None
            ach = d["bytes"] / d["launches"] / (per_launch_ms * 1e-3) / 1e9
            peak, unit, src = peaks.get("hbm_gbs", 6800.0), "GB/s", "MEASURED_PEAKS.json hbm_gbs (of measured)"
            alg = d["bytes"] / d["launches"]
        else:
            if d["flops"] <= 0:
                return None
            alg = d["flops"] / d["launches"]
            if bound.startswith(("tf32", "fp16", "bf16")):
                # achieved = the contraction's algorithmic flops 2 (4p^3)^2 per pair over the launch
                # time.  The tensor pipe issues `mmas` products per algorithmic multiply-add (3 for the
                # hi/lo splits, oz_mmas digit pairs for the sliced FP64-class form); that issue rate is
                # reported apart as tensor_issue_frac and is not the roofline fraction.
                mmas = oz_mmas if bound.startswith("bf16") else 3
                ach = alg / (per_launch_ms * 1e-3) / 1e12
                peak = peaks.get("bf16_tflops", 1909.5) * (0.5 if bound.startswith("tf32") else 1.0)
                unit = "TFLOP/s"
                src = ("TF32 = 1/2 of MEASURED_PEAKS.json bf16_tflops (of measured)" if bound.startswith("tf32")
                       else "MEASURED_PEAKS.json bf16_tflops (FP16/BF16 dense rate, of measured)")
                src += f"; achieved counts algorithmic flops only ({mmas} MMAs issued per multiply-add)"
                extra = {"tensor_issue_frac": mmas * ach / peak, "mmas_per_multiply_add": mmas}
            else:
                ach = alg / (per_launch_ms * 1e-3) / 1e12
                peak = fp64_peak if bound == "fp64" else fp32_peak
                unit, src = "TFLOP/s", f"{bound.upper()} FMA-chain microkernel measured in this run (of measured)"
        r = {"bound": bound, "kernel": name, "achieved": ach, "peak": peak, "unit": unit,
             "frac": ach / peak if peak else None, "peak_source": src,
             "traffic": committed_traffic(name, W.name), "launches": d["launches"],
             "avg_launch_ms": per_launch_ms, "algorithmic_per_launch": alg}
        r.update(extra)
        return r

    rooflines = {}
    for name, d in (prof or {}).items():
        if d["launches"] > 0 and d["ms"] > 0:
            r = roofline_of(name, d)
            if r is not None:
                rooflines[name] = r
    roofline = max(rooflines.values(), key=lambda r: r["launches"] * r["avg_launch_ms"]) if rooflines else None
    # per-solve ideal time: sum over the categories of (algorithmic work / peak of their bound)
    ideal_ms = sum(r["launches"] * r["avg_launch_ms"] * r["frac"] for r in rooflines.values() if r["frac"])
    solve_roofline = {"ideal_ms_per_step": ideal_ms / args.steps, "ms_per_step": total_ms / args.steps,
                      "frac": ideal_ms / total_ms if total_ms else None,
                      "categories": sorted(rooflines),
                      "note": "ideal = sum over counted kernel categories of work / measured peak of the bound"}

    # the mixed path's energy error against the FP64 path, from one untimed FP64 solve
    accuracy = None
    if mixed and not args.no_fp64_check:
        cfg64 = W.config(ibim.PRECISION_FP64)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(ext)
        r64 = ctx.solve_dev(centers.data_ptr(), charges.data_ptr(), radii.data_ptr(), W.mol.n, cfg64)
        b.record(ext)
        b.synchronize()
        ms64 = a.elapsed_time(b)
        rel = abs(r0["energy"] - r64["energy"]) / abs(r64["energy"])
        accuracy = {"energy": r0["energy"], "energy_fp64": r64["energy"], "rel_err_vs_fp64": rel, "tolerance": 1e-4,
                    "within_tolerance": rel <= 1e-4, "fp64_ms_per_solve": ms64,
                    "fp64_solves_per_s": 1e3 / ms64, "speedup_vs_fp64": value / world * ms64 / 1e3,
                    "fp64_gmres_iters": r64["gmres_iters"], "fp64_matvecs": r64["matvecs"]}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            g, _ = ctx.levelset(W.mol.centers, W.mol.radii, cfg)
            grid = g.download()
            tube7 = g.surface(W.thickness).surface7()
            g.close()
            # the reference's matvec count: the FP64 path's products (it reproduces the reference's
            # iteration counts) plus the reference's product A.0 for x0 = 0
            if precision == ibim.PRECISION_FP64:
                ref_mv = r0["matvecs"] + 1
            elif accuracy is not None:
                ref_mv = accuracy["fp64_matvecs"] + 1
            else:
                ref_mv = None
            solve_s, parts = cpu_sample(W, grid_reinit=grid, tube7=tube7, matvecs=ref_mv,
                                        stages=r0["levelset_stages"])
            cpu = cpu_baseline_object(solve_s, parts)
        except Exception as e:  # the baseline is reported, not required
            cpu = {"error": str(e)}

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": statistics.mean(step_ms), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64" if precision == 0 else "f32+f64",
           "data": "synthetic (seeded generator, same shapes as the configuration)",
           "config": dict(W.describe(), precision=args.precision, parallelism=f"replicas{world}",
                          l2="flushed (256 MB write) between steps", tube_points=r0["n_points"]),
           "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99))},
           "e2e": e2e, "gpu_launches": launches, "clocks": clocks, "roofline": roofline, "cpu_baseline": cpu,
           "accuracy": accuracy, "solve_roofline": solve_roofline,
           "rooflines": {k: {f: v[f] for f in ("bound", "achieved", "peak", "unit", "frac", "avg_launch_ms",
                                               "tensor_issue_frac") if f in v}
                         for k, v in rooflines.items()},
           "solve": {k: r0[k] for k in ("energy", "area", "n_points", "gmres_iters", "matvecs", "matvecs_fp64",
                                        "refinements", "residual", "gmres_status", "reinit_steps", "t_levelset_ms",
                                        "t_surface_ms", "t_plan_ms", "t_tree_ms", "t_operators_ms", "t_solve_ms",
                                        "t_energy_ms", "fmm_nodes",
                                        "fmm_v_pairs", "fmm_x_pairs", "fmm_near_pairs", "fmm_operators")},
           "kernels_ms_per_step": {k: round(v["ms"] / args.steps, 3) for k, v in prof.items()},
           "profiled_pass": {"ms_per_step": statistics.mean(prof_ms), "steps": args.steps,
                             "note": "per-category CUDA events around every launch, in a pass after the timed "
                                     "regions; categories on the main stream include waits for SMs held by the "
                                     "near field on the second stream (m2m, p2m)"},
           "peaks_measured": {"fp64_tflops": fp64_peak, "fp32_tflops": fp32_peak,
                              "hbm_gbs": peaks.get("hbm_gbs"), "bf16_tflops": peaks.get("bf16_tflops")}}
    if rank == 0:
        print(json.dumps(out))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_serve(args):
    """Serving sample: Poisson arrivals of whole-solve requests (atom counts log-uniform, kappa
    uniform in [0, 0.15], eps_out 80, h drawn from --hs) through ibim_server; throughput and p50/p99
    latency.  Batch: the same with every request submitted at once (default 256 molecules of
    50-5000 atoms).  The FP64 energy is computed alone for the smallest requests to state the
    mixed path's error."""
    import ibim

    batch = args.workload == "batch"
    nreq = args.requests or (256 if batch else 40)
    rng = np.random.default_rng(3_000_000 if batch else 5_000_000)
    lo, hi = (float(v) for v in (args.atoms or ("50,5000" if batch else "100,2000")).split(","))
    hs = [float(v) for v in args.hs.split(",")]
    reqs = []
    for k in range(nreq):
        n = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        h = float(rng.choice(hs))
        kappa = float(rng.uniform(0.0, 0.15))
        W = workloads.protein(n, (3_000_000 if batch else 4_000_000) + k, h=h, order=5, kappa=kappa)
        reqs.append(W)
    arrivals = np.zeros(nreq) if batch else np.cumsum(rng.exponential(1.0 / args.rate, size=nreq))
    # warm-up request (kernels loaded, memory pool grown), not counted
    W0 = workloads.protein(100, 4_999_999, h=hs[0], order=5, kappa=0.1)
    ctx0 = ibim.Context(0)
    ctx0.solve(W0.mol.centers, W0.mol.charges, W0.mol.radii, W0.config(ibim.PRECISION_MIXED))
    ctx0.close()
    lock = args.batch_mode == "lockstep"
    srv = ibim.Server(0, slots=args.workers if lock else args.slots, hbm_budget_bytes=150e9, lockstep=lock,
                      max_wave=args.max_wave)
    ids, t0 = [], time.perf_counter()
    for W, ta in zip(reqs, arrivals):
        now = time.perf_counter() - t0
        if ta > now:
            time.sleep(ta - now)
        ids.append(srv.submit(W.mol.centers, W.mol.charges, W.mol.radii, W.config(ibim.PRECISION_MIXED)))
    res = [srv.wait(i) for i in ids]
    t_end = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    lat = np.array([r["latency_ms"] for r in res])
    run = np.array([r["run_ms"] for r in res])
    small = sorted(range(len(reqs)), key=lambda k: reqs[k].mol.n)[:args.accuracy_sample]
    ctx = ibim.Context(0)
    errs = []
    for k in small:
        W = reqs[k]
        e64 = ctx.solve(W.mol.centers, W.mol.charges, W.mol.radii, W.config(ibim.PRECISION_FP64))["energy"]
        errs.append(abs(res[k]["energy"] - e64) / abs(e64))
    ctx.close()
    out = {"metric": ("batched: solves/s, all molecules submitted at once (request loop)" if batch else
                      "serving: solves/s with p50/p99 latency (Poisson arrivals, request loop)"),
           "value": len(res) / t_end, "unit": UNIT, "n_gpus": 1, "higher_is_better": True,
           "dtype": "f32+f64", "data": "synthetic (seeded generator)",
           "config": {"workload": "batch" if batch else "serve_sample", "requests": nreq,
                      "offered_rate_per_s": None if batch else args.rate,
                      "mode": "lockstep" if lock else "pool",
                      "threads": args.workers if lock else args.slots, "max_wave": args.max_wave if lock else None,
                      "atoms_range": [lo, hi], "h_choices": hs, "kappa_range": [0.0, 0.15],
                      "eps_out": 80.0, "chebyshev_order": 5, "precision": "mixed", "hbm_budget_gb": 150},
           "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "mean": float(lat.mean())},
           "run_ms": {"p50": float(np.percentile(run, 50)), "mean": float(run.mean())},
           "wall_s": t_end, "atoms_total": int(sum(W.mol.n for W in reqs)),
           "tube_points_total": int(sum(r["n_points"] for r in res)),
           "all_converged": all(r["gmres_status"] == 0 for r in res),
           "rel_err_vs_fp64_smallest": errs, "server": st}
    print(json.dumps(out))
    return 0


def batch_requests(args):
    """The batched configuration: molecules of the seeded generator, atom counts log-uniform in
    50-5,000 (or --atoms), h = 0.5 A, order 5, kappa uniform in [0, 0.15] per molecule."""
    nreq = args.requests or 256
    rng = np.random.default_rng(3_000_000)
    lo, hi = (float(v) for v in (args.atoms or "50,5000").split(","))
    reqs = []
    for k in range(nreq):
        n = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        kappa = float(rng.uniform(0.0, 0.15))
        reqs.append(workloads.protein(n, 3_000_000 + k, h=0.5, order=5, kappa=kappa))
    return reqs, (lo, hi)


def run_batch_lockstep(args):
    """Batched configuration through ibim_batch_solve: all molecules submitted at once, solved in
    lock-step waves (one launch per FMM stage per wave, GMRES advanced together).  Throughput =
    molecules / wall time of the call; latency = when each molecule's wave finished."""
    import ibim

    reqs, (lo, hi) = batch_requests(args)
    mols = [(W.mol.centers, W.mol.charges, W.mol.radii) for W in reqs]
    cfgs = [W.config(ibim.PRECISION_MIXED) for W in reqs]
    ctx = ibim.Context(0)
    # warm-up: one small wave (kernels loaded, memory pool grown)
    ctx.batch_solve(mols[:2], cfgs[:2], max_wave=2, workers=2)
    sampler = ClockSampler()
    sampler.start()
    t0 = time.perf_counter()
    res, st, info = ctx.batch_solve(mols, cfgs, max_wave=args.max_wave, hbm_budget_bytes=150e9,
                                    workers=args.workers, wave_slots=args.wave_slots)
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    lat = np.array([r["done_ms"] for r in res])
    small = sorted(range(len(reqs)), key=lambda k: reqs[k].mol.n)[:args.accuracy_sample]
    errs = []
    for k in small:
        W = reqs[k]
        e64 = ctx.solve(W.mol.centers, W.mol.charges, W.mol.radii, W.config(ibim.PRECISION_FP64))["energy"]
        errs.append(abs(res[k]["energy"] - e64) / abs(e64))
    ctx.close()
    out = {"metric": "batched: solves/s, all molecules submitted at once (lock-step waves on merged plans)",
           "value": len(res) / wall, "unit": UNIT, "n_gpus": 1, "higher_is_better": True,
           "dtype": "f32+f64", "data": "synthetic (seeded generator)",
           "config": {"workload": "batch", "mode": "lockstep", "molecules": len(reqs), "max_wave": args.max_wave,
                      "workers": args.workers, "wave_slots": args.wave_slots, "atoms_range": [lo, hi], "h": 0.5, "kappa_range": [0.0, 0.15],
                      "eps_out": 80.0, "chebyshev_order": 5, "precision": "mixed", "hbm_budget_gb": 150},
           "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "mean": float(lat.mean())},
           "wall_s": wall, "clocks": clocks, "atoms_total": int(sum(W.mol.n for W in reqs)),
           "tube_points_total": int(sum(r["n_points"] for r in res)),
           "all_converged": all(s == 0 and r["gmres_status"] == 0 for s, r in zip(st, res)),
           "rel_err_vs_fp64_smallest": errs, "batch": info,
           "gmres_iters": {"p50": float(np.median([r["gmres_iters"] for r in res])),
                           "max": int(max(r["gmres_iters"] for r in res))}}
    print(json.dumps(out))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch" and args.batch_mode == "lockstep":
        return run_batch_lockstep(args)
    if args.workload in ("serve", "batch"):
        return run_serve(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())

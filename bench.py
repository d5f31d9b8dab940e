#!/usr/bin/env python3
"""Benchmark of the vebisph time step on GB300: particle-steps/s of div_free.

Default workload: the confined cylinder flow (channel 30R x 4R, blockage 0.5, ~4M fluid
particles on a seeded jittered lattice, Oldroyd-B, Re=0.01, Wi=0.6, beta=0.59), FP64.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One JSON line on rank 0.  `value` is fluid particles x steps / device time of K steps with
the state resident in HBM; `e2e` repeats the measurement through the C-ABI with the state
copied host->device before and device->host after every step (pinned host arrays); the
`roofline` object is for the dominant kernel (the persistent BiCGSTAB solver);
`cpu_baseline` times the CPU restatement of the reference (the oracle; the Fortran reference
cannot be compiled: no Fortran compiler on either machine) on this host's cores.
For N > 1 (torchrun) every rank runs an independent replica on its own GPU (the step does
not shard); `value` sums the ranks' particle-steps over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import copy
import json
import os
import pathlib
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s @4M (mixed vs FP64 GPU, 1e-4 rel err); adjoint/forward cost"
UNIT = "particle-steps/s"


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Dist:
    """Replica bookkeeping: torch.distributed (gloo) only for barriers and the max of times."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, out_dir: str | None = None):
        import tempfile
        self.gpu = gpu_index
        self.proc = None
        d = pathlib.Path(out_dir) if out_dir else pathlib.Path(tempfile.mkdtemp(prefix="vebi_bench_"))
        self.path = d / f"clocks_rank{gpu_index}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
        if not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = [ln.split(",") for ln in self.path.read_text().splitlines() if ln.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows)}


def make_case(args):
    from vebisph_gb300 import cases
    if args.case == "cylinder_4m":
        return cases.cylinder(args.particles, Wi=args.wi, seed=args.seed)
    if args.case == "poiseuille_1m":
        return cases.poiseuille(1000, seed=args.seed)
    if args.case == "cavity_1m":
        return cases.cavity(1024, seed=args.seed)
    if args.case == "poiseuille_40":
        return cases.poiseuille(40, seed=args.seed)
    raise SystemExit(f"unknown case {args.case}")


def ppe_bytes_per_iteration(n_rows: int, nnz_off: int, mixed: bool = False) -> float:
    """Algorithmic bytes of one fused BiCGSTAB iteration (closed domain).
    FP64: 2 SpMV x (12 B per off-diagonal slot + 44 B per row: count, diagonal, x_i, gathered
    x, y, one dot operand) + 168 B per row of vector phases (p update 32, mean removal 24, s 24,
    s mean removal 24, x/r update 64).
    Mixed: 2 SpMV x (8 B per slot: FP32 value + column; + 44 B per row: count, FP64 row sum,
    x_i and gathered x as FP32 pairs, y, one dot operand) + 184 B per row of FP64 vector phases
    (p update 32, mean removal + split 24, s 24, s mean removal + split 24, x/r update 64 + 16)."""
    if mixed:
        return 2.0 * (8.0 * nnz_off + 44.0 * n_rows) + 184.0 * n_rows
    return 2.0 * (12.0 * nnz_off + 44.0 * n_rows) + 168.0 * n_rows


def workload_text(args, case, precision: str) -> str:
    Re = (case.Ra / case.Pr) ** 0.5
    common = (f"{case.n_fluid} fluid + {case.nbS} wall particles, dx={case.dx:.4g}, Oldroyd-B Re={Re:.3g} "
              f"Wi={case.El * Re:.3g} beta={case.beta}, {precision}, PPE preconditioner {args.precond}")
    if args.case == "cylinder_4m":
        return f"{case.name}: confined cylinder, channel 30R x 4R, blockage 0.5, periodic x, " + common
    if args.case.startswith("poiseuille"):
        return f"{case.name}: planar Poiseuille channel 1x1, periodic x, walls y=0,1, body force, " + common
    return f"{case.name}: " + common


DATA_TEXT = ("synthetic: seeded jittered lattice (U(-0.01dx,0.01dx)), walls/circle by the reference's "
             "make_boundary_particles rules; no dataset")


def bench_config(args, case, precision: str) -> dict:
    """The workload description both arms print (the same keys and values on both)."""
    return {"workload": workload_text(args, case, precision), "npfb": case.npfb, "n_fluid": case.n_fluid,
            "precision": precision,
            "l2": (f"inputs larger than L2: the pair arrays and the PPE matrix hold {case.npfb * 75 * 40 / 1e9:.2f} GB "
                   "(ELL width 75; link 4 B, three weights 24 B, matrix 12 B per slot), no flush")}


def stage_bandwidth(stage_ms_per_step: dict, n: int, kbar: float, mixed: bool, peak: float) -> dict:
    """Per-stage achieved bandwidth on algorithmic bytes (each array the stage reads or writes
    counted once per element, pair arrays at the mean neighbour count kbar, FP32-stored arrays at
    4 B in the mixed step; a stage's several kernels share its time) over the stage's CUDA-event
    time.  The FP64 pair stages are bound by the FP64 pipe (1.2 TFLOP/s on GB300), not HBM."""
    w = 4.0 if mixed else 8.0
    per_particle = {
        "advect_bin": 90.0,
        "neighbours": 16 + 4 + 4 * kbar + 4,
        "weights": (4 + 3 * w) * kbar + 48,
        "shifting": (4 + 2 * w) * kbar + 64,
        "gradients": (4 + 2 * w) * kbar + 168,   # the three gradient calls fused: one pass over the pairs
        "logconf": 120.0,
        "predictor": (4 + 3 * w) * kbar + 160,
        "ppe_assembly": (24 + 3 * w) * kbar + 84,  # right-hand side, then the matrix (FP64 value + column)
        "pressure_grad": (4 + 2 * w) * kbar + 56,
    }
    out = {}
    for k, b in per_particle.items():
        ms = stage_ms_per_step.get(k)
        if ms:
            gbs = b * n / (ms * 1e-3) / 1e9
            out[k] = {"bytes_per_particle": round(b, 1), "ms": ms, "GB_s": round(gbs, 1), "frac": round(gbs / peak, 4)}
    return out


def mg_bytes_per_iteration(n_rows: int, nnz_off: int, n_cells: int, mixed: bool = False,
                           pairs: float = 5.0) -> float:
    """Algorithmic bytes of one multigrid-preconditioned BiCGSTAB iteration (closed domain),
    pass by pass; k = off-diagonal slots per row.  `pairs` (the mean (cell, value) pairs of A P
    per row) is reported beside the figure; the output pass reads A P by 3x3 direction, eight
    values per row whatever the pair count.

    BiCGSTAB passes: p update 32 (r, v, p; p), v (w, row sum, r_bar; v), s 24 (v, r; s), t (w,
    row sum, s; t), x/r update 64 (the two preconditioned directions, x, t, s, r_bar; x, r).
    The products A M^-1 p and A M^-1 s are the V-cycle's w: FP64 in the FP64 solver (v and t
    32 B each, 184 B in all), FP32 in the mixed one (28 B each, 176 B in all).
    Two V-cycles, particle level:
      mean removal and first sweep: FP64 32 B (q, 1/diag; q, z), mixed 28 (q, FP32 1/diag; q,
        FP32 q and z);
      residual: FP64 36 + 12k (count, diagonal, z_i, q; fr), mixed 20 + 8k (count, FP32 row
        sum, z_i and q; FP32 fr);
      restriction: FP64 12, mixed 8 (cell list entry, fr);
      output: FP64 120 (cell, packed word, z, fr, q, row sum, eight FP64 direction values; the
        direction and w), mixed 68 (the same in FP32 but the FP64 direction, and w in FP32).
    Coarse levels: ~390 B per cell (the cell level's ELL rows read by the residual and the
    smoothing sweep, work vectors, and the geometric sum of the coarser levels)."""
    if mixed:
        fine = 8.0 * nnz_off + (28.0 + 20.0 + 8.0 + 68.0) * n_rows
        krylov = 176.0
    else:
        fine = 12.0 * nnz_off + (32.0 + 36.0 + 12.0 + 120.0) * n_rows
        krylov = 184.0
    return krylov * n_rows + 2.0 * (fine + 390.0 * n_cells)


def cpu_baseline(case, gpu_iters_per_step: float, itermax_sample: int):
    """Time the oracle (CPU restatement of the reference) on this host's cores on a bounded
    sample: one full step whose BiCGSTAB is capped at itermax_sample iterations; the step time
    is scaled to the GPU's iterations per step: t = t_rest + t_solve/iters_sample*iters_gpu."""
    from oracle.oracle import OracleSolver, threads
    o = OracleSolver(case)
    o.set_itermax(itermax_sample)
    o.step()  # warm-up (first touch of the arrays)
    t0 = time.perf_counter()
    s = o.step()
    wall = (time.perf_counter() - t0) * 1e3
    total, solve, iters = s["stage_ms"][14], s["stage_ms"][10], max(s["LS_iters"], 1)
    rest = total - solve
    per_iter = solve / iters
    t_step = rest + per_iter * gpu_iters_per_step
    o.close()
    value = case.n_fluid / (t_step * 1e-3)
    return {"value": value, "unit": UNIT, "cores": threads(), "kind": "port",
            "sample": (f"one oracle step of the same case with BiCGSTAB capped at {itermax_sample} "
                       f"iterations ({iters} run): non-solver {rest:.0f} ms + {per_iter:.1f} ms/iteration "
                       f"scaled to {gpu_iters_per_step:.0f} iterations/step = {t_step:.0f} ms/step; "
                       f"wall {wall:.0f} ms")}


def run_gb300(args, dist: Dist):
    from vebisph_gb300 import abi
    from vebisph_gb300.solver import StepSolver
    import ctypes as C

    case = make_case(args)
    if getattr(args, "perturb", 0.0):  # fluid positions moved by args.perturb * dx (seeded)
        rng = np.random.default_rng(12345)
        case.r[case.nbS:] = case.r[case.nbS:] + args.perturb * case.dx * rng.standard_normal(case.r[case.nbS:].shape)
    if args.itermax:
        case.itermax = args.itermax
    case.ppe_warm_start = 1 if args.warm_start else 0
    case.ppe_precond = abi.PRECOND_MULTIGRID if args.precond == "multigrid" else abi.PRECOND_NONE
    prec = abi.PREC_MIXED if args.precision == "mixed" else abi.PREC_FP64
    sol = StepSolver(case, precision=prec, timing=True)
    n_fluid = case.n_fluid
    # warm-up steps (untimed)
    for _ in range(args.warmup):
        sol.step()
    dist.barrier()
    with ClockSampler(dist.local, args.out_dir) as clk:
        ms, st = sol.run_steps(args.steps)
    dist.barrier()
    # state after warm-up + timed steps (before the e2e steps), for the precision comparison
    fields = {k: sol.get(k)[: case.npfb].copy() for k in ("ux", "uy", "p", "tau11", "tau22", "rx")}
    t_max = dist.max(ms)
    units = dist.sum(float(n_fluid * args.steps))
    value = units / (t_max * 1e-3)
    ls_total = st["LS_iters_total"]
    iters_per_step = ls_total / args.steps
    stage = st["stage_ms"]
    solve_ms = stage[10]
    # roofline of the dominant kernel: the persistent BiCGSTAB launch (one per step)
    cnt = sol.get("ij_count")
    nnz_off = int(cnt.sum())
    mg = case.ppe_precond == abi.PRECOND_MULTIGRID
    if mg:
        cp = sol.get("cellpart")[: case.npfb]
        n_cells = int(np.unique(cp[cp >= 0]).size)
        pairs = float(sol.get("mg_pairs").mean())
        bytes_iter = mg_bytes_per_iteration(case.npfb, nnz_off, n_cells, mixed=prec == abi.PREC_MIXED, pairs=pairs)
    else:
        bytes_iter = ppe_bytes_per_iteration(case.npfb, nnz_off, mixed=prec == abi.PREC_MIXED)
    per_launch_bytes = bytes_iter * iters_per_step
    per_launch_s = solve_ms * 1e-3 / args.steps
    achieved = per_launch_bytes / per_launch_s / 1e9
    peak, peak_kind = peaks()
    traffic = None
    tf = ROOT / "profiles" / "traffic_bicgstab.json"
    if tf.exists():
        tj = json.loads(tf.read_text())
        # measured DRAM bytes per iteration on a small case, scaled by rows x iterations
        traffic = tj["dram_bytes_per_row_iteration"] * case.npfb * iters_per_step
    kname = ("k_bicgstab_mixed<true> (persistent cooperative BiCGSTAB, FP32 SpMV, one launch per step)"
             if prec == abi.PREC_MIXED else "k_bicgstab<true> (persistent cooperative BiCGSTAB, one launch per step)")
    if mg:
        kname = ("k_bicgstab_mixed_mg<true>" if prec == abi.PREC_MIXED else "k_bicgstab_mg<true>") + \
            " (persistent cooperative BiCGSTAB with the multigrid V-cycle; the set-up kernels are in the stage time)"
    if mg:  # measured DRAM bytes per row-iteration of the preconditioned solvers at 1M rows
        tmg = ROOT / "profiles" / ("traffic_bicgstab_multigrid_mixed.json" if prec == abi.PREC_MIXED
                                   else "traffic_bicgstab_multigrid.json")
        traffic = (json.loads(tmg.read_text())["dram_bytes_per_row_iteration"] * case.npfb * iters_per_step
                   if tmg.exists() else None)
    elif prec == abi.PREC_MIXED:
        traffic = None
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic,
            "kernel": kname,
            "peak_kind": f"{peak_kind} hbm_gbs (burst copy)",
            "bytes_per_iteration": bytes_iter, "iterations_per_launch": iters_per_step,
            "mg_pairs_per_row": round(pairs, 3) if mg else None,
            "launch_ms": round(per_launch_s * 1e3, 3)}
    # end to end through the C-ABI with host buffers (pinned), copies inside the timed region:
    # the time loop of a host driver that owns the state in its arrays (the Fortran module
    # arrays behind div_free).  Every step uploads the arrays, steps, and downloads the new
    # state into the same arrays, so the state carries from step to step.
    e2e = None
    if not args.no_e2e:
        n = case.npfb
        host = sol.download()  # the state the GPU holds after the timed steps
        host = {k: np.ascontiguousarray(host[k]) for k in ("r", "u", "tau", "theta", "trace_conf", "inbin", "p")}
        pinned = []
        for a in host.values():
            if sol.lib.vebi_pin_host(a.ctypes.data_as(C.c_void_p), a.nbytes) == 0:
                pinned.append(a)
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
        h2d = sum(host[k].nbytes for k in ("r", "u", "tau", "theta", "trace_conf", "inbin"))
        d2h = sum(host[k].nbytes for k in ("r", "u", "tau", "theta", "trace_conf", "inbin", "p"))
        t_up = t_step = t_down = 0.0
        down_ms = []
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            ta = time.perf_counter()
            sol.upload(host["r"], host["u"], host["tau"], host["theta"], host["trace_conf"], host["inbin"], n)
            tb = time.perf_counter()
            sol.step()
            tc = time.perf_counter()
            sol.lib.vebi_download_state(sol.h, dp(host["r"]), dp(host["u"]), dp(host["tau"]), dp(host["theta"]),
                                        dp(host["p"]), None, None, dp(host["trace_conf"]), None,
                                        host["inbin"].ctypes.data_as(C.POINTER(C.c_uint8)), n)
            td = time.perf_counter()
            t_up, t_step, t_down = t_up + tb - ta, t_step + tc - tb, t_down + td - tc
            down_ms.append(round(1e3 * (td - tc), 2))
        e2e_s = time.perf_counter() - t0
        dist.barrier()
        e2e_s = dist.max(e2e_s)
        pinned_ok = len(pinned) == len(host)
        for a in pinned:
            sol.lib.vebi_unpin_host(a.ctypes.data_as(C.c_void_p))
        k = max(args.e2e_steps, 1)
        e2e = {"value": dist.sum(float(n_fluid * args.e2e_steps)) / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "steps": args.e2e_steps,
               "host_pinned": pinned_ok,
               "ms_per_step": {"upload_call": round(1e3 * t_up / k, 3), "step": round(1e3 * t_step / k, 3),
                               "download": round(1e3 * t_down / k, 3)},
               "download_ms_each_step": down_ms,
               "path": "vebi_upload_state + vebi_step + vebi_download_state on pinned host arrays that carry "
                       "the state from step to step (upload is asynchronous; its copies complete inside the step "
                       "call, whose stats read-back waits for the stream)"}
    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if prec == abi.PREC_FP64 else "f32+f64",
        "data": DATA_TEXT,
        "config": bench_config(args, case, args.precision),
        "parallelism": f"replicas x{dist.world} (the step does not shard; one independent replica per GPU)",
        "LS_iters_per_step": iters_per_step,
        "LS_residual_last": st["LS_residual"],
        "stage_ms_per_step": {abi.STAGE_NAMES[i]: round(v / args.steps, 3) for i, v in enumerate(stage) if v > 0},
        "stage_bandwidth": stage_bandwidth({abi.STAGE_NAMES[i]: v / args.steps for i, v in enumerate(stage) if v > 0},
                                           case.npfb, nnz_off / case.npfb, prec == abi.PREC_MIXED, peak),
        "gpu_launches": st["gpu_launches"],
        "roofline": roof,
        "e2e": e2e,
        "clocks": clk.summary(),
        "nmirror": st["nmirror"], "maxneighbours": st["maxneighbours"],
        "drag": drag_summary(case, st, fields),
    }
    res["_fields"] = fields
    sol.close()
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu:
        res["cpu_baseline"] = cpu_baseline(case, iters_per_step, args.cpu_iters)
    return res


def run_adjoint(args, dist: Dist, ref: dict | None = None) -> dict:
    """Reverse mode on the heated-cavity workload (differentially heated square cavity,
    args.adjoint_side^2 fluid particles, Ra=1e5, Pr=1, Oldroyd-B Wi=0.5, beta=0.5, seeded
    perturbed temperature), FP64 or mixed-precision step (args.adjoint_precision) with the
    reference's PPE solver or the multigrid (args.precond): J = mean kinetic energy
    after a window of args.adjoint steps, dJ/dtheta0 (full field) and dJ/dWi, checkpoints every
    args.checkpoint steps.  Forward cost = the plain steps of the window (captured graph);
    adjoint cost = the reverse sweep, its recompute of every segment included.  With
    args.adjoint_fd > 0, that many seeded directions of theta0, and Wi, are checked by central
    differences of the replayed window (step args.adjoint_eps).  `ref` is the result of another
    run on the same workload (the FP64 window): the directional derivatives along the same
    seeded directions and dJ/dWi are reported against it."""
    from vebisph_gb300 import abi, cases
    from vebisph_gb300.solver import Adjoint, StepSolver
    if dist.rank != 0:
        return None
    side, N, K = args.adjoint_side, args.adjoint, args.checkpoint
    case = cases.cavity(n=side, seed=args.seed, Ra=1.0e5, Pr=1.0, Wi=0.5, beta=0.5)
    case.const_mod = args.adjoint_const_mod
    case.tol = args.adjoint_tol
    if args.precond == "multigrid":
        case.ppe_precond = abi.PRECOND_MULTIGRID
    mixed = args.adjoint_precision == "mixed"
    s = StepSolver(case, precision=abi.PREC_MIXED if mixed else abi.PREC_FP64)
    for _ in range(max(args.warmup, args.adjoint_spinup)):
        s.step()
    st0 = s.download()
    t0 = time.perf_counter()
    _, sf = s.run_steps(N)
    t_fwd = time.perf_counter() - t0
    fwd_iters = sf["LS_iters_total"]
    s.upload(st0["r"], st0["u"], st0["tau"], st0["theta"], st0["trace_conf"], st0["inbin"], case.npfb)
    adj = Adjoint(s, max_steps=N, checkpoint_every=K)
    t0 = time.perf_counter()
    adj.record(N)
    t_rec = time.perf_counter() - t0
    fin = s.download()
    nbS, n = case.nbS, case.npfb
    J = 0.5 * float(np.mean(fin["u"][0, nbS:] ** 2 + fin["u"][1, nbS:] ** 2))
    seed = np.zeros((2, n))
    seed[:, nbS:] = fin["u"][:, nbS:] / (n - nbS)
    t0 = time.perf_counter()
    g = adj.reverse(seed_u=seed)
    t_rev = time.perf_counter() - t0
    def kinetic():
        u = s.download()["u"]
        return 0.5 * float(np.mean(u[0, nbS:] ** 2 + u[1, nbS:] ** 2))

    def direction(k):
        rng = np.random.default_rng(1000 + k)
        d = np.zeros(n)
        d[nbS:] = rng.normal(size=n - nbS)
        return d / np.abs(d).max()

    # central differences of the replayed window (the differentiated map) along seeded
    # unit-max directions of theta0, step args.adjoint_eps; and of Wi, step eps * Wi
    eps = args.adjoint_eps
    fd = []
    t0 = time.perf_counter()
    for k in range(args.adjoint_fd):
        d = direction(k)
        js = []
        for sgn in (1.0, -1.0):
            s.upload(st0["r"], st0["u"], st0["tau"], st0["theta"] + sgn * eps * d, st0["trace_conf"], st0["inbin"], n)
            adj.replay(N)
            js.append(kinetic())
        f = (js[0] - js[1]) / (2 * eps)
        a = float(g["theta"] @ d)
        fd.append({"direction": k, "fd": f, "adjoint": a, "rel_err": abs(f - a) / max(abs(f), 1e-300)})
    fd_wi = None
    if args.adjoint_fd and case.const_mod != 1:
        wi0 = 0.5
        h = eps * wi0
        js = []
        for sgn in (1.0, -1.0):
            s.set_weissenberg(wi0 + sgn * h)
            s.upload(st0["r"], st0["u"], st0["tau"], st0["theta"], st0["trace_conf"], st0["inbin"], n)
            adj.replay(N)
            js.append(kinetic())
        s.set_weissenberg(wi0)
        f = (js[0] - js[1]) / (2 * h)
        fd_wi = {"fd": f, "adjoint": g["wi"], "rel_err": abs(f - g["wi"]) / max(abs(f), 1e-300)}
    t_fd = time.perf_counter() - t0
    # directional derivatives along the same seeded directions, for a run compared with this one
    dirs = [float(g["theta"] @ direction(k)) for k in range(args.adjoint_dirs)]
    vs = None
    if ref is not None:
        rd = ref["directional_derivatives"]
        vs = {"directional_rel_diff": [abs(x - y) / max(abs(y), 1e-300) for x, y in zip(dirs, rd)],
              "dJ_dWi_rel_diff": abs(g["wi"] - ref["dJ_dWi"]) / max(abs(ref["dJ_dWi"]), 1e-300)}
        if ref.get("finite_differences"):
            vs["vs_fp64_fd_rel"] = [abs(x - e["fd"]) / max(abs(e["fd"]), 1e-300)
                                    for x, e in zip(dirs, ref["finite_differences"])]
    adj.close()
    s.close()
    solver = ("the multigrid-preconditioned PPE (forward and transposed)" if args.precond == "multigrid"
              else "the reference's PPE solver")
    model = "Oldroyd-B Wi=0.5 beta=0.5" if case.const_mod != 1 else "Newtonian (const_mod 1) beta=0.5"
    step = ("mixed-precision step (FP32 pair sums and SpMV; the VJP in FP64 on its widened weights, "
            "the transposed solve by the context's mixed solver)" if mixed else "FP64 step")
    return {"workload": f"{case.name}: heated cavity, {n - nbS} fluid + {nbS} wall particles, Ra=1e5 Pr=1 "
                        f"{model}, {step}, {solver}, PPE tol {case.tol:g}, {args.adjoint_spinup} steps "
                        f"of spin-up",
            "precision": args.adjoint_precision,
            "window_steps": N, "checkpoint_every": K, "J": J,
            "forward_ms_per_step": 1e3 * t_fwd / N, "record_ms_per_step": 1e3 * t_rec / N,
            "reverse_ms_per_step": 1e3 * t_rev / N, "adjoint_over_forward": t_rev / t_fwd,
            "forward_LS_iters_per_step": fwd_iters / N, "transposed_LS_iters_per_step": g["ls_iters"] / N,
            "near_pole_particles_per_step": sf["n_near_pole_total"] / N,
            "dJ_dWi": g["wi"], "grad_theta_max_abs": float(np.abs(g["theta"]).max()),
            "grad_theta_abs_percentiles": {str(q): float(np.percentile(np.abs(g["theta"][nbS:]), q))
                                           for q in (50, 99, 99.99, 100)},
            "directional_derivatives": dirs,
            "finite_differences": fd,
            "fd_eps": eps if fd else None,
            "fd_within_1e-5": (f"{sum(e['rel_err'] <= 1e-5 for e in fd)}/{len(fd)}" if fd else None),
            "fd_rel_err_max": max((e["rel_err"] for e in fd), default=None),
            "fd_dJ_dWi": fd_wi,
            "fd_seconds": round(t_fd, 1),
            "vs_fp64_window": vs,
            "timing": "host wall clock around the synchronous calls (each call waits for its GPU work)"}


def run_batch(args, dist: Dist):
    """The batched parameter sweep: args.batch independent Poiseuille/cylinder instances with
    log-uniform fluid counts in 4k-256k, Wi ~ U[0.1, 4], beta ~ U[0.1, 0.9] (seeded), mixed
    precision, advanced together by vebi_batch_step (one CUDA-graph launch per step), against the
    same instances run one by one with the plain FP64 step.  Each instance's velocity error is
    max |u_mixed - u_fp64| / max |u_fp64| after the same steps from the same initial state."""
    from vebisph_gb300 import abi, cases
    from vebisph_gb300.solver import BatchSolver, StepSolver, VebiError

    cl = cases.batch_sweep(args.batch, seed=args.seed)
    mg = args.batch_precond == "multigrid"
    for c in cl:
        c.ppe_precond = abi.PRECOND_MULTIGRID if mg else abi.PRECOND_NONE
    n_fluid = sum(c.n_fluid for c in cl)
    t0 = time.perf_counter()
    bprec = abi.PREC_MIXED if args.batch_precision == "mixed" else abi.PREC_FP64
    b = BatchSolver(cl, precision=bprec)
    t_create = time.perf_counter() - t0
    # divergence guard: each instance fails with its own status if its velocity turns non-finite
    # or passes 100x its flow's velocity scale (the channels and cylinders are scaled to ~1)
    for inst, c in zip(b.instances, cl):
        inst.set_velocity_limit(100.0 * max(1.0, float(np.abs(c.u).max())))
    tune = b.autotune(candidates=tuple(int(v) for v in args.tune.split(",")),
                      coarse_candidates=(tuple(int(v) for v in args.tune_coarse.split(",")) if mg else (2048,)))
    done = 2 * len(tune["ms_per_candidate"])
    for _ in range(args.warmup):
        b.step(1)
    dist.barrier()
    with ClockSampler(dist.local, args.out_dir) as clk:
        ms, stats = b.step(args.steps)
    dist.barrier()
    done += args.warmup + args.steps
    t_max = dist.max(ms)
    fields = [{k: inst.get(k)[: c.npfb].copy() for k in ("ux", "uy", "p")} for inst, c in zip(b.instances, cl)]
    iters = [st["LS_iters_total"] / args.steps for st in stats]
    failed = {i: st["error"] for i, st in enumerate(stats) if st["error"]}
    b.close()
    # only instances that stepped without failure count as work
    n_live = sum(c.n_fluid for i, c in enumerate(cl) if i not in failed)
    value = dist.sum(float(n_live * args.steps)) / (t_max * 1e-3)
    # the same instances one by one, plain FP64, timed over the same K steps (device events)
    serial_ms, serial_units, du, dp, per, spread = 0.0, 0, [], [], [], []
    light = getattr(args, "batch_light", False)  # the default line: speed only, no accuracy reruns
    for i, (c, fm) in enumerate(zip([] if light else cl, fields)):
        s1 = StepSolver(c, precision=abi.PREC_FP64)
        rec = {"i": i, "case": c.name, "n_fluid": c.n_fluid, "El": c.El, "beta": c.beta,
               "batch_error": failed.get(i, 0), "LS_iters_batch": iters[i]}
        try:
            for _ in range(done - args.steps):
                s1.step()
            m1, st1 = s1.run_steps(args.steps)
            serial_ms += m1
            serial_units += c.n_fluid * args.steps
            rec["LS_iters_fp64"] = st1["LS_iters_total"] / args.steps
            ux, uy, pp = (s1.get(k)[: c.npfb] for k in ("ux", "uy", "p"))
            if not (np.isfinite(ux).all() and np.isfinite(uy).all() and np.isfinite(pp).all()):
                rec["fp64_error"] = "non-finite"
            elif i not in failed:
                us = max(np.abs(ux).max(), np.abs(uy).max(), 1e-300)
                rec["du"] = float(max(np.abs(fm["ux"] - ux).max(), np.abs(fm["uy"] - uy).max()) / us)
                rec["dp"] = float(np.abs(fm["p"] - pp).max() / max(np.abs(pp).max(), 1e-300))
                if not np.isfinite(rec["du"]):
                    rec["du"] = float("inf")
                du.append(rec["du"])
                dp.append(rec["dp"])
                # the flow's own sensitivity: FP64 again from a velocity perturbed at FP32 rounding
                # level (relative 6e-8, seeded), same steps
                cp_ = copy.deepcopy(c)
                rng = np.random.default_rng(1000 + i)
                cp_.u = cp_.u * (1.0 + 6e-8 * rng.standard_normal(cp_.u.shape))
                s2 = StepSolver(cp_, precision=abi.PREC_FP64)
                try:
                    for _ in range(done):
                        s2.step()
                    vx, vy = (s2.get(k)[: c.npfb] for k in ("ux", "uy"))
                    rec["fp64_spread"] = float(max(np.abs(vx - ux).max(), np.abs(vy - uy).max()) / us)
                except VebiError:
                    rec["fp64_spread"] = float("inf")
                s2.close()
                spread.append(rec["fp64_spread"])
        except VebiError as e:
            rec["fp64_error"] = e.status
        s1.close()
        per.append(rec)
    serial_value = serial_units / (serial_ms * 1e-3) if serial_ms > 0 else None
    plain = None
    if mg:  # the reference's solver one by one: K steps from the initial state (speed only)
        pms, punits = 0.0, 0
        for c in cases.batch_sweep(args.batch, seed=args.seed):
            s1 = StepSolver(c, precision=abi.PREC_FP64)
            try:
                m1, _ = s1.run_steps(args.steps)
                pms += m1
                punits += c.n_fluid * args.steps
            except VebiError:
                pass
            s1.close()
        plain = {"value": punits / (pms * 1e-3), "unit": UNIT, "ms_per_step": pms / args.steps,
                 "path": "one StepSolver per instance, plain FP64, unpreconditioned PPE (the reference's solver), "
                         f"{args.steps} steps from the initial state"}
    du, dp, spread = np.array(du), np.array(dp), np.array(spread)
    counts = np.array([c.n_fluid for c in cl])
    if args.out_dir:  # the per-instance records
        pathlib.Path(args.out_dir).mkdir(parents=True, exist_ok=True)
        (pathlib.Path(args.out_dir) / f"batch{args.batch}_instances.json").write_text(json.dumps(per))
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if bprec == abi.PREC_MIXED else "f64",
        "data": "synthetic: seeded jittered lattices, walls/circle by the reference's make_boundary_particles rules",
        "config": {"workload": f"batch{args.batch}: {args.batch} independent instances (even: Poiseuille channel, "
                               f"odd: confined cylinder), fluid counts log-uniform 4k-256k, Wi~U[0.1,4], "
                               f"beta~U[0.1,0.9], seed {args.seed}, {args.batch_precision}, PPE preconditioner {args.batch_precond}",
                   "instances": args.batch, "n_fluid_total": n_fluid,
                   "n_fluid_min": int(counts.min()), "n_fluid_max": int(counts.max()),
                   "parallelism": f"batch (one CUDA graph per step, {args.batch} branches) x{dist.world} replicas",
                   "l2": f"inputs larger than L2 (all instances' arrays resident: {n_fluid} particles)",
                   "autotune": tune, "create_s": round(t_create, 2)},
        "gpu_launches": int(sum(st["gpu_launches"] for st in stats)),
        "LS_iters_per_step": {"mean": float(np.mean(iters)), "max": float(np.max(iters))},
        "failed_instances": {"batch": len(failed), "serial_fp64": sum(1 for r in per if "fp64_error" in r),
                             "both": sum(1 for r in per if "fp64_error" in r and r["batch_error"]),
                             "statuses": sorted(set(failed.values()))},
        "serial_fp64": ({"value": serial_value, "unit": UNIT, "ms_per_step": serial_ms / args.steps,
                         "speedup_of_batch": value / serial_value, "counted": "instances that did not fail",
                         "path": "one StepSolver per instance, FP64, same PPE preconditioner as the batch, "
                                 "graph-replayed steps, summed device time"} if serial_value else None),
        "serial_plain_fp64": plain,
        "speedup_vs_serial_plain_fp64": (value / plain["value"]) if plain else None,
        "batch_vs_serial_fp64": ({
            "compared": int(du.size), "note": "instances where neither run failed; u = max|du|/max|u_fp64|",
            "u_rel_median": float(np.median(du)), "u_rel_p90": float(np.percentile(du, 90)),
            "u_within_1e-4": int((du <= 1e-4).sum()), "u_within_1e-3": int((du <= 1e-3).sum()),
            "u_within_1e-2": int((du <= 1e-2).sum()), "p_rel_median": float(np.median(dp)),
            "fp64_spread_median": float(np.median(spread[np.isfinite(spread)])) if np.isfinite(spread).any() else None,
            "u_within_max_1e-4_2x_fp64_spread": int((du <= np.maximum(1e-4, 2.0 * spread)).sum()),
            "spread_note": "fp64_spread: FP64 rerun from velocities perturbed by 6e-8 relative (FP32 rounding) "
                           "after the same steps; the flow's own amplification of rounding-level differences"}
            if du.size else None),
        "roofline": None,
        "clocks": clk.summary(),
    }


def drag_summary(case, st: dict, fields: dict):
    """Force of the fluid on the cylinder after the last timed step and the drag coefficient
    (vebisph_gb300/diagnostics.py)."""
    from vebisph_gb300 import diagnostics
    return diagnostics.drag(case, st["circle_force"], fields["ux"])


def mixed_summary(f64: dict, mx: dict) -> dict:
    """Speed of the mixed step and its difference from the FP64 step after the same steps from
    the same initial state: velocity and pressure (max abs difference / max abs FP64 value),
    the first normal-stress difference N1 = tau_xx - tau_yy at its wake maximum (x > R)."""
    a, b = mx["_fields"], f64["_fields"]
    us = max(np.abs(b["ux"]).max(), np.abs(b["uy"]).max())
    du = max(np.abs(a["ux"] - b["ux"]).max(), np.abs(a["uy"] - b["uy"]).max()) / us
    dp = np.abs(a["p"] - b["p"]).max() / max(np.abs(b["p"]).max(), 1e-300)
    from vebisph_gb300 import diagnostics
    n1a = diagnostics.n1_wake_max(b["rx"], a["tau11"], a["tau22"])
    n1b = diagnostics.n1_wake_max(b["rx"], b["tau11"], b["tau22"])
    dt11 = np.abs(a["tau11"] - b["tau11"]).max() / max(np.abs(b["tau11"]).max(), 1e-300)
    return {"value": mx["value"], "unit": UNIT, "ms_per_step": mx["ms_per_step"],
            "speedup_vs_fp64": mx["value"] / f64["value"], "LS_iters_per_step": mx["LS_iters_per_step"],
            "LS_residual_last": mx["LS_residual_last"], "roofline": mx["roofline"],
            "stage_ms_per_step": mx["stage_ms_per_step"], "gpu_launches": mx["gpu_launches"],
            "rel_diff_vs_fp64": {"u": float(du), "p": float(dp), "tau_xx": float(dt11),
                                 "N1_wake_max": abs(n1a - n1b) / max(abs(n1b), 1e-300)},
            "N1_wake_max": {"mixed": n1a, "fp64": n1b},
            "drag": mx.get("drag"),
            "drag_rel_diff_vs_fp64": (abs(mx["drag"]["F_x"] - f64["drag"]["F_x"]) / abs(f64["drag"]["F_x"])
                                      if mx.get("drag") and f64.get("drag") else None),
            "note": ("both PPE solves stop at the 1000-iteration cap unconverged on this workload (see "
                     "LS_residual_last); on converging cases the mixed velocity stays within 1e-4 of FP64 "
                     "(tests/test_gpu_mixed.py)")}


def multigrid_summary(plain: dict, f64: dict, mx: dict, pert: dict | None = None) -> dict:
    """The opt-in multigrid-preconditioned PPE on the same workload: FP64 and mixed precision,
    both converging to the solver tolerance; speed-ups and the mixed-vs-FP64 differences."""
    keep = ("value", "ms_per_step", "LS_iters_per_step", "LS_residual_last", "stage_ms_per_step", "roofline",
            "gpu_launches", "drag")
    out = {"fp64": {k: f64[k] for k in keep}, "mixed": {k: mx[k] for k in keep}}
    out["speedup_mixed_vs_fp64"] = mx["value"] / f64["value"]
    out["speedup_fp64_vs_plain_fp64"] = f64["value"] / plain["value"]
    out["speedup_mixed_vs_plain_fp64"] = mx["value"] / plain["value"]
    d = mixed_summary(f64, mx)
    out["mixed_vs_fp64"] = {"rel_diff": d["rel_diff_vs_fp64"], "drag_rel_diff": d["drag_rel_diff_vs_fp64"],
                            "N1_wake_max": d["N1_wake_max"]}
    if pert is not None:  # the flow's own sensitivity: FP64 from positions moved at FP32 rounding level
        e = mixed_summary(f64, pert)
        out["fp64_self_spread"] = {"rel_diff": e["rel_diff_vs_fp64"], "drag_rel_diff": e["drag_rel_diff_vs_fp64"],
                                   "perturbation": "fluid positions + 6e-8 dx (seeded normal), FP64, same steps"}
    out["note"] = ("opt-in (ppe_precond = VEBI_PRECOND_MULTIGRID): aggregation multigrid on the cell grid; "
                   "both precisions converge to tol 1e-8 each step, the plain solver stops at its 1000-iteration cap")
    return out


def run_reference(args, dist: Dist):
    """The reference's own CPU path timed on this host: the oracle restatement (the Fortran
    reference has no compiler here), all host threads.

    A full step of the 4M workload takes ~30 s on 16 cores (its BiCGSTAB runs to the
    1000-iteration cap), so the K timed steps are bounded samples: each is a whole step with
    BiCGSTAB capped at args.cpu_iters iterations, and `ms_per_step` is their measured mean.
    `value` is measured too: one full step at the workload's own cap, run once after the
    warm-up (`full_step`), converted to particle-steps/s.  The samples' model -- non-solver
    time + per-iteration time x the full step's iterations -- is reported beside it with its
    error against that full step."""
    if dist.rank != 0:
        return None
    from oracle.oracle import OracleSolver, threads
    case = make_case(args)
    o = OracleSolver(case)
    o.set_itermax(args.cpu_iters)
    for _ in range(args.warmup):
        o.step()
    full = None
    if not args.no_full_step:
        o.set_itermax(case.itermax)
        t0 = time.perf_counter()
        s = o.step()
        full = {"wall_ms": 1e3 * (time.perf_counter() - t0), "LS_iters": s["LS_iters"],
                "LS_residual": s["LS_residual"], "stage_total_ms": s["stage_ms"][14]}
        o.set_itermax(args.cpu_iters)
    tot = solve = wall = 0.0
    iters = 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        s = o.step()
        wall += time.perf_counter() - t0
        tot += s["stage_ms"][14]
        solve += s["stage_ms"][10]
        iters += s["LS_iters"]
    o.close()
    per_iter = solve / max(iters, 1)
    rest = (tot - solve) / args.steps
    sample_ms = 1e3 * wall / args.steps
    model_iters = full["LS_iters"] if full else args.ref_iters
    model_ms = rest + per_iter * model_iters
    if full:
        value = case.n_fluid / (full["wall_ms"] * 1e-3)
        basis = (f"one full step measured after the warm-up: {full['wall_ms']:.0f} ms, "
                 f"{full['LS_iters']} BiCGSTAB iterations (the workload's cap {case.itermax})")
    else:
        value = case.n_fluid / (model_ms * 1e-3)
        basis = f"modelled from the samples at {model_iters:.0f} iterations/step (no full step run)"
    sample = (f"{args.steps} timed oracle steps of the same state, each a whole step with BiCGSTAB capped at "
              f"{args.cpu_iters} iterations: {sample_ms:.0f} ms/step measured (non-solver {rest:.0f} ms + "
              f"{per_iter:.1f} ms/iteration); value: {basis}")
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sample_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": DATA_TEXT,
            "config": bench_config(args, case, "fp64"),
            "impl": "reference",
            "value_measured": full is not None,
            "full_step": full,
            "sampled_step_model": {"ms_per_full_step": model_ms, "iterations": model_iters,
                                   "error_vs_full_step": (model_ms / full["wall_ms"] - 1.0) if full else None},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads(), "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--case", default="cylinder_4m")
    ap.add_argument("--particles", type=float, default=4.0e6)
    ap.add_argument("--wi", type=float, default=0.6)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--precond", choices=["none", "multigrid"], default="none",
                    help="opt-in PPE preconditioner (none = the reference's solver)")
    ap.add_argument("--e2e-steps", type=int, default=0,
                    help="steps of the end-to-end loop (default: the same as --steps)")
    ap.add_argument("--cpu-iters", type=int, default=20, help="BiCGSTAB cap of the CPU sample")
    ap.add_argument("--ref-iters", type=float, default=1001.0,
                    help="iterations/step the reference-arm sample is scaled to")
    ap.add_argument("--itermax", type=int, default=0, help="override the PPE iteration cap (profiling runs)")
    ap.add_argument("--out-dir", default=None,
                    help="folder for the clock samples and the batch's per-instance records (default: a temp folder)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-full-step", action="store_true",
                    help="reference arm: skip the one full step that its value is measured on")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision comparison run")
    ap.add_argument("--no-multigrid", action="store_true", help="skip the multigrid-preconditioned runs")
    ap.add_argument("--batch", type=int, default=0,
                    help="run the batched parameter sweep of this many instances instead")
    ap.add_argument("--batch-precision", choices=["fp64", "mixed"], default="mixed")
    ap.add_argument("--batch-precond", choices=["none", "multigrid"], default="multigrid")
    ap.add_argument("--tune", default="1,2,4", help="solver rows-per-thread candidates of the batch autotuner")
    ap.add_argument("--tune-coarse", default="512,2048,8192",
                    help="coarse-level single-block size candidates of the batch autotuner (multigrid)")
    ap.add_argument("--warm-start", action="store_true",
                    help="opt-in: PPE starts from the previous step's pressure (changes results)")
    ap.add_argument("--adjoint", type=int, default=0,
                    help="measure the reverse mode over a window of this many steps (heated cavity) instead")
    ap.add_argument("--adjoint-side", type=int, default=1024, help="cavity lattice side of the adjoint run")
    ap.add_argument("--checkpoint", type=int, default=20, help="adjoint checkpoint interval")
    ap.add_argument("--adjoint-fd", type=int, default=0, help="finite-difference directions checked at scale")
    ap.add_argument("--adjoint-eps", type=float, default=1.0e-6, help="central-difference step (unit-max directions)")
    ap.add_argument("--adjoint-dirs", type=int, default=8,
                    help="seeded directions whose directional derivatives are reported (and compared across runs)")
    ap.add_argument("--adjoint-tol", type=float, default=1.0e-8, help="PPE tolerance of the adjoint workload")
    ap.add_argument("--adjoint-spinup", type=int, default=20, help="steps run before the adjoint window")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint measurement of the default line")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched sweep of the default line")
    ap.add_argument("--default-adjoint-fd", type=int, default=2,
                    help="central-difference directions of the default line's adjoint (each replays the window twice)")
    ap.add_argument("--adjoint-precision", default="fp64", choices=["fp64", "mixed"],
                    help="arithmetic of the adjoint workload's forward step")
    ap.add_argument("--adjoint-const-mod", type=int, default=2, choices=[1, 2],
                    help="constitutive model of the adjoint workload: 2 Oldroyd-B, 1 Newtonian")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.e2e_steps <= 0:
        args.e2e_steps = args.steps
    if args.batch or (args.impl == "gb300" and not args.no_batch):
        # independent instances run as concurrent graph branches: more hardware queues (set
        # before the first CUDA call of the process)
        os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    dist = Dist()
    if args.impl == "gb300":
        import __graft_entry__ as g
        if dist.local == 0 or not (ROOT / "vebisph_gb300" / "_build" / "libvebi_gb300.so").exists():
            g.build()
        dist.barrier()
        if dist.world > 1:
            # one replica per GPU: pin this rank to its local GPU before the first CUDA call
            vis = os.environ.get("CUDA_VISIBLE_DEVICES")
            ids = vis.split(",") if vis else [str(i) for i in range(dist.world)]
            os.environ["CUDA_VISIBLE_DEVICES"] = ids[dist.local % len(ids)]
        if args.adjoint:
            res = run_adjoint(args, dist)
            if dist.rank == 0:
                print(json.dumps({"adjoint": res}))
            dist.close()
            return
        if args.batch:
            res = run_batch(args, dist)
        else:
            res = run_gb300(args, dist)
        if args.precision == "fp64" and not args.no_mixed and not args.batch:
            # the mixed-precision step on the same workload: its speed and its distance from FP64
            margs = argparse.Namespace(**vars(args))
            margs.precision = "mixed"
            margs.no_e2e = True
            margs.no_cpu = True
            mres = run_gb300(margs, dist)
            res["mixed"] = mixed_summary(res, mres)
        if args.precond == "none" and not args.no_multigrid and not args.batch:
            runs = []
            for p, pert in (("fp64", 0.0), ("mixed", 0.0), ("fp64", 6e-8)):
                gargs = argparse.Namespace(**vars(args))
                gargs.precision, gargs.precond, gargs.no_e2e, gargs.no_cpu = p, "multigrid", True, True
                gargs.perturb = pert
                runs.append(run_gb300(gargs, dist))
            res["multigrid"] = multigrid_summary(res, runs[0], runs[1], runs[2])
        if not args.no_adjoint and not args.batch and dist.rank == 0:
            # the metric's second part: adjoint/forward cost on the heated cavity (1M)
            # the configured window: 200 steps, checkpoints every 20, multigrid PPE; FP64 with
            # central differences (FP64, step 1e-6) along seeded directions and of Wi, then the
            # configuration's mixed-precision step against it
            aargs = argparse.Namespace(**vars(args))
            aargs.adjoint, aargs.checkpoint, aargs.precond = 200, 20, "multigrid"
            aargs.adjoint_tol, aargs.adjoint_fd, aargs.adjoint_const_mod = 1.0e-8, args.default_adjoint_fd, 2
            aargs.adjoint_precision = "fp64"
            aargs.adjoint_dirs = max(args.default_adjoint_fd, 1)
            res["adjoint"] = run_adjoint(aargs, dist)
            aargs.adjoint_precision, aargs.adjoint_fd = "mixed", 0
            res["adjoint_mixed"] = run_adjoint(aargs, dist, ref=res["adjoint"])
            # the same window, Newtonian: the log-conformation update's eigenvalue-gap pole
            # (predictor_mod.F90:213) is absent, so central differences can follow the adjoint
            aargs.adjoint_precision, aargs.adjoint_fd, aargs.adjoint_const_mod = "fp64", args.default_adjoint_fd, 1
            res["adjoint_newtonian"] = run_adjoint(aargs, dist)
        if not args.no_batch and not args.batch and dist.world == 1:
            # the batched sweep (512 instances, mixed + multigrid, autotuned tiles) against the same
            # instances run one by one with the plain FP64 step; speed only (the accuracy
            # comparison is `bench.py --batch 512`)
            bargs = argparse.Namespace(**vars(args))
            bargs.batch, bargs.batch_light, bargs.steps, bargs.warmup = 512, True, 3, 3
            b = run_batch(bargs, dist)
            res["batch"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "config", "LS_iters_per_step",
                                              "failed_instances", "serial_plain_fp64",
                                              "speedup_vs_serial_plain_fp64", "gpu_launches", "clocks")}
        res.pop("_fields", None)
    else:
        from oracle import build as ob
        ob.build()
        res = run_reference(args, dist)
    if dist.rank == 0 and res is not None:
        print(json.dumps(res))
    dist.close()


if __name__ == "__main__":
    main()

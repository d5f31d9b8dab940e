"""Phase timing of the multigrid-preconditioned PPE solver, barrier by barrier.

    python -m vebisph_gb300.barrier_profile [--particles 4e6] [--precision mixed|fp64] [--out FILE]

Builds a diagnostic copy of the library (nvcc -DVEBI_BARRIER_TIMESTAMPS, into
vebisph_gb300/_build_barrier_profile/) in which block 0 of the persistent solver records the
global timer when it arrives at and leaves every grid barrier; the product library is not
touched.  It then runs the confined cylinder with the multigrid preconditioner for 3 warm-up
steps and one recorded step, and prints, for each barrier of a BiCGSTAB iteration, the mean
time block 0 spent working before it (the phase) and waiting in it (the slowest block's
lateness plus the barrier's own latency).  It also records every block's arrival at 64
consecutive barriers, with the SM each block runs on.

With L grid-wide coarse levels an iteration (closed domain) has 4L + 15 barriers, 31 at 4M
(L = 4).  The phases, in order:
  0 p update and its mean; 1 .. 2L+5 the V-cycle on p (1 mean removal + first sweep, 2 fine
  residual, 3 restriction to the cells, then per grid-wide level one fused residual+restriction
  phase, the one-block levels and the coarsest solve, per level one fused prolongation+smoothing
  phase, and the output pass: M^-1 p and A M^-1 p); then v and (r_bar, v); s and its norm; the
  V-cycle on s; t and its products; the x/r update.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent


def build_variant() -> pathlib.Path:
    from . import build
    return build.build(extra=["-DVEBI_BARRIER_TIMESTAMPS"], out_dir=HERE / "_build_barrier_profile")


def phases(arrive: np.ndarray, leave: np.ndarray, period: int) -> dict:
    """Mean work (previous departure to arrival) and wait (arrival to departure) per barrier
    position within an iteration, over the complete iterations recorded."""
    work = (arrive[1:] - leave[:-1]) / 1e3
    wait = (leave - arrive) / 1e3
    full = (len(arrive) - 1) // period
    W = np.zeros(period)
    T = np.zeros(period)
    for k in range(full):
        s = 1 + k * period
        W += work[s - 1:s - 1 + period]
        T += wait[s:s + period]
    return {"iterations": full, "work_us": (W / max(full, 1)).tolist(), "wait_us": (T / max(full, 1)).tolist()}


def arrival_spread(arr: np.ndarray, smid: np.ndarray) -> dict:
    """Per recorded barrier: each block's arrival relative to the earliest block's; summarised
    by the median over barriers of the median and the maximum lateness, and the blocks (with
    their SM) that arrive last most often."""
    nblk = int((arr[0] > 0).sum())
    if nblk == 0:
        return {"blocks": 0, "median_of_median_us": 0.0, "median_of_max_us": 0.0, "often_last": []}
    a = arr[:, :nblk].astype(np.float64)
    rows = a[(a > 0).all(axis=1)]
    late = (rows - rows.min(axis=1, keepdims=True)) / 1e3
    last = np.argmax(late, axis=1)
    counts = np.bincount(last, minlength=nblk)
    often = [(int(b), int(smid[b]), int(counts[b])) for b in np.argsort(counts)[::-1][:8] if counts[b] > 0]
    return {"blocks": nblk, "barriers": int(len(rows)),
            "median_of_median_us": float(np.median(np.median(late, axis=1))),
            "median_of_max_us": float(np.median(late.max(axis=1))),
            "per_barrier_max_us": late.max(axis=1).tolist(),
            "per_barrier_p90_us": np.percentile(late, 90, axis=1).tolist(),
            "per_barrier_last": [(int(b), int(smid[b])) for b in last],
            "lateness_us": np.round(late, 3).tolist(),
            "smid": smid[:nblk].tolist(),
            "often_last": often}


def infer_period(n_barriers: int, iters: int) -> int:
    """Barriers per iteration, 4L + 15 for L grid-wide levels, from a solve's barrier count."""
    est = (n_barriers - 2) / max(iters, 1)
    return int(4 * round((est - 15) / 4) + 15)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--particles", type=float, default=4.0e6)
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--period", type=int, default=0,
                    help="grid barriers per BiCGSTAB iteration (default: from the run, 4L + 15)")
    ap.add_argument("--out", default=None, help="write the raw timestamps and the table as JSON")
    args = ap.parse_args()
    lib_path = build_variant()
    os.environ["VEBI_LIB"] = str(lib_path)
    sys.path.insert(0, str(HERE.parent))
    from vebisph_gb300 import abi, cases
    from vebisph_gb300.solver import StepSolver
    lib = abi.load_library()
    lib.vebi_barrier_timestamps_read.argtypes = [C.c_void_p, C.c_void_p]
    case = cases.cylinder(args.particles, Wi=0.6, seed=0)
    case.ppe_precond = abi.PRECOND_MULTIGRID
    prec = abi.PREC_MIXED if args.precision == "mixed" else abi.PREC_FP64
    s = StepSolver(case, precision=prec, timing=True)
    for _ in range(3):
        s.step()
    lib.vebi_barrier_timestamps_reset()
    st = s.step()
    ts = np.zeros((2, 16384), np.uint64)
    n = C.c_uint(0)
    lib.vebi_barrier_timestamps_read(ts.ctypes.data, C.byref(n))
    n = min(n.value, 16384)
    lib.vebi_barrier_arrivals_read.argtypes = [C.c_void_p, C.c_void_p]
    arr_all = np.zeros((64, 2048), np.uint64)
    smid = np.zeros(2048, np.uint32)
    lib.vebi_barrier_arrivals_read(arr_all.ctypes.data, smid.ctypes.data)
    spread = arrival_spread(arr_all, smid)
    arrive, leave = ts[0, :n].astype(np.float64), ts[1, :n].astype(np.float64)
    period = args.period or infer_period(n, st["LS_iters"])
    table = phases(arrive, leave, period)
    total_us = (leave[-1] - arrive[0]) / 1e3
    print(f"{case.name}, {args.precision}, multigrid: {st['LS_iters']} iterations, {n} barriers, "
          f"{total_us / 1e3:.2f} ms from the first barrier to the last")
    print("barrier  work_us  wait_us")
    for q, (w, t) in enumerate(zip(table["work_us"], table["wait_us"])):
        print(f"{q:7d} {w:8.2f} {t:8.2f}")
    w, t = sum(table["work_us"]), sum(table["wait_us"])
    print(f"per iteration: work {w:.1f} us, wait {t:.1f} us, total {w + t:.1f} us")
    print(f"arrival of every block at barriers 200..263 ({spread['blocks']} blocks), relative to the earliest: "
          f"median of the per-barrier median {spread['median_of_median_us']:.2f} us, of the max "
          f"{spread['median_of_max_us']:.2f} us; blocks last most often: {spread['often_last']}")
    if args.out:
        pathlib.Path(args.out).write_text(json.dumps({"case": case.name, "precision": args.precision,
                                                      "LS_iters": st["LS_iters"], "barriers": n, "period": period,
                                                      "arrive_ns": arrive.tolist(), "leave_ns": leave.tolist(),
                                                      "arrival_spread": spread, **table}))


if __name__ == "__main__":
    main()

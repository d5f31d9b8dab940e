"""Phase timing of the multigrid-preconditioned PPE solver, barrier by barrier.

    python -m vebisph_gb300.barrier_profile [--particles 4e6] [--precision mixed|fp64] [--out FILE]

Builds a diagnostic copy of the library (nvcc -DVEBI_BARRIER_TIMESTAMPS, into
vebisph_gb300/_build_barrier_profile/) in which block 0 of the persistent solver records the
global timer when it arrives at and leaves every grid barrier; the product library is not
touched.  It then runs the confined cylinder with the multigrid preconditioner for 3 warm-up
steps and one recorded step, and prints, for each of the 47 barriers of a BiCGSTAB iteration,
the mean time block 0 spent working before it (the phase) and waiting in it (the slowest
block's lateness plus the barrier's own latency).

The phases of an iteration (closed domain), in order:
  0 p update and its mean; 1-20 the V-cycle on p (1 mean removal + first sweep, 2 fine residual,
  3 restriction to the cells, 4-11 residual/restriction of the grid-wide coarse levels, 12 the
  one-block levels and the coarsest solve, 13-20 prolongation/smoothing back up); 21 the output
  pass (M^-1 p and A M^-1 p); 22 v and (r_bar, v); 23 s and its norm; 24-44 the V-cycle on s and
  its output pass; 45 t and its products; 46 the x/r update.  The grid-wide level count depends on
  the size (4 at 4M); the table is read with the period the run shows.
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--particles", type=float, default=4.0e6)
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--period", type=int, default=47, help="grid barriers per BiCGSTAB iteration")
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
    arrive, leave = ts[0, :n].astype(np.float64), ts[1, :n].astype(np.float64)
    table = phases(arrive, leave, args.period)
    total_us = (leave[-1] - arrive[0]) / 1e3
    print(f"{case.name}, {args.precision}, multigrid: {st['LS_iters']} iterations, {n} barriers, "
          f"{total_us / 1e3:.2f} ms from the first barrier to the last")
    print("barrier  work_us  wait_us")
    for q, (w, t) in enumerate(zip(table["work_us"], table["wait_us"])):
        print(f"{q:7d} {w:8.2f} {t:8.2f}")
    w, t = sum(table["work_us"]), sum(table["wait_us"])
    print(f"per iteration: work {w:.1f} us, wait {t:.1f} us, total {w + t:.1f} us")
    if args.out:
        pathlib.Path(args.out).write_text(json.dumps({"case": case.name, "precision": args.precision,
                                                      "LS_iters": st["LS_iters"], "barriers": n,
                                                      "arrive_ns": arrive.tolist(), "leave_ns": leave.tolist(),
                                                      **table}))


if __name__ == "__main__":
    main()

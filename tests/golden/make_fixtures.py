"""Writes the golden fixtures of tests/golden/ (run here, where the reference checkout exists).

rb_deck_digest.json: SHA-256 digests and scalars of the case deck shipped with the
  reference (source/gen/INDAT, IBOUND, IPART: datclass case 4), parsed with
  vebisph_gb300.cases.read_deck.  tests/test_cases.py checks that the restated generator
  vebisph_gb300.cases.rayleigh_benard_deck() reproduces these digests bit for bit.
oracle_rb_step1.json: a regression summary of one oracle step on that deck.
list_directed.json: the SHA-256 of the shipped IPART text (gfortran list-directed real(8)
  output, datclass.F90:649-651) and sample lines of it and of IBOUND (integer items,
  datclass.F90:686-700): the golden vectors of the library's list-directed formatter.

Usage: python -m tests.golden.make_fixtures <reference checkout>  (the argument is required)
"""
from __future__ import annotations

import hashlib
import json
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from vebisph_gb300 import cases  # noqa: E402


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def deck_summary(c: cases.Case) -> dict:
    return dict(
        npfb=c.npfb, nbS=c.nbS, h=c.h, dx=c.dx, dv=c.dv, Ra=c.Ra, Pr=c.Pr, El=c.El, beta=c.beta,
        ve_nonlinearity=c.ve_nonlinearity, body_force=list(c.body_force), dt_out=c.dt_out,
        r=digest(c.r.astype(np.float64)), u=digest(c.u.astype(np.float64)),
        theta=digest(c.theta.astype(np.float64)), b_node=digest(c.b_node.astype(np.float64)),
        b_edge=digest(c.b_edge.astype(np.float64)), b_type=[int(v) for v in c.b_type],
        b_thermal=[float(v) for v in c.b_thermal], b_vel=[float(v) for v in c.b_vel])


def oracle_summary(c: cases.Case) -> dict:
    from oracle.oracle import OracleSolver
    o = OracleSolver(c)
    s = o.step()
    cnt = o.get("ij_count")
    return dict(LS_iters=s["LS_iters"], nmirror=s["nmirror"], maxneighbours=s["maxneighbours"],
                dt=s["dt"], sum_ij_count=int(cnt.sum()), irelation=digest(o.get("irelation")),
                vrelation=digest(o.get("vrelation")), max_abs_p=s["max_abs_p"], max_abs_v=s["max_abs_v"])


def list_directed_summary(gen: pathlib.Path) -> dict:
    ipart = (gen / "IPART").read_bytes()
    lines = ipart.decode().splitlines()
    ibound = (gen / "IBOUND").read_text().splitlines()
    ints = [ln[:12] for ln in ibound if ln[:12].strip().lstrip("-").isdigit()]
    return dict(ipart_sha256=hashlib.sha256(ipart).hexdigest(), ipart_lines=len(lines),
                ipart_sample={str(i): lines[i] for i in (0, 1, 2, 100, 201, 202, 5000, len(lines) - 1)},
                ibound_integer_items=ints)


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python -m tests.golden.make_fixtures <reference checkout (the vebisph source tree)>")
    ref = pathlib.Path(sys.argv[1])
    deck = cases.read_deck(ref / "source" / "gen")
    (HERE / "rb_deck_digest.json").write_text(json.dumps(deck_summary(deck), indent=1) + "\n")
    (HERE / "oracle_rb_step1.json").write_text(json.dumps(oracle_summary(deck), indent=1) + "\n")
    (HERE / "list_directed.json").write_text(json.dumps(list_directed_summary(ref / "source" / "gen"), indent=1) + "\n")
    print("wrote", HERE / "rb_deck_digest.json", HERE / "oracle_rb_step1.json", HERE / "list_directed.json")


if __name__ == "__main__":
    main()

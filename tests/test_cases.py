"""Case decks: the restated generator reproduces the reference's shipped deck bit for bit,
and every synthetic workload passes the reference's boundary checks."""
import json
import pathlib

import numpy as np
import pytest

from vebisph_gb300 import cases

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"


def test_rb_deck_matches_shipped_deck_digest():
    from tests.golden.make_fixtures import deck_summary
    want = json.loads((GOLDEN / "rb_deck_digest.json").read_text())
    got = deck_summary(cases.rayleigh_benard_deck())
    for k, v in want.items():
        assert got[k] == v, k


def test_poiseuille_counts_and_walls():
    c = cases.poiseuille(40, seed=3)
    # 40 + 1 wall particles per wall line (make_boundary_particles, datclass.F90:779-810)
    assert c.nbS == 82
    assert c.npfb == 82 + 1600
    fl = c.r[c.nbS:]
    assert np.all(np.abs(fl[:, 0] - (np.floor(fl[:, 0] / 0.025) + 0.5) * 0.025) <= 0.01 * 0.025 + 1e-15)
    assert c.body_force == (80.0, 0.0)
    assert c.El == pytest.approx(10.0) and c.Ra == pytest.approx(0.01)


def test_cylinder_small_geometry():
    c = cases.cylinder(n_fluid_target=2.0e4, Wi=0.6, seed=0)
    fl = c.r[c.nbS:]
    rad = np.hypot(fl[:, 0], fl[:, 1])
    assert rad.min() > 1.0  # outside the cylinder (r > R + 0.25dx before jitter)
    assert abs(c.n_fluid - 2.0e4) / 2.0e4 < 0.05
    assert c.nb_circles == 1 and c.c_radius[0] == 1.0
    # mean of the initial parabolic profile is U = 1
    assert abs(fl[:, 0].max() - 15.0) < c.dx


def test_deck_reader_roundtrip(tmp_path):
    c = cases.rayleigh_benard_deck()
    # write a deck in the generator's formats (datclass.F90:649-720) and read it back
    lines = ["F :i_RESTART", f"{c.i_open_domain:5d} :open", f"{c.tmax:18.10f} :tmax",
             f"{c.i_shift_coeff:5d} :shift", f"{c.npfb:7d} :np", f"{c.npfb:7d} :npfb", f"{c.nbS:7d} :nbS",
             f"{c.dt_out:18.10f} :dt_out", f"{c.h:18.10f} :h", f"{c.dx:18.10f} :dx", f"{0.0:18.10f} :dt",
             f"{c.body_force[0]:18.10f}{c.body_force[1]:18.6f} :bf", f"{c.Ra:18.10f} Ra", f"{c.Pr:18.10f} Pr",
             f"{c.El:18.10f} El", f"{c.beta:18.10f} beta", f"{c.dt_coef_cfl:18.10f}{c.dt_coef_visc:18.10f} :dt",
             f"{c.ve_nonlinearity:18.10f} :ve", f"{c.alpha_evss:18.10f} :evss"]
    (tmp_path / "INDAT").write_text("\n".join(lines) + "\n")
    ib = [f"{c.nb_patches} :nb"]
    for i in range(c.nb_patches):
        f = lambda v: repr(float(v))  # noqa: E731
        ib += [f"{f(c.b_node[i][0])} {f(c.b_node[i][1])} :n", f"{f(c.b_edge[i][0])} {f(c.b_edge[i][1])} :e",
               f"{int(c.b_type[i])} :t", f"{f(c.b_vel[i])} :v", f"{f(c.b_thermal[i])} :th"]
        if c.b_type[i] == 2:
            ib.append(f"{int(c.b_periodic_parent[i])} :pp")
    ib.append("0")
    (tmp_path / "IBOUND").write_text("\n".join(ib) + "\n")
    rows = np.column_stack([c.r, c.u, c.theta, np.full(c.npfb, c.dv)])
    np.savetxt(tmp_path / "IPART", rows, fmt="%.17e")
    d = cases.read_deck(tmp_path)
    assert np.array_equal(d.r, c.r) and np.array_equal(d.theta, c.theta)
    assert d.nbS == c.nbS and d.h == c.h and d.El == c.El
    assert list(d.b_periodic_parent) == list(c.b_periodic_parent)

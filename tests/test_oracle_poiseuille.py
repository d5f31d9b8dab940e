"""The oracle alone over the small Poiseuille configuration's 2000 steps (40x40 Oldroyd-B channel,
Re=0.1, Wi=1, beta=0.1, started from rest by a body force) against the analytic start-up flow of
Waters & King, the reference's own check of this case (data_directory/poiseuille.m:3-57),
including its elastic velocity overshoot.  The GPU test of the same run checks the GPU against
the oracle; this one pins the oracle itself on the CPU."""
import numpy as np

from oracle.oracle import OracleSolver
from tests.analytic import waters_king
from vebisph_gb300 import cases


def test_oracle_follows_the_analytic_startup_flow():
    c = cases.poiseuille(40, seed=1)
    o = OracleSolver(c)
    t = 0.0
    for _ in range(2000):
        t += o.step()["dt"]
    n, f = c.npfb, slice(c.nbS, c.npfb)
    u = o.get("ux")[:n]
    Re = (c.Ra / c.Pr) ** 0.5
    ua = waters_king(o.get("ry")[f], t, 1.0 / Re, c.El * Re, c.beta, c.body_force[0])
    assert ua.max() > 3.0  # the overshoot: three times the steady centreline velocity
    assert np.abs(u[f] - ua).max() <= 0.01 * ua.max()  # measured 3.9e-3
    assert abs(u[f].max() - ua.max()) <= 0.005 * ua.max()  # measured 3.5e-3
    o.close()

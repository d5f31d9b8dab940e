"""The small Poiseuille configuration over its full 2000 steps: 40x40 Oldroyd-B channel,
Re=0.1, Wi=1, beta=0.1, started from rest by a body force.  The GPU step stays with the oracle over
the whole run, and both follow the analytic start-up flow (Waters & King), including its elastic
velocity overshoot, to the discretisation error."""
import numpy as np
import pytest

from tests.analytic import waters_king
from vebisph_gb300 import cases

pytestmark = pytest.mark.gpu

STEPS = 2000


def test_poiseuille_2000_steps(built):
    from oracle.oracle import OracleSolver
    from vebisph_gb300.solver import StepSolver
    c = cases.poiseuille(40, seed=1)
    gpu, ref = StepSolver(c), OracleSolver(c)
    t = 0.0
    for _ in range(STEPS):
        sg, so = gpu.step(), ref.step()
        assert sg["dt"] == so["dt"]
        t += sg["dt"]
    n, f = c.npfb, slice(c.nbS, c.npfb)
    ug, uo = gpu.get("ux")[:n], ref.get("ux")[:n]
    umax = np.abs(uo).max()
    assert np.abs(ug - uo).max() <= 1e-6 * umax
    tg, to = gpu.get("tau11")[:n], ref.get("tau11")[:n]
    assert np.abs(tg - to).max() <= 1e-4 * np.abs(to).max()
    # the analytic start-up profile at the same time, at the particles' heights
    Re = (c.Ra / c.Pr) ** 0.5
    ua = waters_king(gpu.get("ry")[f], t, 1.0 / Re, c.El * Re, c.beta, c.body_force[0])
    assert ua.max() > 3.0  # the elastic overshoot: three times the steady centreline velocity
    assert np.abs(ug[f] - ua).max() <= 0.01 * ua.max()
    assert abs(ug[f].max() - ua.max()) <= 0.005 * ua.max()
    gpu.close()
    ref.close()

"""The analytic start-up Poiseuille solution (tests/analytic.py) against its own limits: it is
zero at t=0, tends to the steady parabola, and with no elasticity is the Newtonian series."""
import numpy as np

from tests.analytic import waters_king


def test_limits():
    y = np.linspace(0.0, 1.0, 41)
    steady = 80.0 / (8.0 * 10.0) * 4.0 * y * (1.0 - y)
    assert np.abs(waters_king(y, 0.0, 10.0, 1.0, 0.1, 80.0)).max() < 2e-3  # the series' truncation at t=0
    assert np.abs(waters_king(y, 200.0, 10.0, 1.0, 0.1, 80.0) - steady).max() < 1e-9
    # beta -> 1 (all viscosity from the solvent) approaches the Newtonian start-up
    newt = steady.copy()
    t1 = 10.0 * 0.01
    for n in range(1, 61):
        N = (2 * n - 1) * np.pi
        newt -= 80.0 / (8.0 * 10.0) * 32.0 * np.sin(N * y) / N**3 * np.exp(-N * N * t1)
    assert np.abs(waters_king(y, 0.01, 10.0, 1.0, 0.999999, 80.0) - newt).max() < 1e-4

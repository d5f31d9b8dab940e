"""Flow diagnostics of the confined-cylinder configuration, computed on the host from fields
read back from a context (GPU or oracle alike).

The reference has no force or wake diagnostic; the configuration asks for the drag
coefficient and the peak first normal-stress difference in the wake, so both are defined here
once and shared by the benchmark and the tests:

* drag: the x-force of the fluid on the cylinder from the step's circle-mirror pair terms
  (`vebi_step_stats.circle_force`), as K = F_x / (eta0 U) with eta0 = 1/Re = sqrt(Pr/Ra) and
  U the mean fluid x-velocity;
* N1: max over the wake (fluid and wall particles with x > R, the cylinder being centred at
  x = 0 with R = 1) of tau_xx - tau_yy, tau in the reference's planes (11, 21, 12, 22).
"""
from __future__ import annotations

import numpy as np


def n1_wake_max(rx: np.ndarray, tau11: np.ndarray, tau22: np.ndarray, radius: float = 1.0) -> float:
    wake = rx > radius
    if not wake.any():  # no cylinder: the whole channel
        wake = np.ones_like(wake)
    return float((tau11 - tau22)[wake].max())


def drag(case, circle_force, ux: np.ndarray) -> dict | None:
    if not case.nb_circles:
        return None
    fx, fy = circle_force
    u_mean = float(np.mean(ux[case.nbS:case.npfb]))
    eta0 = (case.Pr / case.Ra) ** 0.5
    return {"F_x": fx, "F_y": fy, "U_mean": u_mean, "K": fx / (eta0 * u_mean)}


def rel(a: float, b: float) -> float:
    """|a - b| relative to |b|."""
    return abs(a - b) / max(abs(b), 1e-300)

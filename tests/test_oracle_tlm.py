"""The FP64 tangent-linear model of the step (oracle.TangentLinear) against central finite
differences of the same map, on the CPU.

The map is n steps with the geometry of the unperturbed trajectory: every step's r* (after
binning) and dt are recorded by the FP64 oracle and replayed when it reruns from perturbed
fields, so the pair lists, weights, mirrors and PPE matrix are the same in every run.  The
tangent-linear model is the same oracle code run over forward-mode dual numbers, which holds
that geometry by construction; its value trajectory is the FP64 oracle's, bit for bit.

J = mean kinetic energy of the fluid particles after the window.  The PPE runs to a relative
residual of 1e-12.  Central differences converge to the tangent at second order in the step, so
each case states the step and the agreement it reaches.
"""
import numpy as np
import pytest

from oracle.oracle import OracleSolver, TangentLinear
from vebisph_gb300 import cases

NSTEPS, SPIN = 6, 15
KEYS = ("r", "u", "tau", "theta", "trace_conf")
ARG = {"u": "du", "tau": "dtau", "theta": "dtheta"}


def kinetic(u, nbS, n):
    return 0.5 * float(np.mean(u[0][nbS:n] ** 2 + u[1][nbS:n] ** 2))


class Window:
    """A spun-up state, the oracle's record of the window from it, and reruns of that window."""

    def __init__(self, case):
        case.tol = 1.0e-12
        case.itermax = 4000
        self.case = case
        self.o = OracleSolver(case)
        for _ in range(SPIN):
            self.o.step()
        self.st0 = self.o.state()
        self.inbin = case.fortran_planes()["inbin"]
        self.o.record_geometry()
        self.J0 = self.run()

    def run(self, **perturbed):
        s = {k: perturbed.get(k, self.st0[k]) for k in KEYS}
        n = self.case.npfb
        self.o.upload(s["r"], s["u"], s["tau"], s["theta"], s["trace_conf"], self.inbin, n)
        for _ in range(NSTEPS):
            self.o.step()
        st = self.o.state()
        return kinetic(st["u"], self.case.nbS, n)

    def direction(self, field, seed):
        case, st0 = self.case, self.st0
        rng = np.random.default_rng(seed)
        shape = st0[field].shape
        d = np.zeros(shape)
        d[..., case.nbS:] = rng.normal(size=shape[:-1] + (case.npfb - case.nbS,))
        if field == "tau":
            d[2] = d[1]  # a symmetric perturbation, as the conformation is
        return d * (max(np.abs(st0[field]).max(), 1.0e-3) / np.abs(d).max())

    def central(self, field, d, eps):
        self.o.replay_geometry()
        jp = self.run(**{field: self.st0[field] + eps * d})
        self.o.replay_geometry()
        jm = self.run(**{field: self.st0[field] - eps * d})
        return (jp - jm) / (2.0 * eps)

    def tangent(self, field, d):
        """dJ . d and the tangent model's own J (its value trajectory)."""
        case, n, nbS = self.case, self.case.npfb, self.case.nbS
        t = TangentLinear(case, state=self.st0)
        t.set_direction(**{ARG[field]: d})
        for _ in range(NSTEPS):
            t.step()
        (ux, dux), (uy, duy) = t.get("ux"), t.get("uy")
        t.close()
        dj = float(np.sum(ux[nbS:n] * dux[nbS:n] + uy[nbS:n] * duy[nbS:n]) / (n - nbS))
        return dj, kinetic((ux, uy), nbS, n)


@pytest.fixture(scope="module")
def cavity():
    """Heated cavity, Oldroyd-B Wi=0.5, Ra=1e4: its conformations separate after the spin-up."""
    return Window(cases.cavity(n=16, seed=3, Ra=1.0e4, Wi=0.5, beta=0.5, amp=2.0e-2))


def test_replay_reproduces_the_record(cavity):
    cavity.o.replay_geometry()
    assert cavity.run() == cavity.J0


def test_tangent_model_values_are_the_step(cavity):
    d = cavity.direction("theta", 1)
    _, j = cavity.tangent("theta", d)
    assert j == cavity.J0


def test_tangent_is_linear_in_the_direction(cavity):
    d = cavity.direction("theta", 2)
    a, _ = cavity.tangent("theta", d)
    b, _ = cavity.tangent("theta", -3.0 * d)
    assert abs(b + 3.0 * a) <= 1.0e-12 * abs(b)


@pytest.mark.parametrize("field,eps,rtol", [("theta", 1.0e-4, 1.0e-9), ("u", 1.0e-4, 1.0e-8),
                                            ("tau", 1.0e-5, 2.0e-8)])
def test_cavity_tangent_matches_central_differences(cavity, field, eps, rtol):
    d = cavity.direction(field, 10)
    tl, _ = cavity.tangent(field, d)
    fd = cavity.central(field, d, eps)
    assert abs(fd) > 0
    assert abs(fd - tl) <= rtol * abs(fd), (fd, tl)


def test_channel_tangent_matches_central_differences():
    """Newtonian Poiseuille: walls, periodic patches, wall-periodic corners, body force."""
    w = Window(cases.poiseuille(24, seed=5, const_mod=1))
    d = w.direction("u", 20)
    tl, _ = w.tangent("u", d)
    fd = w.central("u", d, 1.0e-4)
    assert abs(fd - tl) <= 1.0e-10 * abs(fd), (fd, tl)


@pytest.mark.parametrize("const_mod", [1, 2])
def test_cylinder_tangent_matches_central_differences(const_mod):
    """Confined cylinder (circle mirrors), Newtonian and Oldroyd-B, from the parabolic start."""
    case = cases.cylinder(2.0e3, Wi=0.6, seed=2)
    case.nplink = 96
    case.const_mod = const_mod
    w = Window(case)
    d = w.direction("u", 30)
    tl, _ = w.tangent("u", d)
    fd = w.central("u", d, 1.0e-4)
    assert abs(fd - tl) <= 1.0e-8 * abs(fd), (fd, tl)


@pytest.mark.parametrize("field,eps,rtol", [("theta", 1.0e-3, 1.0e-8), ("tau", 1.0e-4, 1.0e-8)])
def test_ptt_cavity_tangent_matches_central_differences(field, eps, rtol):
    """PTT (ve_nonlinearity 0.25): the relaxation rate follows the conformation's trace."""
    case = cases.cavity(n=16, seed=3, Ra=1.0e4, Wi=0.5, beta=0.5, amp=2.0e-2)
    case.ve_nonlinearity = 0.25
    w = Window(case)
    d = w.direction(field, 40)
    tl, j = w.tangent(field, d)
    assert j == w.J0
    fd = w.central(field, d, eps)
    assert abs(fd - tl) <= rtol * abs(fd), (fd, tl)


@pytest.mark.parametrize("make,rtol", [(lambda: cases.dam_break(20, seed=1), 1.0e-8),
                                       (lambda: cases.free_surface_periodic(30, seed=1), 1.0e-6)])
def test_open_domain_tangent_matches_central_differences(make, rtol):
    """Open domains: free-surface Dirichlet rows, the smoothed PPE and the Jacobi BiCGSTAB (the
    dam break under gravity; the periodic free-surface layer), step 1e-3."""
    w = Window(make())
    d = w.direction("u", 40)
    tl, j = w.tangent("u", d)
    assert j == w.J0
    fd = w.central("u", d, 1.0e-3)
    assert abs(fd - tl) <= rtol * abs(fd), (fd, tl)

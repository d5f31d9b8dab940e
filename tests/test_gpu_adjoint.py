"""Reverse mode of the step (vebi_adjoint_*) against central finite differences of the same
differentiated map (the steps replayed with the recorded geometry), on a small heated cavity
(Oldroyd-B, Ra=1e4) after a spin-up, over a window of 6 steps with checkpoints every 4.

J = mean kinetic energy of the fluid particles after the window.  The PPE runs to a relative
residual of 1e-12 so that its truncation stays far below the differences (step 1e-3 on unit-max
directions: truncation and solver noise are both ~1e-7 relative here)."""
import numpy as np
import pytest

from vebisph_gb300 import abi, cases
from vebisph_gb300.solver import Adjoint, StepSolver

pytestmark = pytest.mark.gpu

NSTEPS, K, SPIN = 6, 4, 15
EPS = 1.0e-3
RTOL = 1.0e-5


def kinetic(state, nbS):
    u = state["u"][:, nbS:]
    return 0.5 * float(np.mean(u[0] ** 2 + u[1] ** 2))


@pytest.fixture(scope="module")
def window():
    case = cases.cavity(n=16, seed=3, Ra=1.0e4, Wi=0.5, beta=0.5, amp=2.0e-2)
    case.tol = 1.0e-12
    case.itermax = 4000
    s = StepSolver(case)
    for _ in range(SPIN):
        s.step()
    st0 = s.download()
    adj = Adjoint(s, max_steps=NSTEPS, checkpoint_every=K)
    adj.record(NSTEPS)
    fin = s.download()
    nbS, n = case.nbS, case.npfb
    seed = np.zeros((2, n))
    seed[:, nbS:] = fin["u"][:, nbS:] / (n - nbS)
    g = adj.reverse(seed_u=seed)
    yield dict(case=case, s=s, adj=adj, st0=st0, J0=kinetic(fin, nbS), g=g)
    adj.close()
    s.close()


def run_from(w, theta=None, u=None, tau=None):
    st0, s = w["st0"], w["s"]
    s.upload(st0["r"], st0["u"] if u is None else u, st0["tau"] if tau is None else tau,
             st0["theta"] if theta is None else theta, st0["trace_conf"], st0["inbin"], st0["r"].shape[1])
    w["adj"].replay(NSTEPS)
    return kinetic(s.download(), w["case"].nbS)


def central(w, field, direction):
    base = w["st0"][field]
    jp = run_from(w, **{field: base + EPS * direction})
    jm = run_from(w, **{field: base - EPS * direction})
    return (jp - jm) / (2.0 * EPS)


def test_replay_reproduces_the_record(window):
    assert run_from(window) == window["J0"]


def test_reverse_uses_the_transposed_solve(window):
    g = window["g"]
    assert g["ls_iters"] > 0
    assert np.all(np.isfinite(g["theta"])) and np.abs(g["theta"]).max() > 0


@pytest.mark.parametrize("k", range(4))
def test_theta_gradient_matches_central_differences(window, k):
    case = window["case"]
    rng = np.random.default_rng(100 + k)
    d = np.zeros(case.npfb)
    d[case.nbS:] = rng.normal(size=case.npfb - case.nbS)
    d /= np.abs(d).max()
    fd = central(window, "theta", d)
    ad = float(window["g"]["theta"] @ d)
    assert abs(fd - ad) <= RTOL * abs(fd), (fd, ad)


@pytest.mark.parametrize("k", range(2))
def test_velocity_gradient_matches_central_differences(window, k):
    case = window["case"]
    rng = np.random.default_rng(200 + k)
    d = np.zeros((2, case.npfb))
    d[:, case.nbS:] = rng.normal(size=(2, case.npfb - case.nbS))
    d *= np.abs(window["st0"]["u"]).max() / np.abs(d).max()
    fd = central(window, "u", d)
    ad = float(np.sum(window["g"]["u"] * d))
    assert abs(fd - ad) <= RTOL * abs(fd), (fd, ad)


@pytest.mark.parametrize("k", range(2))
def test_stress_gradient_matches_central_differences(window, k):
    case = window["case"]
    rng = np.random.default_rng(300 + k)
    d = np.zeros((4, case.npfb))
    d[:, case.nbS:] = rng.normal(size=(4, case.npfb - case.nbS))
    d[2] = d[1]  # a symmetric perturbation, as the conformation is
    d *= np.abs(window["st0"]["tau"]).max() / np.abs(d).max()
    fd = central(window, "tau", d)
    ad = float(np.sum(window["g"]["tau"] * d))
    assert abs(fd - ad) <= RTOL * abs(fd), (fd, ad)


def test_weissenberg_gradient_matches_central_differences(window):
    s, wi, h = window["s"], 0.5, 1.0e-4
    s.set_weissenberg(wi + h)
    jp = run_from(window)
    s.set_weissenberg(wi - h)
    jm = run_from(window)
    s.set_weissenberg(wi)
    fd = (jp - jm) / (2.0 * h)
    ad = window["g"]["wi"]
    assert abs(fd - ad) <= 1.0e-4 * abs(fd), (fd, ad)

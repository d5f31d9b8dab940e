"""Known-answer tests of the CPU oracle (the reference ships none; these pin the restatement).

* the quintic spline integrates to 1 (ad_7 = 7/(478 pi h^2), input.F90:168);
* Shepard sum: sum_j W_ij dv + W(0) dv ~ 1 on a lattice (freesurf_mod.F90:95-100);
* the Bonet-Lok correction makes the gradient of a linear field exact (kernel_calculation.F90:55-66);
* the Morris pair weight gives the Laplacian of a quadratic field (4 for x^2 + y^2, on average);
* calc_eigens reconstructs A = R diag(L) R^T (predictor_mod.F90:253-290);
* at rest the log-conformation step equals the analytic relaxation tau*exp(-dt/Wi) (predictor_mod.F90:318-331);
* the BiCGSTAB solution satisfies the assembled system;
* one step's projection balances a buoyancy that is a pure gradient with the hydrostatic pressure;
* in steady simple shear the log-conformation update converges to the Oldroyd-B relations of
  docs/docs.tex:93-100 (A_xy = Wi g, tau_xx = 2 (Wi g)^2, tau_yy = 0) and to the closed form of
  the linear PTT law stated there, at first order in dt, and from rest it stays at rest (the
  reference's degenerate-eigenvalue branch);
* the oracle is deterministic for any OpenMP thread count;
* a regression summary of one step on the shipped Rayleigh-Benard deck.
"""
import json
import os
import pathlib
import subprocess
import sys

import numpy as np
import pytest

from oracle.oracle import OracleSolver, eigens, logconf_particle
from vebisph_gb300 import cases

ROOT = pathlib.Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def small():
    return OracleSolver(cases.poiseuille(16, seed=0))


def test_kernel_normalisation(small):
    h = small.case.h
    q = np.linspace(0.0, 3.0, 200001)
    w = np.array([small.W(x) for x in q[::50]])
    qq = q[::50]
    integral = np.trapezoid(w * 2.0 * np.pi * qq * h * h, qq)
    assert abs(integral - 1.0) < 1e-6
    # fac is dW/dq / h up to sign convention: fac(q) = W'(q)/q * (1/h) -> check by finite differences
    for x in (0.3, 1.2, 2.5):
        d = (small.W(x + 1e-6) - small.W(x - 1e-6)) / 2e-6
        assert abs(small.fac(x) - d / h) < 1e-6 * abs(d / h)


def test_shepard_sum_on_lattice(small):
    dx, h = small.case.dx, small.case.h
    n = 9
    g = np.arange(-n, n + 1) * dx
    X, Y = np.meshgrid(g, g)
    r = np.hypot(X, Y).ravel()
    s = sum(small.W(v / h) for v in r) * dx * dx
    assert abs(s - 1.0) < 5e-3


def test_gradient_of_linear_field_is_exact():
    c = cases.poiseuille(40, seed=2, const_mod=1)
    a = np.array([0.3, -0.2])
    B = np.array([[0.5, -1.5], [0.7, 0.25]])
    u = c.u.copy()
    u[:] = a + c.r @ B.T
    c.u = u
    c.body_force = (0.0, 0.0)
    o = OracleSolver(c)
    s = o.step()
    dt = s["dt"]
    rs = np.stack([o.get("rsx")[: c.npfb], o.get("rsy")[: c.npfb]], 1)
    # fluid was advected with u0, so u is linear in r*: u = (I + B dt)^-1 (a + B r*)
    M = np.linalg.solve(np.eye(2) + B * dt, B)
    inner = np.arange(c.npfb) >= c.nbS
    inner &= (rs[:, 0] > 0.2) & (rs[:, 0] < 0.8) & (rs[:, 1] > 0.2) & (rs[:, 1] < 0.8)
    g = np.stack([o.get("gradu_x"), o.get("gradu_y"), o.get("gradv_x"), o.get("gradv_y")], 1)[: c.npfb][inner]
    want = np.array([M[0, 0], M[0, 1], M[1, 0], M[1, 1]])
    assert inner.sum() > 500
    assert np.abs(g - want).max() < 1e-9 * np.abs(want).max()


def test_eigen_reconstruction():
    rng = np.random.default_rng(0)
    for _ in range(200):
        Q = rng.normal(size=(2, 2))
        A = Q @ Q.T + 0.1 * np.eye(2)
        L, R = eigens(A)
        back = R @ np.diag(L) @ R.T
        assert np.abs(back - A).max() < 1e-13 * np.abs(A).max()
    L, R = eigens(np.diag([2.0, 3.0]))  # diagonal branch keeps the diagonal order
    assert list(L) == [2.0, 3.0] and np.array_equal(R, np.eye(2))


def test_relaxation_at_rest_matches_closed_form():
    c = cases.poiseuille(24, seed=1)
    c.body_force = (0.0, 0.0)
    c.u[:] = 0.0
    tau0 = np.array([0.12, 0.03, 0.03, -0.05])  # (1,1),(2,1),(1,2),(2,2)
    c.tau = np.tile(tau0, (c.npfb, 1))
    o = OracleSolver(c)
    s = o.step()
    Wi = c.El * np.sqrt(c.Ra / c.Pr)
    e1 = np.exp(-s["dt"] / Wi)  # Oldroyd-B: alpha_R = 1
    for k, nm in enumerate(("tau11", "tau21", "tau12", "tau22")):
        got = o.get(nm)[: c.npfb]
        assert np.abs(got - tau0[k] * e1).max() < 1e-13, nm
    tr = o.get("trace_conf")
    assert np.abs(tr - (2.0 + (tau0[0] + tau0[3]) * e1)).max() < 1e-13


def _ell_matvec(o, x, n):
    cnt = o.get("ij_count")
    k = int(cnt.max())
    col = o.get("ppe_col").reshape(-1, n)[:k]
    val = o.get("ppe_val").reshape(-1, n)[:k]
    mask = np.arange(k)[:, None] < cnt[None, :]
    return o.get("ppe_diag") * x + (np.where(mask, val, 0.0) * x[col]).sum(0)


def steady_shear(Wi, g, eps):
    """Steady simple shear du/dy = g of the linear PTT law of docs/docs.tex (f_R = [1 + eps
    tr(A - I)] (A - I), relaxation rate 1/Wi): with Y = 1 + eps tau_xx, tau_yy = 0,
    tau_xy = Wi g / Y and tau_xx = 2 (Wi g)^2 / Y^2, a cubic in tau_xx solved by Newton.
    eps = 0 is Oldroyd-B: tau_xy = Wi g, tau_xx = 2 (Wi g)^2."""
    wg = Wi * g
    x = 2.0 * wg * wg
    for _ in range(100):
        f = x * (1.0 + eps * x) ** 2 - 2.0 * wg * wg
        x -= f / ((1.0 + eps * x) ** 2 + 2.0 * eps * x * (1.0 + eps * x))
    y = 1.0 + eps * x
    return np.array([x, wg / y, wg / y, 0.0])


def hydrostatic_step(n):
    """One step from rest of the periodic channel with buoyancy theta = sin(pi y) and no body
    force: the pressure's error against the hydrostatic -cos(pi y)/pi (relative to its amplitude)
    and the largest velocity left, relative to the dt theta the predictor adds."""
    c = cases.poiseuille(n, seed=2, const_mod=1)
    c.body_force = (0.0, 0.0)
    c.u = np.zeros_like(c.u)
    c.theta = np.sin(np.pi * c.r[:, 1])
    c.b_thermal = np.zeros(4)
    c.tol = 1.0e-10
    o = OracleSolver(c)
    dt = o.step()["dt"]
    npfb = c.npfb
    y, p = o.get("rsy")[:npfb], o.get("p")[:npfb]
    fl = np.arange(npfb) >= c.nbS
    pa = -np.cos(np.pi * y) / np.pi
    err = np.abs((p - p[fl].mean()) - (pa - pa[fl].mean()))[fl].max() / (1.0 / np.pi)
    vmax = max(np.abs(o.get("ux")[:npfb][fl]).max(), np.abs(o.get("uy")[:npfb][fl]).max())
    return err, vmax / dt


def test_buoyancy_is_balanced_by_the_hydrostatic_pressure():
    """The projection of one step (ppe_solve_in_house_simple_dirichlet.F90, calc_pressure_gradient):
    buoyancy theta e_y with theta = sin(pi y) between no-slip walls (theta = 0 there, b_thermal 0,
    so the wall mirrors' odd reflection continues it exactly) is a pure gradient, balanced by
    P = -cos(pi y)/pi, whose normal derivative vanishes at the walls as the mirrors impose.  The
    step's pressure follows it and the velocity the buoyancy adds is removed, both up to the
    discretisation error, which falls with resolution; a sign or a normalisation error in the
    right-hand side, the Laplacian or the pressure gradient would leave O(1) of either."""
    coarse, fine = hydrostatic_step(24), hydrostatic_step(64)
    assert fine[0] < 0.06 and fine[1] < 0.05, fine
    assert fine[0] < coarse[0] and fine[1] < coarse[1], (coarse, fine)


def test_morris_laplacian_of_a_quadratic():
    """The viscous and heat-diffusion pair weight w_L = 2 r.gradW / (r^2 + 0.01 h^2)
    (kernel_calculation.F90:55-66) makes sum_j (f_i - f_j) w_L the Laplacian: for f = x^2 + y^2
    it averages 4 over the interior of a jittered lattice (pointwise within the operator's
    scatter on disordered particles), which pins its sign and normalisation."""
    c = cases.poiseuille(40, seed=2, const_mod=1)
    c.body_force = (0.0, 0.0)
    o = OracleSolver(c)
    o.step()
    n = c.npfb
    x, y = o.get("rsx"), o.get("rsy")
    cnt, link, wl = o.get("ij_count"), o.get("ij_link"), o.get("w_L")
    kmax = len(link) // n
    link, wl = link.reshape(kmax, n), wl.reshape(kmax, n)
    f = x * x + y * y
    slot = np.arange(kmax)[:, None] < cnt[None, :]
    lap = np.sum(np.where(slot, (f[:n][None, :] - f[link]) * wl, 0.0), axis=0)
    inner = (np.arange(n) >= c.nbS) & (x[:n] > 0.2) & (x[:n] < 0.8) & (y[:n] > 0.2) & (y[:n] < 0.8)
    assert abs(lap[inner].mean() - 4.0) < 0.06, lap[inner].mean()
    assert np.all(np.abs(lap[inner] - 4.0) < 1.0)


@pytest.mark.parametrize("Wi,g,eps", [(1.0, 0.5, 0.0), (0.5, 2.0, 0.0), (2.0, 0.3, 0.0),
                                      (1.0, 1.0, 0.25), (0.5, 2.0, 0.1), (2.0, 0.5, 0.5)])
def test_steady_shear_matches_the_closed_form(Wi, g, eps):
    """Simple shear held for 30 relaxation times from a slightly anisotropic conformation: the
    update's fixed point is the steady state of the Oldroyd-B (eps = 0) or linear PTT law up to
    a first-order splitting error, which falls tenfold with dt."""
    exact = steady_shear(Wi, g, eps)
    errs = []
    for dt in (1.0e-3, 1.0e-4):
        t, trace = logconf_particle([1.0e-2, 1.0e-2, 1.0e-2, 0.0], [0.0, g, 0.0, 0.0], dt, Wi, eps_ptt=eps,
                                    nsteps=int(round(30.0 * Wi / dt)))
        assert abs(trace - (2.0 + t[0] + t[3])) < 1e-12
        err = np.abs(t - exact).max() / np.abs(exact).max()
        assert err < 1.0e-3, (dt, t, exact)
        errs.append(err)
    assert 8.0 < errs[0] / errs[1] < 12.0  # first order in dt


def test_shear_from_rest_stays_at_rest():
    """At A = I both eigenvalues are 1 and R = I (calc_eigens, predictor_mod.F90:253-290); the
    update keeps only the diagonal of R^T grad(u) R in B and puts the shear into the rotation,
    which acts on log A = 0, so a pure shear leaves the conformation at rest.  Stress starts
    growing only once the conformation is anisotropic."""
    t, trace = logconf_particle([0.0, 0.0, 0.0, 0.0], [0.0, 0.5, 0.0, 0.0], 1.0e-3, 1.0, nsteps=5000)
    assert np.all(t == 0.0) and trace == 2.0


def test_bicgstab_solution_satisfies_system():
    c = cases.rayleigh_benard_deck()
    o = OracleSolver(c)
    o.step()
    s = o.step()
    assert s["LS_iters"] < 1000 and s["LS_residual"] <= 1e-8
    n = c.npfb
    p = o.get("p")[:n]
    B = o.get("ppe_B")
    res = B - _ell_matvec(o, p, n)
    # the closed-domain solver works modulo constants (remove_dc): compare without the mean
    res -= res.mean()
    assert np.linalg.norm(res) <= 1e-6 * np.linalg.norm(B)


def test_rb_deck_regression_summary():
    want = json.loads((ROOT / "tests" / "golden" / "oracle_rb_step1.json").read_text())
    from tests.golden.make_fixtures import oracle_summary
    got = oracle_summary(cases.rayleigh_benard_deck())
    for k, v in want.items():
        if isinstance(v, float):
            assert abs(got[k] - v) <= 1e-10 * max(abs(v), 1e-300), k
        else:
            assert got[k] == v, k


def test_oracle_deterministic_across_thread_counts():
    code = ("import hashlib,sys; sys.path.insert(0, %r)\n"
            "from vebisph_gb300 import cases\nfrom oracle.oracle import OracleSolver\n"
            "o = OracleSolver(cases.poiseuille(24, seed=3)); o.step(); o.step()\n"
            "print(hashlib.sha256(o.get('p').tobytes() + o.get('ux').tobytes()).hexdigest())\n") % str(ROOT)
    outs = []
    for nt in ("1", "3"):
        env = dict(os.environ, OMP_NUM_THREADS=nt)
        outs.append(subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                                   check=True).stdout.strip())
    assert outs[0] == outs[1]

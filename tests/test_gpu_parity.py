"""GPU step vs the CPU oracle on the same inputs (FP64): bit-exact cell assignment,
neighbour lists, mirrors, weights and matrix; fields within the tolerances of
tests/parity.py (the PPE solve differs only by reduction order)."""
import numpy as np
import pytest

from tests.parity import compare_step, failures
from vebisph_gb300 import cases

pytestmark = pytest.mark.gpu

CASES = {
    "poiseuille40": lambda: cases.poiseuille(40, seed=1),
    "rb_deck": cases.rayleigh_benard_deck,
    "cylinder20k": lambda: cases.cylinder(2.0e4, Wi=0.6, seed=2),
    "cavity64": lambda: cases.cavity(64, seed=3),
    "poiseuille_newtonian": lambda: cases.poiseuille(32, seed=4, const_mod=1),
    "free_surface_open": lambda: cases.free_surface_periodic(75, seed=5),
    "dam_break_open": lambda: cases.dam_break(40, seed=3),
    "poiseuille_correct_velocity": lambda: _with(cases.poiseuille(40, seed=6), correct_velocity=1),
}


def _with(case, **kw):
    for k, v in kw.items():
        setattr(case, k, v)
    return case


@pytest.fixture(scope="module")
def libs(built):
    from oracle.oracle import OracleSolver
    from vebisph_gb300.solver import StepSolver
    return StepSolver, OracleSolver


@pytest.mark.parametrize("name", sorted(CASES))
def test_one_step_parity(libs, name):
    StepSolver, OracleSolver = libs
    case = CASES[name]()
    gpu, ref = StepSolver(case), OracleSolver(case)
    sg, so = gpu.step(secondary=True), ref.step(secondary=True)
    assert sg["dt"] == so["dt"]
    assert sg["nmirror"] == so["nmirror"] and sg["np"] == so["np"]
    assert sg["maxneighbours"] == so["maxneighbours"]
    assert sg["n_inbin"] == so["n_inbin"]
    assert abs(sg["LS_iters"] - so["LS_iters"]) <= max(5, 0.25 * so["LS_iters"])
    rep = compare_step(gpu, ref, case)
    bad = failures(rep)
    assert not bad, bad
    if case.i_open_domain == 1:  # free-surface identification (freesurf_mod.F90:17-68)
        assert np.array_equal(gpu.get("n_surf")[: case.npfb], ref.get("n_surf")[: case.npfb])
        for nm in ("conc", "div_r"):
            a, b = gpu.get(nm), ref.get(nm)
            assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max(), nm
    # force on the circles (drag/lift diagnostic): pair terms with the new pressure, so the
    # pressure tolerance applies, relative to the force's magnitude
    if case.nb_circles:
        fg, fo = np.array(sg["circle_force"]), np.array(so["circle_force"])
        assert np.abs(fo).max() > 0
        assert np.abs(fg - fo).max() <= 1e-5 * np.abs(fo).max(), (fg, fo)
    else:
        assert sg["circle_force"] == [0.0, 0.0]
    # vorticity diagnostic (secondary_properties) follows the final velocity
    v_g, v_o = gpu.get("vort"), ref.get("vort")
    assert np.abs(v_g - v_o).max() <= 1e-5 * max(np.abs(v_o).max(), 1e-30)
    gpu.close()
    ref.close()


def test_neighbour_sets_order_normalised(libs):
    """Neighbour sets are compared after sorting each list (order normalisation)."""
    StepSolver, OracleSolver = libs
    case = cases.cylinder(2.0e4, Wi=0.3, seed=5)
    gpu, ref = StepSolver(case), OracleSolver(case)
    gpu.step()
    ref.step()
    n = case.npfb
    cg, co = gpu.get("ij_count"), ref.get("ij_count")
    assert np.array_equal(cg, co)
    k = int(co.max())
    lg = gpu.get("ij_link").reshape(-1, n)[:k].T
    lo = ref.get("ij_link").reshape(-1, n)[:k].T
    for i in range(0, n, 7):
        assert sorted(lg[i, :cg[i]]) == sorted(lo[i, :co[i]])


def test_multistep_poiseuille_fields(libs):
    """20 steps: u and r stay within 1e-6 of the oracle; tau within the oracle's own spread.

    GPU and oracle differ only by the order of the PPE reductions (~1e-13 relative in u per
    step).  The log-conformation update divides by (lambda2 - lambda1 + 1e-10)
    (predictor_mod.F90:213), which is near 1e-10 while the conformation tensor is close to the
    identity, so such differences are amplified in tau.  The test measures that amplification
    on the oracle itself -- a second oracle run whose velocity is perturbed by 1e-13 after the
    first step -- and requires the GPU to be no further from the oracle than 10x that spread."""
    StepSolver, OracleSolver = libs
    case = cases.poiseuille(40, seed=7)
    gpu, ref, pert = StepSolver(case), OracleSolver(case), OracleSolver(case)
    n = case.npfb
    for k in range(20):
        sg, so = gpu.step(), ref.step()
        pert.step()
        if k == 0:
            r = np.stack([pert.get("rx")[:n], pert.get("ry")[:n]])
            u = np.stack([pert.get("ux")[:n], pert.get("uy")[:n]]) * (1.0 + 1e-13)
            tau = np.stack([pert.get(nm)[:n] for nm in ("tau11", "tau21", "tau12", "tau22")])
            pert.upload(r, u, tau, pert.get("theta")[:n], pert.get("trace_conf"), np.zeros(n, np.uint8), n)
    groups = {"u": ("ux", "uy"), "r": ("rx", "ry")}
    for names in groups.values():
        scale = max(max(np.abs(ref.get(nm)[:n]).max() for nm in names), 1e-30)
        for name in names:
            a, b = gpu.get(name)[:n], ref.get(name)[:n]
            assert np.abs(a - b).max() / scale < 1e-6, name
    for name in ("tau11", "tau12", "tau21", "tau22"):
        a, b, c = gpu.get(name)[:n], ref.get(name)[:n], pert.get(name)[:n]
        spread = np.abs(c - b).max()
        scale = np.abs(b).max()
        assert np.abs(a - b).max() <= 10.0 * spread + 1e-12 * scale, name
    assert abs(sg["dt"] - so["dt"]) <= 1e-9 * so["dt"]


def test_warm_start_multistep(libs):
    """Opt-in PPE warm start (x0 = previous P): GPU and oracle agree over 5 steps."""
    StepSolver, OracleSolver = libs
    case = _with(cases.poiseuille(40, seed=8), ppe_warm_start=1)
    gpu, ref = StepSolver(case), OracleSolver(case)
    for _ in range(5):
        sg, so = gpu.step(), ref.step()
    n = case.npfb
    us = max(np.abs(ref.get("ux")[:n]).max(), np.abs(ref.get("uy")[:n]).max())
    for nm in ("ux", "uy"):
        assert np.abs(gpu.get(nm)[:n] - ref.get(nm)[:n]).max() < 1e-6 * us, nm
    assert sg["LS_residual"] <= 1e-8 and so["LS_residual"] <= 1e-8

"""The opt-in multigrid-preconditioned PPE (VEBI_PRECOND_MULTIGRID) against the oracle, which
runs the reference's unpreconditioned BiCGSTAB: both stop on the same residual test, so on
cases the reference solves within its iteration cap the fields agree within the FP64 parity
tolerances, in far fewer iterations."""
import numpy as np
import pytest

from tests.parity import TOL, relerr
from vebisph_gb300 import abi, cases

pytestmark = pytest.mark.gpu

CASES = {
    "poiseuille40": lambda: cases.poiseuille(40, seed=1),
    "rb_deck": cases.rayleigh_benard_deck,
    "cylinder20k": lambda: cases.cylinder(2.0e4, Wi=0.6, seed=2),
    "cavity64": lambda: cases.cavity(64, seed=3),
    "free_surface_open": lambda: cases.free_surface_periodic(75, seed=5),
    "dam_break_open": lambda: cases.dam_break(40, seed=3),
}


def _mg(case):
    case.ppe_precond = abi.PRECOND_MULTIGRID
    return case


@pytest.fixture(scope="module")
def libs(built):
    from oracle.oracle import OracleSolver
    from vebisph_gb300.solver import StepSolver
    return StepSolver, OracleSolver


@pytest.mark.parametrize("name", sorted(CASES))
def test_multigrid_step_matches_oracle(libs, name):
    StepSolver, OracleSolver = libs
    gpu, ref = StepSolver(_mg(CASES[name]())), OracleSolver(CASES[name]())
    n = gpu.case.npfb
    for step in range(3):
        sg, so = gpu.step(), ref.step()
        assert sg["error"] == 0 and not (sg["warnings"] & abi.WARN_MAXITER)
        if so["LS_iters"] > 30:
            assert sg["LS_iters"] < so["LS_iters"], (sg["LS_iters"], so["LS_iters"])
        scale_p = max(np.abs(ref.get("p")[:n]).max(), 1e-30)
        assert relerr(gpu.get("p")[:n], ref.get("p")[:n], scale_p) <= TOL["p"], step
        us = max(np.abs(ref.get("ux")[:n]).max(), np.abs(ref.get("uy")[:n]).max(), 1e-30)
        for nm in ("ux", "uy"):
            assert relerr(gpu.get(nm)[:n], ref.get(nm)[:n], us) <= TOL[nm], (step, nm)
    if gpu.case.i_open_domain == 0:  # the zero mean of the reference's iterates is kept
        p = gpu.get("p")[:n]
        assert abs(p.mean()) <= 1e-9 * np.abs(p).max()
    gpu.close()
    ref.close()


def test_multigrid_is_deterministic(libs):
    StepSolver, _ = libs
    out = []
    for _ in range(2):
        s = StepSolver(_mg(cases.cylinder(2.0e4, Wi=0.6, seed=2)))
        for _ in range(2):
            st = s.step()
        out.append((st["LS_iters"], s.get("p").copy(), s.get("ux").copy()))
        s.close()
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1]) and np.array_equal(out[0][2], out[1][2])


@pytest.mark.parametrize("name", ["poiseuille40", "cylinder20k", "free_surface_open", "dam_break_open"])
def test_mixed_multigrid_close_to_fp64(libs, name):
    """Mixed precision with the preconditioner against the FP64 step with it: velocity, and for
    the cylinder the drag, within 1e-4 after three steps (both solves converge)."""
    StepSolver, _ = libs
    a = StepSolver(_mg(CASES[name]()), precision=abi.PREC_FP64)
    b = StepSolver(_mg(CASES[name]()), precision=abi.PREC_MIXED)
    n = a.case.npfb
    for _ in range(3):
        sa, sb = a.step(), b.step()
        assert sb["error"] == 0 and not (sb["warnings"] & abi.WARN_MAXITER)
    us = max(np.abs(a.get("ux")[:n]).max(), np.abs(a.get("uy")[:n]).max())
    for nm in ("ux", "uy"):
        assert relerr(b.get(nm)[:n], a.get(nm)[:n], us) <= 1e-4, nm
    if a.case.nb_circles:
        assert abs(sb["circle_force"][0] - sa["circle_force"][0]) <= 1e-4 * abs(sa["circle_force"][0])
    a.close()
    b.close()


def test_multigrid_with_warm_start_matches_oracle_warm_start(libs):
    """Both opt-ins together: the preconditioned solve starting from the previous pressure
    reaches the oracle's warm-started solution within the pressure tolerance."""
    StepSolver, OracleSolver = libs
    c1 = cases.cylinder(2.0e4, Wi=0.6, seed=2)
    c1.ppe_warm_start = 1
    c2 = cases.cylinder(2.0e4, Wi=0.6, seed=2)
    c2.ppe_warm_start = 1
    gpu, ref = StepSolver(_mg(c1)), OracleSolver(c2)
    n = c1.npfb
    for _ in range(3):
        sg, so = gpu.step(), ref.step()
        assert not (sg["warnings"] & abi.WARN_MAXITER)
    # Both solves stop at 1e-8 of their own first-iteration residual.  From a warm start that
    # residual differs most between the preconditioned and the reference's solve, so the two
    # solutions differ by up to the reference solve's own error: 1.1e-5 measured, 3e-5 allowed.
    scale_p = np.abs(ref.get("p")[:n]).max()
    assert relerr(gpu.get("p")[:n], ref.get("p")[:n], scale_p) <= 3e-5
    assert sg["LS_iters"] < so["LS_iters"]
    gpu.close()
    ref.close()


@pytest.mark.parametrize("prec", [abi.PREC_FP64, abi.PREC_MIXED])
def test_coarse_block_rows_leaves_results_unchanged(libs, prec):
    """The coarse-level tile size (levels run in one block or across the grid) changes which
    threads compute each coarse row, not the row's arithmetic: the fields are bit-identical."""
    StepSolver, _ = libs
    out = []
    for rows in (0, 256, 1 << 20):
        s = StepSolver(_mg(cases.cylinder(2.0e4, Wi=0.6, seed=2)), precision=prec)
        s.set_coarse_block_rows(rows)
        for _ in range(3):
            st = s.step()
        out.append((st["LS_iters"], {nm: s.get(nm) for nm in ("ux", "uy", "p")}))
        s.close()
    for it, f in out[1:]:
        assert it == out[0][0]
        for nm in ("ux", "uy", "p"):
            assert np.array_equal(f[nm], out[0][1][nm]), nm

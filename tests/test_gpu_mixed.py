"""Mixed-precision step (VEBI_PREC_MIXED) against the FP64 GPU step and the FP64 oracle.

FP32 pair sums and an FP32 difference-form SpMV inside the FP64 BiCGSTAB recurrences; on
cases whose PPE converges the velocity stays within 1e-4 of FP64 after 10 steps (the bar of
the mixed step), and the neighbour lists and mirrors are unchanged (positions stay FP64)."""
import numpy as np
import pytest

from vebisph_gb300 import abi, cases

pytestmark = pytest.mark.gpu

CASES = {
    "poiseuille40": lambda: cases.poiseuille(40, seed=1),
    "rb_deck": cases.rayleigh_benard_deck,
    "cylinder20k": lambda: cases.cylinder(2.0e4, Wi=0.6, seed=2),
}


def _run(fn, prec, steps):
    from vebisph_gb300.solver import StepSolver
    c = fn()
    s = StepSolver(c, precision=prec)
    st = [s.step() for _ in range(steps)]
    n = c.npfb
    out = {k: s.get(k)[:n].copy() for k in ("ux", "uy", "p", "rx", "ry")}
    out["ij_count"] = s.get("ij_count")
    out["irelation"] = s.get("irelation")
    s.close()
    return out, st


@pytest.mark.parametrize("name", sorted(CASES))
def test_mixed_matches_fp64(built, name):
    f64, s64 = _run(CASES[name], abi.PREC_FP64, 10)
    mx, smx = _run(CASES[name], abi.PREC_MIXED, 10)
    uscale = max(np.abs(f64["ux"]).max(), np.abs(f64["uy"]).max())
    uerr = max(np.abs(mx["ux"] - f64["ux"]).max(), np.abs(mx["uy"] - f64["uy"]).max()) / uscale
    assert uerr < 1e-4, uerr
    rerr = max(np.abs(mx["rx"] - f64["rx"]).max(), np.abs(mx["ry"] - f64["ry"]).max())
    assert rerr < 1e-6 * case_h(name)
    for a, b in zip(smx, s64):
        assert a["LS_residual"] <= 1e-8 or a["LS_iters"] > 1000
    # the PPE converged in both; its solution agrees where the pressure carries the flow
    if name != "poiseuille40":  # body-force driven: P is ~0 there
        perr = np.abs(mx["p"] - f64["p"]).max() / np.abs(f64["p"]).max()
        assert perr < 1e-4, perr
    # and against the FP64 oracle over the same 10 steps from the same input
    from oracle.oracle import OracleSolver
    ref = OracleSolver(CASES[name]())
    for _ in range(10):
        ref.step()
    n = len(f64["ux"])
    ou = {k: ref.get(k)[:n] for k in ("ux", "uy")}
    ref.close()
    oscale = max(np.abs(ou["ux"]).max(), np.abs(ou["uy"]).max())
    oerr = max(np.abs(mx["ux"] - ou["ux"]).max(), np.abs(mx["uy"] - ou["uy"]).max()) / oscale
    assert oerr < 1e-4, oerr


def case_h(name):
    return CASES[name]().h


def test_mixed_neighbours_and_mirrors_unchanged(built):
    f64, _ = _run(CASES["cylinder20k"], abi.PREC_FP64, 1)
    mx, _ = _run(CASES["cylinder20k"], abi.PREC_MIXED, 1)
    assert np.array_equal(f64["ij_count"], mx["ij_count"])
    assert np.array_equal(f64["irelation"], mx["irelation"])

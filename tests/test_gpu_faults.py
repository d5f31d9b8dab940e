"""Failure paths of the GPU step, injected from the host (no GPU fault is provoked): each
returns the status of the matching `stop` site of the reference, and a fresh context works."""
import numpy as np
import pytest

from vebisph_gb300 import abi, cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def Solver(built):
    from vebisph_gb300.solver import StepSolver, VebiError
    return StepSolver, VebiError


def test_nan_position_goes_to_the_bin(Solver):
    S, _ = Solver
    c = cases.poiseuille(20, seed=0)
    c.r[c.nbS + 5] = [np.nan, 0.5]
    s = S(c).step()
    assert s["n_inbin"] == 1


def test_particle_outside_box_goes_to_the_bin(Solver):
    S, _ = Solver
    c = cases.poiseuille(20, seed=0)
    c.r[c.nbS + 7] = [5.0, 5.0]
    assert S(c).step()["n_inbin"] == 1


def test_all_in_bin_is_an_error(Solver):
    S, E = Solver
    c = cases.poiseuille(8, seed=0)
    c.r[c.nbS:] = [50.0, 50.0]
    with pytest.raises(E) as ei:
        S(c).step()
    assert ei.value.status == 6


@pytest.mark.parametrize("field,value,status", [("nplink", 10, 4), ("nmirror_cap", 10, 7)])
def test_capacity_errors(Solver, field, value, status):
    S, E = Solver
    c = cases.poiseuille(20, seed=0)
    setattr(c, field, value)
    with pytest.raises(E) as ei:
        S(c).step()
    assert ei.value.status == status
    # the GPU is fine: a fresh context steps normally
    assert S(cases.poiseuille(20, seed=0)).step()["status"] == 0


def test_itermax_warning(Solver):
    S, _ = Solver
    c = cases.rayleigh_benard_deck()
    c.itermax = 5
    s = S(c).step()
    assert s["LS_iters"] == 6 and (s["warnings"] & abi.WARN_MAXITER)


def test_box_mismatch_rejected(Solver):
    S, E = Solver
    c = cases.poiseuille(8, seed=0)
    sol = S(c)
    with pytest.raises(E):
        sol.div_free(sol.x_mint - 1.0, sol.y_mint, sol.x_maxt, sol.y_maxt)


def test_grid_barrier_gives_up_and_context_stays_usable(Solver):
    """The solvers' bounded grid barrier, made to run out: one block of a cooperative grid
    never arrives (a wait that nothing ends), the others give up after a short poll limit
    and record VEBI_ERR_TIMEOUT.  The host reads the status; the same process then creates a
    fresh context and steps it normally."""
    import ctypes as C
    S, _ = Solver
    lib = abi.load_library()
    st, ms = C.c_int32(-1), C.c_double(0.0)
    assert lib.vebi_test_barrier_timeout(8, 1 << 14, C.byref(st), C.byref(ms)) == 0, lib.vebi_last_error()
    assert st.value == abi.STATUS["VEBI_ERR_TIMEOUT"], st.value
    assert ms.value < 1000.0, ms.value  # ~1e4 polls of ~64 ns: milliseconds, not the solvers' seconds
    c = cases.poiseuille(20, seed=0)
    s = S(c).step()
    assert s["error"] == 0 and s["LS_iters"] >= 1
    # arguments outside the bounds are refused before anything runs
    assert lib.vebi_test_barrier_timeout(1, 1 << 14, C.byref(st), None) == abi.STATUS["VEBI_ERR_ARG"]
    assert lib.vebi_test_barrier_timeout(8, 1 << 30, C.byref(st), None) == abi.STATUS["VEBI_ERR_ARG"]

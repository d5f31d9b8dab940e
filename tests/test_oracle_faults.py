"""Failure paths of the step, injected on the host into the oracle (no GPU): each maps to a
`stop` site of the reference or to a capacity the reference overruns silently."""
import numpy as np
import pytest

from oracle.oracle import OracleSolver
from vebisph_gb300 import abi, cases


def _state(c):
    f = c.fortran_planes()
    return f


def test_nan_position_goes_to_the_bin():
    c = cases.poiseuille(20, seed=0)
    c.r[c.nbS + 5] = [np.nan, 0.5]
    o = OracleSolver(c)
    s = o.step()
    assert s["n_inbin"] == 1
    assert o.get("ux")[c.nbS + 5] == 0.0 or np.isfinite(o.get("ux")[c.nbS + 5])
    assert np.isfinite(o.get("p")[: c.npfb]).all()


def test_particle_outside_the_box_goes_to_the_bin():
    c = cases.poiseuille(20, seed=0)
    c.r[c.nbS + 7] = [5.0, 5.0]
    o = OracleSolver(c)
    s = o.step()
    assert s["n_inbin"] == 1


def test_all_in_bin_is_an_error():
    c = cases.poiseuille(8, seed=0)
    c.r[c.nbS:] = [50.0, 50.0]
    o = OracleSolver(c)
    with pytest.raises(RuntimeError, match="ALL_IN_BIN"):
        o.step()


def test_cell_capacity_error():
    c = cases.poiseuille(20, seed=0)
    c.nplink = 10  # cells hold ~15 particles at h = 1.3 dx
    o = OracleSolver(c)
    with pytest.raises(RuntimeError, match="CELL_CAPACITY"):
        o.step()


def test_mirror_capacity_error():
    c = cases.poiseuille(20, seed=0)
    c.nmirror_cap = 10
    o = OracleSolver(c)
    with pytest.raises(RuntimeError, match="MIRROR_CAPACITY"):
        o.step()


def test_itermax_warning():
    c = cases.rayleigh_benard_deck()
    c.itermax = 5
    o = OracleSolver(c)
    s = o.step()
    assert s["LS_iters"] == 6 and (s["warnings"] & abi.WARN_MAXITER)


def test_open_boundary_rejected():
    c = cases.poiseuille(8, seed=0)
    c.b_edge = c.b_edge.copy()
    c.b_edge[0] = [0.9, 0.0]  # edges no longer close the polygon (check_boundaries check 1/2)
    with pytest.raises(RuntimeError, match="BOUNDARY"):
        OracleSolver(c)


def test_breakdown_from_rest_is_a_warning():
    # from rest with no forcing the PPE right-hand side is 0: rho = 0, "BICGSTAB Fails"
    c = cases.poiseuille(12, seed=0)
    o = OracleSolver(c)
    s = o.step()
    assert s["warnings"] & abi.WARN_BICGSTAB_BREAKDOWN

"""GPU step vs the CPU oracle at the configurations' own sizes (FP64, same inputs).

The small-case parity tests (test_gpu_parity.py) run at <= 20k particles; here the step is
compared at the sizes the benchmark configurations name, where the cell grid, the ELL width in
use, the mirror capacity and the 4096-element reduction chunks all differ from the small cases:

* the 1000 x 1000 planar Poiseuille channel (1M fluid particles);
* the confined cylinder, channel 30R x 4R, ~4M fluid particles, at Wi = 0.3, 0.6 and 0.9;
* the 1024 x 1024 differentially heated cavity (Ra 1e5, Oldroyd-B Wi 0.5).

Both sides cap BiCGSTAB at the same iteration count (20), which keeps the oracle's step to
seconds on the host's cores; the solver still runs the reference's recurrences on the full
matrix.  The integer and pair arrays are compared bit for bit (cell assignment, neighbour
lists in order and as order-normalised sets, mirror sets, weights, correction matrices, PPE
matrix); the fields within the tolerances of tests/parity.py.

The reference sources followed: neighbour_finding_mod.F90:261-339 (pair list),
mirror_boundaries_mod.F90:18-334 (mirrors), ppe_solve_in_house_simple_dirichlet.F90:60-122
(matrix), linear_solver.F90:275-425 (BiCGSTAB).
"""
import numpy as np
import pytest

from tests.parity import compare_step, failures
from vebisph_gb300 import cases, diagnostics

pytestmark = pytest.mark.gpu

ITERS = 20

CONFIGS = {
    "poiseuille_1m": lambda: cases.poiseuille(1000, seed=0),
    "cylinder_4m_Wi0.3": lambda: cases.cylinder(4.0e6, Wi=0.3, seed=0),
    "cylinder_4m_Wi0.6": lambda: cases.cylinder(4.0e6, Wi=0.6, seed=0),
    "cylinder_4m_Wi0.9": lambda: cases.cylinder(4.0e6, Wi=0.9, seed=0),
    "cavity_1m": lambda: cases.cavity(1024, seed=0),
}


@pytest.fixture(scope="module")
def libs(built):
    from oracle.oracle import OracleSolver
    from vebisph_gb300.solver import StepSolver
    return StepSolver, OracleSolver


def _check_step(gpu, ref, case, sg, so):
    assert sg["dt"] == so["dt"]
    for k in ("nmirror", "np", "maxneighbours", "n_inbin", "LS_iters"):
        assert sg[k] == so[k], (k, sg[k], so[k])
    rep = compare_step(gpu, ref, case)
    bad = failures(rep)
    assert not bad, bad
    # neighbour sets after order normalisation, on a strided subset of the particles
    n = case.npfb
    cnt = ref.get("ij_count")
    k = int(cnt.max())
    sub = np.arange(0, n, 97)
    pad = np.iinfo(np.int32).max
    sets = []
    for side in (gpu, ref):
        link = side.get("ij_link").reshape(-1, n)[:k, sub].copy()
        link[np.arange(k)[:, None] >= cnt[sub][None, :]] = pad
        link.sort(axis=0)
        sets.append(link)
    assert np.array_equal(sets[0], sets[1])
    if case.nb_circles:
        fg, fo = np.array(sg["circle_force"]), np.array(so["circle_force"])
        assert np.abs(fg - fo).max() <= 1e-5 * np.abs(fo).max(), (fg, fo)
        n1g = diagnostics.n1_wake_max(gpu.get("rx")[:n], gpu.get("tau11")[:n], gpu.get("tau22")[:n])
        n1o = diagnostics.n1_wake_max(ref.get("rx")[:n], ref.get("tau11")[:n], ref.get("tau22")[:n])
        assert diagnostics.rel(n1g, n1o) <= 1e-9, (n1g, n1o)


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_config_step_parity(libs, name):
    """One step from the configuration's initial state, then a second step from the oracle's
    state after the first, uploaded to both sides (so the second step's inputs are identical
    too, and its PPE has a developed right-hand side)."""
    StepSolver, OracleSolver = libs
    case = CONFIGS[name]()
    case.itermax = ITERS
    gpu = StepSolver(case)
    ref = OracleSolver(case)
    try:
        sg, so = gpu.step(), ref.step()
        _check_step(gpu, ref, case, sg, so)
        assert so["n_inbin"] == 0  # so the re-uploaded state has no binned particles either
        st = ref.state()
        n = case.npfb
        gpu.upload(st["r"], st["u"], st["tau"], st["theta"], st["trace_conf"], np.zeros(n, np.uint8), n)
        ref.upload(st["r"], st["u"], st["tau"], st["theta"], st["trace_conf"], np.zeros(n, np.uint8), n)
        sg, so = gpu.step(), ref.step()
        _check_step(gpu, ref, case, sg, so)
    finally:
        gpu.close()
        ref.close()

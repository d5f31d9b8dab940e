"""The allocation-free PPE solve (vebi_ppe_solve_noalloc) against the time step's own solve.

Callers that cannot allocate device memory -- a framework whose allocator owns the GPU, or a
real-time loop that must not allocate -- pass their matrix, right-hand side and output in
device memory they already hold; the solve keeps its working vectors in a fixed static array.
This file is collected last (test_zz_*) and needs nothing from the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from vebisph_gb300 import cases

pytestmark = pytest.mark.gpu


def _system(case_fn, steps=2):
    from vebisph_gb300.solver import StepSolver
    case = case_fn()
    sol = StepSolver(case)
    for _ in range(steps):
        s = sol.step()
    n = case.npfb
    out = dict(n=n, cnt=sol.get("ij_count"), col=sol.get("ppe_col"), val=sol.get("ppe_val"),
               diag=sol.get("ppe_diag"), rhs=sol.get("ppe_B"), p=sol.get("p")[:n], iters=s["LS_iters"])
    sol.close()
    return out


SYSTEMS = {
    # closed domains: SPARSE_PBICGSTAB_nonull (linear_solver.F90:275-425)
    "poiseuille40": (lambda: cases.poiseuille(40, seed=11), 1),
    "rb_deck": (cases.rayleigh_benard_deck, 1),
    # an open domain with free-surface rows: the Jacobi SPARSE_PBICGSTAB (linear_solver.F90:82-227)
    "free_surface_open": (lambda: cases.free_surface_periodic(75, seed=5), 0),
}


@pytest.mark.parametrize("which", sorted(SYSTEMS))
def test_noalloc_matches_step_solve_twice(built, which):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device visible to torch")
    from vebisph_gb300 import abi
    lib = abi.load_library()
    fn, closed = SYSTEMS[which]
    sysm = _system(fn)
    n = sysm["n"]
    dev = torch.device("cuda", torch.cuda.current_device())
    g = {k: torch.from_numpy(np.ascontiguousarray(sysm[k])).to(dev) for k in ("cnt", "col", "val", "diag", "rhs")}
    stream = torch.cuda.current_stream()
    ref = sysm["p"]
    for call in range(2):  # the second call reuses the shared array left by the first
        x = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
        iters, resid = C.c_int32(0), C.c_double(0.0)
        st = lib.vebi_ppe_solve_noalloc(
            g["cnt"].data_ptr(), g["col"].data_ptr(), g["val"].data_ptr(), g["diag"].data_ptr(),
            g["rhs"].data_ptr(), x.data_ptr(), n, n, closed, 1.0e-8, 1000, C.c_void_p(stream.cuda_stream),
            C.byref(iters), C.byref(resid))
        assert st == 0, lib.vebi_last_error()
        got = x.cpu().numpy()
        # the step's pressure tolerance (tests/parity.py: p within 1e-5 of its scale)
        err = np.abs(got - ref).max() / max(np.abs(ref).max(), 1e-300)
        assert err < 1e-5, (call, err)
        # BiCGSTAB's iteration count moves with rounding (the step's solver uses fused
        # multiply-adds, this one the reference's separate operations): same order, not equal
        assert abs(iters.value - sysm["iters"]) <= max(5, 0.25 * sysm["iters"]), (call, iters.value)
        assert resid.value <= 1e-8 or iters.value > 1000
    # the asynchronous form: no read-back pointers, so the call only enqueues the solve; the
    # caller's own stream synchronisation makes x readable
    x = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
    st = lib.vebi_ppe_solve_noalloc(
        g["cnt"].data_ptr(), g["col"].data_ptr(), g["val"].data_ptr(), g["diag"].data_ptr(),
        g["rhs"].data_ptr(), x.data_ptr(), n, n, closed, 1.0e-8, 1000, C.c_void_p(stream.cuda_stream),
        None, None)
    assert st == 0, lib.vebi_last_error()
    stream.synchronize()
    got = x.cpu().numpy()
    assert np.isfinite(got).all()
    assert np.abs(got - ref).max() / max(np.abs(ref).max(), 1e-300) < 1e-5


def test_noalloc_rejects_oversized_system(built):
    from vebisph_gb300 import abi
    lib = abi.load_library()
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    st = lib.vebi_ppe_solve_noalloc(dummy, dummy, dummy, dummy, dummy, dummy, abi.NOALLOC_MAX_ROWS + 1,
                                    abi.NOALLOC_MAX_ROWS + 1, 1, 1e-8, 10, None, None, None)
    assert st == 1  # VEBI_ERR_ARG
    assert b"VEBI_NOALLOC_MAX_ROWS" in lib.vebi_last_error()

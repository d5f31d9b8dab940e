"""Batches: instances advanced together through vebi_batch_step give exactly the fields the
same instances give one by one (same kernels, same grids, deterministic reductions)."""
import numpy as np
import pytest

from vebisph_gb300 import abi, cases

pytestmark = pytest.mark.gpu


def _cases():
    return [cases.poiseuille(24, seed=1, Wi=0.5), cases.poiseuille(32, seed=2, Wi=2.0, beta=0.5),
            cases.cylinder(6.0e3, Wi=0.3, seed=3), cases.rayleigh_benard_deck(),
            cases.poiseuille(20, seed=4, const_mod=1), cases.cylinder(1.2e4, Wi=1.5, seed=5, beta=0.8)]


def _with_precond(cl, pc):
    for c in cl:
        c.ppe_precond = pc
    return cl


@pytest.mark.parametrize("prec", [abi.PREC_FP64, abi.PREC_MIXED])
@pytest.mark.parametrize("pc", [abi.PRECOND_NONE, abi.PRECOND_MULTIGRID])
def test_batch_equals_individual_runs(built, prec, pc):
    from vebisph_gb300.solver import BatchSolver, StepSolver
    b = BatchSolver(_with_precond(_cases(), pc), precision=prec)
    ms, stats = b.step(3)
    assert ms > 0 and len(stats) == 6
    for i, c in enumerate(_with_precond(_cases(), pc)):
        s = StepSolver(c, precision=prec)
        for _ in range(3):
            si = s.step()
        assert si["LS_iters"] == stats[i]["LS_iters"]
        for nm in ("ux", "uy", "rx", "p", "tau11"):
            a, r = b.instances[i].get(nm)[: c.npfb], s.get(nm)[: c.npfb]
            assert np.array_equal(a, r), (i, nm)
        s.close()
    b.close()


def test_batch_autotune_keeps_results(built):
    from vebisph_gb300.solver import BatchSolver
    b = BatchSolver(_cases()[:3], precision=abi.PREC_MIXED)
    info = b.autotune(candidates=(1, 4), coarse_candidates=(256, 2048))
    assert info["rows_per_thread"] in (1, 4) and info["coarse_block_rows"] in (256, 2048)
    ms, stats = b.step(1)
    assert all(st["error"] == 0 for st in stats)
    b.close()


def test_failed_instance_is_reported_and_the_others_go_on(built):
    """One instance with a too-small pair capacity fails its step (status 4, the reference's
    `stop` on cell overflow); the batch returns normally, reports the status for that
    instance only, and the other instances match their individual runs exactly."""
    from vebisph_gb300.solver import BatchSolver, StepSolver
    bad = cases.poiseuille(20, seed=0)
    bad.nplink = 10
    cl = [cases.poiseuille(24, seed=1), bad, cases.cylinder(6.0e3, Wi=0.3, seed=3)]
    b = BatchSolver(cl, precision=abi.PREC_MIXED)
    ms, stats = b.step(2)
    assert [st["error"] for st in stats] == [0, 4, 0]
    ms, stats = b.step(1)  # sticky: still reported, the others still step
    assert [st["error"] for st in stats] == [0, 4, 0]
    for i in (0, 2):
        s = StepSolver(cl[i], precision=abi.PREC_MIXED)
        for _ in range(3):
            s.step()
        for nm in ("ux", "uy", "p"):
            assert np.array_equal(b.instances[i].get(nm)[: cl[i].npfb], s.get(nm)[: cl[i].npfb]), (i, nm)
        s.close()
    b.close()


def test_diverging_instance_is_flagged(built):
    """The opt-in divergence guard: an instance whose velocity passes its limit (here a limit
    below the flow's own velocity, standing in for a blow-up) fails with VEBI_ERR_DIVERGED in
    its own stats, sticky like every step failure; the other instances go on unchanged.  A
    NaN velocity in an uploaded state fails the same way."""
    from vebisph_gb300.solver import BatchSolver, StepSolver
    cl = [cases.poiseuille(24, seed=1), cases.cylinder(6.0e3, Wi=0.3, seed=3), cases.poiseuille(20, seed=4)]
    b = BatchSolver(cl, precision=abi.PREC_MIXED)
    for inst in b.instances:
        inst.set_velocity_limit(1.0e3)
    b.instances[1].set_velocity_limit(1.0e-3)  # the cylinder starts at ~1
    ms, stats = b.step(2)
    assert [st["error"] for st in stats] == [0, abi.STATUS["VEBI_ERR_DIVERGED"], 0]
    for i in (0, 2):
        s = StepSolver(cl[i], precision=abi.PREC_MIXED)
        for _ in range(2):
            s.step()
        for nm in ("ux", "uy", "p"):
            assert np.array_equal(b.instances[i].get(nm)[: cl[i].npfb], s.get(nm)[: cl[i].npfb]), (i, nm)
        s.close()
    b.close()
    c = cases.poiseuille(20, seed=5)
    c.u[c.nbS + 3] = [np.nan, 0.0]
    s = StepSolver(c)
    s.set_velocity_limit(1.0e3)
    st = s.lib.vebi_step(s.h, s.x_mint, s.y_mint, s.x_maxt, s.y_maxt, 0, None)
    assert st == abi.STATUS["VEBI_ERR_DIVERGED"], st
    s.set_velocity_limit(0.0)  # off: the reference's behaviour, the NaN particle goes to the bin
    f = c.fortran_planes()
    s.upload(f["r"], f["u"], f["tau"], f["theta"], f["trace_conf"], f["inbin"], f["ld"])
    assert s.step()["n_inbin"] == 1
    s.close()

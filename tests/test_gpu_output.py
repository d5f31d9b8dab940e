"""Output files from the GPU state (vebi_dump_async / vebi_dump_write): the PART dump and the
TEMP_REC.dat restart record hold exactly the fields after the dumped step, in the reference's
column order (output.F90:40-77), also when later steps run while the copies are in flight."""
import numpy as np
import pytest

from vebisph_gb300 import cases

pytestmark = pytest.mark.gpu


def _read_part(path, ve=True):
    rows = [ln.split() for ln in open(path)]
    a = np.array([[float(v) for v in r] for r in rows])
    assert a.shape[1] == (13 if ve else 10)
    return a


def _fields(s, n):
    g = {k: s.get(k)[:n].copy() for k in ("rx", "ry", "ux", "uy", "theta", "p", "a_out", "vort", "tau11", "tau21",
                                          "tau12", "tau22")}
    g["n_surf"] = s.get("n_surf")[:n].copy()
    return g


@pytest.mark.parametrize("binned", [False, True])
def test_part_and_restart_hold_the_dumped_step(built, tmp_path, binned):
    from vebisph_gb300.solver import StepSolver
    c = cases.poiseuille(40, seed=1)
    n = c.npfb
    keep = np.ones(n, bool)
    if binned:  # one particle goes to the bin and is skipped in both files (one step: the
        c.r[c.nbS + 3] = [50.0, 50.0]  # reference's own next step diverges on this input)
        keep[c.nbS + 3] = False
    s = StepSolver(c)
    if not binned:
        s.step()
    s.step(secondary=True)  # vorticity at dump steps (div_free.F90:154)
    want = _fields(s, n)
    s.dump_async()
    if not binned:
        s.step()  # runs while the host copies are in flight; the files keep the dumped step
    s.dump_write(tmp_path / "PART3", tmp_path / "TEMP_REC.dat", time=1.25, dt=1e-3, itime=7, n_dump=3)
    a = _read_part(tmp_path / "PART3")
    assert a.shape[0] == keep.sum()
    cols = ["rx", "ry", "ux", "uy", "theta", "p", None, "a_out", "n_surf", "vort", "tau11", "tau12", "tau22"]
    for k, nm in enumerate(cols):
        if nm is None:
            assert np.all(a[:, k] == 0.0)  # conc exists only in open domains
            continue
        assert np.array_equal(a[:, k], want[nm][keep].astype(float)), nm
    rs = cases.read_restart(tmp_path / "TEMP_REC.dat")
    assert (rs["itime"], rs["time"], rs["n_dump"], rs["npfb"]) == (7, 1.25, 3, int(keep.sum()))
    assert rs["nbS"] == c.nbS and rs["np_inflow"] == 0
    assert np.array_equal(rs["r"][:, 0], want["rx"][keep]) and np.array_equal(rs["u"][:, 1], want["uy"][keep])
    assert np.array_equal(rs["theta"], want["theta"][keep]) and np.array_equal(rs["p"], want["p"][keep])
    assert np.all(rs["dv"] == c.dv)
    for q, nm in enumerate(("tau11", "tau12", "tau21", "tau22")):
        assert np.array_equal(rs["tau"][:, q], want[nm][keep]), nm
    s.close()


def test_background_write_and_readable_restart(built, tmp_path):
    from vebisph_gb300.solver import StepSolver
    c = cases.cylinder(6.0e3, Wi=0.3, seed=3)
    s = StepSolver(c)
    s.step()
    want = _fields(s, c.npfb)
    s.dump_async()
    s.dump_write(None, tmp_path / "R.dat", background=True, restart_readable=True)
    s.step()
    s.dump_wait()
    rs = cases.read_restart(tmp_path / "R.dat", theta=False)
    assert "theta" not in rs
    assert np.array_equal(rs["p"], want["p"]) and np.array_equal(rs["r"][:, 1], want["ry"])
    s.close()


def test_write_without_a_staged_dump_is_an_error(built, tmp_path):
    from vebisph_gb300.solver import StepSolver, VebiError
    s = StepSolver(cases.poiseuille(20, seed=0))
    s.step()
    with pytest.raises(VebiError):
        s.dump_write(tmp_path / "P")
    s.close()

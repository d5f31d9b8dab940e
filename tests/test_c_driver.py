"""A plain-C host driver over the C-ABI (tests/c_driver/vebi_driver.c): it compiles against
include/vebi.h and links the library with gcc alone (CPU), and on the GPU its steps, log records
and dump files equal those of the Python interface on the same input."""
import pathlib
import subprocess

import numpy as np
import pytest

from vebisph_gb300 import abi, cases

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _build(tmp_path):
    exe = tmp_path / "vebi_driver"
    lib = abi.library_path()
    subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-Werror", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "c_driver" / "vebi_driver.c"), "-o", str(exe), "-L", str(lib.parent),
                    "-l:" + lib.name, "-Wl,-rpath," + str(lib.parent)], check=True)
    return exe


def test_driver_compiles_and_links(built, tmp_path):
    assert _build(tmp_path).exists()


def _write_input(path, case):
    f = case.fortran_planes()
    with open(path, "wb") as fh:
        fh.write(bytes(case.params(abi.PREC_FP64)))
        for k in ("r", "u", "tau", "theta", "trace_conf"):
            fh.write(np.ascontiguousarray(f[k], dtype=np.float64).tobytes())
        fh.write(np.ascontiguousarray(f["inbin"], dtype=np.uint8).tobytes())


@pytest.mark.gpu
def test_c_driver_matches_the_python_interface(built, tmp_path):
    from vebisph_gb300.solver import StepSolver
    case = cases.cylinder(6.0e3, Wi=0.6, seed=4)
    n, nsteps = case.npfb, 3
    _write_input(tmp_path / "in.bin", case)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(_build(tmp_path)), str(tmp_path / "in.bin"), str(nsteps), str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    st = np.fromfile(out / "state.bin", dtype=np.float64)
    s = StepSolver(case)
    for k in range(nsteps):
        s.step(secondary=(k == nsteps - 1))
    d = s.download()
    got = {"r": st[: 2 * n], "u": st[2 * n: 4 * n], "tau": st[4 * n: 8 * n], "theta": st[8 * n: 9 * n],
           "p": st[9 * n: 10 * n]}
    for k, v in got.items():
        assert np.array_equal(v, d[k].ravel()[: v.size]), k
    assert len((out / "TIME").read_text().splitlines()) == nsteps
    assert len((out / "LS").read_text().splitlines()) == nsteps
    part = np.loadtxt(out / "PART1")
    assert part.shape[0] == n and np.array_equal(part[:, 5], d["p"][:n])
    s.close()

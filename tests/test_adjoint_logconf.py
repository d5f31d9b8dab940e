"""The adjoint's log-conformation product on the CPU (vebi_adjoint_logconf.cuh is host/device).

logconf_vjp -- three four-direction forward-mode Jacobians chained backwards -- against the
nine-direction forward mode through the whole update, contracted with the same seed, and against
central differences of the FP64 update, over 4000 seeded conformations: general, diagonal
(a21 == 0, the branch whose eigenvector turn is added by hand), at rest (A = I) and with
eigenvalues within 1e-7.  The bounds are in tests/adjoint_logconf/check.cpp."""
import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


def test_chained_product_matches_the_full_jacobian(tmp_path):
    nvcc = shutil.which("nvcc")
    if shutil.which("g++") is None or nvcc is None:
        pytest.skip("needs g++ and the CUDA toolkit's headers")
    CUDA_INCLUDE = pathlib.Path(nvcc).resolve().parent.parent / "include"
    exe = tmp_path / "check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(ROOT / "vebisph_gb300" / "csrc"),
                    "-I", str(CUDA_INCLUDE), "-o", str(exe), str(ROOT / "tests" / "adjoint_logconf" / "check.cpp")],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr

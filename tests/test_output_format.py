"""The list-directed formatter of the output files (vebi_format_list, vebisph_gb300/csrc/
vebi_output.cu) against the reference's own list-directed files: the shipped IPART (written by
datclass.F90:649-651 with gfortran, Makefile FC := gfortran) and IBOUND's integer items.  Host
code only: runs without a GPU."""
import ctypes as C
import hashlib
import json
import pathlib

import pytest

from vebisph_gb300 import cases

GOLDEN = json.loads((pathlib.Path(__file__).resolve().parent / "golden" / "list_directed.json").read_text())


@pytest.fixture(scope="module")
def fmt(built):
    from vebisph_gb300 import abi
    lib = abi.load_library()

    def f(kinds, reals=(), ints=()):
        r = (C.c_double * max(1, len(reals)))(*reals)
        i = (C.c_int32 * max(1, len(ints)))(*ints)
        buf = C.create_string_buffer(4096)
        n = lib.vebi_format_list(kinds.encode(), r, i, buf, 4096)
        assert n > 0
        return buf.raw[:n].decode()
    return f


def test_reproduces_the_shipped_ipart_text(fmt):
    c = cases.rayleigh_benard_deck()
    dxdx = c.dx * c.dx  # write(13,*) ..., dx*dx
    lines = [fmt("rrrrrr", [c.r[i, 0], c.r[i, 1], c.u[i, 0], c.u[i, 1], c.theta[i], dxdx]) for i in range(c.npfb)]
    assert len(lines) == GOLDEN["ipart_lines"]
    for k, want in GOLDEN["ipart_sample"].items():
        assert lines[int(k)] == want + "\n", k
    assert hashlib.sha256("".join(lines).encode()).hexdigest() == GOLDEN["ipart_sha256"]


def test_integer_items_match_ibound(fmt):
    for item in GOLDEN["ibound_integer_items"]:
        assert fmt("i", ints=[int(item)]) == item + "\n"


@pytest.mark.parametrize("v,want", [
    (0.1, "  0.10000000000000001     "),             # F form from 0.1 (17 - 0 decimals)
    (0.09999999999999999, "   9.9999999999999992E-002"),  # below 0.1: E form
    (1.0e16, "   10000000000000000.     "),           # 17 digits before the point
    (1.0e17, "   1.0000000000000000E+017"),           # 1e17: E form
    (-2.5, "  -2.5000000000000000     "),
    (1.0e-300, "   1.0000000000000000E-300"),
    (123456.789, "   123456.78900000000     "),          # k = 6: 11 decimals
])
def test_g_edit_boundaries(fmt, v, want):
    assert fmt("r", [v]) == want + "\n"


def test_cap_too_small_is_rejected(built):
    from vebisph_gb300 import abi
    lib = abi.load_library()
    buf = C.create_string_buffer(10)
    assert lib.vebi_format_list(b"rr", (C.c_double * 2)(1.0, 2.0), None, buf, 10) == -1

"""The library's FP32 <-> FP64 conversions on the integer pipe (vebi_common.cuh: widen, narrow)
against the GPU's own conversions, bit for bit, on 2^26 seeded inputs of every class."""
import ctypes as C

import pytest

from vebisph_gb300 import abi

pytestmark = pytest.mark.gpu


def test_conversions_match_hardware():
    lib = abi.load_library()
    bn, bw = C.c_int64(-1), C.c_int64(-1)
    assert lib.vebi_test_conversions(1 << 26, 20261204, C.byref(bn), C.byref(bw)) == 0, lib.vebi_last_error()
    assert bn.value == 0 and bw.value == 0, (bn.value, bw.value)


def test_conversions_argument_check():
    lib = abi.load_library()
    bn, bw = C.c_int64(0), C.c_int64(0)
    assert lib.vebi_test_conversions(0, 1, C.byref(bn), C.byref(bw)) == abi.STATUS["VEBI_ERR_ARG"]

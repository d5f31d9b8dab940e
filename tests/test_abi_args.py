"""Argument checks of the C-ABI that run before any device work, so they are exercised here
without a GPU: null handles and pointers, empty batches, bad record kinds."""
import ctypes as C

import pytest

from vebisph_gb300 import abi


@pytest.fixture(scope="module")
def lib(built):
    return abi.load_library()


def test_null_arguments_are_rejected(lib):
    h = C.c_void_p()
    assert lib.vebi_create(None, None) == 1  # VEBI_ERR_ARG
    assert lib.vebi_create(None, C.byref(h)) == 1
    assert lib.vebi_step(None, 0.0, 0.0, 1.0, 1.0, 0, None) == 1
    assert lib.vebi_run_steps(None, 0.0, 0.0, 1.0, 1.0, 1, None, None) == 1
    assert lib.vebi_upload_state(None, None, None, None, None, None, None, 0) == 1
    assert lib.vebi_download_state(None, None, None, None, None, None, None, None, None, None, None, 0) == 1
    assert lib.vebi_dump_async(None) == 1
    assert lib.vebi_dump_write(None, None, None, None) == 1
    assert lib.vebi_dump_wait(None) == 1
    assert lib.vebi_set_timing(None, 1) == 1
    assert lib.vebi_set_solver_grid(None, 2) == 1
    assert lib.vebi_destroy(None) == 0
    assert lib.vebi_last_error()  # the last failure left its text


def test_batch_arguments(lib):
    b = C.c_void_p()
    p = abi.VebiParams()
    assert lib.vebi_batch_create(C.byref(p), 0, C.byref(b)) == 1
    assert lib.vebi_batch_create(None, 2, C.byref(b)) == 1
    assert lib.vebi_batch_step(None, 1, None, None) == 1
    assert lib.vebi_batch_get(None, 0, None) == 1
    assert lib.vebi_batch_destroy(None) == 0


def test_record_kinds(lib):
    buf = C.create_string_buffer(256)
    assert lib.vebi_format_list(b"rx", (C.c_double * 2)(1.0, 2.0), None, buf, 256) == -1
    assert lib.vebi_format_list(None, None, None, buf, 256) == -1
    n = lib.vebi_format_list(b"", None, None, buf, 256)
    assert n == 1 and buf.value == b"\n"


def test_adjoint_arguments(lib):
    """The adjoint's entry points reject null handles, and the Weissenberg setter a null context
    or a non-positive value, before any device work."""
    a = C.c_void_p()
    assert lib.vebi_adjoint_create(None, 4, 2, C.byref(a)) == 1
    assert lib.vebi_adjoint_create(None, 4, 2, None) == 1
    assert lib.vebi_adjoint_record(None, 1, None) == 1
    assert lib.vebi_adjoint_replay(None, 1, None) == 1
    assert lib.vebi_adjoint_restore(None, 0) == 1
    assert lib.vebi_adjoint_reverse(None, None, None, None, 1, None, None, None, None, None) == 1
    assert b"adjoint" in lib.vebi_last_error()
    assert lib.vebi_adjoint_destroy(None) == 0
    assert lib.vebi_set_weissenberg(None, 0.5) == 1

"""The C-ABI library builds here (cross-compiled for sm_103a), loads without a GPU and
exports every entry point include/vebi.h declares; the ctypes mirrors match the C layout."""
import pathlib
import re
import subprocess

import ctypes as C
import pytest

from vebisph_gb300 import abi

ROOT = pathlib.Path(__file__).resolve().parent.parent


def header_functions():
    txt = (ROOT / "include" / "vebi.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|const char\*)\s+(vebi_\w+)\s*\(", txt, flags=re.M)))


def test_header_functions_listed():
    assert sorted(abi.EXPORTED_SYMBOLS) == header_functions()


def test_library_exports_every_declared_symbol(built):
    lib = abi.load_library()
    for name in header_functions():
        assert hasattr(lib, name), name
    assert b"sm_103a" in lib.vebi_version()


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "probe.c"
    fields_p = [f for f, _ in abi.VebiParams._fields_]
    fields_s = [f for f, _ in abi.VebiStepStats._fields_]
    fields_d = [f for f, _ in abi.VebiDumpInfo._fields_]
    body = ['#include <stdio.h>', '#include <stddef.h>', '#include "vebi.h"', 'int main(void){',
            'printf("%zu %zu\\n", sizeof(vebi_params), sizeof(vebi_step_stats));']
    body += [f'printf("%zu\\n", offsetof(vebi_params, {f}));' for f in fields_p]
    body += [f'printf("%zu\\n", offsetof(vebi_step_stats, {f}));' for f in fields_s]
    body += ['printf("%zu\\n", sizeof(vebi_dump_info));']
    body += [f'printf("%zu\\n", offsetof(vebi_dump_info, {f}));' for f in fields_d]
    body += ["return 0;}"]
    src.write_text("\n".join(body))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    sp, ss = int(out[0]), int(out[1])
    assert sp == C.sizeof(abi.VebiParams)
    assert ss == C.sizeof(abi.VebiStepStats)
    offs = list(map(int, out[2:]))
    want = [getattr(abi.VebiParams, f).offset for f in fields_p] + \
           [getattr(abi.VebiStepStats, f).offset for f in fields_s] + [C.sizeof(abi.VebiDumpInfo)] + \
           [getattr(abi.VebiDumpInfo, f).offset for f in fields_d]
    assert offs == want


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setenv("VEBI_LIB", str(tmp_path / "nope.so"))
    monkeypatch.setattr(abi, "_lib", None)
    with pytest.raises(RuntimeError):
        abi.load_library()

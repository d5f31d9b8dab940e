"""Build recipe of the CPU oracle (test infrastructure).

g++ on the single restatement file; -ffp-contract=off keeps the arithmetic free of FMA
contraction (gcc contracts by default on aarch64, where the GPU machine runs).
"""
from __future__ import annotations

import pathlib
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
SRC = HERE / "vebi_oracle.cpp"
OUT = HERE / "_build" / "libvebi_oracle.so"


def build(force: bool = False) -> pathlib.Path:
    OUT.parent.mkdir(parents=True, exist_ok=True)
    if not force and OUT.exists() and OUT.stat().st_mtime >= SRC.stat().st_mtime:
        return OUT
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-I", str(HERE.parent / "include"), "-o", str(OUT), str(SRC)]
    subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    print(build(force=True))

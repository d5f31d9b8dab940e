"""Build recipe of the CUDA step library (libvebi_gb300.so) for sm_103a.

Each .cu file compiles to an object in parallel, then nvcc links the shared library.
--fmad=false keeps every FP64 expression un-contracted, as the reference is evaluated;
kernels that want fused multiply-adds call fma() explicitly.  Host code is compiled with
-ffp-contract=off for the same reason (gcc contracts by default on aarch64).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "libvebi_gb300.so"
INCLUDE = HERE.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-I", str(INCLUDE), "-I", str(CSRC)]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if pathlib.Path(cand).exists() else "nvcc"


def sources():
    return sorted(CSRC.glob("*.cu"))


def _stale(out: pathlib.Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False, extra: list | None = None,
          out_dir: pathlib.Path | None = None) -> pathlib.Path:
    """Compile the library into out_dir (default vebisph_gb300/_build); `extra` nvcc flags build
    a variant (e.g. a diagnostic -D flag) that should go to its own out_dir."""
    out = pathlib.Path(out_dir) if out_dir else OUT_DIR
    lib = out / LIB.name
    out.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + [INCLUDE / "vebi.h"]
    nvcc = _nvcc()
    extra = extra or []
    objs = []
    jobs = []
    for src in sources():
        obj = out / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, *ARCH, *NVFLAGS, *extra, "-c", str(src), "-o", str(obj)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
            for j, f in zip(jobs, futs):
                r = f.result()
                if verbose or r.returncode:
                    print(" ".join(j))
                    print(r.stdout + r.stderr)
                if r.returncode:
                    raise RuntimeError(f"nvcc failed on {j[-3]}")
    if force or jobs or _stale(lib, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return lib


if __name__ == "__main__":
    import sys
    print(build(force="-f" in sys.argv, verbose="-v" in sys.argv))

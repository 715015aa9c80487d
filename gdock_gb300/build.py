"""Build the gdock_gb300 shared library (CUDA for sm_103a) in-tree.

``python -m gdock_gb300.build`` compiles every ``csrc/*.cu`` with nvcc in
parallel and links ``gdock_gb300/_build/libgdock_gb300.so``.  ``--debug``
builds the debug variant ``libgdock_gb300_debug.so`` instead: the same code
with the kernels' index checks compiled in (``-DGD_DEBUG_CHECKS``; a failed
check is reported by the call instead of touching memory out of bounds).  Host code is
compiled with ``-ffp-contract=off`` so that host and device arithmetic that
must agree bit for bit (pose frames, transforms) is never fused into FMAs.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libgdock_gb300.so"
LIB_DEBUG = OUT / "libgdock_gb300_debug.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
              f"-I{ROOT / 'include'}", f"-I{CSRC}"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(CSRC.glob("*.cu"))


def _stale(lib: Path) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    deps = list(CSRC.glob("*")) + [ROOT / "include" / "gdock_gb300.h", Path(__file__)]
    return any(d.stat().st_mtime > t for d in deps if d.is_file())


def build(force: bool = False, verbose: bool = False, extra=(), debug: bool = False) -> Path:
    lib = LIB_DEBUG if debug else LIB
    if not force and not _stale(lib):
        return lib
    objdir = OUT / "debug" if debug else OUT
    objdir.mkdir(parents=True, exist_ok=True)
    nv = nvcc()
    flags = [*NVCC_FLAGS, *(["-DGD_DEBUG_CHECKS"] if debug else []), *extra]

    def compile_one(src: Path) -> Path:
        obj = objdir / (src.stem + ".o")
        cmd = [nv, *ARCH, *flags, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, flush=True)
        return obj

    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = OUT / (lib.name + ".tmp")
    cmd = [nv, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    v = "-v" in sys.argv
    print(build(force="-f" in sys.argv, verbose=v, extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else (),
                debug="--debug" in sys.argv))

"""Build libpsfun_gb300.so (sm_103a) in-tree with nvcc.

Every translation unit is compiled in parallel with one -gencode
(compute_103a / sm_103a) and linked into psfun_gb300/lib/libpsfun_gb300.so.
The build is incremental on source/header mtimes, and starts over when the
objects were made on another machine architecture (a stamp file records it).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libpsfun_gb300.so"
INCLUDE = PKG.parent / "include"

SOURCES = ["capi.cu", "krylov.cu", "cg.cu", "batch.cu", "batch_arnoldi.cu", "quadrule.cpp"]
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build psfun_gb300")
    return exe


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


STAMP = LIBDIR / "build_machine.txt"


def _compile(src: str, verbose: bool, fresh: bool) -> Path:
    s = CSRC / src
    obj = LIBDIR / (src + ".o")
    newest = max([s.stat().st_mtime] + [d.stat().st_mtime for d in _deps()])
    if not fresh and obj.exists() and obj.stat().st_mtime >= newest:
        return obj
    cmd = [nvcc(), "-c", str(s), "-o", str(obj), "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
           "-lineinfo", "-I", str(INCLUDE), "-I", str(CSRC)] + GENCODE
    if src.endswith(".cu"):
        cmd += ["--expt-relaxed-constexpr"]
        if verbose:
            cmd += ["-Xptxas", "-v"]
    else:
        cmd = [nvcc(), "-x", "c++", "-c", str(s), "-o", str(obj), "-O3", "-std=c++17",
               "-Xcompiler", "-fPIC", "-I", str(INCLUDE)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False) -> Path:
    LIBDIR.mkdir(parents=True, exist_ok=True)
    machine = platform.machine()
    fresh = not STAMP.exists() or STAMP.read_text().strip() != machine
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, fresh), SOURCES))
    if not fresh and LIB.exists() and LIB.stat().st_mtime >= max(o.stat().st_mtime for o in objs):
        return LIB
    cmd = [nvcc(), "-shared", "-o", str(LIB)] + [str(o) for o in objs] + GENCODE + ["-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    STAMP.write_text(machine + "\n")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))

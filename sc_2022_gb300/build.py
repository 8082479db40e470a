"""Build libsbpmg.so in-tree with nvcc for sm_103a.

Translation units compile in parallel; the shared library lands next to this
file (``sc_2022_gb300/libsbpmg.so``) and the objects in
``sc_2022_gb300/_build/``.  A rebuild is skipped when every object is newer
than its sources and the headers.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIB = PKG / "libsbpmg.so"

SOURCES = ["sbp_kernels.cu", "sbp_high_order.cu", "sbp_varcoef.cu", "sbp_capi.cpp",
           "sbp_op_solver.cpp", "sbp_coarse.cpp", "sbp_tma.cpp", "sbp_csr.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsbpmg")


def _headers():
    return list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *_headers()])


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile and link libsbpmg.so; returns its path."""
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", f"-I{INCLUDE}"]
    procs = []
    objs = []
    for name in SOURCES:
        src = CSRC / name
        obj = BUILD / (name + ".o")
        objs.append(obj)
        if not force and not _stale(obj, src):
            continue
        cmd = [cc, *ARCH, *common, "-c", str(src), "-o", str(obj)]
        if name.endswith(".cu"):
            cmd[1:1] = ["-Xptxas", "-v"] if verbose else []
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((name, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                             text=True)))
    errors = []
    for name, p in procs:
        out, _ = p.communicate()
        if verbose and out:
            print(out, file=sys.stderr)
        if p.returncode != 0:
            errors.append(f"{name}:\n{out}")
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    if force or procs or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart", "-lcusolver",
               "-lpthread",
               "-Xlinker", "--no-undefined"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))

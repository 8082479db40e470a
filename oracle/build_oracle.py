"""Build the C restatement of the reference's CPU sparse path
(oracle/sbp_cpu.c -> oracle/libsbp_cpu.so) with gcc + OpenMP.

Test infrastructure: used by tests/ and by bench.py's CPU baseline legs
only.  The reference itself is Julia; no reference source is compiled.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "sbp_cpu.c"
LIB = HERE / "libsbp_cpu.so"


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime > SRC.stat().st_mtime:
        return LIB
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))

"""Build recipe of the oracle's C restatement (test infrastructure only).

Compiles spmatvec_ref.c into oracle/libnss_oracle.so with gcc and OpenMP,
on whatever host runs it (x86 build host or aarch64 GPU host).  The
reference itself (Fortran + SciFortran + MPI) has no C/C++ source for this
path and no Fortran compiler exists here, so nothing of it is compiled.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "spmatvec_ref.c"
LIB = HERE / "libnss_oracle.so"


def build(verbose: bool = False) -> Path:
    if LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler for the oracle")
    cmd = [cc, "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-o", str(LIB), str(SRC), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)

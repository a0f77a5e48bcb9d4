"""Build recipe of the CUDA extension ``libnssdmrg.so`` (sm_103a only).

Compiles every translation unit of ``csrc/`` with nvcc in parallel and links
one shared library next to this file.  No cmake: the same recipe runs on the
x86 build host and on the aarch64 GPU host.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libnssdmrg.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "--expt-relaxed-constexpr"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(p).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnssdmrg.so")
    return p


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _compile(src: Path, extra: list[str]) -> Path:
    obj = BUILD / (src.stem + ".o")
    deps = [src] + list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.cuh")) + [HERE.parent / "include" / "nssdmrg.h"]
    if obj.exists() and all(obj.stat().st_mtime >= d.stat().st_mtime for d in deps if d.exists()):
        return obj
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile csrc/ into libnssdmrg.so; returns the library path."""
    BUILD.mkdir(exist_ok=True)
    extra = list(extra or [])
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    if LIB.exists() and all(LIB.stat().st_mtime >= o.stat().st_mtime for o in objs):
        return LIB
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcusolver", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_peaks(verbose: bool = False) -> Path:
    """Compile the compute-rate microbenchmark (peaks.cu) next to the objects."""
    BUILD.mkdir(exist_ok=True)
    exe = BUILD / "peaks"
    src = HERE / "peaks.cu"
    if exe.exists() and exe.stat().st_mtime >= src.stat().st_mtime:
        return exe
    r = subprocess.run([nvcc(), *ARCH, "-O3", "-o", str(exe), str(src)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on peaks.cu:\n{r.stderr}")
    if verbose:
        print(f"built {exe}")
    return exe


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])

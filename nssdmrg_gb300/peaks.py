"""Measure the FP64/FP32 CUDA-core rates of the current GPU.

    python -m nssdmrg_gb300.peaks [out.json]

Builds peaks.cu with nvcc (sm_103a) and prints its JSON line; these rates
are the roofline denominators of the plain FP64 and FP32 sector kernels
(the HBM and bf16 tensor peaks come from a copy and a cuBLAS GEMM).
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

from .build import build_peaks


def main(out: str | None = None) -> str:
    exe = build_peaks()
    line = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.strip().splitlines()[-1]
    if out:
        Path(out).write_text(line + "\n")
    print(line)
    return line


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)

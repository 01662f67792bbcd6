"""FP64 arithmetic rates of this GPU: FP64 FMA pipe, FP64 tensor-core MMA (mma.sync m8n8k4)
and FP32 FMA for scale (``python -m fempar_gb300.bench_fp64_rates``).

Builds ``csrc_bench/fp64_rates.cu`` with nvcc for sm_103a into ``_build/fp64_rates`` and runs
it; prints its JSON line (TFLOP/s of each kernel).  These rates decide where FP64 work goes:
the integration and factorisation kernels stay on the FP64 FMA pipe unless the MMA path is
clearly faster.
"""
from __future__ import annotations

import os
import subprocess
import sys

from .build import ARCH, BUILD, nvcc

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc_bench", "fp64_rates.cu")
EXE = os.path.join(BUILD, "fp64_rates")


def build() -> str:
    os.makedirs(BUILD, exist_ok=True)
    if not os.path.exists(EXE) or os.path.getmtime(EXE) < os.path.getmtime(SRC):
        subprocess.run([nvcc(), "-O3", "-std=c++17", "-lineinfo"] + ARCH + [SRC, "-o", EXE], check=True)
    return EXE


def main():
    r = subprocess.run([build()], capture_output=True, text=True)
    sys.stdout.write(r.stdout)
    sys.stderr.write(r.stderr)
    sys.exit(r.returncode)


if __name__ == "__main__":
    main()

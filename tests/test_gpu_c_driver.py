"""The plain-C driver of the C-ABI (tests/c_abi/poisson_driver.c: tutorial_01's serial steps
through include/fempar_gpu.h only) built with gcc and run on the GPU.  Its solution of the
sharp-wave Poisson problem (Q2, 6^3 cells, Jacobi-PCG to 1e-12) equals the oracle's to 1e-10,
with the same dof count and iteration count (+-1)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(ROOT, "fempar_gb300")
SHARP = [50.0, 0.7, -0.05, -0.05, -0.05]


def test_c_driver_runs_and_matches_oracle(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    from fempar_gb300 import build
    build.build()
    exe = tmp_path / "poisson_driver"
    cmd = ["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c_abi", "poisson_driver.c"), "-o", str(exe),
           "-L", LIB_DIR, "-lfempar_gpu", "-Wl,-rpath," + LIB_DIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "x.bin"
    r = subprocess.run([str(exe), "6", "2", "1e-12", str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    tok = r.stdout.split()
    dofs, iters, conv = int(tok[1]), int(tok[3]), int(tok[5])
    x = np.fromfile(out, dtype=np.float64)
    P = O.Problem((6, 6, 6), order=2, source_fn=O.FN_SHARP_WAVE, boundary_fn=O.FN_SHARP_WAVE, fn_param=SHARP)
    ref = P.cg(precond=1, rtol=1e-12, maxit=100000)
    assert conv == 1 and dofs == P.nfree == x.size
    assert abs(iters - ref["iters"]) <= 1, (iters, ref["iters"])
    assert np.linalg.norm(x - ref["x"]) <= 1e-10 * np.linalg.norm(ref["x"])

"""The C-ABI is usable from plain C: tests/c_abi/poisson_driver.c (tutorial_01's serial
steps through include/fempar_gpu.h only) compiles with gcc -std=c11 -Wall -Werror and links
against libfempar_gpu.so.  Running it needs a GPU: tests/test_gpu_c_driver.py runs it there."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(ROOT, "fempar_gb300")


def test_c_driver_compiles_and_links(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    if not os.path.exists(os.path.join(LIB_DIR, "libfempar_gpu.so")):
        pytest.skip("libfempar_gpu.so not built")
    exe = tmp_path / "poisson_driver"
    cmd = ["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c_abi", "poisson_driver.c"), "-o", str(exe),
           "-L", LIB_DIR, "-lfempar_gpu", "-Wl,--allow-shlib-undefined", "-Wl,-rpath," + LIB_DIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert exe.exists()

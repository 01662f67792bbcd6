"""The ctypes mirrors of the C-ABI structs (fempar_gb300/_lib.py) against the header
(include/fempar_gpu.h): size and every field offset, measured by a C program compiled here
with gcc.  A field added on one side only (or reordered) fails here, on the CPU, before any
call crosses the boundary.  The library is not loaded."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# ctypes class name -> C typedef name
PAIRS = {
    "Integrand": "fg_integrand", "MeshInfo": "fg_mesh_info", "PartitionInfo": "fg_partition_info",
    "DofImportSizes": "fg_dof_import_sizes", "SolverParams": "fg_solver_params", "SolveInfo": "fg_solve_info",
    "SpaceInfo": "fg_space_info", "ErrorNorms": "fg_error_norms", "BddcParams": "fg_bddc_params",
    "BddcInfo": "fg_bddc_info", "BatchProblem": "fg_batch_problem", "BatchResult": "fg_batch_result",
    "BatchInfo": "fg_batch_info", "Request": "fg_request", "Result": "fg_result",
}


def _ctypes_classes():
    import importlib.util
    spec = importlib.util.spec_from_file_location("_fg_lib_mirror", os.path.join(ROOT, "fempar_gb300", "_lib.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_struct_layouts_match_the_header(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    L = _ctypes_classes()
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "fempar_gpu.h"', "int main(void) {"]
    for py, c in PAIRS.items():
        cls = getattr(L, py)
        lines.append(f'  printf("{py} size %zu\\n", sizeof({c}));')
        for name, _ in cls._fields_:
            lines.append(f'  printf("{py} {name} %zu\\n", offsetof({c}, {name}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    seen = 0
    for line in out:
        if not line.strip():
            continue
        py, field, val = line.split()
        cls = getattr(L, py)
        if field == "size":
            assert C.sizeof(cls) == int(val), (py, C.sizeof(cls), int(val))
        else:
            assert getattr(cls, field).offset == int(val), (py, field, getattr(cls, field).offset, int(val))
        seen += 1
    assert seen > len(PAIRS)

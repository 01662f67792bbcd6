"""libfempar_gpu.so loads and exports every symbol declared in include/fempar_gpu.h
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        txt = open(os.path.join(ROOT, "include", fn)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b(fg_\w+)\s*\(", txt):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def libpath():
    from fempar_gb300 import build
    return build.build()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert {"fg_ctx_create", "fg_space_create", "fg_assemble", "fg_solve", "fg_system_export_csr"} <= names


def test_library_exports_all_declared(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_list_matches_header():
    from fempar_gb300 import _lib
    assert set(_lib.EXPORTS) == declared_symbols()


def test_status_strings_without_device(libpath):
    from fempar_gb300 import _lib
    L = _lib.lib()
    assert L.fg_status_string(0) == b"FG_OK"
    assert L.fg_status_string(-4) == b"FG_ERR_NOT_CONVERGED"
    assert L.fg_version().startswith(b"fempar-gb300")


def test_default_parameters_match_reference(libpath):
    # iterative_solver_parameters.f90:168-178: rtol 1e-6, atol 0, 1000 iterations, CG stops on res_res
    import ctypes as C
    from fempar_gb300 import _lib
    p = _lib.SolverParams()
    _lib.lib().fg_solver_params_default(C.byref(p))
    assert p.rtol == 1e-6 and p.atol == 0.0 and p.max_iters == 1000 and p.criterion == _lib.FG_RES_RES

"""The Fortran binding module include/fempar_gpu.f90 matches the C-ABI header: its bind(c)
derived types declare the same fields, in the same order, as the C structs of
include/fempar_gpu.h, and every bind(c) function it names is declared in the header.
(No Fortran compiler on the image, so the check is textual.)"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def fortran_types():
    text = open(os.path.join(ROOT, "include", "fempar_gpu.f90")).read()
    out = {}
    for m in re.finditer(r"type, bind\(c\) :: (\w+)\n(.*?)\n\s*end type", text, re.S):
        names = []
        for line in m.group(2).split("\n"):
            line = line.split("!")[0]
            if "::" not in line:
                continue
            decl = line.split("::", 1)[1]
            for item in decl.split(","):
                item = item.strip()
                if item:
                    names.append(re.sub(r"\(.*\)", "", item).strip())
        out[m.group(1)] = names
    return out


def c_struct_fields(name):
    text = open(os.path.join(ROOT, "include", "fempar_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    m = re.search(r"typedef struct \{([^{}]*)\}\s*" + name + r";", text, re.S)
    assert m, name
    names = []
    for decl in m.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        # "type a, b[8], *c" -> a, b, c
        parts = decl.split(",")
        first = parts[0].split()
        names.append(re.sub(r"\[.*\]|\*", "", first[-1]))
        for p in parts[1:]:
            names.append(re.sub(r"\[.*\]|\*", "", p.strip()))
    return names


def test_fortran_types_match_the_header():
    ft = fortran_types()
    assert {"fg_integrand", "fg_solver_params", "fg_solve_info", "fg_bddc_params", "fg_error_norms"} <= set(ft)
    for name, fields in ft.items():
        assert fields == c_struct_fields(name), (name, fields, c_struct_fields(name))


def test_fortran_interfaces_name_header_functions():
    f90 = open(os.path.join(ROOT, "include", "fempar_gpu.f90")).read()
    hdr = open(os.path.join(ROOT, "include", "fempar_gpu.h")).read()
    names = re.findall(r'bind\(c, name="(\w+)"\)', f90)
    assert len(names) >= 20 and "fg_system_spmv_device_noalloc" in names
    for n in names:
        assert re.search(r"\b" + n + r"\s*\(", hdr), n

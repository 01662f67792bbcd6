"""Regenerate the golden fixtures in this folder from the FEMPAR source tree.

Reads the reference's own test data as text (nothing of the reference is run):

* ``Sources/Tests/Serial/test_quadratures/test_quadratures.f90`` -- the hard-coded
  1D Gauss-Legendre nodes/weights for 1..20 points that the reference checks its
  quadrature against (to 1e-10) -> ``gauss_legendre_table.json``.
* ``Tutorials/tutorial_01_poisson_sharp_circular_wave/convergence_plot/uniform_mesh_error_order_{1,2,4,8}``
  -- energy-norm error vs sqrt(#dofs) of the 2D CG tutorial on uniform meshes
  (alpha=200, r=0.7, c=(-0.05,-0.05), Dirichlet on the whole boundary,
  generator script ``generate_convergence_plot_data_files.sh``) ->
  ``tutorial01_convergence.json``.
* ``Sources/Tests/Data/par_test_pb_bddc_linear_elasticity/test1_convergence`` --
  the BDDC elasticity CG iteration log -> ``bddc_elasticity_iterations.json``.
* ``Sources/Tests/Data/{test_poisson,par_test_poisson}/cube_hexas.gid/cube_hexas.mesh`` --
  the hexahedral GiD meshes the reference's test_poisson runs, parsed by the oracle's
  restated reader (``oracle/gid.py``) -> ``gid_cube_hexas.json``.

Usage:  python tests/golden/make_golden.py FEMPAR_SOURCE_TREE
        (or set FEMPAR_SOURCE_TREE in the environment)
"""
import json
import os
import re
import sys

ROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FEMPAR_SOURCE_TREE")
OUT = os.path.dirname(os.path.abspath(__file__))
if __name__ == "__main__" and not ROOT:
    sys.exit("usage: python tests/golden/make_golden.py FEMPAR_SOURCE_TREE")


def gauss_legendre_table():
    path = os.path.join(ROOT, "Sources/Tests/Serial/test_quadratures/test_quadratures.f90")
    txt = open(path).read()
    table = {}
    cur = None
    for line in txt.splitlines():
        m = re.search(r"nlocs\s*==\s*(\d+)", line)
        if m and ("if" in line.lower()):
            cur = int(m.group(1))
            table[cur] = {"x": {}, "w": {}}
            continue
        m = re.search(r"(posgl|weigl)\s*\(\s*(\d+)\s*\)\s*=\s*([-+0-9.eEdD]+)_rp", line)
        if m and cur is not None:
            key = "x" if m.group(1) == "posgl" else "w"
            table[cur][key][int(m.group(2))] = float(m.group(3).replace("d", "e").replace("D", "e"))
    out = {}
    for n, d in sorted(table.items()):
        xs = [d["x"].get(i, 0.0) for i in range(1, n + 1)]
        ws = [d["w"].get(i, 0.0) for i in range(1, n + 1)]
        out[str(n)] = {"x": xs, "w": ws}
    return {"source": "Sources/Tests/Serial/test_quadratures/test_quadratures.f90:29-531",
            "tolerance": 1e-10, "table": out}


def convergence_tables():
    base = os.path.join(ROOT, "Tutorials/tutorial_01_poisson_sharp_circular_wave/convergence_plot")
    out = {}
    for order in (1, 2, 4, 8):
        rows = []
        for line in open(os.path.join(base, f"uniform_mesh_error_order_{order}")):
            parts = line.split()
            if len(parts) == 2:
                rows.append([float(parts[0]), float(parts[1])])
        out[str(order)] = rows
    return {"source": "Tutorials/tutorial_01_poisson_sharp_circular_wave/convergence_plot/uniform_mesh_error_order_{1,2,4,8}",
            "generator": "generate_convergence_plot_data_files.sh: num_dims=2, NX=NY=i*j (i in 10,100,1000; j in 1..9), "
                         "ALPHA=200, CIRCLE_RADIUS=0.7, CIRCLE_CENTER=(-0.05,-0.05), CG formulation",
            "columns": ["sqrt_num_free_dofs", "energy_norm_error"], "tables": out}


def bddc_iterations():
    path = os.path.join(ROOT, "Sources/Tests/Data/par_test_pb_bddc_linear_elasticity/test1_convergence")
    lines = [l.rstrip("\n") for l in open(path)]
    return {"source": "Sources/Tests/Data/par_test_pb_bddc_linear_elasticity/test1_convergence",
            "check": "Sources/Tests/Scripts/par_test_pb_bddc_linear_elasticity:17,29-33 (iterations within 5%)",
            "log": lines}


def gid_meshes():
    sys.path.insert(0, os.path.join(OUT, "..", "..", "oracle"))
    import gid
    out = {}
    for name in ("test_poisson", "par_test_poisson"):
        rel = f"Sources/Tests/Data/{name}/cube_hexas.gid/cube_hexas.mesh"
        m = gid.read_gid(os.path.join(ROOT, rel))
        out[name] = {"source": rel, **{k: (v.tolist() if hasattr(v, "tolist") else v) for k, v in m.items()}}
    return {"reader": "oracle/gid.py (mesh.f90:337-486 restated)", "meshes": out}


if __name__ == "__main__":
    for name, fn in (("gauss_legendre_table.json", gauss_legendre_table),
                     ("tutorial01_convergence.json", convergence_tables),
                     ("bddc_elasticity_iterations.json", bddc_iterations),
                     ("gid_cube_hexas.json", gid_meshes)):
        with open(os.path.join(OUT, name), "w") as f:
            json.dump(fn(), f, indent=1)
        print("wrote", name)

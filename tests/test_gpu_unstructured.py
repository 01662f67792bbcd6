"""Unstructured hexahedral meshes (fg_mesh_create_unstructured / fg_mesh_read_gid) against the
oracle's unstructured route.

Bar:
  * vef ids of every cell, vef set ids, dof numbering, CSR row pointers and column indices:
    bit-exact (reference layout, 1-based upper triangle);
  * matrix entries: |a - o| <= 1e-13 * max_j |o_ij|; right-hand side and Dirichlet values:
    <= 1e-13 (1e-14) of their max;
  * solutions: relative 2-norm error <= 1e-10 (FP64) / 1e-9 (mixed) with rtol 1e-13 / 1e-12;
  * the reference test's exact linear solution: device error norms <= 1e-10.
Meshes: seeded boxes with relabelled vertices, shuffled cells, every cell orientation of the
cube (proper and reflected), moved interior vertices, faces / box edges / corners given with
set ids per side -- the shape of the reference's GiD test meshes.
"""
import numpy as np
import pytest

import gidmesh
import oracle as O

pytestmark = pytest.mark.gpu

MAT_TOL = 1e-13
SHARP = [30.0, 0.35, -0.05, -0.05, -0.05]


@pytest.fixture(scope="module")
def fg():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fempar_gb300 as fg
    from fempar_gb300 import build
    build.build()
    return fg


@pytest.fixture(scope="module")
def ctx(fg):
    return fg.Context(0)


def device_mesh(fg, ctx, m):
    return fg.SerialTriangulation.from_arrays(ctx, m["coords"], m["cells"], m["bvef_ptr"], m["bvef_verts"],
                                              m["bvef_set"])


def assert_matrix_close(irp, ja, val, P):
    oirp, oja, oval = P.csr_upper()
    assert np.array_equal(irp, oirp)
    assert np.array_equal(ja, oja)
    rows = np.repeat(np.arange(P.nfree), np.diff(oirp))
    scale = np.zeros(P.nfree)
    np.maximum.at(scale, rows, np.abs(oval))
    err = np.abs(val - oval) / scale[rows]
    assert err.max() <= MAT_TOL, err.max()


def test_gid_file_and_vefs_match_oracle(fg, ctx, tmp_path):
    m = gidmesh.box_mesh((4, 3, 5), seed=3)
    gidmesh.write_gid(tmp_path / "box.mesh", m)
    tri = fg.SerialTriangulation.from_parameters(ctx, {"STATIC_TRIANG_GENERATE_FROM": "MESH_DATA_FILES",
                                                       "MESH_DIR_PATH": str(tmp_path), "MESH_PREFIX": "box"})
    P = O.UProblem(m, order=1, dirichlet_ids=(1,))
    info = tri.info()
    assert info["unstructured"] == 1
    assert (info["num_cells"], info["num_vertices"]) == (60, 5 * 4 * 6)
    assert (info["num_edges"], info["num_faces"], info["num_vefs"]) == (P.nedges, P.nfaces, P.nvefs)
    cv, vs = tri.get_vefs()
    assert np.array_equal(cv, P.cell_vefs())
    assert np.array_equal(vs, P.vef_sets())
    # the same arrays through the array entry point give the same tables
    tri2 = device_mesh(fg, ctx, m)
    cv2, vs2 = tri2.get_vefs()
    assert np.array_equal(cv2, cv) and np.array_equal(vs2, vs)


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("dirichlet", [(1, 2, 3, 4, 5, 6, 7, 8), (1, 4, 7)])
def test_poisson_parity(fg, ctx, order, dirichlet):
    m = gidmesh.box_mesh((5, 4, 3), seed=order + 10 * len(dirichlet), perturb=0.25)
    nc = len(m["cells"])
    rng = np.random.default_rng(order)
    coef = np.exp(rng.normal(0.0, 1.0, size=nc))
    P = O.UProblem(m, order=order, dirichlet_ids=dirichlet, cell_coef=coef, source_fn=O.FN_SHARP_WAVE,
                   boundary_fn=O.FN_SHARP_WAVE, fn_param=SHARP)
    tri = device_mesh(fg, ctx, m)
    sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=dirichlet)
    assert sp.num_free_dofs == P.nfree and sp.num_dirichlet_dofs == P.ndir
    assert np.array_equal(sp.get_dof_map(), P.dof_map())
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(cell_coef=coef, source_fn=O.FN_SHARP_WAVE,
                                                        boundary_fn=O.FN_SHARP_WAVE, fn_param=SHARP)).compute()
    irp, ja, val = op.get_matrix()
    assert_matrix_close(irp, ja, val, P)
    g, og = op.get_dirichlet_values(), P.dirichlet_values()
    assert np.max(np.abs(g - og)) <= 1e-14 * max(1.0, np.max(np.abs(og)))
    b, ob = op.get_translation(), P.rhs()
    assert np.max(np.abs(b - ob)) <= 1e-13 * np.max(np.abs(ob))
    ref = P.cg(precond=1, rtol=1e-13, maxit=20000)
    for prec, rtol, tol in (("fp64", 1e-13, 1e-10), ("mixed", 1e-12, 1e-9)):
        s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
        s.set_parameters_from_pl({"ILS_RTOL": rtol, "ILS_MAX_NUM_ITERATIONS": 20000, "PRECISION": prec})
        x = s.solve()
        assert s.info()["converged"], prec
        err = np.linalg.norm(x - ref["x"]) / np.linalg.norm(ref["x"])
        assert err <= tol, (prec, err)


@pytest.mark.parametrize("order", [1, 2, 3])
def test_elasticity_parity(fg, ctx, order):
    m = gidmesh.box_mesh((4, 3, 3), seed=21 + order, perturb=0.2)
    E = np.exp(np.random.default_rng(order).normal(0.0, 1.0, size=len(m["cells"])))
    ids = (1, 7, 8)
    P = O.UProblem(m, order=order, kind=O.ELASTICITY, dirichlet_ids=ids, cell_coef=E, nu=0.3,
                   source_fn=O.FN_CONST, fn_param=[0.0, 0.0, -1.0])
    tri = device_mesh(fg, ctx, m)
    sp = fg.SerialFESpace(tri, order=order, ncomp=3, dirichlet_ids=ids)
    assert np.array_equal(sp.get_dof_map(), P.dof_map())
    op = fg.FEAffineOperator(sp, fg.ElasticityIntegration(cell_coef=E, nu=0.3, source_fn=O.FN_CONST,
                                                          fn_param=[0.0, 0.0, -1.0])).compute()
    irp, ja, val = op.get_matrix()
    assert_matrix_close(irp, ja, val, P)
    b, ob = op.get_translation(), P.rhs()
    assert np.max(np.abs(b - ob)) <= 1e-13 * np.max(np.abs(ob))
    ref = P.cg(precond=1, rtol=1e-13, maxit=50000)
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-13, "ILS_MAX_NUM_ITERATIONS": 50000})
    x = s.solve()
    assert np.linalg.norm(x - ref["x"]) <= 1e-10 * np.linalg.norm(ref["x"])


@pytest.mark.parametrize("order", [1, 2, 3])
def test_reference_test_exact_solution_on_device(fg, ctx, order):
    """test_poisson's check on a GiD cube: u = x+y+z on set 1 (faces, box edges and corners
    given with set 1), f = 0; every error norm of the device solution below 1e-10."""
    m = gidmesh.box_mesh((3, 5, 6), seed=5, perturb=0.2, side_sets=False)
    tri = device_mesh(fg, ctx, m)
    sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=[1])
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(source_fn=O.FN_ZERO, boundary_fn=O.FN_LINEAR)).compute()
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-14, "ILS_MAX_NUM_ITERATIONS": 20000})
    x = s.solve()
    e = op.error_norms(x, fg.FG_FN_LINEAR)
    for k in ("mean_norm", "l1_norm", "l2_norm", "linfty_norm", "h1_seminorm", "w1infty_seminorm"):
        assert abs(e[k]) < 1e-10, (k, e[k])


def test_error_norms_match_oracle(fg, ctx):
    m = gidmesh.box_mesh((4, 4, 3), seed=8, perturb=0.2)
    P = O.UProblem(m, order=2, dirichlet_ids=(1, 2, 3, 4, 5, 6, 7, 8), source_fn=O.FN_SHARP_WAVE,
                   boundary_fn=O.FN_SHARP_WAVE, fn_param=SHARP)
    tri = device_mesh(fg, ctx, m)
    sp = fg.SerialFESpace(tri, order=2, dirichlet_ids=list(range(1, 9)))
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(source_fn=O.FN_SHARP_WAVE, boundary_fn=O.FN_SHARP_WAVE,
                                                        fn_param=SHARP)).compute()
    x = P.cg(precond=1, rtol=1e-13, maxit=20000)["x"]
    e = op.error_norms(x, fg.FG_FN_SHARP_WAVE, SHARP)
    o = P.error_norms(x, O.FN_SHARP_WAVE, SHARP)
    for k in ("l2_norm", "h1_seminorm", "linfty_norm"):
        assert abs(e[k] - o[k]) <= 1e-12 * abs(o[k]), (k, e[k], o[k])


def test_bad_meshes_and_bddc_rejected(fg, ctx, tmp_path):
    from fempar_gb300 import FGError
    m = gidmesh.box_mesh((2, 2, 2), seed=1)
    bad = dict(m)
    bad["cells"] = m["cells"].copy()
    bad["cells"][3, 2] = len(m["coords"]) + 5
    with pytest.raises(FGError):
        device_mesh(fg, ctx, bad)
    rep = dict(m)
    rep["cells"] = m["cells"].copy()
    rep["cells"][1, 4] = rep["cells"][1, 0]
    with pytest.raises(FGError):
        device_mesh(fg, ctx, rep)
    with pytest.raises(FGError):
        fg.SerialTriangulation.from_mesh_data_files(ctx, str(tmp_path), "missing")
    tri = device_mesh(fg, ctx, m)
    with pytest.raises(FGError):
        fg.SerialFESpace(tri, order=1, dirichlet_ids=[40])
    sp = fg.SerialFESpace(tri, order=1, dirichlet_ids=[1, 2, 3, 4, 5, 6, 7, 8])
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(source_fn=O.FN_CONST, fn_param=[1.0])).compute()
    with pytest.raises(FGError):
        fg.MLBDDC(op, nsub=(1, 1, 1))


@pytest.mark.parametrize("order", [1, 2, 3])
def test_irregular_mesh_parity(fg, ctx, order):
    """The cube-in-cube mesh refined twice (vertices in 3, 4, 6 and 8 cells), shuffled cells in
    random orientations: vefs, dof map and pattern bit-exact, entries and solution as above."""
    m = gidmesh.cube_in_cube(refine=2, seed=order)
    P = O.UProblem(m, order=order, dirichlet_ids=(1,), source_fn=O.FN_SHARP_WAVE, boundary_fn=O.FN_SHARP_WAVE,
                   fn_param=SHARP)
    tri = device_mesh(fg, ctx, m)
    cv, vs = tri.get_vefs()
    assert np.array_equal(cv, P.cell_vefs()) and np.array_equal(vs, P.vef_sets())
    sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=[1])
    assert np.array_equal(sp.get_dof_map(), P.dof_map())
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(source_fn=O.FN_SHARP_WAVE, boundary_fn=O.FN_SHARP_WAVE,
                                                        fn_param=SHARP)).compute()
    irp, ja, val = op.get_matrix()
    assert_matrix_close(irp, ja, val, P)
    ref = P.cg(precond=1, rtol=1e-13, maxit=20000)
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-13, "ILS_MAX_NUM_ITERATIONS": 20000})
    x = s.solve()
    assert np.linalg.norm(x - ref["x"]) <= 1e-10 * np.linalg.norm(ref["x"])

"""dG (symmetric interior penalty, tutorial_01's second formulation) on the device against the
oracle.

Bar: dof map, CSR row pointers and column indices bit-exact (reference layout, 1-based upper
triangle); entries |a - o| <= 1e-13 * max_j |o_ij| (the device sums a diagonal entry's facet
contributions in local face order, the reference in facet id order); rhs <= 1e-13 * max;
solutions <= 1e-10 (FP64, rtol 1e-13) / 1e-9 (mixed, rtol 1e-12); the reference test's
exact linear solution: device error norms <= 1e-10.
"""
import numpy as np
import pytest

import gidmesh
import oracle as O

pytestmark = pytest.mark.gpu
SHARP = [25.0, 0.3, -0.05, -0.05, -0.05]


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


def perturbed(n, frac, seed):
    rng = np.random.default_rng(seed)
    L = [k + 1 for k in n]
    I, J, K = np.meshgrid(*[np.arange(k) for k in L], indexing="ij")
    I, J, K = (a.transpose(2, 1, 0).ravel() for a in (I, J, K))
    xyz = np.stack([I / n[0], J / n[1], K / n[2]], 1)
    inner = (I > 0) & (I < n[0]) & (J > 0) & (J < n[1]) & (K > 0) & (K < n[2])
    xyz[inner] += rng.uniform(-frac, frac, size=(inner.sum(), 3)) / np.array(n)
    return xyz.ravel()


def check(fg, P, sp, op):
    assert sp.num_free_dofs == P.nfree and sp.num_dirichlet_dofs == 0
    assert np.array_equal(sp.get_dof_map(), P.dof_map())
    irp, ja, val = op.get_matrix()
    oirp, oja, oval = P.csr_upper()
    assert np.array_equal(irp, oirp) and np.array_equal(ja, oja)
    rows = np.repeat(np.arange(P.nfree), np.diff(oirp))
    scale = np.zeros(P.nfree)
    np.maximum.at(scale, rows, np.abs(oval))
    assert (np.abs(val - oval) / scale[rows]).max() <= 1e-13
    b, ob = op.get_translation(), P.rhs()
    assert np.max(np.abs(b - ob)) <= 1e-13 * np.max(np.abs(ob))
    ref = P.cg(precond=1, rtol=1e-13, maxit=50000)
    for prec, rtol, tol in (("fp64", 1e-13, 1e-10), ("mixed", 1e-12, 1e-9)):
        s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
        s.set_parameters_from_pl({"ILS_RTOL": rtol, "ILS_MAX_NUM_ITERATIONS": 50000, "PRECISION": prec})
        x = s.solve()
        assert s.info()["converged"], prec
        assert np.linalg.norm(x - ref["x"]) <= tol * np.linalg.norm(ref["x"]), prec


@pytest.mark.parametrize("order", [1, 2, 3])
def test_dg_structured_parity(fg, ctx, order):
    n = (4, 3, 5)
    xyz = perturbed(n, 0.2, seed=order)
    P = O.Problem(n, order=order, formulation=O.DG, vertex_xyz=xyz, source_fn=O.FN_SHARP_WAVE,
                  boundary_fn=O.FN_SHARP_WAVE, fn_param=SHARP)
    tri = fg.SerialTriangulation(ctx, n, vertex_xyz=xyz)
    sp = fg.SerialFESpace(tri, order=order, dg=True)
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(source_fn=O.FN_SHARP_WAVE, boundary_fn=O.FN_SHARP_WAVE,
                                                        fn_param=SHARP)).compute()
    check(fg, P, sp, op)


@pytest.mark.parametrize("order", [1, 2, 3])
def test_dg_unstructured_parity(fg, ctx, order):
    m = gidmesh.box_mesh((3, 4, 3), seed=30 + order, perturb=0.25)
    P = O.UProblem(m, order=order, dirichlet_ids=(), formulation=O.DG, source_fn=O.FN_SHARP_WAVE,
                   boundary_fn=O.FN_SHARP_WAVE, fn_param=SHARP)
    tri = fg.SerialTriangulation.from_arrays(ctx, m["coords"], m["cells"], m["bvef_ptr"], m["bvef_verts"],
                                             m["bvef_set"])
    sp = fg.SerialFESpace(tri, order=order, dg=True)
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(source_fn=O.FN_SHARP_WAVE, boundary_fn=O.FN_SHARP_WAVE,
                                                        fn_param=SHARP)).compute()
    check(fg, P, sp, op)


@pytest.mark.parametrize("order", [1, 2, 3])
def test_dg_exact_linear_solution(fg, ctx, order):
    """test_poisson -f dG: u = x+y+z weakly on the boundary, f = 0, error norms below 1e-10."""
    m = gidmesh.box_mesh((3, 5, 6), seed=9, perturb=0.2)
    tri = fg.SerialTriangulation.from_arrays(ctx, m["coords"], m["cells"], m["bvef_ptr"], m["bvef_verts"],
                                             m["bvef_set"])
    sp = fg.SerialFESpace(tri, order=order, dg=True)
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(source_fn=O.FN_ZERO, boundary_fn=O.FN_LINEAR)).compute()
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-14, "ILS_MAX_NUM_ITERATIONS": 50000})
    e = op.error_norms(s.solve(), fg.FG_FN_LINEAR)
    for k in ("mean_norm", "l1_norm", "l2_norm", "linfty_norm", "h1_seminorm", "w1infty_seminorm"):
        assert abs(e[k]) < 1e-10, (k, e[k])


def test_dg_rejects_coefficients(fg, ctx):
    from fempar_gb300 import FGError
    tri = fg.SerialTriangulation(ctx, (2, 2, 2))
    sp = fg.SerialFESpace(tri, order=1, dg=True)
    with pytest.raises(FGError):
        fg.FEAffineOperator(sp, fg.PoissonIntegration(cell_coef=np.ones(8) * 2.0)).compute()
    with pytest.raises(FGError):
        fg.MLBDDC(fg.FEAffineOperator(sp, fg.PoissonIntegration()).compute(), nsub=(1, 1, 1))


@pytest.mark.parametrize("order", [1, 2])
def test_dg_irregular_mesh_parity(fg, ctx, order):
    m = gidmesh.cube_in_cube(refine=1, seed=7 + order)
    P = O.UProblem(m, order=order, dirichlet_ids=(), formulation=O.DG, source_fn=O.FN_SHARP_WAVE,
                   boundary_fn=O.FN_SHARP_WAVE, fn_param=SHARP)
    tri = fg.SerialTriangulation.from_arrays(ctx, m["coords"], m["cells"], m["bvef_ptr"], m["bvef_verts"],
                                             m["bvef_set"])
    sp = fg.SerialFESpace(tri, order=order, dg=True)
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(source_fn=O.FN_SHARP_WAVE, boundary_fn=O.FN_SHARP_WAVE,
                                                        fn_param=SHARP)).compute()
    check(fg, P, sp, op)

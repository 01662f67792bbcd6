"""Edge cases against the CPU oracle: single-cell meshes and meshes one cell thick (structured
and unstructured, continuous and dG, Poisson and elasticity), spaces with no free dofs, and
BDDC with one-cell subdomains (no interior dofs for Q1).

Bar as in test_gpu_parity.py: numbering and CSR pattern bit-exact, entries and rhs 1e-13
(row-scaled), solutions 1e-10 at rtol 1e-13."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

CLAMP = [1, 3, 5, 7, 13, 15, 17, 19, 25]
ALL = list(range(1, 27))


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


def pair(fg, ctx, n, order, ids, kind=O.POISSON):
    ncomp = 3 if kind == O.ELASTICITY else 1
    coef = np.exp(np.random.default_rng(n[0] * 7 + order).normal(size=n[0] * n[1] * n[2]))
    fp = [0.0, 0.0, -1.0] if kind == O.ELASTICITY else [1.0]
    P = O.Problem(n, order=order, kind=kind, dirichlet_ids=ids, cell_coef=coef, nu=0.3, source_fn=O.FN_CONST,
                  fn_param=fp)
    tri = fg.SerialTriangulation(ctx, n)
    sp = fg.SerialFESpace(tri, order=order, ncomp=ncomp, dirichlet_ids=ids)
    integ = (fg.ElasticityIntegration(cell_coef=coef, nu=0.3, source_fn=O.FN_CONST, fn_param=fp)
             if kind == O.ELASTICITY else fg.PoissonIntegration(cell_coef=coef, source_fn=O.FN_CONST, fn_param=fp))
    op = fg.FEAffineOperator(sp, integ).compute()
    return P, tri, sp, op


def check_matrix(op, P):
    irp, ja, val = op.get_matrix()
    oirp, oja, oval = P.csr_upper()
    assert np.array_equal(irp, oirp) and np.array_equal(ja, oja)
    if len(oval):
        rows = np.repeat(np.arange(P.nfree), np.diff(oirp))
        scale = np.zeros(P.nfree)
        np.maximum.at(scale, rows, np.abs(oval))
        assert (np.abs(val - oval) / scale[rows]).max() <= 1e-13
    b, ob = op.get_translation(), P.rhs()
    if len(ob):
        assert np.max(np.abs(b - ob)) <= 1e-13 * max(np.max(np.abs(ob)), 1e-300)


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("n,ids", [((1, 1, 1), ALL), ((1, 1, 1), CLAMP), ((8, 1, 1), CLAMP), ((1, 6, 1), ALL),
                                   ((2, 1, 5), [21, 24, 26])])
def test_thin_meshes_match_oracle(fg, ctx, order, n, ids):
    P, tri, sp, op = pair(fg, ctx, n, order, ids)
    assert sp.num_free_dofs == P.nfree and np.array_equal(sp.get_dof_map(), P.dof_map())
    check_matrix(op, P)
    if P.nfree == 0:
        return
    ref = P.cg(precond=1, rtol=1e-13, maxit=100000)
    for prec, tol in (("fp64", 1e-10), ("mixed", 1e-9)):
        s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
        s.set_parameters_from_pl({"ILS_RTOL": 1e-13 if prec == "fp64" else 1e-12, "ILS_MAX_NUM_ITERATIONS": 100000,
                                  "PRECISION": prec})
        x = s.solve()
        assert s.info()["converged"], prec
        assert np.linalg.norm(x - ref["x"]) <= tol * max(np.linalg.norm(ref["x"]), 1e-300), prec


def test_no_free_dofs(fg, ctx):
    """Q1 on one cell with every boundary id Dirichlet: no free dofs; assembly and solve are
    no-ops that succeed (||r_0|| = 0 converges at once, as cg.f90 does)."""
    P, tri, sp, op = pair(fg, ctx, (1, 1, 1), 1, ALL)
    assert P.nfree == 0 and sp.num_free_dofs == 0
    irp, ja, val = op.get_matrix()
    assert list(irp) == [1] and len(ja) == 0
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    x = s.solve()
    assert len(x) == 0 and s.info()["converged"]


@pytest.mark.parametrize("order", [1, 2, 3])
def test_single_cell_elasticity(fg, ctx, order):
    P, tri, sp, op = pair(fg, ctx, (1, 1, 2), order, CLAMP, kind=O.ELASTICITY)
    assert np.array_equal(sp.get_dof_map(), P.dof_map())
    check_matrix(op, P)
    ref = P.cg(precond=1, rtol=1e-13, maxit=100000)
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-13, "ILS_MAX_NUM_ITERATIONS": 100000})
    x = s.solve()
    assert np.linalg.norm(x - ref["x"]) <= 1e-10 * np.linalg.norm(ref["x"])


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("ids", [(1, 2, 3, 4, 5, 6, 7, 8), (1, 7, 8)])
def test_unstructured_single_cell(fg, ctx, order, ids):
    """One hexahedron read as an unstructured mesh: with every boundary set Dirichlet, Q1 has
    no free dofs."""
    import gidmesh
    m = gidmesh.box_mesh((1, 1, 1), seed=5 + order, perturb=0.0)
    P = O.UProblem(m, order=order, dirichlet_ids=ids, source_fn=O.FN_CONST, fn_param=[1.0])
    tri = fg.SerialTriangulation.from_arrays(ctx, m["coords"], m["cells"], m["bvef_ptr"], m["bvef_verts"],
                                             m["bvef_set"])
    sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=list(ids))
    assert sp.num_free_dofs == P.nfree and np.array_equal(sp.get_dof_map(), P.dof_map())
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(source_fn=O.FN_CONST, fn_param=[1.0])).compute()
    check_matrix(op, P)
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-13})
    x = s.solve()
    assert s.info()["converged"]
    if P.nfree:
        ref = P.cg(precond=1, rtol=1e-13, maxit=1000)
        assert np.linalg.norm(x - ref["x"]) <= 1e-10 * np.linalg.norm(ref["x"])


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("n", [(1, 1, 1), (3, 1, 1)])
def test_dg_single_cell_and_thin(fg, ctx, order, n):
    P = O.Problem(n, order=order, formulation=O.DG, source_fn=O.FN_CONST, boundary_fn=O.FN_CONST,
                  fn_param=[1.0])
    tri = fg.SerialTriangulation(ctx, n)
    sp = fg.SerialFESpace(tri, order=order, dg=True)
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(source_fn=O.FN_CONST, boundary_fn=O.FN_CONST,
                                                        fn_param=[1.0])).compute()
    assert np.array_equal(sp.get_dof_map(), P.dof_map())
    check_matrix(op, P)
    ref = P.cg(precond=1, rtol=1e-13, maxit=10000)
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-13, "ILS_MAX_NUM_ITERATIONS": 10000})
    x = s.solve()
    assert np.linalg.norm(x - ref["x"]) <= 1e-10 * np.linalg.norm(ref["x"])


@pytest.mark.parametrize("order,kind", [(1, O.POISSON), (2, O.POISSON), (1, O.ELASTICITY)])
def test_bddc_one_cell_subdomains(fg, ctx, order, kind):
    """Every subdomain one cell: Q1 subdomains have no interior dofs."""
    import torch
    from bddc import BDDCOracle
    n = (4, 3, 2)
    P, tri, sp, op = pair(fg, ctx, n, order, CLAMP, kind=kind)
    ncomp = 3 if kind == O.ELASTICITY else 1
    cuts = [np.arange(k + 1) for k in n]
    Bo = BDDCOracle(P, n, order, ncomp, cuts, use_faces=True)
    M = fg.MLBDDC(op, nsub=n, cuts=cuts, use_faces=True)
    assert M.info()["num_coarse_dofs"] == Bo.ncoarse
    r = np.random.default_rng(4).normal(size=P.nfree)
    zo = Bo.apply(r)
    z = torch.zeros(P.nfree, dtype=torch.float64, device=f"cuda:{ctx.device}")
    M.apply_device(torch.tensor(r, device=z.device), z)
    assert np.linalg.norm(z.cpu().numpy() - zo) <= 1e-10 * np.linalg.norm(zo)
    M.close()

"""2D structured quadrilateral meshes (fg_mesh_create_structured with num_dims = 2) against
the oracle's 2D route: the reference generator's 2D polytope order and set ids (1..8).

Bar as in test_gpu_parity.py: dof numbering and CSR pattern bit-exact, entries and rhs 1e-13
(row-scaled), solutions 1e-10 (FP64, rtol 1e-13) / 1e-9 (mixed, rtol 1e-12)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

ALL2 = list(range(1, 9))
LEFT = [1, 3, 7]  # corners (0,0), (0,1) and the edge x = 0
SHARP = [30.0, 0.35, -0.05, -0.05, 0.0]


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


def perturbed2(n, frac, seed):
    rng = np.random.default_rng(seed)
    J, I = np.meshgrid(np.arange(n[1] + 1), np.arange(n[0] + 1), indexing="ij")
    I, J = I.ravel(), J.ravel()
    xyz = np.stack([I / n[0], J / n[1], np.zeros(I.size)], 1)
    inner = (I > 0) & (I < n[0]) & (J > 0) & (J < n[1])
    xyz[inner, :2] += rng.uniform(-frac, frac, size=(inner.sum(), 2)) / np.array(n)
    return xyz.ravel()


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
    if len(ob) and np.max(np.abs(ob)) > 0:
        assert np.max(np.abs(b - ob)) <= 1e-13 * np.max(np.abs(ob))


def check_solution(fg, op, P):
    ref = P.cg(precond=1, rtol=1e-13, maxit=100000)
    for prec, rtol, tol in (("fp64", 1e-13, 1e-10), ("mixed", 1e-12, 1e-9)):
        s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
        s.set_parameters_from_pl({"ILS_RTOL": rtol, "ILS_MAX_NUM_ITERATIONS": 100000, "PRECISION": prec})
        x = s.solve()
        assert s.info()["converged"], prec
        assert np.linalg.norm(x - ref["x"]) <= tol * np.linalg.norm(ref["x"]), prec


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("n", [(3, 2), (2, 5), (1, 1), (6, 1)])
@pytest.mark.parametrize("ids", ["all", "left", "none", "top"])
def test_dof_map_bit_exact_2d(fg, ctx, order, n, ids):
    d = {"all": ALL2, "left": LEFT, "none": [], "top": [6, 3, 4]}[ids]
    P = O.Problem(n, order=order, num_dims=2, dirichlet_ids=d)
    tri = fg.SerialTriangulation(ctx, n)
    sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=d)
    assert sp.num_free_dofs == P.nfree and sp.num_dirichlet_dofs == P.ndir
    assert np.array_equal(sp.get_dof_map(), P.dof_map())


@pytest.mark.parametrize("order", [1, 2, 3])
def test_poisson_2d_sharp_wave(fg, ctx, order):
    n = (7, 5)
    xyz = perturbed2(n, 0.2, seed=order)
    coef = np.exp(np.random.default_rng(order).normal(size=n[0] * n[1]))
    P = O.Problem(n, order=order, num_dims=2, dirichlet_ids=ALL2, vertex_xyz=xyz, cell_coef=coef,
                  source_fn=O.FN_SHARP_WAVE, boundary_fn=O.FN_SHARP_WAVE, fn_param=SHARP)
    tri = fg.SerialTriangulation(ctx, n, vertex_xyz=xyz)
    sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=ALL2)
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(cell_coef=coef, source_fn=O.FN_SHARP_WAVE,
                                                        boundary_fn=O.FN_SHARP_WAVE, fn_param=SHARP)).compute()
    assert np.array_equal(sp.get_dof_map(), P.dof_map())
    check_matrix(op, P)
    check_solution(fg, op, P)


@pytest.mark.parametrize("order", [1, 2, 3])
def test_poisson_2d_exact_linear(fg, ctx, order):
    """u = x + y is in every Q_p space: the solve reproduces it at the nodes."""
    n = (4, 6)
    xyz = perturbed2(n, 0.2, seed=10 + order)
    tri = fg.SerialTriangulation(ctx, n, vertex_xyz=xyz)
    sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=ALL2)
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(boundary_fn=O.FN_LINEAR)).compute()
    P = O.Problem(n, order=order, num_dims=2, dirichlet_ids=ALL2, vertex_xyz=xyz, boundary_fn=O.FN_LINEAR)
    check_matrix(op, P)
    check_solution(fg, op, P)


@pytest.mark.parametrize("order", [1, 2, 3])
def test_elasticity_2d(fg, ctx, order):
    n = (6, 3)
    xyz = perturbed2(n, 0.15, seed=20 + order)
    E = np.exp(np.random.default_rng(order).normal(0.0, 1.0, size=n[0] * n[1]))
    P = O.Problem(n, order=order, num_dims=2, kind=O.ELASTICITY, dirichlet_ids=LEFT, vertex_xyz=xyz, cell_coef=E,
                  nu=0.3, source_fn=O.FN_CONST, fn_param=[0.0, -1.0])
    tri = fg.SerialTriangulation(ctx, n, vertex_xyz=xyz)
    sp = fg.SerialFESpace(tri, order=order, ncomp=2, dirichlet_ids=LEFT)
    op = fg.FEAffineOperator(sp, fg.ElasticityIntegration(cell_coef=E, nu=0.3, source_fn=O.FN_CONST,
                                                          fn_param=[0.0, -1.0])).compute()
    assert np.array_equal(sp.get_dof_map(), P.dof_map())
    check_matrix(op, P)
    check_solution(fg, op, P)


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("fn", ["sharp", "linear"])
def test_error_norms_2d_match_oracle(fg, ctx, order, fn):
    """Device error norms on quadrilaterals against the oracle's 2D evaluation of the same
    solution vector (error_norms_scalar_t, sbm_error_norms_scalar.i90:67-241)."""
    n = (6, 5)
    xyz = perturbed2(n, 0.2, seed=40 + order)
    f = fg.FG_FN_SHARP_WAVE if fn == "sharp" else fg.FG_FN_LINEAR
    prm = SHARP if fn == "sharp" else []
    tri = fg.SerialTriangulation(ctx, n, vertex_xyz=xyz)
    sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=ALL2)
    src = fg.FG_FN_SHARP_WAVE if fn == "sharp" else fg.FG_FN_ZERO
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(source_fn=src, boundary_fn=f, fn_param=prm)).compute()
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-12, "ILS_MAX_NUM_ITERATIONS": 100000})
    x = s.solve()
    d, cells = op.error_norms(x, f, prm, cell_sq_energy=True)
    P = O.Problem(n, order=order, num_dims=2, dirichlet_ids=ALL2, vertex_xyz=xyz,
                  source_fn=O.FN_SHARP_WAVE if fn == "sharp" else O.FN_ZERO,
                  boundary_fn=O.FN_SHARP_WAVE if fn == "sharp" else O.FN_LINEAR, fn_param=prm)
    o = P.error_norms(x, O.FN_SHARP_WAVE if fn == "sharp" else O.FN_LINEAR, prm)
    scale = max(o["h1_norm"], 1e-300)
    for k, v in o.items():
        ref = scale if k == "mean_norm" else max(abs(v), 1e-14 * scale)
        assert abs(d[k] - v) <= 1e-12 * max(abs(ref), 1e-30) + 1e-14, (k, d[k], v)
    assert abs(np.sqrt(cells.sum()) - d["energy_norm"]) <= 1e-12 * max(d["energy_norm"], 1e-30)
    if fn == "linear":  # u = x + y lies in the space: the error is the solver's
        assert d["h1_norm"] <= 1e-9


def test_2d_unsupported_parts_report_errors(fg, ctx):
    from fempar_gb300 import FGError
    tri = fg.SerialTriangulation(ctx, (3, 3))
    with pytest.raises(FGError):
        fg.SerialFESpace(tri, order=1, dg=True)
    with pytest.raises(FGError):
        fg.SerialFESpace(tri, order=1, ncomp=3)
    with pytest.raises(FGError):
        fg.SerialFESpace(tri, order=1, dirichlet_ids=[12])
    sp = fg.SerialFESpace(tri, order=2, dirichlet_ids=ALL2)
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(source_fn=O.FN_CONST, fn_param=[1.0])).compute()
    with pytest.raises(FGError):
        fg.MLBDDC(op, nsub=(1, 1, 1))


@pytest.mark.parametrize("order", [2, 3])
def test_mixed_solver_finishes_in_fp64_when_fp32_stalls(fg, ctx, order):
    """Plane-strain elasticity to rtol 1e-13: the FP32 segments cannot reach it (before the
    FP64 hand-off the solver reported a non-finite residual); the solve converges to the FP64
    solution."""
    n = (6, 3)
    xyz = perturbed2(n, 0.15, seed=20 + order)
    E = np.exp(np.random.default_rng(order).normal(0.0, 1.0, size=n[0] * n[1]))
    P = O.Problem(n, order=order, num_dims=2, kind=O.ELASTICITY, dirichlet_ids=LEFT, vertex_xyz=xyz, cell_coef=E,
                  nu=0.3, source_fn=O.FN_CONST, fn_param=[0.0, -1.0])
    tri = fg.SerialTriangulation(ctx, n, vertex_xyz=xyz)
    sp = fg.SerialFESpace(tri, order=order, ncomp=2, dirichlet_ids=LEFT)
    op = fg.FEAffineOperator(sp, fg.ElasticityIntegration(cell_coef=E, nu=0.3, source_fn=O.FN_CONST,
                                                          fn_param=[0.0, -1.0])).compute()
    ref = P.cg(precond=1, rtol=1e-13, maxit=100000)
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-13, "ILS_MAX_NUM_ITERATIONS": 100000, "PRECISION": "mixed"})
    x = s.solve()
    assert s.info()["converged"]
    assert s.info()["error_estimate"] <= s.info()["tolerance"]
    assert np.linalg.norm(x - ref["x"]) <= 1e-10 * np.linalg.norm(ref["x"])

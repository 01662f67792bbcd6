"""GPU path (libfempar_gpu.so through its C-ABI) against the CPU oracle.

Bar (stated per test):
  * dof numbering, CSR row pointers and column indices: bit-exact (reference layout,
    1-based upper triangle);
  * matrix entries: |a - o| <= 1e-13 * max_j |o_ij| (row-scaled; entries that cancel
    to ~0 are compared against their row's scale);
  * right-hand side: |b - o| <= 1e-13 * max |o|;
  * solutions: relative 2-norm error <= 1e-10 with both sides solved to rtol 1e-13.
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

MAT_TOL = 1e-13
RHS_TOL = 1e-13
SOL_TOL = 1e-10
SHARP = [50.0, 0.7, -0.05, -0.05, -0.05]
CLAMP = [1, 3, 5, 7, 13, 15, 17, 19, 25]


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


def perturbed_vertices(n, frac, seed):
    rng = np.random.default_rng(seed)
    h = [1.0 / n[0], 1.0 / n[1], 1.0 / n[2]]
    I, J, K = np.meshgrid(np.arange(n[0] + 1), np.arange(n[1] + 1), np.arange(n[2] + 1), indexing="ij")
    I, J, K = I.transpose(2, 1, 0).ravel(), J.transpose(2, 1, 0).ravel(), K.transpose(2, 1, 0).ravel()
    xyz = np.stack([I * h[0], J * h[1], K * h[2]], axis=1)
    interior = (I > 0) & (I < n[0]) & (J > 0) & (J < n[1]) & (K > 0) & (K < n[2])
    d = rng.uniform(-frac, frac, size=xyz.shape) * np.array(h)
    xyz[interior] += d[interior]
    return xyz.ravel()


def build_pair(fg, ctx, n, order, dirichlet=None, source_fn=O.FN_ZERO, boundary_fn=O.FN_ZERO, fn_param=(),
               vertex_xyz=None, cell_coef=None):
    dirichlet = list(range(1, 27)) if dirichlet is None else list(dirichlet)
    P = O.Problem(n, order=order, dirichlet_ids=dirichlet, source_fn=source_fn, boundary_fn=boundary_fn,
                  fn_param=fn_param, vertex_xyz=vertex_xyz, cell_coef=cell_coef)
    tri = fg.SerialTriangulation(ctx, n, vertex_xyz=vertex_xyz)
    sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=dirichlet)
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(source_fn=source_fn, boundary_fn=boundary_fn,
                                                        fn_param=fn_param, cell_coef=cell_coef)).compute()
    return P, tri, sp, op


def assert_matrix_close(irp, ja, val, P):
    oirp, oja, oval = P.csr_upper()
    assert np.array_equal(irp, oirp)
    assert np.array_equal(ja, oja)
    rows = np.repeat(np.arange(P.nfree), np.diff(oirp))
    scale = np.zeros(P.nfree)
    np.maximum.at(scale, rows, np.abs(oval))
    err = np.abs(val - oval) / scale[rows]
    assert err.max() <= MAT_TOL, err.max()


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("n", [(2, 2, 2), (3, 4, 5), (5, 3, 2)])
@pytest.mark.parametrize("dirichlet", ["all", "clamp", "none", "faces"])
def test_dof_map_bit_exact(fg, ctx, order, n, dirichlet):
    ids = {"all": list(range(1, 27)), "clamp": CLAMP, "none": [], "faces": [21, 24, 26]}[dirichlet]
    P = O.Problem(n, order=order, dirichlet_ids=ids)
    tri = fg.SerialTriangulation(ctx, n)
    sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=ids)
    assert sp.num_free_dofs == P.nfree and sp.num_dirichlet_dofs == P.ndir
    assert np.array_equal(sp.get_dof_map(), P.dof_map())


@pytest.mark.parametrize("order", [1, 2, 3])
def test_assembly_sharp_wave(fg, ctx, order):
    n = (6, 5, 4)
    P, tri, sp, op = build_pair(fg, ctx, n, order, source_fn=O.FN_SHARP_WAVE, boundary_fn=O.FN_SHARP_WAVE,
                                fn_param=SHARP)
    irp, ja, val = op.get_matrix()
    assert_matrix_close(irp, ja, val, P)
    g = op.get_dirichlet_values()
    og = P.dirichlet_values()
    assert np.max(np.abs(g - og)) <= 1e-14 * max(1.0, np.max(np.abs(og)))
    b, ob = op.get_translation(), P.rhs()
    assert np.max(np.abs(b - ob)) <= RHS_TOL * np.max(np.abs(ob))


@pytest.mark.parametrize("order", [1, 2])
def test_assembly_perturbed_lognormal(fg, ctx, order):
    n = (5, 4, 6)
    xyz = perturbed_vertices(n, 0.15, seed=7)
    coef = np.exp(np.random.default_rng(3).normal(0.0, 1.0, size=n[0] * n[1] * n[2]))
    P, tri, sp, op = build_pair(fg, ctx, n, order, source_fn=O.FN_CONST, fn_param=[1.0], vertex_xyz=xyz,
                                cell_coef=coef)
    irp, ja, val = op.get_matrix()
    assert_matrix_close(irp, ja, val, P)
    b, ob = op.get_translation(), P.rhs()
    assert np.max(np.abs(b - ob)) <= RHS_TOL * np.max(np.abs(ob))


def test_full_csr_is_expanded_upper(fg, ctx):
    P, tri, sp, op = build_pair(fg, ctx, (4, 4, 4), 2, source_fn=O.FN_CONST, fn_param=[1.0])
    rp, ci, v = op.get_matrix(symmetric_storage=False, one_based=False)
    orp, oci, ov = P.csr_full()
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    rows = np.repeat(np.arange(P.nfree), np.diff(orp))
    scale = np.zeros(P.nfree)
    np.maximum.at(scale, rows, np.abs(ov))
    assert (np.abs(v - ov) / scale[rows]).max() <= MAT_TOL


def test_spmv_device(fg, ctx):
    import torch
    P, tri, sp, op = build_pair(fg, ctx, (5, 6, 4), 2, source_fn=O.FN_CONST, fn_param=[1.0])
    x = np.random.default_rng(1).standard_normal(P.nfree)
    y_ref = P.spmv(x)
    xd = torch.tensor(x, device="cuda")
    yd = torch.empty_like(xd)
    op.apply_device(xd, yd)
    y = yd.cpu().numpy()
    assert np.max(np.abs(y - y_ref)) <= 1e-13 * np.max(np.abs(y_ref))
    # FP32 copy of the matrix
    x32 = xd.float()
    y32 = torch.empty_like(x32)
    op.apply_device(x32, y32, precision=fg.FG_MIXED)
    assert np.max(np.abs(y32.cpu().numpy() - y_ref)) <= 1e-5 * np.max(np.abs(y_ref))


@pytest.mark.parametrize("order,precond", [(1, "identity"), (2, "jacobi"), (3, "jacobi")])
def test_cg_solution_parity(fg, ctx, order, precond):
    n = (5, 4, 6)
    xyz = perturbed_vertices(n, 0.15, seed=11)
    coef = np.exp(np.random.default_rng(5).normal(0.0, 1.0, size=n[0] * n[1] * n[2]))
    P, tri, sp, op = build_pair(fg, ctx, n, order, source_fn=O.FN_CONST, fn_param=[1.0], vertex_xyz=xyz,
                                cell_coef=coef)
    pc = 1 if precond == "jacobi" else 0
    ref = P.cg(precond=pc, rtol=1e-13, maxit=20000)
    s = fg.IterativeLinearSolver().set_type_from_string("CG")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-13, "ILS_MAX_NUM_ITERATIONS": 20000}).set_operators(op, precond)
    x = s.solve()
    assert s.info()["converged"]
    err = np.linalg.norm(x - ref["x"]) / np.linalg.norm(ref["x"])
    assert err <= SOL_TOL, err
    # same stopping decision at the reference default criterion
    ref8 = P.cg(precond=pc, rtol=1e-8, maxit=20000)
    s.set_parameters_from_pl({"ILS_RTOL": 1e-8})
    s.solve()
    assert abs(s.info()["iterations"] - ref8["iters"]) <= 1, (s.info()["iterations"], ref8["iters"])


@pytest.mark.parametrize("crit", ["RES_RES", "RES_RHS", "DELTA_RHS", "DELTA_DELTA", "RES_NRMGIVEN_RHS_NRMGIVEN",
                                  "RES_NRMGIVEN_RES_NRMGIVEN"])
def test_stopping_criteria(fg, ctx, crit):
    P, tri, sp, op = build_pair(fg, ctx, (4, 5, 3), 2, source_fn=O.FN_CONST, fn_param=[1.0])
    code = getattr(O, crit)
    ref = P.cg(precond=1, rtol=1e-7, maxit=5000, criterion=code)
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-7, "ILS_MAX_NUM_ITERATIONS": 5000, "ILS_STOPPING_CRITERIUM": crit})
    s.solve()
    assert abs(s.info()["iterations"] - ref["iters"]) <= 1, (crit, s.info()["iterations"], ref["iters"])


def test_mixed_precision_solution(fg, ctx):
    n = (6, 5, 7)
    xyz = perturbed_vertices(n, 0.15, seed=2)
    coef = np.exp(np.random.default_rng(9).normal(0.0, 1.0, size=n[0] * n[1] * n[2]))
    P, tri, sp, op = build_pair(fg, ctx, n, 2, source_fn=O.FN_CONST, fn_param=[1.0], vertex_xyz=xyz, cell_coef=coef)
    ref = P.cg(precond=1, rtol=1e-13, maxit=20000)
    s = fg.IterativeLinearSolver().set_type_from_string("GPU_MPCG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-12, "ILS_MAX_NUM_ITERATIONS": 20000})
    x = s.solve()
    info = s.info()
    assert info["converged"] and info["outer_iterations"] >= 1
    err = np.linalg.norm(x - ref["x"]) / np.linalg.norm(ref["x"])
    assert err <= 1e-9, err
    # the FP64 residual the refinement loop stops on
    r = P.rhs() - P.spmv(x)
    assert np.linalg.norm(r) <= 1.01e-12 * np.linalg.norm(P.rhs())


def test_exact_linear_solution(fg, ctx):
    for order in (1, 2, 3):
        P, tri, sp, op = build_pair(fg, ctx, (3, 4, 2), order, boundary_fn=O.FN_LINEAR)
        s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
        s.set_parameters_from_pl({"ILS_RTOL": 1e-12, "ILS_MAX_NUM_ITERATIONS": 5000})
        x = s.solve()
        assert P.energy_error(x) < 1e-8


def test_determinism(fg, ctx):
    P, tri, sp, op = build_pair(fg, ctx, (6, 6, 6), 2, source_fn=O.FN_SHARP_WAVE, boundary_fn=O.FN_SHARP_WAVE,
                                fn_param=SHARP)
    _, _, v1 = op.get_matrix(symmetric_storage=False)
    b1 = op.get_translation()
    op.compute()
    _, _, v2 = op.get_matrix(symmetric_storage=False)
    b2 = op.get_translation()
    assert np.array_equal(v1, v2) and np.array_equal(b1, b2)
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-10, "ILS_MAX_NUM_ITERATIONS": 5000})
    x1 = s.solve()
    x2 = s.solve()
    assert np.array_equal(x1, x2)


def test_errors_are_status_codes(fg, ctx):
    from fempar_gb300 import FGError
    tri = fg.SerialTriangulation(ctx, (2, 2, 2))
    with pytest.raises(FGError):
        fg.SerialFESpace(tri, order=7)
    with pytest.raises(FGError):
        fg.SerialFESpace(tri, order=1, dirichlet_ids=[40])
    tri = fg.SerialTriangulation(ctx, (5, 5, 5))
    sp = fg.SerialFESpace(tri, order=1, dirichlet_ids=list(range(1, 27)))
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(source_fn=O.FN_CONST, fn_param=[1.0])).compute()
    s = fg.IterativeLinearSolver().set_operators(op, "identity")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-30, "ILS_MAX_NUM_ITERATIONS": 1})
    s.solve()  # FG_ERR_NOT_CONVERGED is reported in info, x holds the last iterate
    assert not s.info()["converged"] and s.info()["iterations"] == 1
    with pytest.raises(FGError):
        s.solve(raise_on_nonconvergence=True)


@pytest.mark.parametrize("layout", ["stencil", "sell"])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_solver_layouts(fg, ctx, layout, order, monkeypatch):
    """Both solver layouts (lattice-implicit SELL, explicit-column SELL) give the oracle's
    operator and CG solution, on a partly Dirichlet boundary (box positions outside the
    domain and on free boundary nodes)."""
    import torch
    monkeypatch.setenv("FG_SOLVER_LAYOUT", layout)
    n = (5, 3, 4)
    P, tri, sp, op = build_pair(fg, ctx, n, order, dirichlet=CLAMP, source_fn=O.FN_CONST, fn_param=[1.0])
    x = np.random.default_rng(order).standard_normal(P.nfree)
    y_ref = P.spmv(x)
    xd = torch.tensor(x, device="cuda")
    yd = torch.empty_like(xd)
    op.apply_device(xd, yd)
    assert np.max(np.abs(yd.cpu().numpy() - y_ref)) <= 1e-13 * np.max(np.abs(y_ref))
    ref = P.cg(precond=1, rtol=1e-13, maxit=20000)
    for prec in ("fp64", "mixed"):
        s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
        s.set_parameters_from_pl({"ILS_RTOL": 1e-12, "ILS_MAX_NUM_ITERATIONS": 20000, "PRECISION": prec})
        xs = s.solve()
        assert s.info()["converged"], (layout, prec)
        err = np.linalg.norm(xs - ref["x"]) / np.linalg.norm(ref["x"])
        assert err <= 1e-9, (layout, prec, err)


# ---------------------------------------------------------------------------------------
# Linear elasticity (3 components): the heterogeneous irreducible integrand of
# par_test_pb_bddc_linear_elasticity with E per cell, nu = 0.3, body force (0,0,-1).

@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("dirichlet", ["clamp", "all"])
def test_vector_dof_map_bit_exact(fg, ctx, order, dirichlet):
    ids = CLAMP if dirichlet == "clamp" else list(range(1, 27))
    n = (3, 2, 4)
    P = O.Problem(n, order=order, kind=O.ELASTICITY, dirichlet_ids=ids)
    tri = fg.SerialTriangulation(ctx, n)
    sp = fg.SerialFESpace(tri, order=order, ncomp=3, dirichlet_ids=ids)
    assert sp.num_free_dofs == P.nfree and sp.num_dirichlet_dofs == P.ndir
    assert np.array_equal(sp.get_dof_map(), P.dof_map())


def build_elasticity_pair(fg, ctx, n, order, seed=3, perturb=True):
    xyz = perturbed_vertices(n, 0.15, seed=seed) if perturb else None
    E = np.exp(np.random.default_rng(seed).normal(0.0, 1.5, size=n[0] * n[1] * n[2]))
    P = O.Problem(n, order=order, kind=O.ELASTICITY, dirichlet_ids=CLAMP, vertex_xyz=xyz, cell_coef=E, nu=0.3,
                  source_fn=O.FN_CONST, fn_param=[0.0, 0.0, -1.0])
    tri = fg.SerialTriangulation(ctx, n, vertex_xyz=xyz)
    sp = fg.SerialFESpace(tri, order=order, ncomp=3, dirichlet_ids=CLAMP)
    op = fg.FEAffineOperator(sp, fg.ElasticityIntegration(cell_coef=E, nu=0.3, source_fn=O.FN_CONST,
                                                          fn_param=[0.0, 0.0, -1.0])).compute()
    return P, tri, sp, op


@pytest.mark.parametrize("order", [1, 2, 3])
def test_elasticity_assembly(fg, ctx, order):
    P, tri, sp, op = build_elasticity_pair(fg, ctx, (4, 3, 3), order)
    irp, ja, val = op.get_matrix()
    assert_matrix_close(irp, ja, val, P)
    b, ob = op.get_translation(), P.rhs()
    assert np.max(np.abs(b - ob)) <= RHS_TOL * np.max(np.abs(ob))


@pytest.mark.parametrize("order", [1, 2, 3])
def test_elasticity_solution(fg, ctx, order):
    P, tri, sp, op = build_elasticity_pair(fg, ctx, (5, 3, 4), order, seed=8)
    ref = P.cg(precond=1, rtol=1e-13, maxit=50000)
    # mixed to 1e-12: for Q3 (E ~ lognormal, sigma 1.5) the FP32 segments stall near that
    # tolerance and the solver finishes with FP64 PCG iterations
    for prec, tol in (("fp64", SOL_TOL), ("mixed", 1e-9)):
        s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
        s.set_parameters_from_pl({"ILS_RTOL": 1e-13 if prec == "fp64" else 1e-12, "ILS_MAX_NUM_ITERATIONS": 50000,
                                  "PRECISION": prec})
        x = s.solve()
        assert s.info()["converged"], prec
        err = np.linalg.norm(x - ref["x"]) / np.linalg.norm(ref["x"])
        assert err <= tol, (prec, err)


def test_order_4_reported_unsupported(fg, ctx):
    from fempar_gb300 import FGError
    tri = fg.SerialTriangulation(ctx, (2, 2, 2))
    with pytest.raises(FGError):
        sp = fg.SerialFESpace(tri, order=4, ncomp=3, dirichlet_ids=CLAMP)
        fg.FEAffineOperator(sp, fg.ElasticityIntegration(cell_coef=np.ones(8), nu=0.3)).compute()


@pytest.mark.parametrize("tc", ["0", "2"], ids=["float_float", "tensor_cores"])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_fast_integration_matrix_and_mixed_solution(fg, ctx, order, tc, monkeypatch):
    """FG_FAST_INTEGRATION element matrices -- float-float (FG_TC_INTEGRATION=0) or, by default,
    the tensor-core product: entries within 1e-12 of the row scale of the FP64-pipe
    integration (the reference-parity one), pattern identical, and the mixed solve on them
    within 1e-9 of the FP64 drop-in's solution."""
    n = (5, 4, 6)
    xyz = perturbed_vertices(n, 0.15, seed=21)
    k = np.exp(np.random.default_rng(2).normal(size=n[0] * n[1] * n[2]))
    tri = fg.SerialTriangulation(ctx, n, vertex_xyz=xyz)
    sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=list(range(1, 27)))
    sols, mats = [], []
    for fast in (False, True):
        monkeypatch.setenv("FG_TC_INTEGRATION", tc if fast else "0")
        op = fg.FEAffineOperator(sp, fg.PoissonIntegration(cell_coef=k, source_fn=O.FN_CONST, fn_param=[1.0],
                                                           fast_integration=fast)).compute()
        mats.append(op.get_matrix())
        s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
        s.set_parameters_from_pl({"ILS_RTOL": 1e-12, "ILS_MAX_NUM_ITERATIONS": 50000,
                                  "PRECISION": "mixed" if fast else "fp64"})
        sols.append(s.solve())
        op.close()
    (irp, ja, v64), (irp2, ja2, vff) = mats
    assert np.array_equal(irp, irp2) and np.array_equal(ja, ja2)
    rows = np.repeat(np.arange(len(irp) - 1), np.diff(irp))
    scale = np.zeros(len(irp) - 1)
    np.maximum.at(scale, rows, np.abs(v64))
    assert (np.abs(vff - v64) / scale[rows]).max() <= 1e-12
    assert np.linalg.norm(sols[1] - sols[0]) <= 1e-9 * np.linalg.norm(sols[0])


def test_plain_method_32_q1_sharp_wave(fg, ctx):
    """The reference's CPU-runnable case at its size: Poisson on the unit cube, 32^3 Q1, the
    sharp circular wave u = atan(50(|x - c| - 0.7)), c = (-0.05, -0.05, -0.05), as Dirichlet
    data and source, unpreconditioned CG to 1e-8 from x0 = 0.  Numbering, pattern, entries,
    iteration count (+-1) and solution against the oracle."""
    n = (32, 32, 32)
    P, tri, sp, op = build_pair(fg, ctx, n, 1, source_fn=O.FN_SHARP_WAVE, boundary_fn=O.FN_SHARP_WAVE,
                                fn_param=SHARP)
    assert sp.num_free_dofs == P.nfree == 29791
    assert np.array_equal(sp.get_dof_map(), P.dof_map())
    irp, ja, val = op.get_matrix()
    assert_matrix_close(irp, ja, val, P)
    b, ob = op.get_translation(), P.rhs()
    assert np.max(np.abs(b - ob)) <= RHS_TOL * np.max(np.abs(ob))
    ref = P.cg(precond=0, rtol=1e-8, maxit=100000)
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "identity")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-8, "ILS_MAX_NUM_ITERATIONS": 100000})
    x = s.solve()
    assert s.info()["converged"]
    assert abs(s.info()["iterations"] - ref["iters"]) <= 1, (s.info()["iterations"], ref["iters"])
    assert np.linalg.norm(x - ref["x"]) <= 1e-9 * np.linalg.norm(ref["x"])

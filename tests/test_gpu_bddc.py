"""Device BDDC (fg_bddc_* through the C-ABI) against the CPU BDDC restatement.

Bar:
  * apply in FP64: ||z_gpu - z_oracle|| <= 1e-10 ||z_oracle|| (same operator, different
    elimination order: the oracle solves the augmented saddle-point matrix directly);
  * apply with the FP32 factors: <= 1e-4;
  * BDDC-PCG: iteration count within 1 of the oracle's, solution within 1e-9 of the
    oracle's Jacobi-PCG solution at rtol 1e-12;
  * mixed-precision BDDC-PCG (FP32 factors, FP64 Krylov vectors): to 1e-8 converged, error
    <= 1e-7; to 1e-12 within 1e-9 of the oracle's solution, like the FP64 solve (the FP32
    preconditioner costs iterations, not attainable accuracy).
"""
import numpy as np
import pytest

import oracle as O
from bddc import HANDLER_ELASTICITY, WEIGHT_MULTIPLICITY, WEIGHT_STIFFNESS, BDDCOracle

pytestmark = pytest.mark.gpu

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


def perturbed(n, frac, seed):
    rng = np.random.default_rng(seed)
    h = [1.0 / n[0], 1.0 / n[1], 1.0 / n[2]]
    K, J, I = np.meshgrid(np.arange(n[2] + 1), np.arange(n[1] + 1), np.arange(n[0] + 1), indexing="ij")
    I, J, K = I.ravel(), J.ravel(), K.ravel()
    xyz = np.stack([I * h[0], J * h[1], K * h[2]], axis=1)
    interior = (I > 0) & (I < n[0]) & (J > 0) & (J < n[1]) & (K > 0) & (K < n[2])
    xyz[interior] += (rng.uniform(-frac, frac, size=xyz.shape) * np.array(h))[interior]
    return xyz.ravel()


def pair(fg, ctx, n, order, kind, ids, seed=3):
    xyz = perturbed(n, 0.15, seed)
    rng = np.random.default_rng(seed)
    coef = np.exp(rng.normal(0.0, 1.5 if kind == O.ELASTICITY else 1.0, size=n[0] * n[1] * n[2]))
    fp = [0.0, 0.0, -1.0] if kind == O.ELASTICITY else [1.0]
    P = O.Problem(n, order=order, kind=kind, dirichlet_ids=ids, vertex_xyz=xyz, cell_coef=coef, nu=0.3,
                  source_fn=O.FN_CONST, fn_param=fp)
    tri = fg.SerialTriangulation(ctx, n, vertex_xyz=xyz)
    ncomp = 3 if kind == O.ELASTICITY else 1
    sp = fg.SerialFESpace(tri, order=order, ncomp=ncomp, dirichlet_ids=ids)
    integ = (fg.ElasticityIntegration(cell_coef=coef, nu=0.3, source_fn=O.FN_CONST, fn_param=fp)
             if kind == O.ELASTICITY else fg.PoissonIntegration(cell_coef=coef, source_fn=O.FN_CONST, fn_param=fp))
    op = fg.FEAffineOperator(sp, integ).compute()
    return P, (tri, sp), op, ncomp


CASES = [
    # n, order, kind, dirichlet, nsub, jitter, faces, weighting
    ((6, 5, 4), 1, O.POISSON, "all", (3, 2, 2), 0.0, False, WEIGHT_MULTIPLICITY),
    ((6, 6, 4), 2, O.POISSON, "clamp", (3, 2, 2), 0.3, True, WEIGHT_STIFFNESS),
    ((5, 4, 4), 2, O.POISSON, "all", (2, 2, 2), 0.0, False, WEIGHT_STIFFNESS),
    ((6, 4, 4), 1, O.ELASTICITY, "clamp", (3, 2, 2), 0.2, True, WEIGHT_MULTIPLICITY),
    ((4, 4, 4), 2, O.ELASTICITY, "clamp", (2, 2, 2), 0.0, False, WEIGHT_MULTIPLICITY),
]


def ids_of(name):
    return list(range(1, 27)) if name == "all" else CLAMP


@pytest.mark.parametrize("case", CASES)
def test_bddc_apply_matches_oracle(fg, ctx, case):
    import torch
    n, order, kind, ids, nsub, jitter, faces, wt = case
    P, keep, op, ncomp = pair(fg, ctx, n, order, kind, ids_of(ids))
    cuts = fg.bddc_cuts(n, nsub, jitter=jitter, seed=7)
    Bo = BDDCOracle(P, n, order, ncomp, cuts, use_faces=faces, weighting=wt)
    M = fg.MLBDDC(op, nsub=nsub, cuts=cuts, use_faces=faces, weighting=wt)
    info = M.info()
    assert info["num_subdomains"] == nsub[0] * nsub[1] * nsub[2]
    assert info["num_coarse_dofs"] == Bo.ncoarse
    rng = np.random.default_rng(11)
    dev = f"cuda:{ctx.device}"
    for k in range(2):
        r = rng.normal(size=P.nfree)
        zo = Bo.apply(r)
        rt = torch.tensor(r, device=dev)
        z = torch.zeros_like(rt)
        M.apply_device(rt, z)
        err = np.linalg.norm(z.cpu().numpy() - zo) / np.linalg.norm(zo)
        assert err <= 1e-10, err
        z32 = torch.zeros_like(rt)
        M.apply_device(rt, z32, precision=fg.FG_MIXED)
        err32 = np.linalg.norm(z32.cpu().numpy() - zo) / np.linalg.norm(zo)
        assert err32 <= 1e-4, err32
    # run to run: bitwise identical
    z2 = torch.zeros_like(rt)
    M.apply_device(rt, z2)
    assert torch.equal(z, z2)
    M.close()


@pytest.mark.parametrize("case", [CASES[1], CASES[3], CASES[4]])
def test_bddc_pcg_matches_oracle(fg, ctx, case):
    n, order, kind, ids, nsub, jitter, faces, wt = case
    P, keep, op, ncomp = pair(fg, ctx, n, order, kind, ids_of(ids))
    cuts = fg.bddc_cuts(n, nsub, jitter=jitter, seed=7)
    Bo = BDDCOracle(P, n, order, ncomp, cuts, use_faces=faces, weighting=wt)
    xo, ito, oko = Bo.pcg(P, P.rhs(), rtol=1e-12, maxit=1000)
    ref = P.cg(precond=1, rtol=1e-13, maxit=100000)
    M = fg.MLBDDC(op, nsub=nsub, cuts=cuts, use_faces=faces, weighting=wt)
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, M)
    s.set_parameters_from_pl({"ILS_RTOL": 1e-12, "ILS_MAX_NUM_ITERATIONS": 1000})
    x = s.solve()
    inf = s.info()
    assert inf["converged"] and oko
    assert abs(inf["iterations"] - ito) <= 1, (inf["iterations"], ito)
    assert np.linalg.norm(x - ref["x"]) <= 1e-9 * np.linalg.norm(ref["x"])
    # mixed: FP32 preconditioner, FP64 Krylov vectors, to 1e-8
    sm = fg.IterativeLinearSolver().set_type_from_string("GPU_MPCG").set_operators(op, M)
    sm.set_parameters_from_pl({"ILS_RTOL": 1e-8, "ILS_MAX_NUM_ITERATIONS": 1000})
    xm = sm.solve()
    assert sm.info()["converged"]
    assert sm.info()["iterations"] <= inf["iterations"] + 2
    assert np.linalg.norm(xm - ref["x"]) <= 1e-7 * np.linalg.norm(ref["x"])
    sm.set_parameters_from_pl({"ILS_RTOL": 1e-12, "ILS_MAX_NUM_ITERATIONS": 2000})
    xm12 = sm.solve()
    assert sm.info()["converged"]
    assert np.linalg.norm(xm12 - ref["x"]) <= 1e-9 * np.linalg.norm(ref["x"])
    M.close()


RIGID_CASES = [
    # n, order, nsub, jitter, weighting (elasticity, clamped at x = 0)
    ((6, 4, 4), 1, (3, 2, 2), 0.2, WEIGHT_MULTIPLICITY),
    ((4, 4, 4), 2, (2, 2, 2), 0.0, WEIGHT_STIFFNESS),
    ((6, 5, 4), 2, (3, 2, 2), 0.3, WEIGHT_STIFFNESS),
]


@pytest.mark.parametrize("case", RIGID_CASES)
def test_bddc_elasticity_handler_matches_oracle(fg, ctx, case):
    """The elasticity coarse handler: rigid-body face functionals whose rows reach the
    faces' edge and vertex dofs (C_eV != 0 in the device's elimination)."""
    import torch
    n, order, nsub, jitter, wt = case
    P, keep, op, ncomp = pair(fg, ctx, n, order, O.ELASTICITY, CLAMP)
    cuts = fg.bddc_cuts(n, nsub, jitter=jitter, seed=7)
    Bo = BDDCOracle(P, n, order, 3, cuts, use_edges=False, use_faces=True, weighting=wt,
                    coarse_handler=HANDLER_ELASTICITY, vertex_xyz=perturbed(n, 0.15, 3))
    M = fg.MLBDDC(op, nsub=nsub, cuts=cuts, use_edges=False, use_faces=True, weighting=wt,
                  coarse_handler=fg.FG_BDDC_HANDLER_ELASTICITY)
    assert M.info()["num_coarse_dofs"] == Bo.ncoarse
    rng = np.random.default_rng(11)
    dev = f"cuda:{ctx.device}"
    for k in range(2):
        r = rng.normal(size=P.nfree)
        zo = Bo.apply(r)
        rt = torch.tensor(r, device=dev)
        z = torch.zeros_like(rt)
        M.apply_device(rt, z)
        assert np.linalg.norm(z.cpu().numpy() - zo) <= 1e-10 * np.linalg.norm(zo)
        # FP32 factors (the device takes the rotations about each face's centroid, scaled by
        # the face size: the same span as the oracle's rows in the raw coordinates, and a
        # well-conditioned S_e in FP32)
        z32 = torch.zeros_like(rt)
        M.apply_device(rt, z32, precision=fg.FG_MIXED)
        assert np.linalg.norm(z32.cpu().numpy() - zo) <= 1e-4 * np.linalg.norm(zo)
    # iteration counts: within 2 at 1e-10 (the two sides' applies differ by rounding, ~1e-12,
    # which moves the count of these 30-60 iteration solves by one or two)
    xo, ito, oko = Bo.pcg(P, P.rhs(), rtol=1e-10, maxit=1000)
    ref = P.cg(precond=1, rtol=1e-13, maxit=100000)
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, M)
    s.set_parameters_from_pl({"ILS_RTOL": 1e-10, "ILS_MAX_NUM_ITERATIONS": 1000})
    x = s.solve()
    assert s.info()["converged"] and oko
    assert abs(s.info()["iterations"] - ito) <= 2, (s.info()["iterations"], ito)
    assert np.linalg.norm(x - ref["x"]) <= 1e-7 * np.linalg.norm(ref["x"])
    # mixed: FP32 preconditioner, FP64 Krylov vectors, to 1e-8
    sm = fg.IterativeLinearSolver().set_type_from_string("GPU_MPCG").set_operators(op, M)
    sm.set_parameters_from_pl({"ILS_RTOL": 1e-8, "ILS_MAX_NUM_ITERATIONS": 1000})
    xm = sm.solve()
    assert sm.info()["converged"]
    assert np.linalg.norm(xm - ref["x"]) <= 1e-6 * np.linalg.norm(ref["x"])
    # to 1e-12 the FP32 preconditioner reaches the FP64 solution
    sm.set_parameters_from_pl({"ILS_RTOL": 1e-12, "ILS_MAX_NUM_ITERATIONS": 2000})
    xm12 = sm.solve()
    assert sm.info()["converged"]
    assert np.linalg.norm(xm12 - ref["x"]) <= 1e-9 * np.linalg.norm(ref["x"])
    M.close()


NOVERTEX_CASES = [
    # n, order, kind, dirichlet, nsub, jitter, edges, faces, weighting, handler: no primal
    # vertices (the reference test's coarse_space_use_vertices = .false.); the centre
    # subdomains of the first case touch no Dirichlet boundary (floating)
    ((6, 6, 6), 1, O.POISSON, "all", (3, 3, 3), 0.0, True, True, WEIGHT_STIFFNESS, 0),
    ((6, 5, 4), 2, O.POISSON, "all", (3, 2, 2), 0.3, False, True, WEIGHT_MULTIPLICITY, 0),
    ((6, 4, 4), 1, O.ELASTICITY, "clamp", (3, 2, 2), 0.2, True, True, WEIGHT_STIFFNESS, 0),
    ((6, 4, 4), 2, O.ELASTICITY, "clamp", (3, 2, 2), 0.0, False, True, WEIGHT_STIFFNESS, 1),
]


@pytest.mark.parametrize("case", NOVERTEX_CASES)
def test_bddc_without_primal_vertices_matches_oracle(fg, ctx, case):
    """use_vertices = 0: the device adds the constraints to the local matrices as an augmented
    Lagrangian (the same constrained Neumann solutions); the oracle solves the saddle-point
    systems directly.  Same coarse space, applies within 1e-10 (FP32 factors: 1e-4), PCG
    iteration counts within 2 at 1e-10, solutions within 1e-9 of the oracle's Jacobi-PCG."""
    import torch
    n, order, kind, ids, nsub, jitter, edges, faces, wt, handler = case
    P, keep, op, ncomp = pair(fg, ctx, n, order, kind, ids_of(ids))
    cuts = fg.bddc_cuts(n, nsub, jitter=jitter, seed=7)
    Bo = BDDCOracle(P, n, order, ncomp, cuts, use_vertices=False, use_edges=edges, use_faces=faces, weighting=wt,
                    coarse_handler=HANDLER_ELASTICITY if handler else 0,
                    vertex_xyz=perturbed(n, 0.15, 3) if handler else None)
    M = fg.MLBDDC(op, nsub=nsub, cuts=cuts, use_vertices=False, use_edges=edges, use_faces=faces, weighting=wt,
                  coarse_handler=fg.FG_BDDC_HANDLER_ELASTICITY if handler else fg.FG_BDDC_HANDLER_STANDARD)
    assert M.info()["num_coarse_dofs"] == Bo.ncoarse
    rng = np.random.default_rng(5)
    dev = f"cuda:{ctx.device}"
    for k in range(2):
        r = rng.normal(size=P.nfree)
        zo = Bo.apply(r)
        rt = torch.tensor(r, device=dev)
        z = torch.zeros_like(rt)
        M.apply_device(rt, z)
        err = np.linalg.norm(z.cpu().numpy() - zo) / np.linalg.norm(zo)
        assert err <= 1e-10, err
        z32 = torch.zeros_like(rt)
        M.apply_device(rt, z32, precision=fg.FG_MIXED)
        assert np.linalg.norm(z32.cpu().numpy() - zo) <= 1e-4 * np.linalg.norm(zo)
    xo, ito, oko = Bo.pcg(P, P.rhs(), rtol=1e-10, maxit=1000)
    ref = P.cg(precond=1, rtol=1e-13, maxit=100000)
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, M)
    s.set_parameters_from_pl({"ILS_RTOL": 1e-12, "ILS_MAX_NUM_ITERATIONS": 1000})
    x = s.solve()
    assert s.info()["converged"] and oko
    s.set_parameters_from_pl({"ILS_RTOL": 1e-10, "ILS_MAX_NUM_ITERATIONS": 1000})
    s.solve()
    assert abs(s.info()["iterations"] - ito) <= 2, (s.info()["iterations"], ito)
    assert np.linalg.norm(x - ref["x"]) <= 1e-9 * np.linalg.norm(ref["x"])
    M.close()


def test_bddc_elasticity_handler_rejects(fg, ctx):
    from fempar_gb300 import FGError
    P, keep, op, ncomp = pair(fg, ctx, (4, 4, 4), 1, O.ELASTICITY, CLAMP)
    with pytest.raises(FGError):  # the reference's handler asserts no edge constraints
        fg.MLBDDC(op, nsub=(2, 2, 2), use_edges=True, use_faces=True, coarse_handler=fg.FG_BDDC_HANDLER_ELASTICITY)
    P, keep, op, ncomp = pair(fg, ctx, (4, 4, 4), 1, O.POISSON, CLAMP)
    with pytest.raises(FGError):  # rigid-body modes need three components
        fg.MLBDDC(op, nsub=(2, 2, 2), use_edges=False, use_faces=True, coarse_handler=fg.FG_BDDC_HANDLER_ELASTICITY)


def test_bddc_criteria_follow_cg(fg, ctx):
    n, order, kind, ids, nsub, jitter, faces, wt = CASES[0]
    P, keep, op, ncomp = pair(fg, ctx, n, order, kind, ids_of(ids))
    M = fg.MLBDDC(op, nsub=nsub)
    for crit in ("RES_RES", "RES_RHS", "DELTA_RHS", "DELTA_DELTA", "RES_NRMGIVEN_RHS_NRMGIVEN",
                 "RES_NRMGIVEN_RES_NRMGIVEN"):
        s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, M)
        s.set_parameters_from_pl({"ILS_RTOL": 1e-9, "ILS_STOPPING_CRITERIUM": crit})
        s.solve()
        assert s.info()["converged"], crit
        assert s.info()["error_estimate"] <= s.info()["tolerance"]


def test_bddc_reassembly_refreshes_numerical_setup(fg, ctx):
    """Doubling the coefficient doubles A: after numerical_setup M^-1 halves."""
    import torch
    tri = fg.SerialTriangulation(ctx, (4, 4, 4), vertex_xyz=perturbed((4, 4, 4), 0.15, 5))
    sp = fg.SerialFESpace(tri, order=2, dirichlet_ids=CLAMP)
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(coef_const=1.0, source_fn=O.FN_CONST, fn_param=[1.0]))
    op.compute()
    M = fg.MLBDDC(op, nsub=(2, 2, 2))
    r = torch.tensor(np.random.default_rng(3).normal(size=sp.num_free_dofs), device=f"cuda:{ctx.device}")
    z1 = torch.zeros_like(r)
    M.apply_device(r, z1)
    op.integration = fg.PoissonIntegration(coef_const=2.0, source_fn=O.FN_CONST, fn_param=[1.0])
    op.compute()
    M.numerical_setup()
    z2 = torch.zeros_like(r)
    M.apply_device(r, z2)
    assert torch.allclose(z2, 0.5 * z1, rtol=1e-12, atol=1e-14 * float(z1.abs().max()))


def test_bddc_rejects_bad_parameters(fg, ctx):
    from fempar_gb300 import FGError
    P, keep, op, ncomp = pair(fg, ctx, (4, 4, 2), 1, O.POISSON, list(range(1, 27)))
    with pytest.raises(FGError):  # no coarse constraints at all
        fg.MLBDDC(op, nsub=(2, 2, 2), use_vertices=False, use_edges=False, use_faces=False)
    with pytest.raises(FGError):
        fg.MLBDDC(op, nsub=(5, 1, 1))
    with pytest.raises(FGError):
        fg.MLBDDC(op, nsub=(2, 1, 1), cuts=[[0, 3, 3], [0, 4], [0, 2]])


@pytest.mark.parametrize("order", [1, 2])
def test_subparts_with_one_material_reduce_to_the_box_objects(fg, ctx, order):
    """With one material the subparts are the subdomains: the physics-based partition's face
    objects are the box faces and its weights the multiplicities, so the preconditioner equals
    the faces-only one with multiplicity weights (same coarse space, applies equal to 1e-12)."""
    import torch
    n = (6, 4, 4)
    tri = fg.SerialTriangulation(ctx, n, vertex_xyz=perturbed(n, 0.15, 3))
    sp = fg.SerialFESpace(tri, order=order, ncomp=3, dirichlet_ids=CLAMP)
    op = fg.FEAffineOperator(sp, fg.ElasticityIntegration(coef_const=2.5, nu=0.3, source_fn=fg.FG_FN_CONST,
                                                          fn_param=[0.0, 0.0, -1.0])).compute()
    cuts = fg.bddc_cuts(n, (3, 2, 2), jitter=0.2, seed=7)
    common = dict(nsub=(3, 2, 2), cuts=cuts, use_vertices=False, use_edges=False, use_faces=True,
                  coarse_handler=fg.FG_BDDC_HANDLER_ELASTICITY)
    Mp = fg.MLBDDC(op, weighting=fg.FG_BDDC_WEIGHT_SUBPART, use_subparts=True, **common)
    Mb = fg.MLBDDC(op, weighting=fg.FG_BDDC_WEIGHT_MULTIPLICITY, **common)
    assert Mp.info()["num_coarse_dofs"] == Mb.info()["num_coarse_dofs"]
    r = torch.randn(sp.num_free_dofs, dtype=torch.float64, device=f"cuda:{ctx.device}")
    zp, zb = torch.zeros_like(r), torch.zeros_like(r)
    Mp.apply_device(r, zp)
    Mb.apply_device(r, zb)
    assert float((zp - zb).norm() / zb.norm()) <= 1e-12
    Mp.close()
    Mb.close()

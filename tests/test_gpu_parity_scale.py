"""GPU path against the oracle at real sizes, on the benchmark's own input distributions.

Poisson (the headline workload's distribution at 40^3 instead of 128^3): unit cube, Q2,
interior vertices perturbed U(-0.15h, 0.15h) per component, k = exp(N(0,1)) per cell, f = 1,
u = 0 on the whole boundary, Jacobi-PCG from x0 = 0 (inputs from bench.workload, the
generator of the benchmark).  Elasticity (the 3D elasticity configuration's integrand): 16^3
Q2, E = exp(N(0,1.5)) per cell, nu = 0.3, clamped at x = 0, body force (0,0,-1).

Bar:
  * dof numbering, CSR row pointers and column indices: bit-exact;
  * matrix entries within 1e-13 of their row's largest entry; rhs within 1e-13 of its largest;
  * FP64 solutions, both sides to rtol 1e-13: within 1e-10 (relative 2-norm);
  * the benchmark's two arms at rtol 1e-8 (FP64 drop-in; mixed precision on the float-float
    element matrices) against the oracle's solution at rtol 1e-13: within 1e-8.
The oracle assembles on all host threads (the same CSR, bit for bit, as its serial
restatement) and its PCG sums in thread order (results equal to the serial ones to rounding).
"""
import os

import numpy as np
import pytest

import oracle as O
from bench import workload

pytestmark = pytest.mark.gpu

MAT_TOL = 1e-13
RHS_TOL = 1e-13
SOL_TOL = 1e-10
ARM_TOL = 1e-8
CLAMP = [1, 3, 5, 7, 13, 15, 17, 19, 25]
THREADS = max(1, len(os.sched_getaffinity(0)))


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


def assert_system_matches(op, P):
    irp, ja, val = op.get_matrix()
    oirp, oja, oval = P.csr_upper()
    assert np.array_equal(irp, oirp), "row pointers differ"
    assert np.array_equal(ja, oja), "column indices differ"
    rows = np.repeat(np.arange(P.nfree), np.diff(oirp))
    scale = np.zeros(P.nfree)
    np.maximum.at(scale, rows, np.abs(oval))
    err = (np.abs(val - oval) / scale[rows]).max()
    assert err <= MAT_TOL, err
    b, ob = op.get_translation(), P.rhs()
    assert np.abs(b - ob).max() <= RHS_TOL * np.abs(ob).max()


def solve(fg, op, rtol, precision):
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": rtol, "ILS_MAX_NUM_ITERATIONS": 200000, "PRECISION": precision})
    x = s.solve()
    assert s.info()["converged"], (precision, rtol)
    return x, s.info()


def rel(x, ref):
    return float(np.linalg.norm(x - ref) / np.linalg.norm(ref))


def test_poisson_q2_perturbed_lognormal_40(fg, ctx):
    n = 40
    xyz, coef = workload(n)
    P = O.Problem((n, n, n), order=2, vertex_xyz=xyz, cell_coef=coef, source_fn=O.FN_CONST, fn_param=[1.0],
                  nthreads=THREADS)
    tri = fg.SerialTriangulation(ctx, (n, n, n), vertex_xyz=xyz)
    sp = fg.SerialFESpace(tri, order=2, dirichlet_ids=fg.ALL_BOUNDARY_IDS)
    assert np.array_equal(sp.get_dof_map(), P.dof_map()), "dof map differs"
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(cell_coef=coef, source_fn=fg.FG_FN_CONST,
                                                       fn_param=[1.0])).compute()
    assert_system_matches(op, P)
    ref = P.cg(precond=1, rtol=1e-13, maxit=200000, nthreads=THREADS)
    assert ref["converged"]
    x13, _ = solve(fg, op, 1e-13, "fp64")
    assert rel(x13, ref["x"]) <= SOL_TOL
    # the benchmark's arms: FP64 drop-in and mixed precision (float-float element matrices)
    x64, i64 = solve(fg, op, 1e-8, "fp64")
    fast = fg.FEAffineOperator(sp, fg.PoissonIntegration(cell_coef=coef, source_fn=fg.FG_FN_CONST, fn_param=[1.0],
                                                         fast_integration=True)).compute()
    xmx, imx = solve(fg, fast, 1e-8, "mixed")
    e64, emx = rel(x64, ref["x"]), rel(xmx, ref["x"])
    print(f"40^3 Q2 Poisson: FP64 {i64['iterations']} its err {e64:.2e}; mixed {imx['iterations']} its err {emx:.2e}")
    assert e64 <= ARM_TOL and emx <= ARM_TOL, (e64, emx)


def test_elasticity_q2_lognormal_clamped_16(fg, ctx):
    n = 16
    rng = np.random.Generator(np.random.PCG64(20261204))
    E = np.exp(rng.normal(0.0, 1.5, size=n ** 3))
    P = O.Problem((n, n, n), order=2, kind=O.ELASTICITY, dirichlet_ids=CLAMP, cell_coef=E, nu=0.3,
                  source_fn=O.FN_CONST, fn_param=[0.0, 0.0, -1.0], nthreads=THREADS)
    tri = fg.SerialTriangulation(ctx, (n, n, n))
    sp = fg.SerialFESpace(tri, order=2, ncomp=3, dirichlet_ids=CLAMP)
    assert np.array_equal(sp.get_dof_map(), P.dof_map()), "dof map differs"
    op = fg.FEAffineOperator(sp, fg.ElasticityIntegration(cell_coef=E, nu=0.3, source_fn=fg.FG_FN_CONST,
                                                          fn_param=[0.0, 0.0, -1.0])).compute()
    assert_system_matches(op, P)
    ref = P.cg(precond=1, rtol=1e-13, maxit=400000, nthreads=THREADS)
    assert ref["converged"]
    x13, _ = solve(fg, op, 1e-13, "fp64")
    assert rel(x13, ref["x"]) <= SOL_TOL
    x64, i64 = solve(fg, op, 1e-8, "fp64")
    xmx, imx = solve(fg, op, 1e-8, "mixed")
    e64, emx = rel(x64, ref["x"]), rel(xmx, ref["x"])
    print(f"16^3 Q2 elasticity: FP64 {i64['iterations']} its err {e64:.2e}; mixed {imx['iterations']} its err {emx:.2e}")
    assert e64 <= ARM_TOL and emx <= ARM_TOL, (e64, emx)

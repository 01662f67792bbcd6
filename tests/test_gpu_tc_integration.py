"""Poisson element matrices on the tensor cores against the FP64-pipe integration kernel.

The tensor-core path computes all cells' element matrices as one product G T^T, with FP64
emulated by digit slicing on tcgen05.  T (upper pairs x 6 NQ) holds the reference-gradient
products; G holds each cell's |det J| w k J^-1 J^-T entries per Gauss point.
FG_TC_INTEGRATION selects it: 0 off, 1 for FP64 integration, 2 (default) also for
float-float requests.  The oracle parity tests (`test_gpu_parity.py`) run it by default.

Checks here:

* Assembled CSR values: within K 2^-52 (K = 6 NQ, the FP64 dot-product bound of the
  contraction: 1.1e-14 for Q1, 3.6e-14 for Q2, 8.5e-14 for Q3) of each row's largest entry
  of the FP64-pipe kernel's (FG_TC_INTEGRATION=0).  Measured 2.0e-15 for Q2, 1.2e-14 for
  Q3.  The right-hand side (source part and the strong-Dirichlet lifting through the
  unpacked element matrices) meets the same bar against its largest entry.  Q1-Q3,
  perturbed vertices, lognormal coefficients, sharp-wave Dirichlet data.
* Fast-integration requests compute the geometric factors G in float-float on the FP32
  pipe.  Their matrices must be within 1e-12 of the FP64-pipe kernel's, the float-float
  kernel's bar.  The mixed-precision solve on them reaches the FP64 drop-in's solution
  to 1e-9.
* A bounded wait of the product that runs out (test switch) makes the assembly return
  FG_ERR_TIMEOUT; the next assembly on the same context is correct.
* Where the context's HBM budget has no room for the product's scratch, the assembly runs
  the FP64-pipe kernel instead: same matrix bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHARP = [50.0, 0.7, -0.05, -0.05, -0.05]


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
    h = np.array([1.0 / n[0], 1.0 / n[1], 1.0 / n[2]])
    K, J, I = np.meshgrid(np.arange(n[2] + 1), np.arange(n[1] + 1), np.arange(n[0] + 1), indexing="ij")
    I, J, K = I.ravel(), J.ravel(), K.ravel()
    xyz = np.stack([I * h[0], J * h[1], K * h[2]], axis=1)
    inner = (I > 0) & (I < n[0]) & (J > 0) & (J < n[1]) & (K > 0) & (K < n[2])
    xyz[inner] += rng.uniform(-frac, frac, size=(inner.sum(), 3)) * h
    return xyz.ravel()


def operator(fg, ctx, n, order, seed=0, fast=False):
    xyz = perturbed(n, 0.15, seed)
    coef = np.exp(np.random.default_rng(seed + 1).normal(0.0, 1.0, size=n[0] * n[1] * n[2]))
    tri = fg.SerialTriangulation(ctx, n, vertex_xyz=xyz)
    sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=fg.ALL_BOUNDARY_IDS)
    integ = fg.PoissonIntegration(source_fn=fg.FG_FN_SHARP_WAVE, boundary_fn=fg.FG_FN_SHARP_WAVE, fn_param=SHARP,
                                  cell_coef=coef, fast_integration=fast)
    return tri, sp, fg.FEAffineOperator(sp, integ)


def matrix_rhs(op):
    irp, ja, val = op.get_matrix(symmetric_storage=False, one_based=False)
    return irp, ja, val, op.get_translation()


def assert_close(a, b, tol):
    irp, ja, val, rhs = a
    irp2, ja2, val2, rhs2 = b
    assert np.array_equal(irp, irp2) and np.array_equal(ja, ja2)
    rows = np.repeat(np.arange(len(irp) - 1), np.diff(irp))
    scale = np.zeros(len(irp) - 1)
    np.maximum.at(scale, rows, np.abs(val2))
    err = (np.abs(val - val2) / scale[rows]).max()
    assert err <= tol, err
    assert np.abs(rhs - rhs2).max() <= tol * np.abs(rhs2).max()


@pytest.mark.parametrize("n,order", [((14, 11, 9), 1), ((10, 9, 8), 2), ((6, 5, 7), 3)])
def test_tensor_core_element_matrices_match_fp64_pipe(fg, ctx, monkeypatch, n, order):
    tri, sp, op = operator(fg, ctx, n, order)
    monkeypatch.setenv("FG_TC_INTEGRATION", "0")
    ref = matrix_rhs(op.compute())
    monkeypatch.setenv("FG_TC_INTEGRATION", "1")
    tc = matrix_rhs(op.compute())
    assert_close(tc, ref, 6 * (order + 1) ** 3 * 2.0 ** -52)


@pytest.mark.parametrize("n,order", [((14, 11, 9), 1), ((10, 9, 8), 2), ((6, 5, 7), 3)])
def test_fast_requests_float_float_geometry(fg, ctx, monkeypatch, n, order):
    """Fast-integration requests run the geometric factors in float-float (FP32 pipe): matrix
    and right-hand side within 1e-12 of the FP64-pipe kernel's (the float-float integration
    kernel's bar; measured ~1e-14)."""
    tri, sp, op = operator(fg, ctx, n, order)
    monkeypatch.setenv("FG_TC_INTEGRATION", "0")
    ref = matrix_rhs(op.compute())
    _, _, op2 = operator(fg, ctx, n, order, fast=True)
    monkeypatch.setenv("FG_TC_INTEGRATION", "2")
    ff = matrix_rhs(op2.compute())
    assert_close(ff, ref, 1e-12)


def test_mixed_solve_on_tensor_core_element_matrices(fg, ctx, monkeypatch):
    tri, sp, op = operator(fg, ctx, (16, 14, 12), 2, seed=4)
    monkeypatch.setenv("FG_TC_INTEGRATION", "0")
    op.compute()
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-12, "ILS_MAX_NUM_ITERATIONS": 20000, "PRECISION": "fp64"})
    x64 = s.solve()
    _, _, op2 = operator(fg, ctx, (16, 14, 12), 2, seed=4, fast=True)
    monkeypatch.setenv("FG_TC_INTEGRATION", "2")
    op2.compute()
    s2 = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op2, "jacobi")
    s2.set_parameters_from_pl({"ILS_RTOL": 1e-12, "ILS_MAX_NUM_ITERATIONS": 20000, "PRECISION": "mixed"})
    xm = s2.solve()
    assert s2.info()["converged"]
    assert np.linalg.norm(xm - x64) <= 1e-9 * np.linalg.norm(x64)


def test_bounded_wait_runs_out_in_the_assembly(fg, ctx, monkeypatch):
    from fempar_gb300 import FGError
    tri, sp, op = operator(fg, ctx, (12, 10, 8), 2, seed=9)
    monkeypatch.setenv("FG_TC_INTEGRATION", "0")
    ref = matrix_rhs(op.compute())
    monkeypatch.setenv("FG_TC_INTEGRATION", "1")
    monkeypatch.setenv("FG_OZ_TEST_DROP_STAGE", "2")
    with pytest.raises(FGError) as ei:
        op.compute()
    assert "FG_ERR_TIMEOUT" in str(ei.value)
    monkeypatch.delenv("FG_OZ_TEST_DROP_STAGE")
    assert_close(matrix_rhs(op.compute()), ref, 6 * 27 * 2.0 ** -52)


def test_budget_without_room_for_the_product_falls_back(fg, ctx, monkeypatch):
    n = (12, 10, 8)
    monkeypatch.setenv("FG_TC_INTEGRATION", "0")
    ca = fg.Context(0)
    _, _, opa = operator(fg, ca, n, 2, seed=5)
    ref = matrix_rhs(opa.compute())
    used_direct = ca.memory()[0]
    monkeypatch.setenv("FG_TC_INTEGRATION", "2")
    opa.compute()
    assert ca.memory()[0] - used_direct > 4 << 20   # the product's scratch is held by the system
    cb = fg.Context(0, hbm_budget_bytes=used_direct + (2 << 20))
    _, _, opb = operator(fg, cb, n, 2, seed=5)
    got = matrix_rhs(opb.compute())
    assert np.array_equal(got[2], ref[2]) and np.array_equal(got[3], ref[3])
    assert cb.memory()[0] <= used_direct + (2 << 20)

"""fg_system_spmv_device_noalloc, the SpMV entry point for callers that cannot allocate
device memory (a serving loop whose HBM is reserved up front, a host framework whose
caching allocator owns the device memory).

Called through the C-ABI and checked against fg_system_spmv_device on the same system,
on two calls in a row with different inputs, with the tolerances of test_gpu_parity.py
(FP64: 1e-13 of the largest entry; the FP32 copy: 1e-5): Poisson Q2 and elasticity Q2 on
the lattice-implicit solver layout, Poisson Q2 on the explicit-column SELL layout.  Also
checks that the calls leave the library's device allocations unchanged and the caller's
current device as it was, that a system without free dofs returns FG_OK, and that a
system larger than the FG_NOALLOC_SCRATCH_BYTES staging array is refused with
FG_ERR_BADARG.  This file is collected last, so a run that stops at the first failure has
run everything else first.
"""
import os
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-13
FP32_TOL = 1e-5


@pytest.fixture(scope="module")
def fg():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fempar_gb300 as fg
    from fempar_gb300 import build
    build.build()
    return fg


def _system(fg, ctx, n, order, kind="poisson", layout=None, dirichlet_ids=None):
    rng = np.random.default_rng(4)
    coef = np.exp(rng.normal(0.0, 1.0, size=n[0] * n[1] * n[2]))
    old = os.environ.pop("FG_SOLVER_LAYOUT", None)
    if layout:
        os.environ["FG_SOLVER_LAYOUT"] = layout
    try:
        tri = fg.SerialTriangulation(ctx, n)
        ids = fg.CLAMP_X0_IDS if dirichlet_ids is None else dirichlet_ids
        if kind == "elasticity":
            sp = fg.SerialFESpace(tri, order=order, ncomp=3, dirichlet_ids=ids)
            integ = fg.ElasticityIntegration(cell_coef=coef, nu=0.3, source_fn=fg.FG_FN_CONST,
                                             fn_param=[0.0, 0.0, -1.0])
        else:
            sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=ids)
            integ = fg.PoissonIntegration(cell_coef=coef, source_fn=fg.FG_FN_CONST, fn_param=[1.0])
    finally:
        os.environ.pop("FG_SOLVER_LAYOUT", None)
        if old is not None:
            os.environ["FG_SOLVER_LAYOUT"] = old
    op = fg.FEAffineOperator(sp, integ)
    return tri, sp, op.compute()


CASES = [((9, 7, 8), 2, "poisson", None, 0), ((5, 4, 6), 2, "elasticity", None, 0), ((7, 6, 5), 2, "poisson", "sell", 1)]


@pytest.mark.parametrize("n,order,kind,layout,want_layout", CASES, ids=["poisson_q2", "elasticity_q2", "poisson_q2_sell"])
def test_noalloc_spmv_matches_spmv_device(fg, n, order, kind, layout, want_layout):
    import torch
    from fempar_gb300 import _lib as L
    lib = L.lib()
    ctx = fg.Context(0)
    tri, sp, op = _system(fg, ctx, n, order, kind, layout)
    assert sp.info.solver_layout == want_layout
    n = sp.num_free_dofs
    gen = torch.Generator(device="cuda").manual_seed(11)
    for prec, dt, tol in ((L.FG_FP64, torch.float64, FP64_TOL), (L.FG_MIXED, torch.float32, FP32_TOL)):
        for call in range(2):
            x = torch.randn(n, dtype=dt, device="cuda", generator=gen)
            y = torch.full_like(x, float("nan"))
            used0 = ctx.memory()[0]
            torch_alloc0 = torch.cuda.memory_allocated()
            dev0 = torch.cuda.current_device()
            st = lib.fg_system_spmv_device_noalloc(op.h, prec, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()))
            assert st == L.FG_OK, lib.fg_last_error()
            assert torch.cuda.current_device() == dev0
            assert ctx.memory()[0] == used0, "the no-allocation SpMV allocated device memory"
            assert torch.cuda.memory_allocated() == torch_alloc0
            y_ref = torch.empty_like(x)
            op.apply_device(x, y_ref, prec)
            scale = y_ref.abs().max().item()
            err = (y - y_ref).abs().max().item()
            assert np.isfinite(err) and err <= tol * scale, (prec, call, err, scale)


def test_noalloc_spmv_without_free_dofs(fg):
    import torch
    from fempar_gb300 import _lib as L
    lib = L.lib()
    ctx = fg.Context(0)
    # Q1 on a 1x1x1 mesh with every boundary set Dirichlet: no free dofs
    tri, sp, op = _system(fg, ctx, (1, 1, 1), 1, dirichlet_ids=fg.ALL_BOUNDARY_IDS)
    assert sp.num_free_dofs == 0
    x = torch.zeros(1, dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    for prec in (L.FG_FP64, L.FG_MIXED):
        st = lib.fg_system_spmv_device_noalloc(op.h, prec, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()))
        assert st == L.FG_OK, lib.fg_last_error()


def test_noalloc_spmv_rejects_oversize(fg):
    import torch
    from fempar_gb300 import _lib as L
    lib = L.lib()
    ctx = fg.Context(0)
    # 64^3 Q2: padded lattice of 133^3 = 2,352,637 entries > 2,097,152 FP64 entries
    tri, sp, op = _system(fg, ctx, (64, 64, 64), 2)
    if sp.info.solver_vec_len <= 2_097_152:
        pytest.skip("solver layout smaller than the scratch limit")
    n = sp.num_free_dofs
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    st = lib.fg_system_spmv_device_noalloc(op.h, L.FG_FP64, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()))
    assert st == -1, st  # FG_ERR_BADARG
    assert b"no-allocation scratch" in lib.fg_last_error()

"""The row gather that writes the lattice-implicit solver layout directly (structured 3D
continuous spaces; the CSR values are derived from that layout only when exported).

* Reassembly with new coefficients: the exported matrix and the solution of the reassembled
  system equal a fresh assembly's bit for bit (the CSR view is rebuilt after every numeric
  phase), for Poisson Q1-Q3 and elasticity Q1-Q2.
* The same operator as the CSR route: the explicit-column SELL layout (assembled through
  the CSR) and the direct lattice-implicit layout give the same exported matrix, bit for
  bit, and FP64 solutions within 1e-12.
"""

import numpy as np
import pytest

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


def integration(fg, kind, coef):
    if kind == "elasticity":
        return fg.ElasticityIntegration(cell_coef=coef, nu=0.3, source_fn=fg.FG_FN_CONST, fn_param=[0.0, 0.0, -1.0])
    return fg.PoissonIntegration(cell_coef=coef, source_fn=fg.FG_FN_CONST, fn_param=[1.0])


def space(fg, ctx, n, order, kind):
    tri = fg.SerialTriangulation(ctx, n)
    if kind == "elasticity":
        return tri, fg.SerialFESpace(tri, order=order, ncomp=3, dirichlet_ids=CLAMP)
    return tri, fg.SerialFESpace(tri, order=order, dirichlet_ids=fg.ALL_BOUNDARY_IDS)


def solve(fg, op):
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-12, "ILS_MAX_NUM_ITERATIONS": 50000})
    return s.solve()


@pytest.mark.parametrize("order,kind", [(1, "poisson"), (2, "poisson"), (3, "poisson"), (1, "elasticity"),
                                        (2, "elasticity")])
def test_reassembly_rebuilds_the_exported_matrix(fg, ctx, order, kind):
    n = (5, 4, 6)
    rng = np.random.default_rng(order)
    k1, k2 = np.exp(rng.normal(size=(2, n[0] * n[1] * n[2])))
    tri, sp = space(fg, ctx, n, order, kind)
    op = fg.FEAffineOperator(sp, integration(fg, kind, k1)).compute()
    m1 = op.get_matrix()
    op.integration = integration(fg, kind, k2)
    op.compute()
    m2 = op.get_matrix()
    x2 = solve(fg, op)
    fresh = fg.FEAffineOperator(sp, integration(fg, kind, k2)).compute()
    mf = fresh.get_matrix()
    xf = solve(fg, fresh)
    for a, b in zip(m2, mf):
        assert np.array_equal(a, b)
    assert not np.array_equal(m1[2], m2[2])
    assert np.array_equal(x2, xf)


@pytest.mark.parametrize("order,kind", [(2, "poisson"), (3, "poisson"), (2, "elasticity")])
def test_direct_layout_equals_csr_route(fg, ctx, order, kind, monkeypatch):
    n = (4, 5, 3)
    coef = np.exp(np.random.default_rng(7).normal(size=n[0] * n[1] * n[2]))
    out = {}
    for layout in ("stencil", "sell"):
        if layout == "sell":
            monkeypatch.setenv("FG_SOLVER_LAYOUT", "sell")
        else:
            monkeypatch.delenv("FG_SOLVER_LAYOUT", raising=False)
        tri, sp = space(fg, ctx, n, order, kind)
        assert sp.info.solver_layout == (1 if layout == "sell" else 0)
        op = fg.FEAffineOperator(sp, integration(fg, kind, coef)).compute()
        out[layout] = (op.get_matrix(), solve(fg, op), op.get_translation())
    (ms, xs, bs), (mc, xc, bc) = out["stencil"], out["sell"]
    for a, b in zip(ms, mc):
        assert np.array_equal(a, b)
    assert np.array_equal(bs, bc)
    assert np.linalg.norm(xs - xc) <= 1e-12 * np.linalg.norm(xc)

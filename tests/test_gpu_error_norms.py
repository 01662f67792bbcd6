"""Device error norms (fg_system_error_norms) against the oracle's restatement of
error_norms_scalar_t (same solution vector on both sides, so only the norm evaluation is
compared): every norm within 1e-12 relative; per-cell squared energy errors sum to the
energy norm; h-refinement rates of a smooth exact solution."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

SHARP = [50.0, 0.7, -0.05, -0.05, -0.05]
SMOOTH = [2.0, 0.5, -0.05, -0.05, -0.05]


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


def solve(fg, ctx, n, order, fn, prm, xyz=None):
    tri = fg.SerialTriangulation(ctx, n, vertex_xyz=xyz)
    sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=list(range(1, 27)))
    src = fg.FG_FN_SHARP_WAVE if fn == fg.FG_FN_SHARP_WAVE else fg.FG_FN_ZERO
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(source_fn=src, boundary_fn=fn, fn_param=prm)).compute()
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-12, "ILS_MAX_NUM_ITERATIONS": 100000})
    return (tri, sp), op, s.solve()


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("fn", ["sharp", "linear"])
def test_error_norms_match_oracle(fg, ctx, order, fn):
    n = (4, 3, 5)
    xyz = perturbed(n, 0.15, 3)
    f = fg.FG_FN_SHARP_WAVE if fn == "sharp" else fg.FG_FN_LINEAR
    prm = SHARP if fn == "sharp" else []
    keep, op, x = solve(fg, ctx, n, order, f, prm, xyz)
    d, cells = op.error_norms(x, f, prm, cell_sq_energy=True)
    P = O.Problem(n, order=order, vertex_xyz=xyz, source_fn=O.FN_SHARP_WAVE if fn == "sharp" else O.FN_ZERO,
                  boundary_fn=O.FN_SHARP_WAVE if fn == "sharp" else O.FN_LINEAR, fn_param=prm)
    o = P.error_norms(x, O.FN_SHARP_WAVE if fn == "sharp" else O.FN_LINEAR, prm)
    scale = max(o["h1_norm"], 1e-300)
    # absolute floor: for u = x + y + z the error is the solver's (~1e-11), and a pointwise
    # gradient error is a difference of O(1) values that two summation orders reproduce to
    # ~nd u max|grad u| (nd <= 64 dofs, |grad u| = sqrt(3)): ~1e-14-1e-13
    floor = 1e-13 if fn == "linear" else 1e-14
    for k, v in o.items():
        ref = scale if k in ("mean_norm",) else max(abs(v), 1e-14 * scale)
        assert abs(d[k] - v) <= 1e-12 * max(abs(ref), 1e-30) + floor, (k, d[k], v)
    assert abs(np.sqrt(cells.sum()) - d["energy_norm"]) <= 1e-12 * max(d["energy_norm"], 1e-30)
    assert abs(d["energy_norm"] - d["h1_seminorm"]) <= 1e-12 * max(d["h1_seminorm"], 1e-30)
    if fn == "linear":  # u = x + y + z lies in the space: the error is the solver's
        assert d["h1_norm"] <= 1e-9


@pytest.mark.parametrize("order", [1, 2])
def test_error_norm_rates_under_refinement(fg, ctx, order):
    errs = []
    for n in (6, 12):
        keep, op, x = solve(fg, ctx, (n, n, n), order, fg.FG_FN_SHARP_WAVE, SMOOTH)
        errs.append(op.error_norms(x, fg.FG_FN_SHARP_WAVE, SMOOTH))
    l2_rate = np.log2(errs[0]["l2_norm"] / errs[1]["l2_norm"])
    h1_rate = np.log2(errs[0]["h1_seminorm"] / errs[1]["h1_seminorm"])
    assert l2_rate > order + 0.7 and h1_rate > order - 0.3, (l2_rate, h1_rate)


def test_energy_norm_weights_the_coefficient(fg, ctx):
    tri = fg.SerialTriangulation(ctx, (3, 3, 3))
    sp = fg.SerialFESpace(tri, order=1, dirichlet_ids=list(range(1, 27)))
    k = np.linspace(0.5, 3.0, 27)
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(cell_coef=k, boundary_fn=fg.FG_FN_SHARP_WAVE,
                                                       fn_param=SHARP)).compute()
    x = np.zeros(sp.num_free_dofs)
    d, cells = op.error_norms(x, fg.FG_FN_SHARP_WAVE, SHARP, cell_sq_energy=True)
    d1 = op.error_norms(x, fg.FG_FN_SHARP_WAVE, SHARP)
    assert d["energy_norm"] == d1["energy_norm"]
    assert d["energy_norm"] != d["h1_seminorm"]

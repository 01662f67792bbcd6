"""Quadrature-point coordinates at the boundary (fg_space_get_qp_coords) and a user-defined
source evaluated there.

tutorial_01's integrate_galerkin evaluates its own source function at the physical quadrature
points of every cell (modules :107,124).  A caller of the C-ABI does the same with the
exported coordinates and passes the values as FG_FN_QP_VALUES:

* the coordinates equal the oracle's (cell_map quadrature points, sbm_cell_map.i90:673-686)
  within 1e-14 on a perturbed structured mesh and on the reference's GiD cube mesh, from the
  host and the device export;
* the sharp-wave source written here in numpy (f = -lap atan(alpha(|x-c| - r))), evaluated at
  those points, assembles the same right-hand side as the built-in FG_FN_SHARP_WAVE
  (1e-12 of the largest entry) and the same matrix (bit for bit).
"""
import numpy as np
import pytest

import gidmesh
import oracle as O

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


def sharp_wave_source(xyz, alpha, r, c):
    """-lap u for u = atan(alpha (rho - r)), rho = |x - c| (3D)."""
    d = xyz - np.asarray(c)
    rho = np.sqrt((d * d).sum(axis=-1))
    s = 1.0 + (alpha * (rho - r)) ** 2
    return 2.0 * alpha ** 3 * (rho - r) / s ** 2 - 2.0 * alpha / (rho * s)


def perturbed(n, seed):
    rng = np.random.default_rng(seed)
    I, J, K = np.meshgrid(*(np.arange(m + 1) for m in n), indexing="ij")
    I, J, K = (a.transpose(2, 1, 0).ravel() for a in (I, J, K))
    xyz = np.stack([I / n[0], J / n[1], K / n[2]], axis=1)
    inner = (I > 0) & (I < n[0]) & (J > 0) & (J < n[1]) & (K > 0) & (K < n[2])
    xyz[inner] += rng.uniform(-0.15, 0.15, size=(inner.sum(), 3)) / np.array(n)
    return xyz.ravel()


@pytest.mark.parametrize("order", [1, 2, 3])
def test_qp_coords_match_oracle_structured(fg, ctx, order):
    import torch
    n = (5, 4, 6)
    xyz = perturbed(n, order)
    P = O.Problem(n, order=order, vertex_xyz=xyz)
    tri = fg.SerialTriangulation(ctx, n, vertex_xyz=xyz)
    sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=fg.ALL_BOUNDARY_IDS)
    q = sp.get_qp_coords()
    assert q.shape == (P.ncells, P.nq, 3)
    assert np.abs(q - P.qp_coords()).max() <= 1e-14
    d = torch.empty(q.size, dtype=torch.float64, device="cuda")
    sp.get_qp_coords(out=d)
    assert np.abs(d.cpu().numpy().reshape(q.shape) - q).max() <= 1e-15


@pytest.mark.parametrize("order", [1, 2])
def test_qp_coords_match_oracle_gid(fg, ctx, order):
    m = gidmesh.reference_mesh("test_poisson")
    P = O.UProblem(m, order=order, dirichlet_ids=(1,))
    tri = fg.SerialTriangulation.from_arrays(ctx, m["coords"], m["cells"], m["bvef_ptr"], m["bvef_verts"],
                                             m["bvef_set"])
    sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=[1])
    assert np.abs(sp.get_qp_coords() - P.qp_coords()).max() <= 1e-14


@pytest.mark.parametrize("order", [1, 2])
def test_user_source_at_qp_equals_builtin(fg, ctx, order):
    n = (6, 5, 4)
    xyz = perturbed(n, 10 + order)
    tri = fg.SerialTriangulation(ctx, n, vertex_xyz=xyz)
    sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=fg.ALL_BOUNDARY_IDS)
    f = sharp_wave_source(sp.get_qp_coords(), SHARP[0], SHARP[1], SHARP[2:5]).ravel()
    user = fg.FEAffineOperator(sp, fg.PoissonIntegration(source_fn=fg.FG_FN_QP_VALUES, qp_source=f,
                                                         boundary_fn=fg.FG_FN_SHARP_WAVE, fn_param=SHARP)).compute()
    builtin = fg.FEAffineOperator(sp, fg.PoissonIntegration(source_fn=fg.FG_FN_SHARP_WAVE,
                                                            boundary_fn=fg.FG_FN_SHARP_WAVE,
                                                            fn_param=SHARP)).compute()
    bu, bb = user.get_translation(), builtin.get_translation()
    assert np.abs(bu - bb).max() <= 1e-12 * np.abs(bb).max()
    for a, b in zip(user.get_matrix(), builtin.get_matrix()):
        assert np.array_equal(a, b)

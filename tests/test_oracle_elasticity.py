"""The oracle's linear-elasticity integrand on the CPU, pinned by properties of the exact
stiffness operator (sbm_irreducible_discrete_integration.i90:100-121 restated in
oracle/fempar_oracle.cpp): with no Dirichlet dofs the assembled matrix has the rigid-body
modes in its null space, and a uniform strain (linear displacement) leaves only boundary
rows nonzero (the interior rows of K u are the discrete equilibrium of a constant stress).
Meshes are affine images of the unit box, so node coordinates are the affine map of the
lattice and every Q_p space holds linear fields exactly."""
import numpy as np
import pytest

import oracle as O

AFFINE3 = np.array([[1.0, 0.2, 0.1], [0.05, 0.9, 0.15], [0.1, -0.1, 1.1]])
SHIFT3 = np.array([0.3, -0.2, 0.5])
AFFINE2 = np.array([[1.0, 0.3], [-0.2, 0.8]])
SHIFT2 = np.array([0.1, 0.4])


def vertices(n, dim):
    if dim == 3:
        K, J, I = np.meshgrid(np.arange(n[2] + 1), np.arange(n[1] + 1), np.arange(n[0] + 1), indexing="ij")
        ref = np.stack([I.ravel() / n[0], J.ravel() / n[1], K.ravel() / n[2]], 1)
        return ref @ AFFINE3.T + SHIFT3
    J, I = np.meshgrid(np.arange(n[1] + 1), np.arange(n[0] + 1), indexing="ij")
    ref = np.stack([I.ravel() / n[0], J.ravel() / n[1]], 1)
    xy = ref @ AFFINE2.T + SHIFT2
    return np.concatenate([xy, np.zeros((xy.shape[0], 1))], 1)


def dof_positions(P, n, order, dim):
    """Physical node coordinates and component of every free dof (affine meshes)."""
    dm = P.dof_map()
    np1 = order + 1
    nn = np1 ** dim
    xs = np.zeros((P.nfree, dim))
    comp = np.zeros(P.nfree, dtype=int)
    interior = np.zeros(P.nfree, dtype=bool)
    for c in range(P.ncells):
        ci = [c % n[0], (c // n[0]) % n[1], c // (n[0] * n[1])][:dim]
        for loc in range(dm.shape[1]):
            g = dm[c, loc]
            if g <= 0:
                continue
            a, cc = loc % nn, loc // nn
            ai = [a % np1, (a // np1) % np1, a // (np1 * np1)][:dim]
            lat = np.array([(order * ci[d] + ai[d]) / (order * n[d]) for d in range(dim)])
            xs[g - 1] = lat @ (AFFINE3 if dim == 3 else AFFINE2).T + (SHIFT3 if dim == 3 else SHIFT2)
            comp[g - 1] = cc
            interior[g - 1] = all(0 < order * ci[d] + ai[d] < order * n[d] for d in range(dim))
    return xs, comp, interior


def rigid_modes(xs, comp, dim):
    modes = []
    for t in range(dim):
        modes.append((comp == t).astype(float))
    if dim == 2:
        modes.append(np.where(comp == 0, xs[:, 1], -xs[:, 0]))
    else:
        modes.append(np.where(comp == 0, xs[:, 1], np.where(comp == 1, -xs[:, 0], 0.0)))
        modes.append(np.where(comp == 0, -xs[:, 2], np.where(comp == 2, xs[:, 0], 0.0)))
        modes.append(np.where(comp == 1, xs[:, 2], np.where(comp == 2, -xs[:, 1], 0.0)))
    return modes


@pytest.mark.parametrize("dim,n", [(3, (2, 3, 2)), (2, (3, 4))])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_rigid_modes_are_in_the_null_space(dim, n, order):
    nv = int(np.prod([k + 1 for k in n]))
    P = O.Problem(n, order=order, num_dims=dim, kind=O.ELASTICITY, dirichlet_ids=[], nu=0.3,
                  vertex_xyz=vertices(n, dim).ravel(),
                  cell_coef=np.exp(np.random.default_rng(order).normal(size=int(np.prod(n)))))
    xs, comp, _ = dof_positions(P, n, order, dim)
    scale = np.abs(P.csr_full()[2]).max()
    for r in rigid_modes(xs, comp, dim):
        assert np.abs(P.spmv(r)).max() <= 1e-11 * scale * max(1.0, np.abs(r).max())
    assert nv > 0


@pytest.mark.parametrize("dim,n", [(3, (3, 3, 3)), (2, (4, 3))])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_uniform_strain_is_in_equilibrium_inside(dim, n, order):
    """u = B x with symmetric B: constant stress, zero divergence.  With one coefficient the
    interior rows of K u vanish; the boundary rows carry the tractions."""
    P = O.Problem(n, order=order, num_dims=dim, kind=O.ELASTICITY, dirichlet_ids=[], nu=0.3,
                  vertex_xyz=vertices(n, dim).ravel(), cell_coef=np.full(int(np.prod(n)), 2.5))
    xs, comp, interior = dof_positions(P, n, order, dim)
    B = np.array([[0.3, 0.1, -0.2], [0.1, -0.4, 0.05], [-0.2, 0.05, 0.2]])[:dim, :dim]
    u = np.einsum("ij,nj->ni", B, xs)[np.arange(P.nfree), comp]
    Ku = P.spmv(u)
    scale = np.abs(P.csr_full()[2]).max() * np.abs(u).max()
    assert np.abs(Ku[interior]).max() <= 1e-11 * scale
    assert np.abs(Ku[~interior]).max() > 1e-6 * scale   # the boundary carries the tractions


def test_reference_pb_bddc_problem_rhs_norm():
    """The rhs of the reference's physics-based BDDC test problem (channels with E jump 1e8,
    u = x+y+z on the boundary): 1e-6 ||b|| equals the tolerance the reference printed,
    3.708160389E+02, to its 10 significant digits."""
    import pb_elasticity_case as pb
    P = O.Problem(pb.N, order=1, kind=O.ELASTICITY, limits=list(pb.LIMITS), cell_coef=pb.cell_modulus(), nu=pb.NU,
                  source_fn=O.FN_ZERO, boundary_fn=O.FN_LINEAR, dirichlet_ids=list(range(1, 27)))
    tol = pb.RTOL * float(np.linalg.norm(P.rhs()))
    assert abs(tol - pb.TOLERANCE) <= 0.5e-7, tol

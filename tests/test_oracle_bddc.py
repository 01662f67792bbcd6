"""The CPU BDDC restatement (oracle/bddc.py) and the box-partition helper, no GPU.

The reference's own BDDC test (par_test_pb_bddc_linear_elasticity, 11 iterations) needs
MPI, a physics-based partition and PARDISO; it is not reproduced.  The oracle is checked
here on properties that any correct BDDC has: a symmetric positive definite operator, the
exact inverse when there is one subdomain, a CG iteration count well below Jacobi's, and
the same solution as the Jacobi-preconditioned CG of the oracle.
"""
import numpy as np
import pytest

import oracle as O
from bddc import WEIGHT_MULTIPLICITY, WEIGHT_STIFFNESS, BDDCOracle

CLAMP = [1, 3, 5, 7, 13, 15, 17, 19, 25]


def problem(n, order, kind, ids, seed=0):
    rng = np.random.default_rng(seed)
    coef = np.exp(rng.normal(0, 1, size=n[0] * n[1] * n[2]))
    return O.Problem(n, order=order, kind=kind, dirichlet_ids=ids, cell_coef=coef, source_fn=O.FN_CONST,
                     fn_param=[0, 0, -1] if kind == O.ELASTICITY else [1.0])


def even(n, nsub):
    return [np.array([(k * n[d]) // nsub[d] for k in range(nsub[d] + 1)]) for d in range(3)]


@pytest.mark.parametrize("case", [
    ((6, 5, 4), 1, O.POISSON, "all", (3, 2, 2), False, WEIGHT_MULTIPLICITY),
    ((4, 4, 3), 2, O.POISSON, "clamp", (2, 2, 1), True, WEIGHT_STIFFNESS),
    ((4, 3, 3), 1, O.ELASTICITY, "clamp", (2, 2, 2), False, WEIGHT_MULTIPLICITY),
])
def test_oracle_bddc_is_spd_and_beats_jacobi(case):
    n, order, kind, ids, nsub, faces, wt = case
    P = problem(n, order, kind, list(range(1, 27)) if ids == "all" else CLAMP)
    B = BDDCOracle(P, n, order, 3 if kind == O.ELASTICITY else 1, even(n, nsub), use_faces=faces, weighting=wt)
    rng = np.random.default_rng(1)
    u, v = rng.normal(size=P.nfree), rng.normal(size=P.nfree)
    Mu, Mv = B.apply(u), B.apply(v)
    assert abs(u @ Mv - v @ Mu) <= 1e-12 * abs(u @ Mv)
    assert u @ Mu > 0 and v @ Mv > 0
    x, it, ok = B.pcg(P, P.rhs(), rtol=1e-10, maxit=500)
    ref = P.cg(precond=1, rtol=1e-10, maxit=50000)
    assert ok and it < ref["iters"]
    assert np.linalg.norm(x - ref["x"]) <= 1e-7 * np.linalg.norm(ref["x"])


def test_oracle_bddc_single_subdomain_is_exact():
    n = (3, 3, 2)
    P = problem(n, 2, O.POISSON, list(range(1, 27)))
    B = BDDCOracle(P, n, 2, 1, even(n, (1, 1, 1)))
    x, it, ok = B.pcg(P, P.rhs(), rtol=1e-12, maxit=10)
    assert ok and it == 1


def test_bddc_cuts_partition_rules():
    from fempar_gb300.fe import bddc_cuts
    cuts = bddc_cuts((96, 96, 96), (8, 8, 8), jitter=0.08, seed=20261203)
    for c in cuts:
        assert c[0] == 0 and c[-1] == 96 and np.all(np.diff(c) >= 1)
    w = [np.diff(c) for c in cuts]
    counts = np.einsum("i,j,k->ijk", w[0], w[1], w[2])
    assert counts.min() >= 0.7 * 1728 and counts.max() <= 1.3 * 1728
    even_cuts = bddc_cuts((6, 6, 6), (3, 2, 1))
    assert [list(c) for c in even_cuts] == [[0, 2, 4, 6], [0, 3, 6], [0, 6]]


# ---------------------------------------------------------------------------------------
# Elasticity coarse handler (sbm_elasticity_coarse_fe_handler.i90): rigid-body face rows

@pytest.mark.parametrize("order", [1, 2])
def test_rigid_face_rows_reproduce_the_mode_gram_matrix(order):
    """On an undeformed mesh each face is a flat rectangle and the modes are linear, so
    C_face applied to the nodal interpolant of mode k is (1/|F|) int_F r_m . r_k exactly,
    computed here from the rectangle's moments."""
    from bddc import HANDLER_ELASTICITY, _rigid_modes
    n, nsub = (4, 4, 4), (2, 2, 2)
    P = problem(n, order, O.ELASTICITY, CLAMP)
    B = BDDCOracle(P, n, order, 3, even(n, nsub), use_faces=True, use_edges=False, coarse_handler=HANDLER_ELASTICITY)
    dm = P.dof_map()
    nn = (order + 1) ** 3
    # coordinates and component of every free dof
    xyz = np.zeros((P.nfree, 3))
    comp = np.zeros(P.nfree, dtype=int)
    for c in range(P.ncells):
        ci, cj, ck = c % n[0], (c // n[0]) % n[1], c // (n[0] * n[1])
        for loc in range(dm.shape[1]):
            g = dm[c, loc]
            if g <= 0:
                continue
            a, cc = loc % nn, loc // nn
            ai, aj, ak = a % (order + 1), (a // (order + 1)) % (order + 1), a // (order + 1) ** 2
            xyz[g - 1] = [(order * ci + ai) / (order * n[0]), (order * cj + aj) / (order * n[1]),
                          (order * ck + ak) / (order * n[2])]
            comp[g - 1] = cc
    inv = {v: k for k, v in B.coarse_index.items()}
    # subdomain 1 (x in [0.5, 1]): its face on the y cut plane touches no clamped node
    s = 1
    S = B.subs[s]
    key = next(inv[ci][0] for ci in S["cidx"] if inv[ci][0][0] == 2 and inv[ci][0][1] == 1)
    rows = [i for i, ci in enumerate(S["cidx"]) if inv[ci][0] == key]
    assert len(rows) == 6
    Cf = S["C"][rows]
    R = np.array([[_rigid_modes(xyz[g])[m, comp[g]] for g in S["gl"]] for m in range(6)])
    got = Cf @ R.T
    # face: y = 0.5, x in [0.5, 1], z in [0, 0.5]; monomial moments over the rectangle
    x0, x1, z0, z1, y = 0.5, 1.0, 0.0, 0.5, 0.5

    def mom(px, pz):
        return (x1 ** (px + 1) - x0 ** (px + 1)) / (px + 1) * (z1 ** (pz + 1) - z0 ** (pz + 1)) / (pz + 1)

    area = mom(0, 0)
    # r . r' for the six modes as polynomials in x, z at fixed y: evaluate with a tensor Gauss rule
    gx, gw = np.polynomial.legendre.leggauss(3)
    G = np.zeros((6, 6))
    for xs, wx in zip(gx, gw):
        for zs, wz in zip(gx, gw):
            X = np.array([x0 + (x1 - x0) * (xs + 1) / 2, y, z0 + (z1 - z0) * (zs + 1) / 2])
            Rm = _rigid_modes(X)
            G += wx * wz * (x1 - x0) * (z1 - z0) / 4 * (Rm @ Rm.T)
    assert np.allclose(got, G / area, rtol=1e-12, atol=1e-14)
    # translations: the rows of a component sum to one (partition of unity)
    for m in range(3):
        assert abs(Cf[m][comp[S["gl"]] == m].sum() - 1.0) < 1e-13


def test_elasticity_handler_spd_and_converges():
    from bddc import HANDLER_ELASTICITY
    n, nsub = (6, 4, 4), (3, 2, 2)
    P = problem(n, 2, O.ELASTICITY, CLAMP, seed=4)
    cuts = [np.array([0, 2, 3, 6]), np.array([0, 2, 4]), np.array([0, 1, 4])]
    B = BDDCOracle(P, n, 2, 3, cuts, use_faces=True, use_edges=False, coarse_handler=HANDLER_ELASTICITY,
                   weighting=WEIGHT_STIFFNESS)
    Bv = BDDCOracle(P, n, 2, 3, cuts, use_faces=False, use_edges=False, coarse_handler=HANDLER_ELASTICITY,
                    weighting=WEIGHT_STIFFNESS)
    rng = np.random.default_rng(1)
    u, v = rng.normal(size=P.nfree), rng.normal(size=P.nfree)
    Mu, Mv = B.apply(u), B.apply(v)
    assert abs(u @ Mv - v @ Mu) <= 1e-12 * abs(u @ Mv)
    assert u @ Mu > 0
    x, it, ok = B.pcg(P, P.rhs(), rtol=1e-10, maxit=500)
    xv, itv, okv = Bv.pcg(P, P.rhs(), rtol=1e-10, maxit=500)
    ref = P.cg(precond=1, rtol=1e-11, maxit=50000)
    assert ok and okv and it < itv < ref["iters"]
    assert np.linalg.norm(x - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    with pytest.raises(ValueError):
        BDDCOracle(P, n, 2, 3, cuts, use_faces=True, use_edges=True, coarse_handler=HANDLER_ELASTICITY)

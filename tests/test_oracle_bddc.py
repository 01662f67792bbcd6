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

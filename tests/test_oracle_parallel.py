"""The oracle's multi-threaded assembly and PCG (used to time the reference path and to solve
the full-size workload on the host) against its serial restatement of the reference.

Assembly: the CSR (row pointers, columns, values), rhs and COO entry count built by chunks of
cells on several threads equal the serial COO append + sort_and_compress's bit for bit
(Poisson Q1-Q3 on perturbed meshes, elasticity Q2).  PCG: the threaded symmetric-storage
SpMV and the full-CSR gather form give the serial iteration count (+-1) and solutions within
1e-12 (they sum in another order)."""
import numpy as np
import pytest

import oracle as O
from bench import workload


@pytest.mark.parametrize("n,order,kind", [(7, 1, O.POISSON), (6, 2, O.POISSON), (4, 3, O.POISSON),
                                          (4, 2, O.ELASTICITY)])
def test_threaded_assembly_is_bit_identical(n, order, kind):
    xyz, coef = workload(n, seed=5)
    kw = dict(order=order, kind=kind, vertex_xyz=xyz, cell_coef=coef, source_fn=O.FN_CONST,
              fn_param=[1.0, 0.5, -1.0], dirichlet_ids=[1, 3, 5, 7, 13, 15, 17, 19, 25])
    A = O.Problem((n, n, n), nthreads=1, **kw)
    B = O.Problem((n, n, n), nthreads=5, **kw)
    for a, b in zip(A.csr_upper(), B.csr_upper()):
        assert np.array_equal(a, b)
    assert np.array_equal(A.rhs(), B.rhs())
    assert A.coo_entries == B.coo_entries


@pytest.mark.parametrize("nth", [3, -3])
def test_threaded_pcg_matches_serial(nth):
    xyz, coef = workload(8, seed=6)
    P = O.Problem((8, 8, 8), order=2, vertex_xyz=xyz, cell_coef=coef, source_fn=O.FN_CONST, fn_param=[1.0])
    a = P.cg(precond=1, rtol=1e-12, maxit=10000)
    b = P.cg(precond=1, rtol=1e-12, maxit=10000, nthreads=nth, times=True, history=True)
    assert a["converged"] and b["converged"] and abs(a["iters"] - b["iters"]) <= 1
    assert np.linalg.norm(a["x"] - b["x"]) <= 1e-12 * np.linalg.norm(a["x"])
    assert np.all(np.diff(b["times"]) >= 0) and len(b["history"]) == b["iters"]

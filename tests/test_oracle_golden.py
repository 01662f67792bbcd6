"""The CPU oracle against the reference's own golden data (no GPU).

* Gauss-Legendre nodes/weights vs the table of test_quadratures.f90 (1e-10, as the
  reference checks itself).
* Energy-norm errors of the 2D CG tutorial vs the published convergence tables
  (uniform_mesh_error_order_{1,2,4,8}; written with 10 significant digits).
* Exact reproduction of a linear solution (test_poisson: u = x+y+z, f = 0, CG
  rtol 1e-12; the reference checks error norms < 1e-6).
"""
import json
import os

import numpy as np
import pytest

import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_gauss_legendre_table():
    d = json.load(open(os.path.join(GOLD, "gauss_legendre_table.json")))
    tol = d["tolerance"]
    for n, ref in d["table"].items():
        n = int(n)
        x, w = O.gauss_legendre(n)
        rx = np.array(ref["x"])
        rw = np.array(ref["w"])
        # the reference compares each tabulated node with both symmetric positions
        for i in range(n):
            errx = min(abs(rx[i] - x[i]), abs(rx[n - 1 - i] - x[i]))
            assert errx <= tol, (n, i)
        assert np.max(np.abs(np.sort(rw) - np.sort(w))) <= tol, n


@pytest.mark.parametrize("order,nrows", [(1, 3), (2, 2), (4, 1)])
def test_tutorial01_convergence_table(order, nrows):
    d = json.load(open(os.path.join(GOLD, "tutorial01_convergence.json")))
    rows = d["tables"][str(order)][:nrows]
    for sqrt_ndofs, err_ref in rows:
        # sqrt(#free dofs) = p*NX - 1 on an NX x NX mesh with the whole boundary Dirichlet
        nx = int(round((sqrt_ndofs + 1) / order))
        P = O.Problem([nx, nx], order=order, num_dims=2, source_fn=O.FN_SHARP_WAVE, boundary_fn=O.FN_SHARP_WAVE,
                      fn_param=[200.0, 0.7, -0.05, -0.05, -0.05])
        assert np.sqrt(P.nfree) == pytest.approx(sqrt_ndofs)
        r = P.cg(rtol=1e-14, maxit=200000)
        assert r["converged"]
        e = P.energy_error(r["x"])
        # the table holds 10 significant digits
        assert abs(e - err_ref) <= 6e-10 * err_ref, (order, nx, e, err_ref)


@pytest.mark.parametrize("order", [1, 2, 3])
def test_exact_linear_solution_3d(order):
    P = O.Problem([3, 4, 2], order=order, source_fn=O.FN_ZERO, boundary_fn=O.FN_LINEAR)
    r = P.cg(rtol=1e-12, maxit=5000)
    assert r["converged"]
    assert P.energy_error(r["x"]) < 1e-8


def test_csr_upper_layout_and_symmetry():
    P = O.Problem([3, 3, 3], order=2, source_fn=O.FN_CONST, fn_param=[1.0])
    irp, ja, val = P.csr_upper()
    assert irp[0] == 1 and irp[-1] == len(ja) + 1
    for r in range(P.nfree):
        cols = ja[irp[r] - 1: irp[r + 1] - 1]
        assert cols[0] == r + 1  # diagonal first (matvec_symmetric_storage relies on it)
        assert np.all(np.diff(cols) > 0)
    # symmetric-storage SpMV equals the full matrix product
    rp, ci, v = P.csr_full()
    x = np.random.default_rng(0).standard_normal(P.nfree)
    y_full = np.array([np.dot(v[rp[i]:rp[i + 1]], x[ci[rp[i]:rp[i + 1]]]) for i in range(P.nfree)])
    assert np.allclose(P.spmv(x), y_full, rtol=1e-12, atol=1e-12)


def test_dof_numbering_counts():
    # free dofs of a Q_p space on n^3 cells with the whole boundary Dirichlet: (p n - 1)^3
    for p, n in [(1, 4), (2, 3), (3, 2)]:
        P = O.Problem([n, n, n], order=p)
        assert P.nfree == (p * n - 1) ** 3
        assert P.ndir == (p * n + 1) ** 3 - (p * n - 1) ** 3
        m = P.dof_map()
        assert m.shape == (n ** 3, (p + 1) ** 3)
        free = m[m > 0]
        assert set(np.unique(free)) == set(range(1, P.nfree + 1))
        assert set(np.unique(-m[m < 0])) == set(range(1, P.ndir + 1))


def test_dirichlet_first_visit_order():
    # Dirichlet ids are numbered in (cell, vef) first-visit order: the first cell
    # (0,0,0) owns vertex 1, whose dof is -1.
    P = O.Problem([2, 2, 2], order=1)
    m = P.dof_map()
    assert m[0, 0] == -1
    # first free dof is the first interior vertex met in cell order: (1,1,1) is vertex 8 of cell 0
    assert m[0, 7] == 1


def test_elasticity_clamped_counts():
    clamp = [1, 3, 5, 7, 13, 15, 17, 19, 25]
    P = O.Problem([2, 2, 2], order=2, kind=O.ELASTICITY, dirichlet_ids=clamp, cell_coef=np.ones(8), nu=0.3,
                  source_fn=O.FN_CONST, fn_param=[0.0, 0.0, -1.0])
    # lattice 5^3 nodes, 25 on x=0 clamped, 3 components
    assert P.ndir == 25 * 3
    assert P.nfree == (125 - 25) * 3
    r = P.cg(precond=1, rtol=1e-10, maxit=5000)
    assert r["converged"]

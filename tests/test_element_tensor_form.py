"""The tensor form behind the tensor-core Poisson element matrices, checked on the CPU with numpy.

For a trilinear cell and the Poisson integrand k grad(phi_a) . grad(phi_b):

    E_ab = sum_q w_q |det J_q| k (J_q^-T r_a(q)) . (J_q^-T r_b(q))
         = sum_{q, m} T[ab][6q + m] G[6q + m],

where r_a(q) is the reference gradient of shape a at Gauss point q and
G[6q + m] = w_q |det J_q| k (J_q^-1 J_q^-T)_m, for m over the entries 00 11 22 01 02 12.
T[ab][6q + m] is r_a,j r_b,j on the diagonal m = jj and r_a,j r_b,k + r_a,k r_b,j off it.
This is the table the library builds once per space: the same for every cell.  Checked for
Q1-Q3 on randomly perturbed cells, to 1e-13 of the largest entry.
"""
import numpy as np
import pytest


def lagrange_1d(p, x):
    """Values and derivatives of the degree-p Lagrange basis on equispaced nodes of [-1, 1]."""
    nodes = np.linspace(-1.0, 1.0, p + 1)
    v = np.ones((p + 1, len(x)))
    d = np.zeros((p + 1, len(x)))
    for i in range(p + 1):
        others = [nodes[j] for j in range(p + 1) if j != i]
        den = np.prod([nodes[i] - o for o in others])
        v[i] = np.prod([x - o for o in others], axis=0) / den
        for skip in range(len(others)):
            d[i] += np.prod([x - o for j, o in enumerate(others) if j != skip], axis=0) / den
    return v, d


def reference_gradients(p, nq1):
    """r[a, q, :] for shapes a = i + (p+1)(j + (p+1)k) and Gauss points q likewise, weights w[q]."""
    x, w1 = np.polynomial.legendre.leggauss(nq1)
    v, d = lagrange_1d(p, x)
    n = p + 1
    r = np.zeros((n ** 3, nq1 ** 3, 3))
    w = np.zeros(nq1 ** 3)
    for qk in range(nq1):
        for qj in range(nq1):
            for qi in range(nq1):
                q = qi + nq1 * (qj + nq1 * qk)
                w[q] = w1[qi] * w1[qj] * w1[qk]
                for k in range(n):
                    for j in range(n):
                        for i in range(n):
                            a = i + n * (j + n * k)
                            r[a, q] = [d[i, qi] * v[j, qj] * v[k, qk], v[i, qi] * d[j, qj] * v[k, qk],
                                       v[i, qi] * v[j, qj] * d[k, qk]]
    return r, w, x


def jacobians(verts, nq1):
    """J[q][i][j] = dX_i/dxi_j of the trilinear map with vertices verts[8, 3] (x fastest)."""
    r1 = reference_gradients(1, nq1)[0]  # gradients of the 8 trilinear shapes
    return np.einsum("kqj,ki->qij", r1, verts)


@pytest.mark.parametrize("p", [1, 2, 3])
def test_element_matrix_equals_table_times_geometric_factors(p):
    rng = np.random.default_rng(p)
    nq1 = p + 1
    r, w, x = reference_gradients(p, nq1)
    verts = np.array([[i, j, k] for k in (0, 1) for j in (0, 1) for i in (0, 1)], dtype=float) * 0.1
    verts += rng.uniform(-0.02, 0.02, size=verts.shape)
    kc = np.exp(rng.normal())
    J = jacobians(verts, nq1)
    Jinv = np.linalg.inv(J)
    det = np.abs(np.linalg.det(J))
    # direct: physical gradients g = J^-T r
    g = np.einsum("qji,aqj->aqi", Jinv, r)
    E = np.einsum("q,aqi,bqi->ab", w * det * kc, g, g)
    # tensor form
    M = np.einsum("qjl,qkl->qjk", Jinv, Jinv) * (w * det * kc)[:, None, None]  # J^-1 J^-T
    jk = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
    G = np.array([[M[q, j, k] for (j, k) in jk] for q in range(len(w))]).ravel()
    nd = r.shape[0]
    T = []
    for a in range(nd):
        for b in range(a, nd):
            row = []
            for q in range(len(w)):
                ra, rb = r[a, q], r[b, q]
                row += [ra[0] * rb[0], ra[1] * rb[1], ra[2] * rb[2], ra[0] * rb[1] + ra[1] * rb[0],
                        ra[0] * rb[2] + ra[2] * rb[0], ra[1] * rb[2] + ra[2] * rb[1]]
            T.append(row)
    T = np.array(T)
    assert T.shape == (nd * (nd + 1) // 2, 6 * len(w))
    Ep = T @ G
    iu = np.triu_indices(nd)
    assert np.max(np.abs(Ep - E[iu])) <= 1e-13 * np.max(np.abs(E))

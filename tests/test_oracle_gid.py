"""The oracle's unstructured-mesh route (GiD reader, vef generation, boundary set ids, dof
numbering with own-dof permutations), pinned on the reference's own test meshes.

Pin: the reference's test_poisson runs its GiD cube meshes with orders 1-3, Dirichlet data
u = x+y+z on set 1, f = 0, and requires every error norm of the discrete solution below
1e-6 (Sources/Tests/Serial/test_poisson/modules/test_poisson_driver.f90:562-600,
Sources/Tests/Scripts/test_poisson:215-235).  The exact recovery needs the boundary set ids
handed from faces to their edges and vertices and conforming own-dof permutations, so the
same check on meshes with every cell orientation pins both.  Bar here: 1e-10.
"""

import numpy as np
import pytest

import gid
import gidmesh
import oracle as O

def ref_mesh(name):
    return gidmesh.reference_mesh(name)


def exact_linear_errors(mesh, order):
    P = O.UProblem(mesh, order=order, dirichlet_ids=(1,), source_fn=O.FN_ZERO, boundary_fn=O.FN_LINEAR)
    r = P.cg(precond=1, rtol=1e-14, maxit=20000)
    assert r["converged"]
    return P, P.error_norms(r["x"], O.FN_LINEAR)


@pytest.mark.parametrize("name", ["test_poisson", "par_test_poisson"])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_reference_meshes_recover_linear_solution(name, order):
    m = ref_mesh(name)
    P, e = exact_linear_errors(m, order)
    for k in ("mean_norm", "l1_norm", "l2_norm", "linfty_norm", "h1_seminorm", "w1infty_seminorm"):
        assert abs(e[k]) < 1e-10, (k, e[k])
    # a box of a x b x c hexahedra: Euler counts of its vefs
    nv = m["coords"].shape[0]
    assert P.nvefs == nv + P.nedges + P.nfaces
    assert nv - P.nedges + P.nfaces - P.ncells == 1


def test_reference_mesh_counts():
    m = ref_mesh("test_poisson")
    P = O.UProblem(m, order=1, dirichlet_ids=(1,), boundary_fn=O.FN_LINEAR)
    # 3 x 5 x 6 cells: 4*6*7 vertices, edges and faces of the box lattice
    assert (m["cells"].shape[0], m["coords"].shape[0]) == (90, 168)
    assert (P.nedges, P.nfaces) == (3 * 6 * 7 + 4 * 5 * 7 + 4 * 6 * 6, 4 * 5 * 6 + 3 * 6 * 6 + 3 * 5 * 7)
    # every boundary vertex is Dirichlet once the face sets reach their closure
    assert P.ndir == 168 - 2 * 4 * 5 and P.nfree == 2 * 4 * 5


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("seed", [0, 1])
def test_all_orientations_recover_linear_solution(order, seed):
    m = gidmesh.box_mesh((3, 4, 2), seed=seed, perturb=0.25, side_sets=False)
    _, e = exact_linear_errors(m, order)
    assert e["l2_norm"] < 1e-10 and e["h1_seminorm"] < 1e-10 and e["linfty_norm"] < 1e-10


def test_gid_writer_reader_round_trip(tmp_path):
    m = gidmesh.box_mesh((2, 3, 2), seed=4)
    for c_order in (True, False):
        p = tmp_path / f"box{int(c_order)}.mesh"
        gidmesh.write_gid(p, m, c_order=c_order)
        r = gid.read_gid(str(p))
        assert np.array_equal(r["cells"], m["cells"])
        assert np.allclose(r["coords"], m["coords"], rtol=0, atol=1e-15)
        for k in ("bvef_ptr", "bvef_verts", "bvef_set"):
            assert np.array_equal(r[k], m[k])


def test_vef_sets_cover_the_boundary_closure():
    m = gidmesh.box_mesh((3, 2, 4), seed=2)
    P = O.UProblem(m, order=2, dirichlet_ids=(1, 2, 3, 4, 5, 6, 7, 8), boundary_fn=O.FN_LINEAR)
    cv = P.cell_vefs() - 1
    sets = P.vef_sets()
    cnt = np.bincount(cv.ravel(), minlength=P.nvefs)
    nv = m["coords"].shape[0]
    faces = np.arange(nv + P.nedges, P.nvefs)
    bfaces = faces[cnt[faces] == 1]
    assert len(bfaces) == 2 * (3 * 2 + 2 * 4 + 3 * 4)
    assert np.all(sets[bfaces] > 0)
    # vertices and edges of boundary faces have sets; interior vefs have none
    on_bnd = np.zeros(P.nvefs, bool)
    codes = list(O.polytope_codes(3))
    for c in range(P.ncells):
        for f in range(20, 26):
            if cnt[cv[c, f]] == 1:
                on_bnd[cv[c, f]] = True
                a, t = codes[f] & 7, codes[f] >> 3
                verts = {a | s for s in range(8) if (s & ~t) == 0}
                for f2 in range(20):
                    a2, t2 = codes[f2] & 7, codes[f2] >> 3
                    if {a2 | s for s in range(8) if (s & ~t2) == 0} <= verts:
                        on_bnd[cv[c, f2]] = True
    assert np.all(sets[on_bnd] > 0) and np.all(sets[~on_bnd] == 0)
    # full Dirichlet boundary: the solution of the linear data is exact
    r = P.cg(precond=1, rtol=1e-14, maxit=20000)
    assert P.error_norms(r["x"], O.FN_LINEAR)["l2_norm"] < 1e-10


def test_unstructured_matches_structured_oracle_on_a_box():
    """Same box through both routes (cells in lattice order, lexicographic vertices): the
    vertex values of the sharp-wave solution agree."""
    n = (4, 3, 5)
    m = gidmesh.box_mesh(n, seed=0, perturb=0.0, shuffle=False, orient=False, side_sets=False)
    prm = (25.0, 0.3, -0.05, -0.05, -0.05)
    U = O.UProblem(m, order=1, dirichlet_ids=(1,), source_fn=O.FN_SHARP_WAVE, boundary_fn=O.FN_SHARP_WAVE,
                   fn_param=prm)
    S = O.Problem(n, order=1, source_fn=O.FN_SHARP_WAVE, boundary_fn=O.FN_SHARP_WAVE, fn_param=prm)
    xu = U.cg(precond=1, rtol=1e-14, maxit=20000)["x"]
    xs = S.cg(precond=1, rtol=1e-14, maxit=20000)["x"]
    assert U.nfree == S.nfree and U.ndir == S.ndir
    # both place vertex dofs at the lattice vertices: map through the coordinates
    du, ds = U.dof_map(), S.dof_map()
    cu = m["coords"][m["cells"] - 1]   # (nc, 8, 3)
    valu, vals = {}, {}
    for c in range(U.ncells):
        for a in range(8):
            key = tuple(np.round(cu[c, a], 12))
            if du[c, a] > 0:
                valu[key] = xu[du[c, a] - 1]
    L = np.array(n) + 1
    for c in range(S.ncells):
        i, j, k = c % n[0], (c // n[0]) % n[1], c // (n[0] * n[1])
        for a in range(8):
            v = np.array([i + (a & 1), j + ((a >> 1) & 1), k + ((a >> 2) & 1)]) / np.array(n)
            if ds[c, a] > 0:
                vals[tuple(np.round(v, 12))] = xs[ds[c, a] - 1]
    assert valu.keys() == vals.keys()
    d = max(abs(valu[k] - vals[k]) for k in valu)
    assert d < 1e-12 * max(abs(v) for v in vals.values())


@pytest.mark.parametrize("refine", [0, 1, 2])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_irregular_cube_in_cube_recovers_linear_solution(refine, order):
    """Vertices in 3, 4, 6 and 8 cells; shuffled cells in random orientations."""
    m = gidmesh.cube_in_cube(refine=refine, seed=refine + order)
    _, e = exact_linear_errors(m, order)
    assert e["l2_norm"] < 1e-10 and e["h1_seminorm"] < 1e-10 and e["linfty_norm"] < 1e-10

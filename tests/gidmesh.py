"""Seeded unstructured hexahedral test meshes and a writer of the GiD problem-type format.

Test helper: a box of n0 x n1 x n2 hexahedra whose vertices are relabelled at random, whose
interior vertices are moved (the trilinear map stays valid), whose cells come in random
order, each with its 8 vertices listed in one of the cube's 48 (or 24 proper) orientations,
and whose boundary is given as faces (set id per side), box edges and box corners -- the
shape of the reference's GiD test meshes.  Arrays use the keys of ``oracle.gid.read_gid``.
"""
from __future__ import annotations

import itertools
import json
import os

import numpy as np

GOLDEN_GID = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gid_cube_hexas.json")

PERMU_3DQ1 = (1, 2, 4, 3, 5, 6, 8, 7)


def cube_orientations(proper_only=False):
    """Maps new local vertex -> old local vertex (lexicographic bits) for the cube's symmetries."""
    out = []
    for perm in itertools.permutations(range(3)):
        inv = sum(1 for a in range(3) for b in range(a + 1, 3) if perm[a] > perm[b])
        for flips in range(8):
            det = (-1) ** inv * (-1) ** bin(flips).count("1")
            if proper_only and det < 0:
                continue
            m = []
            for b in range(8):
                old = 0
                for d in range(3):
                    old |= (((b >> d) & 1) ^ ((flips >> d) & 1)) << perm[d]
                m.append(old)
            out.append(m)
    return out


def box_mesh(n=(3, 4, 5), seed=0, perturb=0.2, shuffle=True, orient=True, proper_only=False,
             side_sets=True, limits=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)):
    rng = np.random.default_rng(seed)
    nx, ny, nz = n
    L = np.array([nx + 1, ny + 1, nz + 1])
    nv = int(np.prod(L))
    lat = np.arange(nv)
    I, J, K = lat % L[0], (lat // L[0]) % L[1], lat // (L[0] * L[1])
    ijk = np.stack([I, J, K], 1).astype(float)
    lo = np.array(limits[0::2], dtype=float)
    hi = np.array(limits[1::2], dtype=float)
    h = (hi - lo) / np.array(n, dtype=float)
    interior = (I > 0) & (I < nx) & (J > 0) & (J < ny) & (K > 0) & (K < nz)
    xyz = lo + ijk * h
    if perturb > 0:
        xyz[interior] += rng.uniform(-perturb, perturb, size=(int(interior.sum()), 3)) * h
    relabel = rng.permutation(nv) if shuffle else np.arange(nv)   # lattice vertex -> new id (0-based)
    coords = np.zeros((nv, 3))
    coords[relabel] = xyz
    orients = cube_orientations(proper_only)
    cells = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                base = [(i + (b & 1)) + L[0] * ((j + ((b >> 1) & 1)) + L[1] * (k + ((b >> 2) & 1))) for b in range(8)]
                m = orients[rng.integers(len(orients))] if orient else list(range(8))
                cells.append([relabel[base[m[b]]] + 1 for b in range(8)])
    cells = np.array(cells, dtype=np.int32)
    if shuffle:
        cells = cells[rng.permutation(len(cells))]

    def vid(i, j, k):
        return int(relabel[i + L[0] * (j + L[1] * k)]) + 1

    given = []  # (vertices, set)
    sides = [(0, 0), (0, nx), (1, 0), (1, ny), (2, 0), (2, nz)]
    for sid, (d, val) in enumerate(sides, start=1):
        a, b = [e for e in range(3) if e != d]
        for u in range(n[a]):
            for v in range(n[b]):
                quad = []
                for du, dv in ((0, 0), (1, 0), (1, 1), (0, 1)):
                    c = [0, 0, 0]
                    c[d], c[a], c[b] = val, u + du, v + dv
                    quad.append(vid(*c))
                r = rng.integers(4)
                given.append((quad[r:] + quad[:r], sid if side_sets else 1))
    for d in range(3):
        a, b = [e for e in range(3) if e != d]
        for va in (0, n[a]):
            for vb in (0, n[b]):
                for t in range(n[d]):
                    c0, c1 = [0, 0, 0], [0, 0, 0]
                    c0[a] = c1[a] = va
                    c0[b] = c1[b] = vb
                    c0[d], c1[d] = t, t + 1
                    e = [vid(*c0), vid(*c1)]
                    if rng.integers(2):
                        e = e[::-1]
                    given.append((e, 7 if side_sets else 1))
    for c in itertools.product((0, nx), (0, ny), (0, nz)):
        given.append(([vid(*c)], 8 if side_sets else 1))
    order = rng.permutation(len(given)) if shuffle else np.arange(len(given))
    given = [given[i] for i in order]
    bptr = np.zeros(len(given) + 1, dtype=np.int64)
    bptr[1:] = np.cumsum([len(g[0]) for g in given])
    return {"dim": 3, "coords": coords, "cells": cells, "cell_set": np.zeros(len(cells), np.int32),
            "cell_geo": np.ones(len(cells), np.int32), "bvef_ptr": bptr,
            "bvef_verts": np.array([v for g in given for v in g[0]], dtype=np.int32),
            "bvef_set": np.array([g[1] for g in given], dtype=np.int32),
            "bvef_geo": np.ones(len(given), np.int32)}


def write_gid(path, mesh, c_order=True):
    """Write a mesh in the GiD problem-type format (hexahedra in GiD's order when c_order)."""
    cells = np.asarray(mesh["cells"])
    if c_order:
        out = np.zeros_like(cells)
        for i, p in enumerate(PERMU_3DQ1):
            out[:, p - 1] = cells[:, i]
        cells = out
    nb = len(mesh["bvef_ptr"]) - 1
    lines = [f"MESH dimension  3  order  {0 if c_order else 1}  types  1  elements {len(cells):10d}"
             f"  vertices {len(mesh['coords']):10d}  vefs {nb:10d}", "coordinates"]
    for i, x in enumerate(mesh["coords"], start=1):
        lines.append(f"{i:11d} {x[0]:.16e} {x[1]:.16e} {x[2]:.16e}")
    lines += ["end coordinates", "elements"]
    for i, c in enumerate(cells, start=1):
        lines.append(f"{i:8d} {8:8d} " + " ".join(f"{v:8d}" for v in c) + f" {0:8d} {1:8d}")
    lines += ["end elements", "vefs"]
    bp, bv, bs = mesh["bvef_ptr"], mesh["bvef_verts"], mesh["bvef_set"]
    for i in range(nb):
        vs = bv[bp[i]:bp[i + 1]]
        lines.append(f"{i + 1:11d} {len(vs):8d} " + " ".join(f"{v:8d}" for v in vs) + f" {bs[i]:8d} {1:8d}")
    lines += ["end vefs", ""]
    with open(path, "w") as f:
        f.write("\n".join(lines))


def cube_in_cube(refine=0, inner=(0.3, 0.7), seed=None):
    """The classic irregular hexahedral mesh: an inner cube inside the unit cube joined to it
    by 6 frustum cells (inner corners lie in 4 cells, outer corners in 3), split `refine`
    times into 8 by the trilinear map of each cell.  Boundary: the outer faces, edges and
    corners with set id 1.  With `seed`, cells are shuffled and listed in random orientations."""
    lo, hi = inner
    verts = {}

    def vid(key, x):
        if key not in verts:
            verts[key] = (len(verts) + 1, np.array(x, dtype=float))
        return verts[key][0]

    def outer(b):
        return vid(("o",) + tuple(b), [float(v) for v in b])

    def inn(b):
        return vid(("i",) + tuple(b), [lo + (hi - lo) * v for v in b])

    cells = [[inn([(k >> 0) & 1, (k >> 1) & 1, (k >> 2) & 1]) for k in range(8)]]
    for d in range(3):
        for s in (0, 1):
            cell = []
            for k in range(8):
                b = [(k >> 0) & 1, (k >> 1) & 1, (k >> 2) & 1]
                layer_outer = (b[d] == 0) if s == 0 else (b[d] == 1)
                bb = list(b)
                bb[d] = s
                cell.append(outer(bb) if layer_outer else inn(bb))
            cells.append(cell)
    bfaces = []
    for d in range(3):
        a, c = [e for e in range(3) if e != d]
        for s in (0, 1):
            q = []
            for (u, v) in ((0, 0), (1, 0), (1, 1), (0, 1)):
                b = [0, 0, 0]
                b[d], b[a], b[c] = s, u, v
                q.append(outer(b))
            bfaces.append(q)
    bedges = []
    for d in range(3):
        a, c = [e for e in range(3) if e != d]
        for u in (0, 1):
            for v in (0, 1):
                b0, b1 = [0, 0, 0], [0, 0, 0]
                b0[a] = b1[a] = u
                b0[c] = b1[c] = v
                b1[d] = 1
                bedges.append([outer(b0), outer(b1)])
    bverts = [[outer([(k >> 0) & 1, (k >> 1) & 1, (k >> 2) & 1])] for k in range(8)]
    coords = {v[0]: v[1] for v in verts.values()}
    for _ in range(refine):
        newc = []
        mid = {}

        def key_mid(ids):
            return tuple(sorted(ids))

        def point(ids):
            k = key_mid(ids)
            if k not in mid:
                nid = len(coords) + 1
                coords[nid] = np.mean([coords[i] for i in ids], axis=0)
                mid[k] = nid
            return mid[k]

        for cell in cells:
            # trilinear points at parametric (0, 1/2, 1) per direction
            X = np.array([coords[v] for v in cell])

            def tri(t):
                w = [(1 - t[0], t[0]), (1 - t[1], t[1]), (1 - t[2], t[2])]
                return sum(w[0][k & 1] * w[1][(k >> 1) & 1] * w[2][(k >> 2) & 1] * X[k] for k in range(8))

            grid = {}
            for i in range(3):
                for j in range(3):
                    for k in range(3):
                        t = (i / 2, j / 2, k / 2)
                        # the vertices of the n-face holding the point name it, so cells that
                        # share an edge or face share its midpoint
                        span = [cell[b] for b in range(8)
                                if all(t[d] == 0.5 or ((b >> d) & 1) == int(t[d]) for d in range(3))]
                        if len(span) == 1:
                            grid[(i, j, k)] = span[0]
                        else:
                            nid = point(span)
                            coords[nid] = tri(t)
                            grid[(i, j, k)] = nid
            for ci in range(2):
                for cj in range(2):
                    for ck in range(2):
                        newc.append([grid[(ci + (b & 1), cj + ((b >> 1) & 1), ck + ((b >> 2) & 1))] for b in range(8)])
        nb = []
        for q in bfaces:
            e = [point([q[a], q[(a + 1) % 4]]) for a in range(4)]
            c = point(list(q))
            nb += [[q[0], e[0], c, e[3]], [e[0], q[1], e[1], c], [c, e[1], q[2], e[2]], [e[3], c, e[2], q[3]]]
        bfaces = nb
        ne = []
        for e in bedges:
            m = point(e)
            ne += [[e[0], m], [m, e[1]]]
        bedges = ne
        cells = newc
    coords_arr = np.array([coords[i] for i in range(1, len(coords) + 1)])
    cells = np.array(cells, dtype=np.int32)
    rng = np.random.default_rng(seed) if seed is not None else None
    if rng is not None:
        orients = cube_orientations()
        cells = np.array([[c[m] for m in orients[rng.integers(len(orients))]] for c in cells], dtype=np.int32)
        cells = cells[rng.permutation(len(cells))]
    given = [(q, 1) for q in bfaces] + [(e, 1) for e in bedges] + [(v, 1) for v in bverts]
    bptr = np.zeros(len(given) + 1, dtype=np.int64)
    bptr[1:] = np.cumsum([len(g[0]) for g in given])
    return {"dim": 3, "coords": coords_arr, "cells": cells, "cell_set": np.zeros(len(cells), np.int32),
            "cell_geo": np.ones(len(cells), np.int32), "bvef_ptr": bptr,
            "bvef_verts": np.array([v for g in given for v in g[0]], dtype=np.int32),
            "bvef_set": np.array([g[1] for g in given], dtype=np.int32),
            "bvef_geo": np.ones(len(given), np.int32)}


def reference_mesh(name):
    """The reference's cube_hexas GiD mesh of test `name` ("test_poisson" or "par_test_poisson"),
    as tests/golden/make_golden.py parsed it from
    Sources/Tests/Data/<name>/cube_hexas.gid/cube_hexas.mesh (keys of ``oracle.gid.read_gid``)."""
    m = json.load(open(GOLDEN_GID))["meshes"][name]
    types = {"coords": np.float64, "cells": np.int32, "cell_set": np.int32, "cell_geo": np.int32,
             "bvef_ptr": np.int64, "bvef_verts": np.int32, "bvef_set": np.int32, "bvef_geo": np.int32}
    return {"dim": m["dim"], **{k: np.asarray(m[k], dtype=t) for k, t in types.items()}}

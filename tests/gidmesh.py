"""Seeded unstructured hexahedral test meshes and a writer of the GiD problem-type format.

Test helper: a box of n0 x n1 x n2 hexahedra whose vertices are relabelled at random, whose
interior vertices are moved (the trilinear map stays valid), whose cells come in random
order, each with its 8 vertices listed in one of the cube's 48 (or 24 proper) orientations,
and whose boundary is given as faces (set id per side), box edges and box corners -- the
shape of the reference's GiD test meshes.  Arrays use the keys of ``oracle.gid.read_gid``.
"""
from __future__ import annotations

import itertools

import numpy as np

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

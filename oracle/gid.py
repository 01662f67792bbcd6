"""Reader of FEMPAR's GiD problem-type mesh files, restated for the oracle.

TEST INFRASTRUCTURE ONLY: the checker for the product reader (``fg_mesh_read_gid``).
Only tests/ import this module.

Follows ``Sources/Lib/Geometry/Mesh/mesh.f90:337-486``
(``read_fempar_gid_problem_type_format_file_unit``):

* header ``MESH dimension D order O types T elements NC vertices NV vefs NB``;
* ``coordinates`` ... ``end coordinates``: ``id x y [z]``;
* ``elements`` ... ``end elements``: ``id nnode v_1 .. v_nnode set geo``;
* ``vefs`` ... ``end vefs``: ``id nnodb v_1 .. v_nnodb set geo`` (the given boundary vefs);
* when the header's order is 0 ("c order", GiD's counter-clockwise vertex order) the vertices
  of every hexahedron are reordered to FEMPAR's lexicographic ("z") order by
  ``permu_3DQ1 = (1, 2, 4, 3, 5, 6, 8, 7)`` (``mesh.f90:52``, ``:458-485``).

Sections are found, as in the reference, by the first five characters of a line.
"""
from __future__ import annotations

import numpy as np

PERMU_3DQ1 = (1, 2, 4, 3, 5, 6, 8, 7)


def _section(lines, i, head):
    while i < len(lines) and lines[i][:5] != head:
        i += 1
    return i + 1


def read_gid(path: str) -> dict:
    """Arrays of one mesh file: 1-based vertex ids, z-ordered hexahedra."""
    with open(path) as f:
        lines = f.read().split("\n")
    t = lines[0].split()
    hdr = {t[k].lower(): int(t[k + 1]) for k in range(1, len(t) - 1, 2)}
    dim, order = hdr["dimension"], hdr["order"]
    nelem, npoin = hdr["elements"], hdr["vertices"]
    coords = np.zeros((npoin, 3))
    i = _section(lines, 0, "coord")
    while lines[i][:5] != "end c":
        tok = lines[i].split()
        coords[int(tok[0]) - 1, :dim] = [float(x) for x in tok[1:1 + dim]]
        i += 1
    cells, cset, cgeo = [None] * nelem, np.zeros(nelem, np.int32), np.zeros(nelem, np.int32)
    i = _section(lines, i, "eleme")
    while lines[i][:5] != "end e":
        tok = [int(x) for x in lines[i].split()]
        e, nn = tok[0] - 1, tok[1]
        cells[e] = tok[2:2 + nn]
        cset[e], cgeo[e] = tok[2 + nn], tok[3 + nn]
        i += 1
    i = _section(lines, i, "vefs")
    bptr, bverts, bset, bgeo = [0], [], [], []
    rows = {}
    while i < len(lines) and lines[i][:5] != "end v":
        tok = [int(x) for x in lines[i].split()]
        rows[tok[0]] = tok
        i += 1
    for k in sorted(rows):
        tok = rows[k]
        nb = tok[1]
        bverts.extend(tok[2:2 + nb])
        bset.append(tok[2 + nb])
        bgeo.append(tok[3 + nb])
        bptr.append(len(bverts))
    if order == 0:
        for e in range(nelem):
            if dim == 3 and len(cells[e]) == 8:
                cells[e] = [cells[e][p - 1] for p in PERMU_3DQ1]
    if any(len(c) != 8 for c in cells):
        raise ValueError("only hexahedral meshes")
    return {"dim": dim, "coords": coords, "cells": np.array(cells, dtype=np.int32), "cell_set": cset,
            "cell_geo": cgeo, "bvef_ptr": np.array(bptr, dtype=np.int64),
            "bvef_verts": np.array(bverts, dtype=np.int32), "bvef_set": np.array(bset, dtype=np.int32),
            "bvef_geo": np.array(bgeo, dtype=np.int32)}

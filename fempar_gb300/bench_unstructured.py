"""Unstructured-mesh benchmark: the headline Poisson workload through the mesh-data-files route
(``python -m fempar_gb300.bench_unstructured``).

Workload (seeded, synthetic): the geometry and coefficients of the structured headline (unit
cube, n^3 hexahedra, interior vertices perturbed by U(-0.15h, 0.15h), Q2, k = exp(N(0,1)) per
cell, f = 1, Dirichlet on the whole boundary, Jacobi-PCG to 1e-8) handed over as an
unstructured mesh: explicit cell vertex lists with every cell's vertices in a seeded random
orientation of the cube (48 symmetries), boundary given as faces, box edges and corners with
set id 1 -- the shape of the reference's GiD meshes.  Optionally the mesh is written to and read
back from a GiD file (``--gid-file``).

Times: mesh (vef generation and set ids on the device), space (node and dof numbering,
sparsity, SELL layout), numeric assembly (FP64 and float-float integration), PCG (mixed and
FP64); and the same problem on the structured lattice, whose solution the unstructured one
must reproduce node by node (max relative difference reported).

Prints one JSON line.
"""
from __future__ import annotations

import argparse
import itertools
import json
import os
import tempfile
import time

import numpy as np

from . import _lib as L
from .fe import Context, FEAffineOperator, IterativeLinearSolver, PoissonIntegration, SerialFESpace, SerialTriangulation

SEED = 20261203


def orientations():
    """The cube's 48 symmetries as maps new local vertex -> old local vertex, with the matching
    axis permutation and flips (new axis d runs along old axis perm[d], reversed if flip d)."""
    out = []
    for perm in itertools.permutations(range(3)):
        for flips in range(8):
            m = []
            for b in range(8):
                old = 0
                for d in range(3):
                    old |= (((b >> d) & 1) ^ ((flips >> d) & 1)) << perm[d]
                m.append(old)
            out.append((m, perm, flips))
    return out


def workload(n, seed=SEED):
    """Vertices and per-cell coefficients of the structured headline (same seed and draws)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    h = 1.0 / n
    nv = n + 1
    k, j, i = np.meshgrid(np.arange(nv), np.arange(nv), np.arange(nv), indexing="ij")
    xyz = np.stack([i * h, j * h, k * h], axis=-1).reshape(-1, 3)
    ii, jj, kk = i.ravel(), j.ravel(), k.ravel()
    interior = (ii > 0) & (ii < n) & (jj > 0) & (jj < n) & (kk > 0) & (kk < n)
    d = rng.uniform(-0.15 * h, 0.15 * h, size=xyz.shape)
    xyz[interior] += d[interior]
    coef = np.exp(rng.normal(0.0, 1.0, size=n ** 3))
    return xyz, coef


def unstructured_box(n, seed=SEED + 1):
    """Cells (1-based, random orientation per cell), orientation ids, given boundary vefs."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nv = n + 1
    c = np.arange(n ** 3)
    ci, cj, ck = c % n, (c // n) % n, c // (n * n)
    base = np.stack([(ci + (b & 1)) + nv * ((cj + ((b >> 1) & 1)) + nv * (ck + ((b >> 2) & 1))) for b in range(8)], 1)
    ors = orientations()
    table = np.array([o[0] for o in ors], dtype=np.int64)
    o = rng.integers(len(ors), size=n ** 3)
    cells = np.take_along_axis(base, table[o], axis=1).astype(np.int32) + 1

    def vid(a, b, cc):
        return a + nv * (b + nv * cc) + 1

    quads, edges = [], []
    u, v = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    u, v = u.ravel(), v.ravel()
    for d in range(3):
        a, b = [e for e in range(3) if e != d]
        for val in (0, n):
            corner = []
            for du, dv in ((0, 0), (1, 0), (1, 1), (0, 1)):
                x = [None, None, None]
                x[d], x[a], x[b] = np.full(u.size, val), u + du, v + dv
                corner.append(vid(*x))
            quads.append(np.stack(corner, 1))
    t = np.arange(n)
    for d in range(3):
        a, b = [e for e in range(3) if e != d]
        for va in (0, n):
            for vb in (0, n):
                x0, x1 = [None] * 3, [None] * 3
                x0[a] = x1[a] = np.full(n, va)
                x0[b] = x1[b] = np.full(n, vb)
                x0[d], x1[d] = t, t + 1
                edges.append(np.stack([vid(*x0), vid(*x1)], 1))
    quads = np.concatenate(quads)
    edges = np.concatenate(edges)
    corners = np.array([[vid(a, b, cc)] for a in (0, n) for b in (0, n) for cc in (0, n)])
    verts = np.concatenate([quads.ravel(), edges.ravel(), corners.ravel()]).astype(np.int32)
    ptr = np.concatenate([[0], np.cumsum([4] * len(quads) + [2] * len(edges) + [1] * len(corners))]).astype(np.int64)
    sets = np.ones(len(ptr) - 1, dtype=np.int32)
    return cells, o, ptr, verts, sets


def write_gid(path, xyz, cells, ptr, verts, sets):
    """GiD problem-type file (hexahedra in GiD's order, header order 0)."""
    permu = (1, 2, 4, 3, 5, 6, 8, 7)
    gidc = np.zeros_like(cells)
    for i, p in enumerate(permu):
        gidc[:, p - 1] = cells[:, i]
    nb = len(ptr) - 1
    with open(path, "w") as f:
        f.write(f"MESH dimension  3  order  0  types  1  elements {len(cells):10d}  vertices {len(xyz):10d}"
                f"  vefs {nb:10d}\ncoordinates\n")
        ids = np.arange(1, len(xyz) + 1)
        np.savetxt(f, np.column_stack([ids, xyz]), fmt=["%d", "%.17e", "%.17e", "%.17e"])
        f.write("end coordinates\nelements\n")
        e = np.column_stack([np.arange(1, len(cells) + 1), np.full(len(cells), 8), gidc, np.zeros(len(cells), int),
                             np.ones(len(cells), int)])
        np.savetxt(f, e, fmt="%d")
        f.write("end elements\nvefs\n")
        for i in range(nb):
            vs = verts[ptr[i]:ptr[i + 1]]
            f.write(f"{i + 1} {len(vs)} " + " ".join(str(x) for x in vs) + f" {sets[i]} 1\n")
        f.write("end vefs\n")


def node_map_q2(o):
    """Per cell, unstructured local Q2 node -> structured local node, from the orientation."""
    ors = orientations()
    table = np.zeros((len(ors), 27), dtype=np.int64)
    for t, (_, perm, flips) in enumerate(ors):
        for a in range(27):
            new = (a % 3, (a // 3) % 3, a // 9)
            old = [0, 0, 0]
            for d in range(3):
                old[perm[d]] = 2 - new[d] if (flips >> d) & 1 else new[d]
            table[t, a] = old[0] + 3 * (old[1] + 3 * old[2])
    return table[o]


def run(n=128, rtol=1e-8, device=0, gid_file=False, structured=True):
    xyz, coef = workload(n)
    cells, o, ptr, verts, sets = unstructured_box(n)
    ctx = Context(device)
    out = {"metric": "Poisson Q2 on an unstructured hexahedral mesh: DOF/s to 1e-8 (assembly + Jacobi-PCG)",
           "n": n, "cells": int(n ** 3)}
    t0 = time.perf_counter()
    if gid_file:
        d = tempfile.mkdtemp()
        write_gid(os.path.join(d, "box.mesh"), xyz, cells, ptr, verts, sets)
        out["gid_write_s"] = time.perf_counter() - t0
        out["gid_file_mb"] = os.path.getsize(os.path.join(d, "box.mesh")) / 1e6
        t0 = time.perf_counter()
        tri = SerialTriangulation.from_mesh_data_files(ctx, d, "box")
        out["gid_read_and_mesh_ms"] = (time.perf_counter() - t0) * 1e3
    else:
        tri = SerialTriangulation.from_arrays(ctx, xyz, cells, ptr, verts, sets)
        out["mesh_ms"] = (time.perf_counter() - t0) * 1e3
    out["mesh"] = tri.info()
    t0 = time.perf_counter()
    sp = SerialFESpace(tri, order=2, dirichlet_ids=[1])
    out["space_ms"] = (time.perf_counter() - t0) * 1e3
    out["dofs"] = sp.num_free_dofs
    out["nnz_full"] = sp.info.nnz_full
    integ = PoissonIntegration(cell_coef=coef, source_fn=L.FG_FN_CONST, fn_param=[1.0])
    fast = PoissonIntegration(cell_coef=coef, source_fn=L.FG_FN_CONST, fn_param=[1.0], fast_integration=True)
    res = {}
    for name, ig, prec in (("fp64", integ, "fp64"), ("mixed", fast, "mixed")):
        op = FEAffineOperator(sp, ig)
        op.compute()                      # warm (attributes, allocations)
        t0 = time.perf_counter()
        op.compute()
        t_asm = (time.perf_counter() - t0) * 1e3
        s = IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
        s.set_parameters_from_pl({"ILS_RTOL": rtol, "ILS_MAX_NUM_ITERATIONS": 200000, "PRECISION": prec})
        x = s.solve()
        inf = s.info()
        step = t_asm + inf["solve_ms"]
        res[name] = x
        out[name] = {"assembly_ms": t_asm, "iterations": inf["iterations"], "solve_ms": inf["solve_ms"],
                     "ms_per_iteration": inf["solve_ms"] / max(inf["iterations"], 1), "step_ms": step,
                     "dof_per_s": sp.num_free_dofs / (step * 1e-3), "converged": inf["converged"]}
        op.close()
    xm, x64 = res["mixed"], res["fp64"]
    out["mixed_vs_fp64"] = float(np.linalg.norm(xm - x64) / np.linalg.norm(x64))
    if structured:
        dmu = sp.get_dof_map()
        sp.close()
        tri.close()
        trs = SerialTriangulation(ctx, (n, n, n), vertex_xyz=xyz.ravel())
        sps = SerialFESpace(trs, order=2, dirichlet_ids=list(range(1, 27)))
        op = FEAffineOperator(sps, integ)
        op.compute()
        t0 = time.perf_counter()
        op.compute()
        t_asm = (time.perf_counter() - t0) * 1e3
        s = IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
        s.set_parameters_from_pl({"ILS_RTOL": rtol, "ILS_MAX_NUM_ITERATIONS": 200000, "PRECISION": "fp64"})
        xs = s.solve()
        inf = s.info()
        out["structured_fp64"] = {"assembly_ms": t_asm, "iterations": inf["iterations"], "solve_ms": inf["solve_ms"],
                                  "dof_per_s": sps.num_free_dofs / ((t_asm + inf["solve_ms"]) * 1e-3)}
        dms = sps.get_dof_map()
        nm = node_map_q2(o)
        du = dmu.ravel()
        ds = np.take_along_axis(dms, nm, axis=1).ravel()
        keep = du > 0
        assert np.all(ds[keep] > 0)
        diff = np.abs(x64[du[keep] - 1] - xs[ds[keep] - 1])
        out["max_rel_diff_vs_structured"] = float(diff.max() / np.abs(xs).max())
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--gid-file", action="store_true", help="write the mesh as a GiD file and read it back")
    ap.add_argument("--no-structured", action="store_true")
    a = ap.parse_args()
    print(json.dumps(run(a.n, gid_file=a.gid_file, structured=not a.no_structured)))


if __name__ == "__main__":
    main()

"""Partitioned dof numbering and dof_import of FEMPAR's parallel FE space, restated for the oracle.

TEST INFRASTRUCTURE ONLY: the checker for ``fg_partition_*``.  Only tests/ import this module.

A structured mesh of n0 x n1 x n2 cells split into np0 x np1 x np2 box parts (n_d divisible by
np_d), as ``uniform_hex_mesh_generator`` does for a task (part ids 1-based, lexicographic):

* local cells (``uniform_hex_mesh_generator.f90:255-360``): walking the part's box extended by
  one ghost layer towards every neighbour part, in lexicographic order, cells next to a ghost
  layer are "interface" cells and go to the end of the local list in reverse visiting order;
  the others keep their visiting order at the front;
* local free dofs: the serial numbering run over the local cells in that order
  (``sbm_serial_fe_space.i90:2623-2884``): per cell its interior dofs, then its vefs' own dofs
  on first visit; Dirichlet dofs are the global ones;
* interface couplings (``sbm_par_fe_space.i90:1877-2034``): one column per (local interface
  dof, other part sharing it) holding (neighbour part, number of sharing parts, non-consecutive
  dof ggid) -- the ggid built from the largest global cell id around the dof's vef and the
  dof's position in that cell (``:1103-1118``); columns sorted lexicographically
  (``sort.f90``), owners decided by ``:2737-2853``: a dof shared by two parts goes to the larger
  part id for the first half of each neighbour's run and to the smaller one for the rest; a dof
  shared by more parts goes to the largest part id;
* ``dof_import_create`` (``dof_import.f90:102-213``) and the interior-then-interface
  renumbering (``:365-421``, ``sbm_par_fe_space.i90:449-470``).
"""
from __future__ import annotations

import numpy as np

import oracle as O

OWNER, NON_OWNER, UNCOUPLED = -2, -3, -1
GGID_SHIFT = 40   # bits of the cell part of a non-consecutive dof ggid


def part_cells(n, nparts, part_id):
    """Global cell ids (0-based) of part part_id (1-based) in local order."""
    npx = list(nparts)
    pid = part_id - 1
    pijk = [pid % npx[0], (pid // npx[0]) % npx[1], pid // (npx[0] * npx[1])]
    nloc = [n[d] // npx[d] for d in range(3)]
    left = [1 if pijk[d] > 0 else 0 for d in range(3)]
    right = [1 if pijk[d] < npx[d] - 1 else 0 for d in range(3)]
    tot = [nloc[d] + left[d] + right[d] for d in range(3)]
    first = [pijk[d] * nloc[d] - left[d] for d in range(3)]
    interior, itfc = [], []
    for k in range(tot[2]):
        for j in range(tot[1]):
            for i in range(tot[0]):
                ijk = (i, j, k)
                ghost = any((left[d] and ijk[d] == 0) or (right[d] and ijk[d] == tot[d] - 1) for d in range(3))
                if ghost:
                    continue
                g = [first[d] + ijk[d] for d in range(3)]
                cid = g[0] + n[0] * (g[1] + n[1] * g[2])
                if any((left[d] and ijk[d] == 1) or (right[d] and ijk[d] == tot[d] - 2) for d in range(3)):
                    itfc.append(cid)
                else:
                    interior.append(cid)
    return interior + itfc[::-1]


def cell_part(n, nparts, c):
    i, j, k = c % n[0], (c // n[0]) % n[1], c // (n[0] * n[1])
    nloc = [n[d] // nparts[d] for d in range(3)]
    return 1 + i // nloc[0] + nparts[0] * (j // nloc[1] + nparts[1] * (k // nloc[2]))


def build(P, nparts):
    """Per part: l2g (local free dof -> global free id, 1-based, final numbering) and the
    dof_import fields.  P is a structured oracle Problem."""
    n = [int(v) for v in P.params.n]
    nparts = [int(v) for v in nparts]
    assert all(n[d] % nparts[d] == 0 for d in range(3))
    num_parts = nparts[0] * nparts[1] * nparts[2]
    dm = P.dof_map()
    nd = P.nd
    codes = list(O.polytope_codes(3))
    ncomp = 3 if P.params.kind == O.ELASTICITY else 1
    order = P.params.order
    own = [list(O.own_dofs(3, order, ncomp, f + 1)) for f in range(27)]   # n-faces 1-based there
    nfaces = 27
    # numbering walk: interior (last n-face) first, then the 26 vefs
    walk = [nfaces - 1] + list(range(nfaces - 1))
    parts = []
    sharers = {}   # global free id -> set of parts
    for p in range(1, num_parts + 1):
        cells = part_cells(n, nparts, p)
        seen = {}
        l2g = []
        for c in cells:
            for f in walk:
                for s in own[f]:
                    g = int(dm[c, s])
                    if g > 0 and g not in seen:
                        seen[g] = len(l2g)
                        l2g.append(g)
        for g in l2g:
            sharers.setdefault(g, set()).add(p)
        parts.append({"cells": cells, "l2g": l2g, "g2l": seen})
    # largest cell around each dof (over the whole mesh) and the dof's position in it
    maxcell = {}
    for c in range(P.ncells):
        for s in range(nd):
            g = int(dm[c, s])
            if g > 0 and (g not in maxcell or c >= maxcell[g][0]):
                maxcell[g] = (c, s)
    for p, part in enumerate(parts, start=1):
        cols = []
        for g, loc in part["g2l"].items():
            sh = sharers[g]
            if len(sh) < 2:
                continue
            c, s = maxcell[g]
            key = c + (s << GGID_SHIFT)
            mx = max(sh)
            for q in sorted(sh - {p}):
                cols.append([q, len(sh), key, loc, mx])
        cols.sort(key=lambda r: (r[0], r[1], r[2]))
        flags = [0] * len(cols)
        i = 0
        while i < len(cols):
            if cols[i][1] == 2:
                s0 = i
                while i < len(cols) and cols[i][1] == 2 and cols[i][0] == cols[s0][0]:
                    i += 1
                size = i - s0
                first_owner = p == max(p, cols[s0][0])
                for j in range(s0, i):
                    in_first = j < s0 + size // 2
                    flags[j] = OWNER if in_first == first_owner else NON_OWNER
            else:
                if p == cols[i][4]:
                    flags[i] = OWNER
                elif cols[i][0] == cols[i][4]:
                    flags[i] = NON_OWNER
                else:
                    flags[i] = UNCOUPLED
                i += 1
        # dof_import_create (1-based local ids)
        nloc = len(part["l2g"])
        weight = np.ones(nloc)
        list_rcv, list_snd, rcv, snd = [], [], {}, {}
        itfc = set()
        for col, fl in zip(cols, flags):
            q, loc = col[0], col[3] + 1
            if fl == OWNER:
                if q not in rcv:
                    rcv[q] = []
                    list_rcv.append(q)
                rcv[q].append(loc)
            elif fl == NON_OWNER:
                if q not in snd:
                    snd[q] = []
                    list_snd.append(q)
                snd[q].append(loc)
                weight[loc - 1] = 0.0
            itfc.add(loc)
        unpack = [v for q in list_rcv for v in rcv[q]]
        pack = [v for q in list_snd for v in snd[q]]
        rcv_ptrs = np.cumsum([1] + [len(rcv[q]) for q in list_rcv])
        snd_ptrs = np.cumsum([1] + [len(snd[q]) for q in list_snd])
        n_int = nloc - len(itfc)
        # interior first, then interface (pack order, then unpack order)
        perm = [-1] * (nloc + 1)
        cur = n_int + 1
        for v in pack + unpack:
            if perm[v] == -1:
                perm[v] = cur
                cur += 1
        cur = 1
        for v in range(1, nloc + 1):
            if perm[v] == -1:
                perm[v] = cur
                cur += 1
        pack = [perm[v] for v in pack]
        unpack = [perm[v] for v in unpack]
        w2 = np.zeros(nloc)
        l2g = np.zeros(nloc, dtype=np.int64)
        for v in range(1, nloc + 1):
            w2[perm[v] - 1] = weight[v - 1]
            l2g[perm[v] - 1] = part["l2g"][v - 1]
        part.update({"num_dofs": nloc, "num_interior": n_int, "num_interface": len(itfc), "weight": w2,
                     "list_rcv": list_rcv, "rcv_ptrs": list(rcv_ptrs), "unpack_idx": unpack,
                     "list_snd": list_snd, "snd_ptrs": list(snd_ptrs), "pack_idx": pack, "l2g": l2g})
        del part["g2l"]
    return parts


def comm(parts, vals):
    """par_scalar_array_t%comm (par_scalar_array.f90:498-533) on per-part arrays: non-owners
    send their interface values, owners add them (in list_rcv order), then owners send back
    and non-owners overwrite."""
    out = [v.copy() for v in vals]
    idx = {p: i for i, p in enumerate(range(1, len(parts) + 1))}
    # stage 1: p receives from each q in list_rcv the values q packed for p
    for p, part in enumerate(parts, start=1):
        for k, q in enumerate(part["list_rcv"]):
            qpart = parts[idx[q]]
            kk = qpart["list_snd"].index(p)
            src = qpart["pack_idx"][qpart["snd_ptrs"][kk] - 1:qpart["snd_ptrs"][kk + 1] - 1]
            dst = part["unpack_idx"][part["rcv_ptrs"][k] - 1:part["rcv_ptrs"][k + 1] - 1]
            for s, d in zip(src, dst):
                out[p - 1][d - 1] = out[p - 1][d - 1] + vals[q - 1][s - 1]
    final = [v.copy() for v in out]
    # stage 2: owners send back (unpack lists), non-owners overwrite (pack lists)
    for p, part in enumerate(parts, start=1):
        for k, q in enumerate(part["list_snd"]):
            qpart = parts[idx[q]]
            kk = qpart["list_rcv"].index(p)
            src = qpart["unpack_idx"][qpart["rcv_ptrs"][kk] - 1:qpart["rcv_ptrs"][kk + 1] - 1]
            dst = part["pack_idx"][part["snd_ptrs"][k] - 1:part["snd_ptrs"][k + 1] - 1]
            for s, d in zip(src, dst):
                final[p - 1][d - 1] = out[q - 1][s - 1]
    return final

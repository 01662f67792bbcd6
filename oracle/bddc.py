"""Two-level BDDC preconditioner restated on the CPU with dense numpy algebra.

TEST INFRASTRUCTURE ONLY: the checker for the GPU BDDC path.  Only tests/ import it.

It follows FEMPAR's mlbddc for one level of subdomains and a directly solved coarse
problem, on the element matrices and dof map of the oracle (``oracle.Problem``):

* apply, steps 1-5 (interior Dirichlet correction, interface residual update, weighted
  coarse + constrained-Neumann correction, weighted sum, harmonic extension):
  ``Sources/Lib/LinearAlgebra/Preconditioner/sbm_base_mlbddc.i90:909-1009``;
* the constrained Neumann problem is the augmented matrix [A_i C_i^T; C_i 0] solved
  directly (``:261-297,:522-542,:1479-1526``); the coarse basis Phi_i is the first block of
  its solution for right-hand sides [0; I] (``:558-595``);
* the coarse matrix is sum_i R_ci^T (Phi_i^T A_i Phi_i) R_ci (``:598-662,:771-828``),
  solved directly (``:1011-1026``);
* one coarse dof per object and field component; its constraint row is the average of
  that component over the object's free dofs
  (``Sources/Lib/Integration/FESpace/sbm_standard_coarse_fe_handler.i90:28-219``);
* weights W = 1 / (number of subdomains around the dof) (``:221-295``), or, as an option,
  the diagonal-stiffness weights diag(A_i) / sum_j diag(A_j);
* or, with ``coarse_handler=HANDLER_ELASTICITY``, the elasticity coarse handler
  (``Sources/Lib/Integration/FESpace/sbm_elasticity_coarse_fe_handler.i90``): one coarse dof
  per vertex and component, no edge constraints (``:110-111``), and six per face whose
  constraint rows are the face integrals of the shape functions times the rigid-body modes
  (translations, then r4 = (y,-x,0), r5 = (-z,0,x), r6 = (0,z,-y), ``:37-73``) divided by
  the face measure (strategy CI, ``:180-381``), over the subdomain's own cells.

Subdomains are boxes of cells given by cut positions per axis.  Objects are classified
from the box grid: an interface node that lies on a slab plane in all three directions is
a vertex, a node on two interior cut planes (and inside a slab along the third axis) an
edge point, a node on one interior cut plane a face point.  Edges and faces are grouped
by the planes and slabs they lie in (a face point on the domain boundary belongs to the
slab next to it: the same two subdomains share it).
"""
from __future__ import annotations

import numpy as np

WEIGHT_MULTIPLICITY, WEIGHT_STIFFNESS = 0, 1
HANDLER_STANDARD, HANDLER_ELASTICITY = 0, 1

_MODES = 6  # rigid-body modes in 3D: 3 translations + 3 rotations


def _lagrange(p, i, x):
    """Lagrange basis i of order p on the equispaced nodes of [-1, 1] at x."""
    nodes = -1.0 + 2.0 * np.arange(p + 1) / p
    v = 1.0
    for j in range(p + 1):
        if j != i:
            v *= (x - nodes[j]) / (nodes[i] - nodes[j])
    return v


def _rigid_modes(x):
    """Values r_m[comp] of the six rigid-body modes at point x (rows m)."""
    return np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0],
                     [x[1], -x[0], 0.0], [-x[2], 0.0, x[0]], [0.0, x[2], -x[1]]])


def _slab_index(X, pos):
    """Index of the slab plane X lies on, or of the slab that contains X."""
    k = int(np.searchsorted(pos, X, side="right")) - 1
    return min(k, len(pos) - 2) if X != pos[k] else k


class BDDCOracle:
    def __init__(self, problem, n, order, ncomp, cuts, use_vertices=True, use_edges=True, use_faces=False,
                 weighting=WEIGHT_MULTIPLICITY, coarse_handler=HANDLER_STANDARD, vertex_xyz=None):
        P = problem
        p = order
        self.n = [int(v) for v in n]
        self.cuts = [np.asarray(c, dtype=np.int64) for c in cuts]
        nsub = [len(c) - 1 for c in self.cuts]
        self.nsub = nsub
        self.nfree = P.nfree
        dm = P.dof_map()
        nn = (p + 1) ** 3
        nd = nn * ncomp
        nx, ny, nz = self.n
        ncells = nx * ny * nz
        # lattice node and component of every free dof (1-based ids in the dof map)
        lat = np.zeros((self.nfree, 3), dtype=np.int64)
        comp_of = np.zeros(self.nfree, dtype=np.int64)
        cell_sub = np.zeros(ncells, dtype=np.int64)
        parts = [set() for _ in range(self.nfree)]
        sub_cells = [[] for _ in range(nsub[0] * nsub[1] * nsub[2])]
        for c in range(ncells):
            ci, cj, ck = c % nx, (c // nx) % ny, c // (nx * ny)
            si = int(np.searchsorted(self.cuts[0], ci, side="right")) - 1
            sj = int(np.searchsorted(self.cuts[1], cj, side="right")) - 1
            sk = int(np.searchsorted(self.cuts[2], ck, side="right")) - 1
            s = si + nsub[0] * (sj + nsub[1] * sk)
            cell_sub[c] = s
            sub_cells[s].append(c)
            for loc in range(nd):
                g = dm[c, loc]
                if g <= 0:
                    continue
                a, cc = loc % nn, loc // nn
                ai, aj, ak = a % (p + 1), (a // (p + 1)) % (p + 1), a // ((p + 1) ** 2)
                lat[g - 1] = (p * ci + ai, p * cj + aj, p * ck + ak)
                comp_of[g - 1] = cc
                parts[g - 1].add(s)
        self.parts = parts
        pos = [p * c for c in self.cuts]
        # object key of each interface dof
        keys = {}
        for g in range(self.nfree):
            if len(parts[g]) < 2:
                continue
            X = lat[g]
            on_cut = [X[d] in set(pos[d][1:-1].tolist()) for d in range(3)]
            plane = [X[d] in set(pos[d].tolist()) for d in range(3)]
            idx = [_slab_index(int(X[d]), pos[d]) for d in range(3)]
            if all(plane):
                key = (0, int(X[0]), int(X[1]), int(X[2]))
            elif sum(on_cut) == 2:
                a = [d for d in range(3) if not plane[d]][0]
                key = (1, a) + tuple(idx)
            else:
                # a face: the cut plane and the slabs along the other axes (points on the
                # domain boundary join the face: the same two subdomains share them)
                d = on_cut.index(True)
                slab = [min(int(np.searchsorted(pos[e], X[e], side="right")) - 1, len(pos[e]) - 2) for e in range(3)]
                key = (2, d) + tuple(idx[e] if e == d else slab[e] for e in range(3))
            keys[g] = key
        use = {0: use_vertices, 1: use_edges, 2: use_faces}
        rigid = coarse_handler == HANDLER_ELASTICITY
        if rigid and (ncomp != 3 or use_edges):
            raise ValueError("the elasticity coarse handler needs 3 components and no edge constraints")
        if rigid:
            # faces: six functionals per face object; vertices: one per component
            objs = sorted({(k, int(comp_of[g])) for g, k in keys.items() if k[0] == 0 and use[0]} |
                          {(k, mode) for k in keys.values() if k[0] == 2 and use[2] for mode in range(_MODES)})
        else:
            objs = sorted({(k, int(comp_of[g])) for g, k in keys.items() if use[k[0]]})
        self.coarse_index = {kc: i for i, kc in enumerate(objs)}
        self.ncoarse = len(objs)
        obj_dofs = {kc: [] for kc in objs}
        for g, k in keys.items():
            kc = (k, int(comp_of[g]))
            if kc in obj_dofs:
                obj_dofs[kc].append(g)
        if vertex_xyz is None:
            K3, J3, I3 = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
            vertex_xyz = np.stack([I3.ravel() / nx, J3.ravel() / ny, K3.ravel() / nz], axis=1)
        xyz = np.asarray(vertex_xyz, dtype=np.float64).reshape(-1, 3)
        lat_dof = {(int(lat[g, 0]), int(lat[g, 1]), int(lat[g, 2]), int(comp_of[g])): g for g in range(self.nfree)}
        gx, gw = np.polynomial.legendre.leggauss(p + 1)

        def face_rows(key, s, loc, m):
            """The six constraint rows of face object `key` seen from subdomain s."""
            d = key[1]
            b, c = [e for e in range(3) if e != d]
            sidx = [s % nsub[0], (s // nsub[0]) % nsub[1], s // (nsub[0] * nsub[1])]
            lo_c = [int(self.cuts[e][sidx[e]]) for e in range(3)]
            hi_c = [int(self.cuts[e][sidx[e] + 1]) for e in range(3)]
            plane = int(self.cuts[d][key[2 + d]])
            ca, side = (plane, 0) if plane == lo_c[d] else (plane - 1, 1)
            rows = np.zeros((_MODES, m))
            meas = 0.0
            for cc in range(lo_c[c], hi_c[c]):
                for cb in range(lo_c[b], hi_c[b]):
                    V = np.zeros((2, 2, 3))
                    for u in range(2):
                        for v in range(2):
                            I3 = [0, 0, 0]
                            I3[d], I3[b], I3[c] = ca + side, cb + u, cc + v
                            V[u, v] = xyz[I3[0] + (nx + 1) * (I3[1] + (ny + 1) * I3[2])]
                    for t, wt in zip(gx, gw):
                        for s_, ws in zip(gx, gw):
                            fs, ft = [(1 - s_) / 2, (1 + s_) / 2], [(1 - t) / 2, (1 + t) / 2]
                            x = sum(fs[u] * ft[v] * V[u, v] for u in range(2) for v in range(2))
                            dxs = sum((u - 0.5) * ft[v] * V[u, v] for u in range(2) for v in range(2))
                            dxt = sum(fs[u] * (v - 0.5) * V[u, v] for u in range(2) for v in range(2))
                            f = ws * wt * np.linalg.norm(np.cross(dxs, dxt))
                            meas += f
                            R = _rigid_modes(x)
                            for j in range(p + 1):
                                for i in range(p + 1):
                                    Nv = _lagrange(p, i, s_) * _lagrange(p, j, t)
                                    P3 = [0, 0, 0]
                                    P3[d], P3[b], P3[c] = p * (ca + side), p * cb + i, p * cc + j
                                    for comp in range(3):
                                        g = lat_dof.get((P3[0], P3[1], P3[2], comp))
                                        if g is not None and g in loc:
                                            rows[:, loc[g]] += Nv * R[:, comp] * f
            return rows / meas

        # per-subdomain local problems
        self.subs = []
        for s, cells in enumerate(sub_cells):
            gl = sorted({int(dm[c, l]) - 1 for c in cells for l in range(nd) if dm[c, l] > 0})
            loc = {g: i for i, g in enumerate(gl)}
            m = len(gl)
            K = np.zeros((m, m))
            for c in cells:
                em, _ = P.elmat(c)
                ids = [loc.get(int(dm[c, l]) - 1, -1) if dm[c, l] > 0 else -1 for l in range(nd)]
                for a in range(nd):
                    if ids[a] < 0:
                        continue
                    for b in range(nd):
                        if ids[b] >= 0:
                            K[ids[a], ids[b]] += em[a, b]
            gl = np.array(gl, dtype=np.int64)
            iface = np.array([len(parts[g]) > 1 for g in gl])
            if rigid:
                my_objs = sorted(({(keys[g], int(comp_of[g])) for g in gl if g in keys} |
                                  {(keys[g], mode) for g in gl if g in keys for mode in range(_MODES)})
                                 & set(self.coarse_index))
            else:
                my_objs = sorted({(keys[g], int(comp_of[g])) for g in gl if g in keys} & set(obj_dofs))
            C = np.zeros((len(my_objs), m))
            frows = {}
            for r, kc in enumerate(my_objs):
                if rigid and kc[0][0] == 2:
                    if kc[0] not in frows:
                        frows[kc[0]] = face_rows(kc[0], s, loc, m)
                    C[r] = frows[kc[0]][kc[1]]
                    continue
                ds = obj_dofs[kc]
                for g in ds:
                    C[r, loc[g]] = 1.0 / len(ds)
            self.subs.append({"gl": gl, "K": K, "iface": iface, "C": C,
                              "cidx": np.array([self.coarse_index[kc] for kc in my_objs], dtype=np.int64)})
        # weights
        if weighting == WEIGHT_STIFFNESS:
            dsum = np.zeros(self.nfree)
            for S in self.subs:
                dsum[S["gl"]] += np.diag(S["K"])
            for S in self.subs:
                S["w"] = np.diag(S["K"]) / dsum[S["gl"]]
        else:
            for S in self.subs:
                S["w"] = np.array([1.0 / len(parts[g]) for g in S["gl"]])
        # constrained Neumann matrices, coarse basis, coarse matrix
        Kc = np.zeros((self.ncoarse, self.ncoarse))
        for S in self.subs:
            K, C = S["K"], S["C"]
            m, nc = K.shape[0], C.shape[0]
            aug = np.zeros((m + nc, m + nc))
            aug[:m, :m] = K
            aug[:m, m:] = C.T
            aug[m:, :m] = C
            S["aug"] = aug
            rhs = np.zeros((m + nc, nc))
            rhs[m:, :] = np.eye(nc)
            Phi = np.linalg.solve(aug, rhs)[:m, :] if nc else np.zeros((m, 0))
            S["Phi"] = Phi
            Kc[np.ix_(S["cidx"], S["cidx"])] += Phi.T @ K @ Phi
            I = np.where(~S["iface"])[0]
            S["I"] = I
            S["G"] = np.where(S["iface"])[0]
            S["KII"] = K[np.ix_(I, I)]
        self.Kc = Kc

    def apply(self, r):
        r = np.array(r, dtype=np.float64)
        y = np.zeros(self.nfree)
        # 1) delta_I = A_II^-1 r_I ; 2) y_I = delta_I
        dI = {}
        for s, S in enumerate(self.subs):
            d = np.linalg.solve(S["KII"], r[S["gl"][S["I"]]]) if len(S["I"]) else np.zeros(0)
            dI[s] = d
            y[S["gl"][S["I"]]] = d
        # 3) r_G -= sum_i A_GI^i delta_I^i ; r_I = 0
        for s, S in enumerate(self.subs):
            if len(S["I"]):
                r[S["gl"][S["G"]]] -= S["K"][np.ix_(S["G"], S["I"])] @ dI[s]
        isint = np.zeros(self.nfree, dtype=bool)
        for S in self.subs:
            isint[S["gl"][S["I"]]] = True
        r[isint] = 0.0
        # 4) weighted coarse + constrained Neumann corrections, weighted sum
        fc = np.zeros(self.ncoarse)
        loc_r = []
        for S in self.subs:
            rs = S["w"] * r[S["gl"]]
            loc_r.append(rs)
            fc[S["cidx"]] += S["Phi"].T @ rs
        uc = np.linalg.solve(self.Kc, fc) if self.ncoarse else fc
        dG = np.zeros(self.nfree)
        for S, rs in zip(self.subs, loc_r):
            m, nc = S["K"].shape[0], S["C"].shape[0]
            sol = np.linalg.solve(S["aug"], np.concatenate([rs, np.zeros(nc)]))[:m]
            d = S["Phi"] @ uc[S["cidx"]] + sol
            dG[S["gl"]] += S["w"] * d
        dG[isint] = 0.0
        y[~isint] = dG[~isint]
        # 5) y_I -= A_II^-1 A_IG delta_G
        for S in self.subs:
            if len(S["I"]):
                t = S["K"][np.ix_(S["I"], S["G"])] @ dG[S["gl"][S["G"]]]
                y[S["gl"][S["I"]]] -= np.linalg.solve(S["KII"], t)
        return y

    def pcg(self, problem, b, rtol=1e-8, maxit=1000):
        """PCG with this preconditioner, res_res criterion, zero initial guess; the update
        sequence of cg.f90:101-238 (see orc_cg)."""
        A = problem.spmv
        x = np.zeros(self.nfree)
        r = np.array(b, dtype=np.float64)
        z = self.apply(r)
        rz = float(r @ z)
        p = z.copy()
        test = rtol * np.linalg.norm(r)
        it = 0
        while True:
            it += 1
            Ap = A(p)
            pAp = float(Ap @ p)
            alpha = rz / pAp if pAp != 0.0 else 0.0
            x += alpha * p
            r -= alpha * Ap
            err = np.linalg.norm(r)
            if err <= test or it >= maxit:
                break
            z = self.apply(r)
            beta = 1.0 / rz
            rz = float(r @ z)
            beta *= rz
            p = z + beta * p
        return x, it, err <= test

"""ctypes wrapper of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: the checker for the GPU path.  Only tests/,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm
import this module; the product package ``fempar_gb300`` never does.

The oracle restates FEMPAR's serial path (mesh -> dof numbering -> integration ->
COO -> CSR -> CG); ``fempar_oracle.h`` lists the reference file:line each part
follows.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

POISSON, ELASTICITY = 0, 1
CG, DG = 0, 1
FN_ZERO, FN_CONST, FN_SHARP_WAVE, FN_LINEAR, FN_QP_VALUES = 0, 1, 2, 3, 4
RES_RES, RES_RHS, DELTA_RHS, DELTA_DELTA, RES_NRMGIVEN_RHS_NRMGIVEN, RES_NRMGIVEN_RES_NRMGIVEN = range(6)

ALL_BOUNDARY_3D = list(range(1, 27))
ALL_BOUNDARY_2D = list(range(1, 9))


class _Params(C.Structure):
    _fields_ = [
        ("num_dims", C.c_int),
        ("n", C.c_int * 3),
        ("limits", C.c_double * 6),
        ("vertex_xyz", C.c_void_p),
        ("order", C.c_int),
        ("kind", C.c_int),
        ("dirichlet_ids", C.c_int * 27),
        ("n_dirichlet_ids", C.c_int),
        ("cell_coef", C.c_void_p),
        ("nu", C.c_double),
        ("source_fn", C.c_int),
        ("fn_param", C.c_double * 8),
        ("qp_source", C.c_void_p),
        ("boundary_fn", C.c_int),
        ("translated_jacobian", C.c_int),
        ("nthreads", C.c_int),
        ("formulation", C.c_int),
    ]


class _UMesh(C.Structure):
    _fields_ = [
        ("num_vertices", C.c_int64),
        ("coords", C.c_void_p),
        ("num_cells", C.c_int64),
        ("cell_vertices", C.c_void_p),
        ("num_given_vefs", C.c_int64),
        ("given_vef_ptr", C.c_void_p),
        ("given_vef_vertices", C.c_void_p),
        ("given_vef_set", C.c_void_p),
    ]


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (plain g++)."""
    src = os.path.join(HERE, "fempar_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp, i64, i32, dbl = C.c_void_p, C.c_int64, C.c_int, C.c_double
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.POINTER(_Params)]
        L.orc_destroy.argtypes = [vp]
        L.orc_create_unstructured.restype = vp
        L.orc_create_unstructured.argtypes = [C.POINTER(_Params), C.POINTER(_UMesh)]
        L.orc_num_vefs.restype = i64
        L.orc_num_vefs.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.orc_get_cell_vefs.argtypes = [vp, vp]
        L.orc_get_vef_sets.argtypes = [vp, vp]
        for name in ("orc_num_cells", "orc_num_free", "orc_num_dirichlet", "orc_nnz_upper", "orc_coo_entries"):
            getattr(L, name).restype = i64
            getattr(L, name).argtypes = [vp]
        for name in ("orc_dofs_per_cell", "orc_qp_per_cell"):
            getattr(L, name).restype = i32
            getattr(L, name).argtypes = [vp]
        L.orc_get_dof_map.argtypes = [vp, vp]
        L.orc_get_csr_upper.argtypes = [vp, vp, vp, vp]
        L.orc_get_rhs.argtypes = [vp, vp]
        L.orc_get_dirichlet_values.argtypes = [vp, vp]
        L.orc_get_elmat.argtypes = [vp, i64, vp, vp]
        L.orc_get_timings.argtypes = [vp, vp]
        L.orc_get_qp_coords.argtypes = [vp, vp]
        L.orc_cg.restype = i32
        L.orc_cg.argtypes = [vp, i32, dbl, dbl, i32, i32, vp, vp, vp, C.POINTER(C.c_int), vp, i32]
        L.orc_cg_timed.restype = i32
        L.orc_cg_timed.argtypes = [vp, i32, dbl, dbl, i32, i32, vp, vp, vp, C.POINTER(C.c_int), vp, i32, vp]
        L.orc_spmv.argtypes = [vp, vp, vp]
        L.orc_energy_error.restype = dbl
        L.orc_energy_error.argtypes = [vp, vp]
        L.orc_error_norms.restype = None
        L.orc_error_norms.argtypes = [vp, vp, C.c_int, vp, vp]
        L.orc_gauss_legendre.argtypes = [i32, vp, vp]
        L.orc_own_dofs.restype = i32
        L.orc_own_dofs.argtypes = [i32, i32, i32, i32, vp]
        L.orc_polytope_codes.restype = i32
        L.orc_polytope_codes.argtypes = [i32, vp]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def gauss_legendre(n: int):
    x = np.zeros(n)
    w = np.zeros(n)
    lib().orc_gauss_legendre(n, _ptr(x), _ptr(w))
    return x, w


def polytope_codes(num_dims: int):
    out = np.zeros(27, dtype=np.int32)
    k = lib().orc_polytope_codes(num_dims, _ptr(out))
    return out[:k]


def own_dofs(num_dims: int, order: int, ncomp: int, iface: int):
    out = np.zeros(4096, dtype=np.int32)
    k = lib().orc_own_dofs(num_dims, order, ncomp, iface, _ptr(out))
    return out[:k]


class Problem:
    """One assembled problem of the oracle (mesh, dofs, CSR upper 1-based, rhs)."""

    def __init__(self, n, order=1, num_dims=3, kind=POISSON, dirichlet_ids=None, limits=None,
                 vertex_xyz=None, cell_coef=None, nu=0.3, source_fn=FN_ZERO, fn_param=(),
                 qp_source=None, boundary_fn=FN_ZERO, translated_jacobian=False, nthreads=1, formulation=CG):
        P = _Params()
        P.num_dims = num_dims
        n = list(n) + [1] * (3 - len(n))
        for i in range(3):
            P.n[i] = int(n[i])
        lim = limits if limits is not None else [0.0, 1.0] * 3
        for i in range(6):
            P.limits[i] = float(lim[i]) if i < len(lim) else 0.0
        self._keep = []
        if vertex_xyz is not None:
            vertex_xyz = np.ascontiguousarray(vertex_xyz, dtype=np.float64)
            self._keep.append(vertex_xyz)
        if cell_coef is not None:
            cell_coef = np.ascontiguousarray(cell_coef, dtype=np.float64)
            self._keep.append(cell_coef)
        if qp_source is not None:
            qp_source = np.ascontiguousarray(qp_source, dtype=np.float64)
            self._keep.append(qp_source)
        P.vertex_xyz = _ptr(vertex_xyz)
        P.cell_coef = _ptr(cell_coef)
        P.qp_source = _ptr(qp_source)
        P.order = order
        P.kind = kind
        ids = dirichlet_ids if dirichlet_ids is not None else (ALL_BOUNDARY_3D if num_dims == 3 else ALL_BOUNDARY_2D)
        for i, v in enumerate(ids):
            P.dirichlet_ids[i] = int(v)
        P.n_dirichlet_ids = len(ids)
        P.nu = nu
        P.source_fn = source_fn
        for i, v in enumerate(fn_param):
            P.fn_param[i] = float(v)
        P.boundary_fn = boundary_fn
        P.translated_jacobian = int(bool(translated_jacobian))
        P.nthreads = int(nthreads)
        P.formulation = int(formulation)
        self.params = P
        self.h = self._create(P)
        if not self.h:
            raise ValueError("oracle rejected the parameters")
        L = lib()
        self.ncells = L.orc_num_cells(self.h)
        self.nd = L.orc_dofs_per_cell(self.h)
        self.nq = L.orc_qp_per_cell(self.h)
        self.nfree = L.orc_num_free(self.h)
        self.ndir = L.orc_num_dirichlet(self.h)
        self.nnz_upper = L.orc_nnz_upper(self.h)
        self.coo_entries = L.orc_coo_entries(self.h)

    def _create(self, P):
        return lib().orc_create(C.byref(P))

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().orc_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def dof_map(self):
        out = np.zeros(self.ncells * self.nd, dtype=np.int32)
        lib().orc_get_dof_map(self.h, _ptr(out))
        return out.reshape(self.ncells, self.nd)

    def csr_upper(self):
        irp = np.zeros(self.nfree + 1, dtype=np.int64)
        ja = np.zeros(self.nnz_upper, dtype=np.int32)
        val = np.zeros(self.nnz_upper, dtype=np.float64)
        lib().orc_get_csr_upper(self.h, _ptr(irp), _ptr(ja), _ptr(val))
        return irp, ja, val

    def rhs(self):
        out = np.zeros(self.nfree)
        lib().orc_get_rhs(self.h, _ptr(out))
        return out

    def dirichlet_values(self):
        out = np.zeros(self.ndir)
        lib().orc_get_dirichlet_values(self.h, _ptr(out))
        return out

    def elmat(self, cell):
        em = np.zeros((self.nd, self.nd))
        ev = np.zeros(self.nd)
        lib().orc_get_elmat(self.h, int(cell), _ptr(em), _ptr(ev))
        return em.T.copy(), ev  # stored column-major

    def qp_coords(self):
        out = np.zeros((self.ncells, self.nq, 3))
        lib().orc_get_qp_coords(self.h, _ptr(out))
        return out

    def timings(self):
        t = np.zeros(3)
        lib().orc_get_timings(self.h, _ptr(t))
        return {"setup": t[0], "integrate": t[1], "compress": t[2]}

    def spmv(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.nfree)
        lib().orc_spmv(self.h, _ptr(x), _ptr(y))
        return y

    def cg(self, b=None, precond=0, rtol=1e-6, atol=0.0, maxit=1000, criterion=RES_RES, x0=None,
           history=False, nthreads=1, times=False):
        """PCG (cg.f90).  history: per-iteration error estimate; times: seconds from the call's
        start to the end of each iteration.  nthreads > 1: threaded symmetric-storage SpMV;
        nthreads < -1: |nthreads| threads on a full-CSR row-gather SpMV."""
        b = self.rhs() if b is None else np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.nfree)
        it = C.c_int(0)
        hist = np.zeros(maxit) if history else None
        tim = np.zeros(maxit) if times else None
        x0 = None if x0 is None else np.ascontiguousarray(x0, dtype=np.float64)
        rc = lib().orc_cg_timed(self.h, precond, rtol, atol, maxit, criterion, _ptr(b), _ptr(x0), _ptr(x),
                                C.byref(it), _ptr(hist), nthreads, _ptr(tim))
        out = {"x": x, "iters": it.value, "converged": rc == 0}
        if history:
            out["history"] = hist[: it.value]
        if times:
            out["times"] = tim[: it.value]
        return out

    def error_norms(self, x, fn, fn_param=()):
        """mean, l1, l2, linfty, h1_seminorm, h1, w1infty_seminorm, w1infty (finalised)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        prm = np.zeros(8)
        prm[:len(fn_param)] = fn_param
        o = np.zeros(6)
        lib().orc_error_norms(self.h, _ptr(x), int(fn), _ptr(prm), _ptr(o))
        return {"mean_norm": o[0], "l1_norm": o[1], "l2_norm": np.sqrt(o[2]), "linfty_norm": o[3],
                "h1_seminorm": np.sqrt(o[4]), "h1_norm": np.sqrt(o[2] + o[4]), "w1infty_seminorm": o[5],
                "w1infty_norm": o[3] + o[5]}

    def energy_error(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        return lib().orc_energy_error(self.h, _ptr(x))

    def csr_full(self):
        """Full symmetric CSR (0-based, sorted columns) expanded from the upper layout."""
        irp, ja, val = self.csr_upper()
        n = self.nfree
        rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(irp))
        cols = ja.astype(np.int64) - 1
        off = rows != cols
        r2 = np.concatenate([rows, cols[off]])
        c2 = np.concatenate([cols, rows[off]])
        v2 = np.concatenate([val, val[off]])
        order = np.lexsort((c2, r2))
        r2, c2, v2 = r2[order], c2[order], v2[order]
        rp = np.zeros(n + 1, dtype=np.int64)
        np.add.at(rp, r2 + 1, 1)
        rp = np.cumsum(rp)
        return rp, c2.astype(np.int32), v2


class UProblem(Problem):
    """The oracle on an unstructured hexahedral mesh (``gid.read_gid`` arrays or the same keys):
    vefs generated by first appearance, boundary set ids from the given vefs, dirichlet_ids
    are the mesh's set ids."""

    def __init__(self, mesh, order=1, dirichlet_ids=(1,), **kw):
        m = _UMesh()
        coords = np.ascontiguousarray(mesh["coords"], dtype=np.float64)
        cells = np.ascontiguousarray(mesh["cells"], dtype=np.int32)
        bptr = np.ascontiguousarray(mesh["bvef_ptr"], dtype=np.int64)
        bv = np.ascontiguousarray(mesh["bvef_verts"], dtype=np.int32)
        bs = np.ascontiguousarray(mesh["bvef_set"], dtype=np.int32)
        self._mesh_keep = [coords, cells, bptr, bv, bs]
        m.num_vertices = coords.shape[0]
        m.coords = _ptr(coords)
        m.num_cells = cells.shape[0]
        m.cell_vertices = _ptr(cells)
        m.num_given_vefs = bptr.size - 1
        m.given_vef_ptr = _ptr(bptr)
        m.given_vef_vertices = _ptr(bv)
        m.given_vef_set = _ptr(bs)
        self._umesh = m
        super().__init__((1, 1, 1), order=order, num_dims=3, dirichlet_ids=list(dirichlet_ids), **kw)
        ne, nf = C.c_int64(0), C.c_int64(0)
        self.nvefs = lib().orc_num_vefs(self.h, C.byref(ne), C.byref(nf))
        self.nedges, self.nfaces = ne.value, nf.value

    def _create(self, P):
        return lib().orc_create_unstructured(C.byref(P), C.byref(self._umesh))

    def cell_vefs(self):
        out = np.zeros(self.ncells * 26, dtype=np.int32)
        lib().orc_get_cell_vefs(self.h, _ptr(out))
        return out.reshape(self.ncells, 26)

    def vef_sets(self):
        out = np.zeros(self.nvefs, dtype=np.int32)
        lib().orc_get_vef_sets(self.h, _ptr(out))
        return out

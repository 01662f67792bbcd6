"""Host-side mirror of FEMPAR's interfaces for the GB300 path.

The objects wrap the C-ABI handles of libfempar_gpu.so and keep the reference's
names and call order, so a driver reads like the reference's tutorial drivers
(Tutorials/tutorial_01_poisson_sharp_circular_wave/tutorial_01_poisson_sharp_circular_wave.f90):

    ctx   = Context()
    tri   = SerialTriangulation(ctx, [32, 32, 32])              # triangulation%create
    space = SerialFESpace(tri, order=1, dirichlet_ids=range(1,27))  # fe_space%create
    op    = FEAffineOperator(space, PoissonIntegration(...))    # fe_affine_operator%create
    op.compute()                                                 # fe_affine_operator%compute
    solver = IterativeLinearSolver(); solver.set_type_from_string("CG")
    solver.set_parameters_from_pl({"ILS_RTOL": 1e-8}); solver.set_operators(op, "jacobi")
    x = solver.solve(op.get_translation())                       # iterative_linear_solver%solve

Errors raise FGError (the C-ABI never aborts).  Arrays are numpy (host) or, for the
``*_device`` methods, torch CUDA tensors.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def _ptr(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


class Context:
    """One device, one CUDA stream, an HBM budget (serial_context_t + environment_t)."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        h = C.c_void_p()
        L.check(L.lib().fg_ctx_create(device, hbm_budget_bytes, C.byref(h)), "fg_ctx_create")
        self.h = h
        self.device = device

    def memory(self):
        used, budget = C.c_uint64(), C.c_uint64()
        L.check(L.lib().fg_ctx_memory(self.h, C.byref(used), C.byref(budget)), "fg_ctx_memory")
        return used.value, budget.value

    def stream_handle(self) -> int:
        """cudaStream_t of the context (e.g. for torch.cuda.ExternalStream)."""
        s = C.c_void_p()
        L.check(L.lib().fg_ctx_get_stream(self.h, C.byref(s)), "fg_ctx_get_stream")
        return s.value or 0

    def kernel_launches(self) -> int:
        c = C.c_int64()
        L.check(L.lib().fg_ctx_kernel_launches(self.h, C.byref(c)), "fg_ctx_kernel_launches")
        return c.value

    def close(self):
        if getattr(self, "h", None):
            L.lib().fg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SerialTriangulation:
    """Hexahedral mesh (serial_triangulation_t): structured (uniform_hex_mesh_t) from the
    constructor, unstructured from mesh data files or arrays (``from_parameters``,
    ``from_mesh_data_files``, ``from_arrays``)."""

    def __init__(self, ctx: Context, n, limits=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0), vertex_xyz=None):
        """``n`` of length 3 gives hexahedra, of length 2 quadrilaterals (num_dims = 2); vertex
        coordinates are 3 per vertex in both cases (z ignored in 2D)."""
        self.ctx = ctx
        self.unstructured = False
        self.num_dims = len(n)
        if self.num_dims not in (2, 3):
            raise ValueError("n must have 2 or 3 entries")
        self.n = [int(v) for v in n] + ([1] if self.num_dims == 2 else [])
        nn = (C.c_int32 * 3)(*self.n)
        lim = list(limits) + [0.0, 0.0] * (3 - len(limits) // 2)
        lim = (C.c_double * 6)(*[float(v) for v in lim[:6]])
        vx = None
        nverts = (self.n[0] + 1) * (self.n[1] + 1) * (self.n[2] + 1 if self.num_dims == 3 else 1)
        if vertex_xyz is not None:
            vx = np.ascontiguousarray(vertex_xyz, dtype=np.float64)
            if vx.size != 3 * nverts:
                raise ValueError(f"vertex_xyz must hold {3 * nverts} values")
        h = C.c_void_p()
        L.check(L.lib().fg_mesh_create_structured(ctx.h, self.num_dims, nn, lim, _ptr(vx), C.byref(h)),
                "fg_mesh_create_structured")
        self.h = h
        self.num_cells = self.n[0] * self.n[1] * (self.n[2] if self.num_dims == 3 else 1)

    @classmethod
    def _wrap(cls, ctx, h):
        self = cls.__new__(cls)
        self.ctx = ctx
        self.h = h
        self.unstructured = True
        self.num_dims = 3
        self.n = None
        self.num_cells = self.info()["num_cells"]
        return self

    @classmethod
    def from_parameters(cls, ctx: Context, parameters: dict):
        """serial_triangulation_t%create(parameters): STATIC_TRIANG_GENERATE_FROM =
        MESH_DATA_FILES reads MESH_DIR_PATH/MESH_PREFIX.mesh; STRUCT_HEX_MESH_GENERATOR takes
        NUM_CELLS_X_DIR (and DOMAIN_LIMITS) like the structured constructor."""
        how = parameters.get("STATIC_TRIANG_GENERATE_FROM", "STRUCT_HEX_MESH_GENERATOR")
        if how == "MESH_DATA_FILES":
            return cls.from_mesh_data_files(ctx, parameters["MESH_DIR_PATH"], parameters["MESH_PREFIX"])
        if how == "STRUCT_HEX_MESH_GENERATOR":
            return cls(ctx, parameters["NUM_CELLS_X_DIR"],
                       parameters.get("DOMAIN_LIMITS", (0.0, 1.0, 0.0, 1.0, 0.0, 1.0)))
        raise ValueError(f"STATIC_TRIANG_GENERATE_FROM = {how!r}")

    @classmethod
    def from_mesh_data_files(cls, ctx: Context, dir_path: str, prefix: str):
        """Read <dir_path>/<prefix>.mesh (GiD, fempar problem type) -- fg_mesh_read_gid."""
        h = C.c_void_p()
        L.check(L.lib().fg_mesh_read_gid(ctx.h, str(dir_path).encode(), str(prefix).encode(), C.byref(h)),
                "fg_mesh_read_gid")
        return cls._wrap(ctx, h)

    @classmethod
    def from_arrays(cls, ctx: Context, coords, cells, given_vef_ptr=None, given_vef_vertices=None,
                    given_vef_set=None):
        """Unstructured mesh from arrays: coords (nv, 3); cells (nc, 8) 1-based vertex ids in the
        lexicographic local order; given boundary vefs as CSR (ptr, 1-based vertices, set ids)."""
        xyz = np.ascontiguousarray(coords, dtype=np.float64)
        cv = np.ascontiguousarray(cells, dtype=np.int32)
        nb = 0 if given_vef_ptr is None else len(given_vef_ptr) - 1
        bp = np.ascontiguousarray(given_vef_ptr if nb else [0], dtype=np.int64)
        bv = np.ascontiguousarray(given_vef_vertices if nb else [0], dtype=np.int32)
        bs = np.ascontiguousarray(given_vef_set if nb else [0], dtype=np.int32)
        h = C.c_void_p()
        L.check(L.lib().fg_mesh_create_unstructured(ctx.h, xyz.shape[0], _ptr(xyz), cv.shape[0], _ptr(cv), nb,
                                                     _ptr(bp), _ptr(bv), _ptr(bs), C.byref(h)),
                "fg_mesh_create_unstructured")
        return cls._wrap(ctx, h)

    def info(self):
        i = L.MeshInfo()
        L.check(L.lib().fg_mesh_get_info(self.h, C.byref(i)), "fg_mesh_get_info")
        return {k: getattr(i, k) for k, _ in L.MeshInfo._fields_}

    def get_vefs(self):
        """(cell vef ids (ncells, 26), 1-based; set id of every vef) -- unstructured meshes."""
        inf = self.info()
        cv = np.zeros(inf["num_cells"] * 26, dtype=np.int32)
        vs = np.zeros(inf["num_vefs"], dtype=np.int32)
        L.check(L.lib().fg_mesh_get_vefs(self.h, _ptr(cv), _ptr(vs)), "fg_mesh_get_vefs")
        return cv.reshape(-1, 26), vs

    def close(self):
        if getattr(self, "h", None):
            L.lib().fg_mesh_destroy(self.h)
            self.h = None


class SerialFESpace:
    """Lagrangian FE space with strong Dirichlet dofs (serial_fe_space_t); ``dg=True`` builds the
    discontinuous space of tutorial_01's interior-penalty formulation (scalar, weak boundary
    data, no Dirichlet ids)."""

    def __init__(self, triangulation: SerialTriangulation, order: int = 1, ncomp: int = 1, dirichlet_ids=(),
                 dg: bool = False):
        self.triangulation = triangulation
        self.dg = bool(dg)
        h = C.c_void_p()
        if self.dg:
            if ncomp != 1 or len(list(dirichlet_ids)):
                raise ValueError("the dG space is scalar and takes its boundary data weakly")
            L.check(L.lib().fg_space_create_dg(triangulation.h, order, C.byref(h)), "fg_space_create_dg")
        else:
            ids = np.ascontiguousarray(list(dirichlet_ids), dtype=np.int32)
            L.check(L.lib().fg_space_create(triangulation.h, order, ncomp, _ptr(ids) if ids.size else None,
                                            int(ids.size), C.byref(h)), "fg_space_create")
        self.h = h
        info = L.SpaceInfo()
        L.check(L.lib().fg_space_get_info(h, C.byref(info)), "fg_space_get_info")
        self.info = info
        self.order = order
        self.ncomp = ncomp
        self.num_free_dofs = info.num_free
        self.num_dirichlet_dofs = info.num_dirichlet
        self.dofs_per_cell = info.dofs_per_cell
        self.qp_per_cell = info.qp_per_cell
        self.num_cells = info.num_cells

    def release_pattern(self):
        """Free the CSR pattern after lean assembly (fg_space_release_pattern)."""
        L.check(L.lib().fg_space_release_pattern(self.h), "fg_space_release_pattern")

    def get_dof_map(self):
        """lst_dofs_gids, shape (ncells, dofs_per_cell), reference convention."""
        out = np.zeros(self.num_cells * self.dofs_per_cell, dtype=np.int32)
        L.check(L.lib().fg_space_get_dof_map(self.h, _ptr(out)), "fg_space_get_dof_map")
        return out.reshape(self.num_cells, self.dofs_per_cell)

    def get_dirichlet_coords(self):
        out = np.zeros(3 * self.num_dirichlet_dofs)
        L.check(L.lib().fg_space_get_dirichlet_coords(self.h, _ptr(out)), "fg_space_get_dirichlet_coords")
        return out.reshape(-1, 3)

    def get_qp_coords(self, out=None):
        """Physical quadrature-point coordinates, (num_cells, qp_per_cell, 3): where a
        user-defined source is evaluated before passing it as FG_FN_QP_VALUES.  out: an
        optional torch CUDA float64 tensor of that many entries (filled on the device)."""
        info = self.info
        if out is not None:
            L.check(L.lib().fg_space_get_qp_coords(self.h, _ptr(out), 1), "fg_space_get_qp_coords")
            return out
        xyz = np.zeros((info.num_cells, info.qp_per_cell, 3))
        L.check(L.lib().fg_space_get_qp_coords(self.h, _ptr(xyz), 0), "fg_space_get_qp_coords")
        return xyz

    def close(self):
        if getattr(self, "h", None):
            L.lib().fg_space_destroy(self.h)
            self.h = None


class DiscreteIntegration:
    """Description of discrete_integration_t%integrate_galerkin for the device kernels."""

    def __init__(self, kind=L.FG_POISSON, cell_coef=None, coef_const=1.0, nu=0.3, source_fn=L.FG_FN_ZERO,
                 fn_param=(), qp_source=None, boundary_fn=L.FG_FN_ZERO, dirichlet_values=None,
                 fast_integration=False):
        """fast_integration: float-float element matrices (FG_FAST_INTEGRATION), for mixed solves."""
        self.kind = kind
        self.fast_integration = fast_integration
        self.cell_coef = cell_coef
        self.coef_const = coef_const
        self.nu = nu
        self.source_fn = source_fn
        self.fn_param = list(fn_param)
        self.qp_source = qp_source
        self.boundary_fn = boundary_fn
        self.dirichlet_values = dirichlet_values

    def to_c(self):
        g = L.Integrand()
        L.lib().fg_integrand_default(C.byref(g))
        keep = []
        on_dev = None

        def arr(a):
            nonlocal on_dev
            if a is None:
                return None
            if hasattr(a, "data_ptr"):
                on_dev = True if on_dev in (None, True) else self._mixed()
                keep.append(a)
                return a.data_ptr()
            on_dev = False if on_dev in (None, False) else self._mixed()
            a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            return a.ctypes.data

        g.kind = self.kind
        g.cell_coef = arr(self.cell_coef)
        g.coef_const = self.coef_const
        g.nu = self.nu
        g.source_fn = self.source_fn
        for i, v in enumerate(self.fn_param):
            g.fn_param[i] = float(v)
        g.qp_source = arr(self.qp_source)
        g.boundary_fn = self.boundary_fn
        g.dirichlet_values = arr(self.dirichlet_values)
        g.flags = (L.FG_INPUTS_ON_DEVICE if on_dev else 0) | (L.FG_FAST_INTEGRATION if self.fast_integration else 0)
        return g, keep

    @staticmethod
    def _mixed():
        raise ValueError("integrand arrays must be all host (numpy) or all device (torch) arrays")


def PoissonIntegration(**kw):
    return DiscreteIntegration(kind=L.FG_POISSON, **kw)


def ElasticityIntegration(**kw):
    return DiscreteIntegration(kind=L.FG_ELASTICITY, **kw)


class FEAffineOperator:
    """fe_affine_operator_t: integrate + assemble into CSR (+FP32 copy) and rhs on the device."""

    def __init__(self, space: SerialFESpace, integration: DiscreteIntegration, lean: bool = False):
        """lean: keep only what a solve needs (FG_LEAN_SYSTEM; no export / reassembly / BDDC)."""
        self.space = space
        self.integration = integration
        self.lean = lean
        self.h = None

    def compute(self):
        g, keep = self.integration.to_c()
        if self.lean:
            g.flags |= L.FG_LEAN_SYSTEM
        if self.h is None:
            h = C.c_void_p()
            L.check(L.lib().fg_assemble(self.space.h, C.byref(g), C.byref(h)), "fg_assemble")
            self.h = h
        else:
            L.check(L.lib().fg_system_reassemble(self.h, C.byref(g)), "fg_system_reassemble")
        del keep
        return self

    def get_matrix(self, symmetric_storage=True, one_based=True):
        """(irp, ja, val) of the assembled matrix; the reference layout by default."""
        n = self.space.num_free_dofs
        nnz = self.space.info.nnz_upper if symmetric_storage else self.space.info.nnz_full
        irp = np.zeros(n + 1, dtype=np.int64)
        ja = np.zeros(nnz, dtype=np.int32)
        val = np.zeros(nnz, dtype=np.float64)
        L.check(L.lib().fg_system_export_csr(self.h, int(symmetric_storage), int(one_based), _ptr(irp), _ptr(ja),
                                             _ptr(val)), "fg_system_export_csr")
        return irp, ja, val

    def get_translation(self):
        out = np.zeros(self.space.num_free_dofs)
        L.check(L.lib().fg_system_export_rhs(self.h, _ptr(out)), "fg_system_export_rhs")
        return out

    def get_dirichlet_values(self):
        out = np.zeros(self.space.num_dirichlet_dofs)
        L.check(L.lib().fg_system_export_dirichlet_values(self.h, _ptr(out)), "fg_system_export_dirichlet_values")
        return out

    def apply_device(self, x, y, precision=L.FG_FP64):
        """y = A x with torch CUDA tensors (float64, or float32 for precision=FG_MIXED)."""
        import torch
        n = self.space.num_free_dofs
        want = torch.float32 if precision == L.FG_MIXED else torch.float64
        for t in (x, y):
            if not (t.is_cuda and t.is_contiguous() and t.dtype == want and t.numel() == n):
                raise ValueError(f"x and y must be contiguous CUDA {want} tensors of {n} entries")
        L.check(L.lib().fg_system_spmv_device(self.h, precision, _ptr(x), _ptr(y)), "fg_system_spmv_device")
        return y

    def apply_solver_layout_device(self, x_slot, y_slot, precision=L.FG_FP64, reps=1):
        """reps launches of the solver's SpMV on solver-layout vectors, not synchronised."""
        import torch
        n = self.space.info.solver_vec_len
        want = torch.float32 if precision == L.FG_MIXED else torch.float64
        for t in (x_slot, y_slot):
            if not (t.is_cuda and t.is_contiguous() and t.dtype == want and t.numel() == n):
                raise ValueError(f"solver-layout vectors must be contiguous CUDA {want} tensors of {n} entries")
        L.check(L.lib().fg_system_spmv_solver_layout_device(self.h, precision, _ptr(x_slot), _ptr(y_slot), reps),
                "fg_system_spmv_solver_layout_device")
        return y_slot

    def error_norms(self, x, exact_fn=L.FG_FN_ZERO, fn_param=(), cell_sq_energy=False):
        """Norms of u - u_h for the solution x (numpy, num_free_dofs, or a torch CUDA tensor)
        against the analytic exact_fn (error_norms_scalar_t%compute for every scalar norm
        type, plus the tutorial's energy norm).  Returns a dict (and the per-cell squared
        energy errors if cell_sq_energy)."""
        n = self.space.num_free_dofs
        on_dev = hasattr(x, "data_ptr")
        if not on_dev:
            x = np.ascontiguousarray(x, dtype=np.float64)
        if (x.numel() if on_dev else x.size) != n:
            raise ValueError("x must have num_free_dofs entries")
        prm = np.zeros(8)
        prm[:len(fn_param)] = fn_param
        cells = np.zeros(self.space.num_cells) if cell_sq_energy else None
        out = L.ErrorNorms()
        L.check(L.lib().fg_system_error_norms(self.h, _ptr(x), int(on_dev), int(exact_fn), _ptr(prm), _ptr(cells),
                                              C.byref(out)), "fg_system_error_norms")
        d = {k: getattr(out, k) for k, _ in L.ErrorNorms._fields_}
        return (d, cells) if cell_sq_energy else d

    def close(self):
        if getattr(self, "h", None):
            L.lib().fg_system_destroy(self.h)
            self.h = None


_CRITERIA = {"RES_RES": L.FG_RES_RES, "RES_RHS": L.FG_RES_RHS, "DELTA_RHS": L.FG_DELTA_RHS,
             "DELTA_DELTA": L.FG_DELTA_DELTA, "RES_NRMGIVEN_RHS_NRMGIVEN": L.FG_RES_NRMGIVEN_RHS_NRMGIVEN,
             "RES_NRMGIVEN_RES_NRMGIVEN": L.FG_RES_NRMGIVEN_RES_NRMGIVEN}


def bddc_cuts(n, nsub, jitter=0.0, seed=20261203):
    """Cell cut positions of a box partition: nsub[d] slabs per direction, widths jittered
    by up to +-jitter (fraction of the even width) with a seeded generator, each >= 1."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cuts = []
    for d in range(3):
        nd, ns = int(n[d]), int(nsub[d])
        base = nd / ns
        w = np.full(ns, base)
        if jitter > 0 and ns > 1:
            w = w * (1.0 + rng.uniform(-jitter, jitter, size=ns))
        c = np.concatenate([[0.0], np.cumsum(w)])
        c = np.round(c * nd / c[-1]).astype(np.int64)
        for k in range(1, ns + 1):
            c[k] = max(c[k], c[k - 1] + 1)
        for k in range(ns - 1, -1, -1):
            c[k] = min(c[k], c[k + 1] - 1)
        c[0], c[-1] = 0, nd
        cuts.append(c.astype(np.int32))
    return cuts


class MLBDDC:
    """mlbddc_t on box subdomains (two levels; coarse problem solved directly).

    Mirrors mlbddc_t's life cycle (sbm_base_mlbddc.i90:162-474): construction does the
    symbolic and numerical setup from the operator's element matrices;
    ``numerical_setup()`` refreshes it after ``FEAffineOperator.compute()`` on new data.
    Parameters follow the reference's coarse-space switches (coarse_space_use_vertices /
    edges / faces), the standard handler's multiplicity weighting and the choice of coarse
    FE handler: ``coarse_handler=FG_BDDC_HANDLER_ELASTICITY`` selects the elasticity handler
    (rigid-body face functionals, no edge constraints: pass ``use_edges=False``)."""

    def __init__(self, A: FEAffineOperator, nsub=(2, 2, 2), cuts=None, use_vertices=True, use_edges=True,
                 use_faces=False, weighting=L.FG_BDDC_WEIGHT_MULTIPLICITY,
                 coarse_handler=L.FG_BDDC_HANDLER_STANDARD, use_subparts=False):
        p = L.BddcParams()
        L.lib().fg_bddc_params_default(C.byref(p))
        for d in range(3):
            p.nsub[d] = int(nsub[d])
        self._cuts = None
        if cuts is not None:
            self._cuts = np.ascontiguousarray(np.concatenate([np.asarray(c, dtype=np.int32) for c in cuts]))
            p.cuts = self._cuts.ctypes.data
        p.use_vertices, p.use_edges, p.use_faces = int(use_vertices), int(use_edges), int(use_faces)
        p.weighting = int(weighting)
        p.coarse_handler = int(coarse_handler)
        p.use_subparts = int(use_subparts)
        self.A = A
        h = C.c_void_p()
        L.check(L.lib().fg_bddc_create(A.h, C.byref(p), C.byref(h)), "fg_bddc_create")
        self.h = h

    def numerical_setup(self):
        L.check(L.lib().fg_bddc_numerical_setup(self.h), "fg_bddc_numerical_setup")

    def info(self):
        i = L.BddcInfo()
        L.check(L.lib().fg_bddc_get_info(self.h, C.byref(i)), "fg_bddc_get_info")
        return {k: getattr(i, k) for k, _ in L.BddcInfo._fields_}

    def apply_device(self, r, z, precision=L.FG_FP64):
        """z = M^-1 r on torch CUDA float64 tensors of num_free_dofs entries."""
        n = self.A.space.num_free_dofs
        for t in (r, z):
            if t.numel() != n or t.dtype.itemsize != 8 or not t.is_contiguous():
                raise ValueError("r and z must be contiguous float64 tensors of num_free_dofs entries")
        L.check(L.lib().fg_bddc_apply_device(self.h, precision, _ptr(r), _ptr(z)), "fg_bddc_apply_device")

    def close(self):
        if getattr(self, "h", None):
            L.lib().fg_bddc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class IterativeLinearSolver:
    """iterative_linear_solver_t with the CG type (FP64 reference CG or mixed precision)."""

    def __init__(self):
        p = L.SolverParams()
        L.lib().fg_solver_params_default(C.byref(p))
        self.params = p
        self.A = None
        self.M = None
        self.last_info = None

    def set_type_from_string(self, name: str):
        if name.upper() not in ("CG", "GPU_CG", "GPU_MPCG"):
            raise ValueError(f"solver type {name} is not built on the device (CG only)")
        if name.upper() == "GPU_MPCG":
            self.params.precision = L.FG_MIXED
        return self

    def set_parameters_from_pl(self, pl: dict):
        """Keys of iterative_solver_parameters.f90:76-81 (+ the device-only ones)."""
        for k, v in pl.items():
            K = k.upper()
            if K == "ILS_RTOL":
                self.params.rtol = float(v)
            elif K == "ILS_ATOL":
                self.params.atol = float(v)
            elif K == "ILS_MAX_NUM_ITERATIONS":
                self.params.max_iters = int(v)
            elif K == "ILS_STOPPING_CRITERIUM":
                self.params.criterion = _CRITERIA[str(v).upper()]
            elif K == "PRECISION":
                self.params.precision = L.FG_MIXED if str(v).lower() in ("mixed", "fp32") else L.FG_FP64
            elif K == "INNER_RTOL":
                self.params.inner_rtol = float(v)
            elif K == "INNER_MAX_NUM_ITERATIONS":
                self.params.inner_max_iters = int(v)
            elif K == "CHECK_EVERY":
                self.params.check_every = int(v)
            else:
                raise KeyError(k)
        return self

    def set_operators(self, A: FEAffineOperator, M="identity"):
        """M: "identity", "jacobi" or an MLBDDC built on A."""
        self.A = A
        self.M = M if isinstance(M, MLBDDC) else None
        if self.M is not None:
            self.params.precond = L.FG_PREC_BDDC
        else:
            self.params.precond = L.FG_PREC_JACOBI if str(M).lower() == "jacobi" else L.FG_PREC_NONE
        return self

    def solve(self, b=None, x0=None, raise_on_nonconvergence=False, out=None):
        n = self.A.space.num_free_dofs
        x = np.zeros(n) if out is None else out
        if x.dtype != np.float64 or x.size != n or not x.flags.c_contiguous:
            raise ValueError("out must be a contiguous float64 array of num_free_dofs entries")
        info = L.SolveInfo()
        bb = None if b is None else np.ascontiguousarray(b, dtype=np.float64)
        xx0 = None if x0 is None else np.ascontiguousarray(x0, dtype=np.float64)
        if self.M is not None:
            st = L.lib().fg_bddc_solve(self.M.h, C.byref(self.params), _ptr(bb), _ptr(xx0), _ptr(x), C.byref(info))
        else:
            st = L.lib().fg_solve(self.A.h, C.byref(self.params), _ptr(bb), _ptr(xx0), _ptr(x), C.byref(info))
        if st != L.FG_OK and (st != L.FG_ERR_NOT_CONVERGED or raise_on_nonconvergence):
            raise L.FGError(st, "fg_solve")
        self.last_info = info
        return x

    def solve_device(self, b=None, x0=None, x=None):
        """Device-resident solve with torch CUDA tensors (float64)."""
        import torch
        n = self.A.space.num_free_dofs
        if x is None:
            x = torch.empty(n, dtype=torch.float64, device=f"cuda:{self.A.space.triangulation.ctx.device}")
        info = L.SolveInfo()
        if self.M is not None:
            st = L.lib().fg_bddc_solve_device(self.M.h, C.byref(self.params), _ptr(b), _ptr(x0), _ptr(x),
                                              C.byref(info))
        else:
            st = L.lib().fg_solve_device(self.A.h, C.byref(self.params), _ptr(b), _ptr(x0), _ptr(x), C.byref(info))
        if st not in (L.FG_OK, L.FG_ERR_NOT_CONVERGED):
            raise L.FGError(st, "fg_solve_device")
        self.last_info = info
        return x

    def info(self):
        i = self.last_info
        return None if i is None else {"iterations": i.iterations, "outer_iterations": i.outer_iterations,
                                       "converged": bool(i.converged), "error_estimate": i.error_estimate,
                                       "tolerance": i.tolerance, "solve_ms": i.solve_ms}

/*
 * fempar_gpu.h -- C-ABI of libfempar_gpu.so, the GB300 (sm_103a) implementation of
 * FEMPAR's data-parallel hot path: cell-wise Galerkin integration, global sparse
 * assembly into CSR, and the preconditioned CG solve.
 *
 * Conventions
 *   - Every function returns fg_status (FG_OK = 0; errors < 0).  Nothing aborts.
 *   - Handles are opaque and owned by the caller (fg_*_destroy).  A handle lives on
 *     the context's device and CUDA stream; calls on one context are serialised.
 *   - Host arrays passed in are copied; exports write into caller-allocated host
 *     buffers.  Functions named *_device take device pointers instead.
 *   - Global dof ids follow the reference: free dofs 1..nfree, strong-Dirichlet dofs
 *     -1..-ndirichlet (numbered first, in cell/vef visit order).
 *   - The parity export of the matrix is the reference's storage: 1-based CSR, upper
 *     triangle (j >= i) when symmetric_storage = 1.  Row pointers are int64 (the
 *     reference uses int32; a 96^3 Q2 elasticity matrix does not fit int32).
 *
 * Each entry point cites the reference interface it replaces (paths relative to the
 * fempar source tree).
 */
#ifndef FEMPAR_GPU_H
#define FEMPAR_GPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t fg_status;
enum {
  FG_OK = 0,
  FG_ERR_BADARG = -1,
  FG_ERR_OOM = -2,            /* device allocation failed or HBM budget exceeded */
  FG_ERR_CUDA = -3,           /* CUDA runtime error (fg_last_error has the text)   */
  FG_ERR_NOT_CONVERGED = -4,  /* solver hit max_iters; x holds the last iterate    */
  FG_ERR_NUMERIC = -5,        /* NaN/Inf met (input or breakdown)                  */
  FG_ERR_TIMEOUT = -6,        /* a bounded device wait ran out                     */
  FG_ERR_UNSUPPORTED = -7,    /* order / dimension / kind not built                */
  FG_ERR_NO_DEVICE = -8
};

typedef struct fg_ctx fg_ctx;
typedef struct fg_mesh fg_mesh;
typedef struct fg_space fg_space;
typedef struct fg_system fg_system;

/* Integrand kinds (discrete_integration_t extensions of the drivers). */
enum { FG_POISSON = 0, FG_ELASTICITY = 1 };

/* Analytic source / boundary functions. */
enum {
  FG_FN_ZERO = 0,
  FG_FN_CONST = 1,        /* fn_param[0..ncomp-1]                                   */
  FG_FN_SHARP_WAVE = 2,   /* u = atan(a(|x-c|-r)), f = -lap u; fn_param = a, r, cx, cy, cz */
  FG_FN_LINEAR = 3,       /* u = x+y+z, f = 0                                       */
  FG_FN_QP_VALUES = 4     /* source given at quadrature points: ncells*nq*ncomp     */
};

/* Flags of fg_integrand.flags.  FG_INPUTS_ON_DEVICE: the arrays are device pointers.
 * FG_LEAN_SYSTEM (fg_assemble only): keep only what a solve needs — the element matrices
 * are freed right after the scatter (before the solver layout is allocated) and the CSR
 * values after the solver layout and the Jacobi diagonal are filled; export, reassembly and
 * BDDC on such a system return FG_ERR_UNSUPPORTED.  Peak device memory of an assembly drops
 * from elmat + CSR + layout to max(elmat + CSR, CSR + layout). */
enum { FG_INPUTS_ON_DEVICE = 1, FG_LEAN_SYSTEM = 2, FG_FAST_INTEGRATION = 4 };
/* Poisson element matrices.  By default those of all cells are one FP64 product, emulated on
 * the tensor cores: the cells' geometric factors times a table shared by all cells.  They
 * match the FP64-pipe integration to ~1e-15 of the row scale, with reference parity.
 * FG_FAST_INTEGRATION asks for float-float accuracy (~2^-44, meant for FG_MIXED solves, whose
 * FP64 copy of the matrix feeds the residual refinement).  Its geometric factors are then
 * computed in float-float on the FP32 pipe (GB300's FP64 rate is ~1/70 of FP32's): ~2e-14 of
 * the row scale.  The environment variable FG_TC_INTEGRATION selects the path: 2 (default)
 * the tensor cores for both requests; 1 for FP64 requests only, with the float-float
 * integration kernel (~2e-13) for fast ones; 0 neither.  Where the context's HBM budget has
 * no room for the product's scratch (~7 KB per Q2 cell), the assembly uses the direct
 * kernels. */

typedef struct {
  int kind;                        /* FG_POISSON / FG_ELASTICITY                     */
  const double* cell_coef;         /* per-cell diffusion k (Poisson) or Young's E; NULL = coef_const */
  double coef_const;
  double nu;                       /* Poisson ratio (elasticity)                     */
  int source_fn;                   /* FG_FN_*                                        */
  double fn_param[8];
  const double* qp_source;         /* FG_FN_QP_VALUES                                */
  int boundary_fn;                 /* Dirichlet data when dirichlet_values == NULL   */
  const double* dirichlet_values;  /* optional: ndirichlet values (fixed dof values) */
  int flags;                       /* FG_INPUTS_ON_DEVICE                            */
} fg_integrand;

/* Solver selection (iterative_linear_solver_t parameters). */
enum { FG_PREC_NONE = 0, FG_PREC_JACOBI = 1 };
enum { FG_FP64 = 0, FG_MIXED = 1 };
/* Stopping criteria, cg.f90 names. */
enum { FG_RES_RES = 0, FG_RES_RHS = 1, FG_DELTA_RHS = 2, FG_DELTA_DELTA = 3,
       FG_RES_NRMGIVEN_RHS_NRMGIVEN = 4, FG_RES_NRMGIVEN_RES_NRMGIVEN = 5 };

typedef struct {
  int precond;          /* FG_PREC_*                                                  */
  int precision;        /* FG_FP64: reference CG in FP64; FG_MIXED: FP32 inner PCG + FP64 refinement */
  int criterion;        /* FG_RES_RES (default in the reference)                      */
  double rtol;          /* default 1e-6 (iterative_solver_parameters.f90:168-178)    */
  double atol;          /* default 0                                                  */
  int max_iters;        /* default 1000                                               */
  double inner_rtol;    /* FG_MIXED: reliable-update threshold delta: the FP32 recursive residual
                           is replaced by the FP64 true residual each time it has dropped by
                           this factor (0 = 0.1)                                          */
  int inner_max_iters;  /* reserved (0)                                                   */
  int check_every;      /* iterations between host-side convergence polls (0 = auto)  */
} fg_solver_params;

typedef struct {
  int iterations;       /* CG iterations (FG_MIXED: total inner iterations)           */
  int outer_iterations; /* FG_MIXED: refinement steps (FP64 residuals)               */
  int converged;
  double error_estimate;/* last value of the stopping-criterion quantity              */
  double tolerance;     /* rtol*|.|+atol the criterion compared against                */
  double solve_ms;      /* device time of the solve                                    */
  int64_t kernel_launches; /* kernels of this library launched by the solve (graph nodes included) */
} fg_solve_info;

typedef struct {
  int num_dims, order, ncomp;
  int dofs_per_cell, qp_per_cell;
  int64_t num_cells, num_free, num_dirichlet;
  int64_t nnz_full, nnz_upper;
  int64_t solver_vec_len;  /* entries of a vector in the solver's own layout (>= num_free) */
  int64_t solver_entries;  /* matrix entries stored by the solver's layout (>= nnz_full: padding) */
  int32_t solver_layout;   /* 0 = lattice-implicit SELL (no column indices), 1 = explicit-column SELL */
} fg_space_info;

const char* fg_status_string(fg_status s);
/* Text of the last error raised on this host thread. */
const char* fg_last_error(void);
/* Library version string. */
const char* fg_version(void);

/* Execution context: one device, one stream, an HBM budget (0 = all free memory).
 * Replaces serial_context_t/environment_t setup (Sources/Lib/Tools/execution_context.f90:63-145). */
fg_status fg_ctx_create(int device, uint64_t hbm_budget_bytes, fg_ctx** out);
fg_status fg_ctx_destroy(fg_ctx* ctx);
/* Bytes currently allocated by the context's objects. */
fg_status fg_ctx_memory(fg_ctx* ctx, uint64_t* in_use, uint64_t* budget);
/* The context's CUDA stream (cudaStream_t) for callers that order their own work or
 * record events around the library's kernels. */
fg_status fg_ctx_get_stream(fg_ctx* ctx, void** stream);
/* Kernels launched by this context so far (assembly, symbolic phase and solves). */
fg_status fg_ctx_kernel_launches(fg_ctx* ctx, int64_t* count);

/* Structured hexahedral mesh of [lim0,lim1]x[lim2,lim3]x[lim4,lim5] with n[0]*n[1]*n[2] cells,
 * cells lexicographic (x fastest).  vertex_xyz (nullable) gives 3*(n0+1)(n1+1)(n2+1) coordinates in
 * x-fastest lattice order (interleaved xyz) for a perturbed geometry; the map stays trilinear.
 * num_dims = 2: quadrilaterals of [lim0,lim1]x[lim2,lim3] with n[0]*n[1] cells (n[2] ignored),
 * vertex_xyz of 3*(n0+1)(n1+1) values (z ignored), bilinear map, boundary set ids 1..8 (the
 * generator's 2D polytope order; 9 interior).  On 2D meshes: continuous spaces (Poisson, ncomp
 * 1; plane-strain elasticity, ncomp 2) of orders 1-3, assembly, CSR export, the solvers and
 * error norms; the dG space, BDDC and partitions return FG_ERR_UNSUPPORTED.
 * Replaces uniform_hex_mesh_t%generate_part_local_mesh + serial_triangulation_t%create
 * (Sources/Lib/Geometry/Tools/uniform_hex_mesh_generator.f90:145-647,
 *  Sources/Lib/Geometry/Triangulation/sbm_serial_triangulation.i90:29-201). */
fg_status fg_mesh_create_structured(fg_ctx* ctx, int num_dims, const int32_t n[3], const double limits[6],
                                    const double* vertex_xyz, fg_mesh** out);
fg_status fg_mesh_destroy(fg_mesh* mesh);

/* Unstructured hexahedral mesh: num_vertices vertices (3 coordinates each, interleaved),
 * num_cells cells of 8 vertex ids each (1-based, in the reference FE's lexicographic local
 * order: bit 0 = x, bit 1 = y, bit 2 = z of the reference cell) and the given boundary vefs
 * (vertex ids of vertex k of vef i at given_vef_vertices[given_vef_ptr[i] + k]; 1, 2 or 4
 * vertices) with their set ids.  Edges and faces are generated on the device in the
 * reference's first-appearance order; set ids are assigned and handed from boundary faces to
 * their edges and vertices as the reference does.
 * Replaces serial_triangulation_t%create from mesh data files
 * (Sources/Lib/Geometry/Triangulation/sbm_serial_triangulation.i90:120-188,
 *  Sources/Lib/Geometry/Triangulation/sbm_fine_triangulation.i90:115-527). */
fg_status fg_mesh_create_unstructured(fg_ctx* ctx, int64_t num_vertices, const double* vertex_xyz,
                                      int64_t num_cells, const int32_t* cell_vertices, int64_t num_given_vefs,
                                      const int64_t* given_vef_ptr, const int32_t* given_vef_vertices,
                                      const int32_t* given_vef_set, fg_mesh** out);
/* Read <dir_path>/<prefix>.mesh (GiD, fempar problem type: header, coordinates, elements,
 * vefs; hexahedra in GiD order are reordered to the lexicographic one when the header's order
 * is 0) and build the unstructured mesh.  Only 3D hexahedral meshes are accepted.
 * Replaces mesh_t%read_fempar_gid_problem_type_format
 * (Sources/Lib/Geometry/Mesh/mesh.f90:337-504). */
fg_status fg_mesh_read_gid(fg_ctx* ctx, const char* dir_path, const char* prefix, fg_mesh** out);

typedef struct {
  int64_t num_cells, num_vertices, num_edges, num_faces, num_vefs;
  int32_t unstructured;             /* 1 for fg_mesh_create_unstructured / fg_mesh_read_gid */
  int32_t max_cells_around_vertex;  /* unstructured meshes                                 */
} fg_mesh_info;
fg_status fg_mesh_get_info(fg_mesh* mesh, fg_mesh_info* info);
/* Unstructured meshes: the vef ids of every cell (26 per cell, 1-based: vertices, edges,
 * faces in the reference FE's local order) and the set id of every vef (either may be NULL).
 * The reference's lst_vefs_gids and vefs_set (sbm_fine_triangulation.i90:115-527). */
fg_status fg_mesh_get_vefs(fg_mesh* mesh, int32_t* cell_vefs, int32_t* vef_set_ids);

/* Lagrangian FE space of order 1..3 with ncomp components (1 = scalar, 3 = vector),
 * global dof numbering and strong Dirichlet dofs on the boundary set ids listed
 * (polytope ids 1..26 of the structured generator; the mesh file's set ids 1..31 on an
 * unstructured mesh).
 * Replaces serial_fe_space_t%create + set_up_strong_dirichlet_bcs + generate_global_dof_numbering
 * (Sources/Lib/Integration/FESpace/sbm_serial_fe_space.i90:28-298,525-716,2423-2884). */
fg_status fg_space_create(fg_mesh* mesh, int order, int ncomp, const int32_t* dirichlet_ids, int n_ids,
                          fg_space** out);
fg_status fg_space_destroy(fg_space* space);
/* Discontinuous Lagrangian space of order 1..3 (scalar) for tutorial_01's symmetric interior
 * penalty formulation: every dof belongs to one cell (ids c*nn + a + 1, cell-local order), no
 * strong Dirichlet dofs.  fg_assemble on it takes the Poisson integrand with k = 1: volume terms,
 * interior-facet and boundary-facet (weak Dirichlet data boundary_fn) terms with C_IP = 10 p^2.
 * Replaces serial_fe_space_t%create with fe_space_type_dg and dg_discrete_integration_t
 * (Tutorials/tutorial_01_poisson_sharp_circular_wave/modules/
 *  tutorial_01_poisson_sharp_circular_wave_modules.f90:146-322). */
fg_status fg_space_create_dg(fg_mesh* mesh, int order, fg_space** out);
/* Free the space's CSR pattern (row pointers and column indices) once its systems are
 * assembled lean (FG_LEAN_SYSTEM): solves keep working, further assemblies and exports
 * return FG_ERR_UNSUPPORTED.  No counterpart in the reference (serving memory control). */
fg_status fg_space_release_pattern(fg_space* space);
fg_status fg_space_get_info(fg_space* space, fg_space_info* info);
/* lst_dofs_gids: ncells*dofs_per_cell int32 in the reference's cell-local dof order
 * (fe_space.f90:636-637). */
fg_status fg_space_get_dof_map(fg_space* space, int32_t* lst_dofs_gids);
/* Physical coordinates (3 per dof) of the Dirichlet nodes, in Dirichlet-id order, for callers
 * that interpolate their own boundary function (interpolate_dirichlet_values,
 * sbm_serial_fe_space.i90:997-1176). */
fg_status fg_space_get_dirichlet_coords(fg_space* space, double* xyz);
/* Physical coordinates of every cell's quadrature points, xyz[(cell*qp_per_cell + q)*3 + l]
 * (x fastest over the tensor Gauss rule), for callers that evaluate their own source function
 * at the quadrature points -- what a discrete_integration_t's integrate_galerkin does through
 * fe_cell_iterator%get_quadrature_points_coordinates (cell_map quadrature points,
 * sbm_cell_map.i90:673-686; tutorial_01 modules :107,124) -- and pass the values as
 * FG_FN_QP_VALUES.  on_device: xyz is a device pointer (num_cells*qp_per_cell*3 doubles).
 * 3D hexahedral meshes. */
fg_status fg_space_get_qp_coords(fg_space* space, double* xyz, int on_device);

/* Numeric assembly: integrate every cell, impose strong Dirichlet lifting and assemble the
 * global CSR matrix (+ FP32 copy) and right-hand side on the device, deterministically.
 * Replaces fe_affine_operator_t%compute -> discrete_integration_t%integrate_galerkin ->
 * fe_cell_iterator_t%assembly -> sparse_assembler_t -> sparse_matrix_t%convert
 * (Sources/Lib/Integration/FEOperator/sbm_fe_affine_operator.i90:15-34,
 *  Sources/Lib/Integration/FEOperator/sparse_assembler.f90:58-205,
 *  Sources/Lib/LinearAlgebra/SparseMatrix/base_sparse_matrix.f90:3469-3513,4121-4829). */
fg_status fg_assemble(fg_space* space, const fg_integrand* integrand, fg_system** out);
/* Re-run the numeric phase on an existing system (same space, new coefficients/data). */
fg_status fg_system_reassemble(fg_system* sys, const fg_integrand* integrand);
fg_status fg_system_destroy(fg_system* sys);

/* Parity export of the matrix: symmetric_storage = 1 gives the reference's upper-triangle
 * layout, 0 the full matrix; one_based = 1 gives the reference's 1-based indices.
 * irp has nfree+1 entries, ja/val nnz (fg_space_info.nnz_upper or nnz_full).
 * Replaces sparse_matrix_t's CSR state (csr_sparse_matrix.f90:44-115). */
fg_status fg_system_export_csr(fg_system* sys, int symmetric_storage, int one_based,
                               int64_t* irp, int32_t* ja, double* val);
/* Right-hand side (fe_affine_operator_t%get_translation, fe_operator.f90:113-183). */
fg_status fg_system_export_rhs(fg_system* sys, double* rhs);
/* Dirichlet values used in the lifting (fe_function_t%get_fixed_dof_values). */
fg_status fg_system_export_dirichlet_values(fg_system* sys, double* g);

/* y = A x on the device (precision FG_FP64 or FG_MIXED for the FP32 copy), device pointers.
 * Replaces sparse_matrix_t%apply (sparse_matrix.f90:1264-1276, csr_sparse_matrix.f90:626-672). */
fg_status fg_system_spmv_device(fg_system* sys, int precision, const void* x, void* y);
/* y = A x like fg_system_spmv_device, for callers that must not allocate device memory.
 * No counterpart in the reference: FEMPAR's sparse_matrix_t%apply runs on host arrays.
 *
 * Who needs it: a serving loop that pre-reserves all of its HBM and may not grow it, or a
 * host framework whose caching allocator owns the device memory (a cudaMalloc behind its
 * back can fail or fragment its pool).  fg_system_spmv_device stages x and y in the
 * solver's padded layout in work buffers the system allocates on first use; this variant
 * stages them instead in one file-scope device array of FG_NOALLOC_SCRATCH_BYTES (32 MiB)
 * that the library holds on every GPU that loads it, until the process exits.  With lazy
 * module loading (the CUDA default) that array is loaded on a device at the first call
 * there, outside the context's HBM budget: make the first call before reserving HBM.
 *
 * Limit: 2 * fg_space_info.solver_vec_len * (8 for FG_FP64, 4 for FG_MIXED) bytes must fit
 * the array (solver_vec_len <= 2,097,152 in FP64, <= 4,194,304 in FP32); larger systems are
 * rejected with FG_ERR_BADARG and a message in fg_last_error().  x and y are device
 * pointers of num_free entries (double, or float for FG_MIXED).  A system without free
 * dofs returns FG_OK at once.
 * The first call on a device looks up the array's device address there (once per
 * device), so make that first call before any stream capture.  All calls share the one
 * array: calls that overlap on the GPU (other host threads, other contexts of the same
 * device) race on it; serialise them.  The call is synchronous (it returns after the
 * result is in y) and leaves the caller's current device unchanged.
 * Calls no cudaMalloc/cudaFree and no allocating library routine. */
#define FG_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
fg_status fg_system_spmv_device_noalloc(fg_system* sys, int precision, const void* x, void* y);
/* reps launches of the solver's own SpMV kernel on vectors already in the solver's layout
 * (fg_space_info.solver_vec_len entries each, FP64 or FP32 per precision; entries that are
 * not free dofs must be finite), queued on the context's stream without synchronising; for
 * timing the kernel alone.  Same operator as sparse_matrix_t%apply in a permuted basis.
 * The caller guarantees the buffer lengths: the library cannot check raw pointers. */
fg_status fg_system_spmv_solver_layout_device(fg_system* sys, int precision, const void* x_slot, void* y_slot,
                                              int reps);

/* PCG solve of A x = b.  b == NULL uses the assembled right-hand side; x0 == NULL is the zero
 * initial guess (base_iterative_linear_solver.f90:281-282).  Host pointers.
 * Replaces iterative_linear_solver_t%solve -> cg_t (Sources/Lib/LinearAlgebra/IterativeLinearSolver/
 * iterative_linear_solver.f90:124-131, cg.f90:101-407) with jacobi_preconditioner_t
 * (Sources/Lib/LinearAlgebra/Preconditioner/jacobi_preconditioner.f90:356-412). */
fg_status fg_solve(fg_system* sys, const fg_solver_params* params, const double* b, const double* x0,
                   double* x, fg_solve_info* info);
/* Same, device pointers (b may be NULL; x0 NULL = zero guess; x written on the device). */
fg_status fg_solve_device(fg_system* sys, const fg_solver_params* params, const double* b_dev,
                          const double* x0_dev, double* x_dev, fg_solve_info* info);

/* Norms of the error u - u_h of a discrete solution (free-dof values x, num_free entries;
 * Dirichlet dofs take the system's fixed values) against an analytic u = FG_FN_* with
 * fn_param, per cell at the Gauss points and summed over the cells.  Replaces
 * error_norms_scalar_t%compute for the scalar norms (Sources/Lib/Integration/ErrorNorms/
 * sbm_error_norms_scalar.i90:67-241, finalize_norm error_norms.f90:174-221) and the
 * tutorial's energy-norm error estimator (tutorial_01 modules :542-679: cell_sq_energy,
 * nullable host array of num_cells values sum_q k |grad e|^2 |det J| w).  Scalar fields. */
typedef struct {
  double mean_norm, l1_norm, l2_norm, linfty_norm;
  double h1_seminorm, h1_norm, w1infty_seminorm, w1infty_norm;
  double energy_norm;     /* sqrt(sum_K k_K |grad e|^2_K) (k = 1: the tutorial's estimator) */
} fg_error_norms;
fg_status fg_system_error_norms(fg_system* sys, const double* x, int32_t x_on_device, int32_t fn,
                                const double* fn_param, double* cell_sq_energy, fg_error_norms* out);

/* Partitioned assembly: the structured mesh of a continuous space split into
 * np0 x np1 x np2 box parts (cells per direction divisible by the parts) as FEMPAR's parallel
 * FE space does for its tasks -- local cells, local dof numbering, interface couplings with the
 * reference's owner rule, dof_import (nearest-neighbour exchange lists) and the
 * interior-then-interface renumbering -- with all parts resident on this context's device.
 * Replaces par_fe_space_t%generate_global_dof_numbering / compute_dof_import
 * (Sources/Lib/Integration/FESpace/sbm_par_fe_space.i90:425-470,707-793,1877-2034,2737-2853),
 * dof_import_t (Sources/Lib/LinearAlgebra/Vector/dof_import.f90:102-213,365-421). */
typedef struct fg_partition fg_partition;
typedef struct {
  int32_t num_parts;
  int64_t num_local_dofs;    /* all parts' local free dofs (interface dofs once per part) */
  int64_t max_part_dofs;
  int64_t num_couplings;     /* interface columns over all parts */
  int64_t nnz_full;          /* entries of the subassembled matrices */
  int64_t nnz_upper;         /* their upper-triangle entries (symmetric-storage export) */
  int64_t num_dirichlet;     /* strong Dirichlet dofs (global ids shared by every part) */
} fg_partition_info;
typedef struct {
  int32_t num_dofs, num_interior_dofs, num_interface_dofs;
  int32_t num_rcv, num_snd, num_unpack, num_pack;
  int64_t num_cells;
  int64_t first_local_dof;   /* offset of the part in the concatenated local-dof vectors */
} fg_dof_import_sizes;
fg_status fg_partition_create(fg_space* space, const int32_t num_parts_x_dir[3], fg_partition** out);
fg_status fg_partition_destroy(fg_partition* partition);
fg_status fg_partition_get_info(fg_partition* partition, fg_partition_info* info);
/* dof_import_t of part part_id (1-based): sizes, then the arrays (1-based like the reference;
 * any pointer may be NULL): l2g = global free dof id of each local dof, weight, list_rcv,
 * rcv_ptrs (num_rcv+1), unpack_idx, list_snd, snd_ptrs (num_snd+1), pack_idx, and the part's
 * cells (global ids, 0-based) in local order. */
fg_status fg_partition_get_dof_import_sizes(fg_partition* partition, int32_t part_id, fg_dof_import_sizes* sizes);
fg_status fg_partition_get_dof_import(fg_partition* partition, int32_t part_id, int32_t* l2g, double* weight,
                                      int32_t* list_rcv, int32_t* rcv_ptrs, int32_t* unpack_idx,
                                      int32_t* list_snd, int32_t* snd_ptrs, int32_t* pack_idx, int64_t* cells);
/* Subassembled local systems of every part (block-diagonal matrix over the concatenated local
 * dofs; each part's rhs sums only its own cells): the assembler of par_fe_space_t.
 * Export/SpMV through the usual fg_system_* calls on the concatenated local space. */
fg_status fg_partition_assemble(fg_partition* partition, const fg_integrand* integrand, fg_system** out);
/* x (device, concatenated local dofs) <- comm(x): subassembled -> assembled interface values
 * (par_scalar_array_t%comm, Sources/Lib/LinearAlgebra/Vector/par_scalar_array.f90:498-533). */
fg_status fg_partition_comm_device(fg_partition* partition, double* x);
/* Partitioned (Jacobi-)PCG on a subassembled system: SpMV + comm, weighted dots
 * (par_scalar_array.f90:303-345), res_res criterion; x_global (host, num_free of the global
 * space) receives the owners' values. */
fg_status fg_partition_solve(fg_partition* partition, fg_system* subassembled, const fg_solver_params* params,
                             double* x_global, fg_solve_info* info);

/* ---------------------------------------------------------------------------------------
 * BDDC preconditioner (two levels: box subdomains of cells and a coarse problem).
 * Replaces mlbddc_t (Sources/Lib/LinearAlgebra/Preconditioner/mlbddc.f90,
 * sbm_base_mlbddc.i90:162-1527) built on a par_fe_space_t with the standard coarse FE
 * handler (Sources/Lib/Integration/FESpace/sbm_standard_coarse_fe_handler.i90): the same
 * apply (interior correction, weighted coarse + constrained-Neumann correction, weighted
 * sum, harmonic extension; sbm_base_mlbddc.i90:909-1009), one coarse dof per object and
 * component with per-component averages as constraints (:121-219), multiplicity weights
 * (:221-295).  The subdomain and coarse matrices are factorised by FP64 Cholesky on the
 * device (the reference calls a sparse direct solver).  Objects come from the box grid:
 * interface nodes on slab planes in all three directions are vertices (primal, or with
 * use_vertices = 0 interface dofs without coarse dofs: the constrained Neumann problems are
 * then solved with the constraints added to the local matrix as an augmented Lagrangian,
 * which leaves the operator unchanged), nodes on two interior cut planes edge points, on
 * one a face point.  Subdomain matrices are dense: the library refuses (FG_ERR_OOM) a
 * partition whose dense local matrices do not fit the context's HBM budget. */
typedef struct fg_bddc fg_bddc;
enum { FG_PREC_BDDC = 2 };
enum { FG_BDDC_WEIGHT_MULTIPLICITY = 0, FG_BDDC_WEIGHT_STIFFNESS = 1, FG_BDDC_WEIGHT_SUBPART = 2 };
/* Coarse FE handler.  STANDARD: sbm_standard_coarse_fe_handler.i90 (one coarse dof per
 * object and component, algebraic averages).  ELASTICITY: elasticity_pb_bddc_l1_coarse_fe_handler_t
 * (sbm_elasticity_coarse_fe_handler.i90:75-381): 3 coarse dofs per vertex, no edge
 * constraints (use_edges must be 0), and per face 6 functionals -- the 3 translations and 3
 * rotations r4 = (y,-x,0), r5 = (-z,0,x), r6 = (0,z,-y) -- each the face integral of the
 * shape functions times the mode over the face measure (strategy "CI", :180-381); a face's
 * rows reach its edge and vertex dofs.  The rotations are taken about the face's centroid and
 * scaled by its size: the same span of functionals, hence the same preconditioner, with a
 * constraint Schur complement that stays well-conditioned for the FP32 factors.
 * Vector-valued (3-component) spaces only. */
enum { FG_BDDC_HANDLER_STANDARD = 0, FG_BDDC_HANDLER_ELASTICITY = 1 };
typedef struct {
  int32_t nsub[3];         /* subdomains per direction                                     */
  const int32_t* cuts;     /* NULL: even split; else nsub[0]+1, nsub[1]+1, nsub[2]+1 increasing
                              cell indices per direction, from 0 to n[d]                   */
  int32_t use_vertices;    /* coarse_space_use_vertices                                     */
  int32_t use_edges;       /* coarse_space_use_edges                                       */
  int32_t use_faces;       /* coarse_space_use_faces                                       */
  int32_t weighting;       /* FG_BDDC_WEIGHT_MULTIPLICITY (reference standard handler) or
                              FG_BDDC_WEIGHT_STIFFNESS (diag(A_i) / sum_j diag(A_j))        */
  int32_t coarse_handler;  /* FG_BDDC_HANDLER_STANDARD (default) or FG_BDDC_HANDLER_ELASTICITY */
  int32_t use_subparts;    /* physics-based partition (the reference's pb_bddc): a subdomain's
                              cells split into subparts (face-connected cells of equal cell
                              coefficient); interface dofs are grouped by the subparts around
                              them, a face object being the dofs whose cells belong to exactly
                              two subparts, one on each side; with FG_BDDC_WEIGHT_SUBPART the
                              weight of subdomain i is the sum of the coefficients of its
                              subparts around the dof over that of all of them
                              (sbm_elasticity_coarse_fe_handler.i90:422-516).  Elasticity
                              handler, faces only (use_edges = 0)                          */
} fg_bddc_params;
typedef struct {
  int32_t num_subdomains;
  int32_t max_local_dofs;
  int64_t num_interface_dofs;
  int64_t num_coarse_dofs;
  double symbolic_ms, numeric_ms;
  uint64_t device_bytes;
  double factor_flops;     /* FP64 flops of the batched subdomain partial Cholesky        */
  double factor_ms;        /* its device time in the last numerical setup (CUDA events)   */
  double coarse_ms;        /* coarse assembly + factorisation + inverse, device time      */
} fg_bddc_info;
void fg_bddc_params_default(fg_bddc_params* p);
/* symbolic_setup + numerical_setup (sbm_base_mlbddc.i90:162-201,437-474) on the system's
 * current element matrices.  The system must stay alive while the preconditioner does. */
fg_status fg_bddc_create(fg_system* sys, const fg_bddc_params* params, fg_bddc** out);
/* numerical_setup again after fg_system_reassemble (same mesh, space and partition). */
fg_status fg_bddc_numerical_setup(fg_bddc* bddc);
fg_status fg_bddc_get_info(fg_bddc* bddc, fg_bddc_info* info);
/* z = M^-1 r (base_mlbddc_apply, sbm_base_mlbddc.i90:853-1009) on device vectors of
 * num_free FP64 entries in free-dof order.  precision FG_MIXED applies the FP32 copies of
 * the factors (inputs and outputs stay FP64). */
fg_status fg_bddc_apply_device(fg_bddc* bddc, int precision, const double* r_dev, double* z_dev);
/* PCG preconditioned by the BDDC (cg.f90:101-407 with mlbddc_t as the preconditioner):
 * params as for fg_solve (precond is ignored; every stopping criterion is supported).
 * FG_FP64: all FP64.  FG_MIXED: FP64 Krylov vectors, SpMV and dots; FP32 preconditioner
 * (factors, local vectors and the two SpMVs inside the apply). */
fg_status fg_bddc_solve(fg_bddc* bddc, const fg_solver_params* params, const double* b, const double* x0,
                        double* x, fg_solve_info* info);
fg_status fg_bddc_solve_device(fg_bddc* bddc, const fg_solver_params* params, const double* b_dev,
                               const double* x0_dev, double* x_dev, fg_solve_info* info);
fg_status fg_bddc_destroy(fg_bddc* bddc);

/* ---------------------------------------------------------------------------------------
 * Batched independent Poisson problems in one persistent launch.  No counterpart in the
 * reference (FEMPAR solves one problem per program); each problem is the tutorial /
 * test_poisson path: -div(k grad u) = f on the unit cube with n^3 uniform hexahedra, Q1-Q3
 * Lagrangian elements, (order+1)^3 Gauss points, constant k, f given at the Gauss points,
 * u = 0 on the whole boundary, Jacobi-PCG (cg.f90:101-238, jacobi_preconditioner.f90:356-412)
 * to ||b - A x|| <= rtol ||b|| + atol.  Assembly (the load vector; the operator is applied
 * matrix-free from the uniform cell matrix) and the solve are fused in one cooperative
 * kernel; FP32 CG with float-float (~2^-48) solution, right-hand side and true residuals.
 * A plan (fg_batch_create) fixes the problems' sizes and buffers, schedules teams of CTAs,
 * picks the block size (threads = 0: the fastest of 128/256/512 on this batch, timed once)
 * and captures the launch in a CUDA graph; fg_batch_run re-runs it on the current source
 * values. */
typedef struct fg_batch fg_batch;
typedef struct {
  int32_t n;                 /* cells per direction                                      */
  int32_t order;             /* 1..3                                                     */
  double coef;               /* diffusion coefficient k > 0                              */
  const double* qp_source;   /* n^3 (order+1)^3 values of f at the Gauss points: cells in
                                lexicographic order, points x fastest (FG_FN_QP_VALUES)   */
  double* x;                 /* out: (order n - 1)^3 values at the interior lattice nodes,
                                x fastest (node (i,j,k), 1 <= i,j,k <= order n - 1)       */
} fg_batch_problem;
typedef struct {
  int32_t status;            /* FG_OK, FG_ERR_NOT_CONVERGED, FG_ERR_NUMERIC, FG_ERR_TIMEOUT */
  int32_t iterations;
  int32_t refinements;       /* float-float true residuals computed                      */
  int32_t team;              /* CTAs that solved the problem                             */
  double rel_residual;       /* last ||b - A x|| / ||b||                                 */
} fg_batch_result;
typedef struct {
  int32_t threads, ctas, max_team, teams_gt1, graph;
  int64_t total_dofs;
  double predicted_balance;  /* planner's estimate: mean CTA load / the longest            */
  double run_ms;             /* last fg_batch_run (device events, copies included)         */
  double autotune_ms;
  double team_share;         /* team sizing chosen (with threads) by the autotuner: a problem
                                gets ceil(work / (team_share x a CTA's share)) CTAs         */
} fg_batch_info;
/* flags: FG_INPUTS_ON_DEVICE = qp_source and x are device pointers (read / written in place
 * at every run); otherwise host pointers, copied in and out by every run.  params: rtol,
 * atol, max_iters, inner_rtol (reliable-update factor, 0 = 0.1); the rest is ignored. */
fg_status fg_batch_create(fg_ctx* ctx, int32_t nprob, const fg_batch_problem* problems, int32_t flags,
                          const fg_solver_params* params, int32_t threads, fg_batch** out);
/* results: NULL or nprob entries.  Returns the worst status over the problems. */
fg_status fg_batch_run(fg_batch* batch, fg_batch_result* results);
fg_status fg_batch_get_info(fg_batch* batch, fg_batch_info* info);
fg_status fg_batch_destroy(fg_batch* batch);

/* ---------------------------------------------------------------------------------------
 * Serving: a device-resident request loop.  No counterpart in the reference (FEMPAR runs
 * one problem per program); built from the entry points above.  Worker threads each own a
 * context (its own CUDA stream) on one device; a request (mesh, FE space, integrand,
 * solver parameters) is admitted when its estimated device footprint fits the remaining
 * HBM budget, queued per size class (log2 of its dofs) and taken oldest-first among the
 * classes whose head fits; admitted requests run concurrently and overlap on the GPU.
 * Each request's mesh, matrix and Krylov state live on the device until its solution is
 * copied out; a request whose footprint exceeds the whole budget is refused at submit.
 * Results do not depend on what else runs: kernels use fixed grids and reductions. */
typedef struct fg_server fg_server;

typedef struct {
  int kind;                     /* FG_POISSON / FG_ELASTICITY                          */
  int32_t n[3];                 /* cells per direction (unit cube)                     */
  int order;                    /* 1..3                                                */
  const double* cell_coef;      /* host, ncells (copied at submit); NULL = coef_const  */
  double coef_const, nu;
  int source_fn;                /* FG_FN_ZERO / FG_FN_CONST                            */
  double fn_param[8];
  const int32_t* dirichlet_ids; /* copied at submit                                    */
  int n_ids;
  fg_solver_params solver;
} fg_request;

typedef struct {
  fg_status status;             /* of the request's own calls                          */
  int iterations, outer_iterations;
  int64_t num_free;
  double t_queue_ms;            /* submit -> start                                     */
  double t_run_ms;              /* start -> solution on the host                       */
  double t_total_ms;            /* submit -> solution on the host                      */
  double solve_ms;              /* device time of the solve                            */
  uint64_t footprint_bytes;
} fg_result;

/* Estimated device bytes of a request (admission unit) and its free-dof count. */
fg_status fg_request_footprint(const fg_request* req, uint64_t* bytes, int64_t* num_free);
fg_status fg_server_create(int device, uint64_t hbm_budget_bytes, int nworkers, fg_server** out);
fg_status fg_server_submit(fg_server* srv, const fg_request* req, uint64_t* ticket);
/* Wait up to timeout_ms (< 0: forever) for a request; FG_ERR_TIMEOUT if not finished. */
fg_status fg_server_wait(fg_server* srv, uint64_t ticket, int timeout_ms, fg_result* res);
/* Copy the solution (num_free doubles, reference dof order) and release the request. */
fg_status fg_server_take_solution(fg_server* srv, uint64_t ticket, double* x);
/* Peak device bytes reserved by admitted requests so far. */
fg_status fg_server_stats(fg_server* srv, uint64_t* peak_reserved, int64_t* completed);
fg_status fg_server_destroy(fg_server* srv);

/* ---------------------------------------------------------------------------------------
 * Dense FP64 product on the bf16 tensor cores: C = alpha A B^T + beta C with A m x k,
 * B n x k, C m x n; element (i, l) of A at A[i*a_rs + l*a_cs] (likewise B, C), device
 * pointers, on the context's stream, synchronous.  B = NULL: B = A (needs n = m).
 * flags: FG_DENSE_LOWER writes only the elements with i >= j.  FP64 is emulated by 7 signed
 * 8-bit digits per value and row (Ozaki scheme) with 56 bits below the row's maximum; the
 * result is within ~k 2^-53 max|A_i.| max|B_j.| of the exact product (the FP64 dot-product
 * bound), plus the FP64 rounding of the update.  No counterpart in the
 * reference (its dense factorisations call MKL / PARDISO); the building block of the BDDC
 * set-up's factorisations.  Returns FG_ERR_TIMEOUT if a bounded device wait ran out. */
#define FG_DENSE_LOWER 1
fg_status fg_dense_gemm_nt(fg_ctx* ctx, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
                           int64_t a_rs, int64_t a_cs, const double* B, int64_t b_rs, int64_t b_cs, double beta,
                           double* C, int64_t c_rs, int64_t c_cs, int32_t flags);

/* Default parameters (reference defaults: CG, res_res, rtol 1e-6, 1000 iterations). */
void fg_solver_params_default(fg_solver_params* p);
void fg_integrand_default(fg_integrand* g);

#ifdef __cplusplus
}
#endif
#endif

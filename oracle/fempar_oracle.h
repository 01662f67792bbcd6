/*
 * fempar_oracle.h -- CPU restatement of FEMPAR's serial assembly + CG path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU path:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
 * arm may load it.  The product library (libfempar_gpu.so) never links it.
 *
 * What it restates (reference paths are relative to the fempar source tree):
 *   structured hex/quad mesh     Sources/Lib/Geometry/Tools/uniform_hex_mesh_generator.f90:145-647
 *   unstructured hex mesh vefs   Sources/Lib/Geometry/Triangulation/sbm_fine_triangulation.i90:115-527,
 *                                Sources/Lib/Geometry/Triangulation/sbm_base_static_triangulation.i90:697-739
 *   polytope n-faces, nodes      Sources/Lib/Integration/ReferenceFE/sbm_polytope.i90:175-433,640-860
 *   own-dof lists, components    Sources/Lib/Integration/ReferenceFE/sbm_lagrangian_reference_fe.i90:1072-1153,1240-1285,1549-1758
 *   Dirichlet-first numbering    Sources/Lib/Integration/FESpace/sbm_serial_fe_space.i90:525-716
 *   free dof numbering           Sources/Lib/Integration/FESpace/sbm_serial_fe_space.i90:2623-2884
 *                                Sources/Lib/Integration/FESpace/sbm_fe_cell_iterator.i90:352-856
 *   Gauss-Legendre quadrature    Sources/Lib/Integration/ReferenceFE/sbm_quadrature.i90:767-823
 *   1D Lagrange basis            Sources/Lib/Integration/ReferenceFE/sbm_polynomial.i90:61-109
 *   tensor-product shapes        Sources/Lib/Integration/ReferenceFE/sbm_tensor_product_polynomial.i90:28-120
 *   Jacobian / invmtx            Sources/Lib/Integration/ReferenceFE/sbm_base_map.i90:100-106,
 *                                Sources/Lib/Integration/Tools/field.f90:763-787,
 *                                Sources/Lib/Integration/ReferenceFE/sbm_cell_map.i90:245-369,
 *                                Sources/Lib/Integration/ReferenceFE/sbm_cell_integrator.i90:448-500
 *   physical gradients           Sources/Lib/Integration/ReferenceFE/sbm_lagrangian_reference_fe.i90:1306-1342
 *   Poisson integrand            Tutorials/tutorial_01_poisson_sharp_circular_wave/modules/...modules.f90:71-137
 *   dG interior penalty          ...modules.f90:146-322; facet geometry: Sources/Lib/Integration/ReferenceFE/
 *                                sbm_facet_integrator.i90:212-264, sbm_facet_map.i90:74-128, sbm_cell_map.i90:429-461
 *   elasticity integrand         Sources/Tests/Par/par_test_pb_bddc_linear_elasticity/modules/
 *                                sbm_irreducible_discrete_integration.i90:46-135
 *   Dirichlet lifting            Sources/Lib/Integration/FESpace/sbm_fe_cell_iterator.i90:1610-1637
 *   COO append (upper, >=1)      Sources/Lib/LinearAlgebra/SparseMatrix/base_sparse_matrix.f90:3469-3513
 *   sort_and_compress            Sources/Lib/LinearAlgebra/SparseMatrix/base_sparse_matrix.f90:4121-4829
 *   CSR SpMV (sym. storage)      Sources/Lib/LinearAlgebra/SparseMatrix/csr_sparse_matrix.f90:545-623
 *   extract_diagonal             Sources/Lib/LinearAlgebra/SparseMatrix/csr_sparse_matrix.f90:4231-4256
 *   CG + stopping criteria       Sources/Lib/LinearAlgebra/IterativeLinearSolver/cg.f90:101-407
 *   Jacobi                       Sources/Lib/LinearAlgebra/Preconditioner/jacobi_preconditioner.f90:356-412
 *   energy-norm true error       Tutorials/tutorial_01_poisson_sharp_circular_wave/modules/...modules.f90:542-679
 */
#ifndef FEMPAR_ORACLE_H
#define FEMPAR_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Integrand kinds. */
enum { ORC_POISSON = 0, ORC_ELASTICITY = 1 };

/* Source / boundary function ids (scalar problems). */
enum {
  ORC_FN_ZERO = 0,          /* f = 0                                        */
  ORC_FN_CONST = 1,         /* f = fn_param[0]                              */
  ORC_FN_SHARP_WAVE = 2,    /* tutorial_01: u = atan(a(|x-c|-r)), f = -lap u  (params a, r, cx, cy, cz) */
  ORC_FN_LINEAR = 3,        /* test_poisson: u = x+y(+z), f = 0             */
  ORC_FN_QP_VALUES = 4      /* source given per quadrature point (ncells*nq) */
};

typedef struct {
  int num_dims;             /* 2 or 3                                        */
  int n[3];                 /* cells per direction                           */
  double limits[6];         /* xmin,xmax,ymin,ymax,zmin,zmax                 */
  const double* vertex_xyz; /* optional 3*(n0+1)(n1+1)(n2+1) coordinates, x-fastest lattice; NULL = uniform */
  int order;                /* Lagrange order p                              */
  int kind;                 /* ORC_POISSON / ORC_ELASTICITY                  */
  int dirichlet_ids[27];    /* polytope boundary set ids that are Dirichlet  */
  int n_dirichlet_ids;
  const double* cell_coef;  /* optional per-cell k (Poisson) or E (elasticity); NULL = 1 */
  double nu;                /* Poisson ratio (elasticity)                    */
  int source_fn;            /* ORC_FN_*                                      */
  double fn_param[8];       /* parameters of the analytic functions / const  */
  const double* qp_source;  /* ORC_FN_QP_VALUES: ncells*nq*ncomp values      */
  int boundary_fn;          /* ORC_FN_* for the Dirichlet data               */
  int translated_jacobian;  /* 1 = reuse cell-1 Jacobian (reference structured-mesh shortcut) */
  int nthreads;             /* threads for the assembly (1 = the reference's serial COO append and
                               sort_and_compress; >1 = the same CSR, bit for bit, built by chunks
                               of cells on that many threads) */
  int formulation;          /* ORC_CG, or ORC_DG: tutorial_01's interior-penalty dG (Poisson, k = 1) */
} orc_params;

enum { ORC_CG = 0, ORC_DG = 1 };

typedef struct orc_problem orc_problem;

/* Unstructured hexahedral mesh, as the GiD reader hands it to the serial triangulation
 * (sbm_serial_triangulation.i90:120-188): vertices, cells (8 vertex ids each, 1-based, in the
 * reference FE's lexicographic local order) and the given boundary vefs with their set ids.
 * Vefs are generated by first appearance (sbm_fine_triangulation.i90:115-315), given set ids
 * assigned (:317-444) and handed from boundary faces to their edges/vertices (:453-527). */
typedef struct {
  int64_t num_vertices;
  const double* coords;               /* 3*num_vertices                       */
  int64_t num_cells;
  const int32_t* cell_vertices;       /* 8*num_cells, 1-based                 */
  int64_t num_given_vefs;
  const int64_t* given_vef_ptr;       /* num_given_vefs+1 offsets             */
  const int32_t* given_vef_vertices;  /* 1-based vertex ids                   */
  const int32_t* given_vef_set;       /* set id of each given vef             */
} orc_umesh;

/* Build mesh, dof numbering, Dirichlet values, element integration, COO and CSR. */
orc_problem* orc_create(const orc_params* p);
void orc_destroy(orc_problem* h);
/* Same on an unstructured hexahedral mesh (num_dims 3; n, limits, vertex_xyz unused;
 * dirichlet_ids are the mesh's set ids, 1..63). */
orc_problem* orc_create_unstructured(const orc_params* p, const orc_umesh* m);
/* Vefs of the unstructured mesh: total (vertices + edges + faces), edges and faces. */
int64_t orc_num_vefs(const orc_problem* h, int64_t* num_edges, int64_t* num_faces);
void orc_get_cell_vefs(const orc_problem* h, int32_t* out);   /* ncells*26, 1-based vef gids */
void orc_get_vef_sets(const orc_problem* h, int32_t* out);    /* nvefs set ids               */

/* Sizes. */
int64_t orc_num_cells(const orc_problem* h);
int     orc_dofs_per_cell(const orc_problem* h);
int     orc_qp_per_cell(const orc_problem* h);
int64_t orc_num_free(const orc_problem* h);
int64_t orc_num_dirichlet(const orc_problem* h);
int64_t orc_nnz_upper(const orc_problem* h);
int64_t orc_coo_entries(const orc_problem* h);

/* Copies out (caller-allocated). */
void orc_get_dof_map(const orc_problem* h, int32_t* lst_dofs_gids);      /* ncells*nd, reference convention */
void orc_get_csr_upper(const orc_problem* h, int64_t* irp, int32_t* ja, double* val); /* 1-based */
void orc_get_rhs(const orc_problem* h, double* rhs);                     /* nfree */
void orc_get_dirichlet_values(const orc_problem* h, double* g);          /* ndir  */
void orc_get_elmat(const orc_problem* h, int64_t cell, double* elmat, double* elvec); /* before lifting of elvec? no: after */

/* Physical quadrature-point coordinates of every cell (sbm_cell_map.i90:673-686): ncells*nq*3. */
void orc_get_qp_coords(const orc_problem* h, double* xyz);

/* Stage timings of orc_create (seconds): mesh+numbering, integration+COO, sort_and_compress. */
void orc_get_timings(const orc_problem* h, double* t3);

/* Stopping criteria (cg.f90 names). */
enum { ORC_RES_RES = 0, ORC_RES_RHS = 1, ORC_DELTA_RHS = 2, ORC_DELTA_DELTA = 3,
       ORC_RES_NRMGIVEN_RHS_NRMGIVEN = 4, ORC_RES_NRMGIVEN_RES_NRMGIVEN = 5 };

/* PCG on the assembled upper-triangle CSR (symmetric-storage SpMV).
 * precond: 0 = identity, 1 = Jacobi.  x0 may be NULL (zero initial guess).
 * history (optional, length maxit) receives the per-iteration error estimate. */
int orc_cg(const orc_problem* h, int precond, double rtol, double atol, int maxit, int criterion,
           const double* b, const double* x0, double* x, int* iters, double* history, int nthreads);

/* orc_cg with per-iteration timestamps: it_time (optional, length maxit) receives the seconds
 * from the call's start (its set-up included) to the end of each iteration.  With
 * nthreads > 1 the SpMV is the symmetric-storage kernel on nthreads threads (each thread's
 * rows, transposed contributions past its rows in a private buffer added in thread order)
 * and reductions are summed in thread order: deterministic for a thread count, equal to the
 * serial kernel's results to rounding.  nthreads < -1: the same on -nthreads threads with the
 * matrix first expanded to a full CSR and a row-gather SpMV (twice the bytes, no scatter). */
int orc_cg_timed(const orc_problem* h, int precond, double rtol, double atol, int maxit, int criterion,
                 const double* b, const double* x0, double* x, int* iters, double* history, int nthreads,
                 double* it_time);

/* y = A x with the reference symmetric-storage kernel. */
void orc_spmv(const orc_problem* h, const double* x, double* y);

/* Energy-norm true error sqrt(sum_K int_K |grad(u - u_h)|^2) for the analytic solution of
 * boundary_fn (sharp wave or linear), u_h given by free values x and the Dirichlet values. */
double orc_energy_error(const orc_problem* h, const double* x);
/* Scalar error norms of x against the analytic fn (sbm_error_norms_scalar.i90:115-241),
 * before finalize_norm: out = mean, l1, l2^2, linfty, |grad e|^2, w1infty. */
void orc_error_norms(const orc_problem* h, const double* x, int fn, const double* prm, double* out);

/* Gauss-Legendre nodes/weights on [-1,1] (n points). */
void orc_gauss_legendre(int n, double* x, double* w);

/* Reference-FE tables used by the GPU library's own tables (for cross-checks):
 * own-dof list of n-face `iface` (1-based polytope index, volume last). Returns count. */
int orc_own_dofs(int num_dims, int order, int ncomp, int iface, int32_t* out);
/* polytope n-face codes sorted (returns count, 9 in 2D / 27 in 3D) */
int orc_polytope_codes(int num_dims, int32_t* codes);

#ifdef __cplusplus
}
#endif
#endif

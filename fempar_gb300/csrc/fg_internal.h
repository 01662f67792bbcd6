// fg_internal.h -- internal types of libfempar_gpu.so (not part of the C-ABI).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "../../include/fempar_gpu.h"

#define FG_MAX_ORDER 3
#define FG_MAX_NN 64          // nodes per cell, Q3 hex
#define FG_MAX_NQ 64          // quadrature points per cell, Q3 hex

namespace fg {

void set_error(const char* fmt, ...);

#define FG_CUDA_TRY(expr)                                                                   \
  do {                                                                                      \
    cudaError_t e_ = (expr);                                                                \
    if (e_ != cudaSuccess) {                                                                \
      ::fg::set_error("%s:%d %s: %s", __FILE__, __LINE__, #expr, cudaGetErrorString(e_));   \
      return e_ == cudaErrorMemoryAllocation ? FG_ERR_OOM : FG_ERR_CUDA;                     \
    }                                                                                       \
  } while (0)

#define FG_TRY(expr)                   \
  do {                                 \
    fg_status s_ = (expr);             \
    if (s_ != FG_OK) return s_;        \
  } while (0)

// Host-side reference-element tables for a Lagrangian hex FE of order p with ncomp
// components, and the Q1 geometry map, evaluated at the (p+1)^3 Gauss points.
struct RefTables {
  int dim = 3, order = 1, ncomp = 1;
  int nn = 0;        // nodes per cell (p+1)^3
  int nd = 0;        // dofs per cell nn*ncomp
  int nq = 0;        // quadrature points (p+1)^3
  int codes[27];     // polytope n-face codes sorted by (dim, code); volume last
  int code2idx[64];  // inverse of codes (-1 if absent)
  std::vector<double> qw;     // nq
  std::vector<double> shp;    // nn*nq     shape values
  std::vector<double> shg;    // nn*nq*3   reference gradients
  std::vector<double> gshp;   // 8*nq      Q1 geometry shapes
  std::vector<double> gshg;   // 8*nq*3    Q1 geometry gradients
  std::vector<double> gnod;   // 8*nn      Q1 geometry shapes at the FE nodes
  void build(int order, int ncomp);
  // quadrilateral (dim 2): (p+1)^2 nodes and points, 9 n-faces (anchor | free << 2), 4
  // geometry nodes; gradients keep 3 slots with the third zero
  void build2d(int order, int ncomp);
};

// One row class of the lattice-implicit SELL layout (fg_stencil.cu).
struct StencilClass {
  int64_t vbase;   // first value of the class in class-by-class storage (set-up only)
  int64_t sbase;   // first slice of the class in class-by-class numbering (set-up only)
  int64_t nrows;   // rows of the class
  int lo[3], w[3]; // box start (relative to the row's node) and width per direction
  int B, Bp;       // box entries (all components) and the 4-padded count
  int offbase;     // first entry of the class in the offset table
  int64_t ownoff;  // start of the class's sub-lattice in the solver vector
};

enum { FG_LAYOUT_STENCIL = 0, FG_LAYOUT_SELL = 1 };

// Device copy of the tables in one buffer.
struct DevTables {
  double* base = nullptr;
  const double* qw;
  const double* shp;
  const double* shg;
  const double* gshp;
  const double* gshg;
  const double* gnod;
  size_t bytes = 0;
  // reference gradients as float-float pairs (hi, lo), for the float-float integration
  float* fbase = nullptr;
  const float* shgh;
  const float* shgl;
};

}  // namespace fg

struct fg_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  uint64_t budget = 0;
  uint64_t in_use = 0;
  int64_t launches = 0;           // kernels launched through this context
  std::map<void*, size_t> allocs;
};

struct fg_mesh {
  fg_ctx* ctx = nullptr;
  int dim = 3;
  int n[3] = {0, 0, 0};
  double limits[6];
  int64_t ncells = 0, nverts = 0;
  double* d_coords = nullptr;  // 3*nverts, interleaved xyz, x-fastest lattice (structured)
  // unstructured hexahedral mesh (fg_mesh_create_unstructured, fg_mesh_read_gid); n = {ncells,1,1}
  bool unst = false;
  int64_t nedges = 0, nfaces = 0, nvefs = 0;
  int max_vcells = 0;              // most cells around one vertex
  int32_t* d_cellvert = nullptr;   // 8*ncells vertex ids, 0-based, lexicographic local order
  int32_t* d_cellvef = nullptr;    // 26*ncells vef ids (vertices, edges, faces), 0-based
  int32_t* d_vset = nullptr;       // nvefs boundary set ids
  int64_t* d_vowner = nullptr;     // nedges+nfaces: first cell * 32 + local n-face
  int32_t* d_vnbr = nullptr;       // nedges+nfaces: cells holding the vef
  int64_t* d_vptr = nullptr;       // nverts+1 offsets of the cells around each vertex
  int32_t* d_vcells = nullptr;     // cells around each vertex, ascending
};

struct fg_space {
  fg_mesh* mesh = nullptr;
  fg::RefTables tab;
  fg::DevTables dtab;
  int order = 1, ncomp = 1;
  int Ln[3];                      // lattice nodes per direction: p*n+1
  int64_t nlat = 0;               // lattice nodes
  uint32_t dirmask = 0;           // bit s set: boundary set id s is strong Dirichlet
  int64_t nfree = 0, ndir = 0;
  int32_t* d_latdof = nullptr;    // nlat*ncomp: +id free (1-based), -id Dirichlet, 0 never
  int32_t* d_free2lat = nullptr;  // nfree: lattice slot L*ncomp+comp of each free dof
  int32_t* d_dir2lat = nullptr;   // ndir: lattice slot of each Dirichlet dof
  // full CSR pattern of the free-dof matrix, 0-based sorted columns
  int64_t nnz = 0;
  int64_t* d_rowptr = nullptr;    // nfree+1
  int32_t* d_col = nullptr;       // nnz
  int64_t nnz_upper = 0;
  int box_cap = 0;                // power-of-two capacity of a row's neighbour box
  // SELL-C-sigma pattern of the same matrix (solver layout, slot order)
  int64_t nslices = 0, sell_nnz = 0;
  int32_t* d_perm = nullptr;      // slot -> row
  int32_t* d_iperm = nullptr;     // row -> slot
  int64_t* d_sptr = nullptr;      // nslices+1 entry offsets
  int32_t* d_scol = nullptr;      // sell_nnz column slots
  // solver layout: FG_LAYOUT_STENCIL (lattice-implicit SELL, default) or FG_LAYOUT_SELL
  int layout = 0;
  int64_t nvec = 0;               // solver vector length
  int32_t* d_row2vec = nullptr;   // free row -> solver vector index
  // lattice-implicit SELL
  int halo = 0, Pn[3] = {0, 0, 0};
  int st_ncls = 0;
  int64_t st_nslices = 0, st_nvals = 0;
  fg::StencilClass* d_st_cls = nullptr;
  int32_t* d_st_off = nullptr;    // box offsets per class
  uint8_t* d_st_scls = nullptr;   // class of each slice
  int64_t* d_st_voff = nullptr;   // first value of each slice (slices are stored interleaved)
  int32_t* d_st_row = nullptr;    // 32*st_nslices: solver vector index of each row slot
  int32_t* d_row2st = nullptr;    // free row -> row slot
  int32_t* d_st_slot2row = nullptr;  // 32*st_nslices: free row of each row slot (-1: padding)
  int st_max_bp = 0;              // largest Bp of the classes
  std::vector<fg::StencilClass> h_st_cls;
  double* d_tcT = nullptr;        // Poisson element tensor T (upper pairs x 6 NQ), tensor-core path
  float* d_tcff = nullptr;        // float-float tables of its fast-integration geometry kernel
  // unstructured mesh: nodes (nlat of them) are vertices, edge, face and cell interior nodes
  int32_t* d_cellnode = nullptr;  // nn*ncells node ids
  int64_t* d_nptr = nullptr;      // nlat+1 offsets of the cells around each node
  int64_t* d_ncl = nullptr;       // (cell << 6 | local node), ascending per node
  int max_ncells = 0;             // most cells around one node
  int row_cap = 0;                // power of two >= the longest row
  // explicit node table (unstructured meshes, partitioned spaces): row gather through the
  // cells around each node instead of the lattice
  bool explicit_nodes = false;
  // discontinuous Galerkin space (fg_space_create_dg): cell-interior dofs, face neighbours
  bool dg = false;
  int32_t* d_dgnbr = nullptr;     // 6*ncells: neighbour across local face lf, -1 on the boundary
  int8_t* d_dgnbrface = nullptr;  // 6*ncells: the neighbour's local face
};

struct fg_system {
  fg_space* space = nullptr;
  double* d_val = nullptr;        // nnz FP64
  float* d_val32 = nullptr;       // nnz FP32 copy (mixed precision)
  double* d_rhs = nullptr;        // nfree
  double* d_gvals = nullptr;      // ndir Dirichlet values
  double* d_elmat = nullptr;      // ncells*nd*nd element matrices (scratch of the numeric phase)
  double* d_elvec = nullptr;      // ncells*nd
  double* d_coef = nullptr;       // ncells
  double* d_qpsrc = nullptr;      // optional per-qp source
  double* d_sval = nullptr;       // sell_nnz FP64 values (SELL layout)
  float* d_sval32 = nullptr;      // sell_nnz FP32 values (SELL layout)
  double* d_tval = nullptr;       // st_nvals FP64 values (lattice-implicit SELL layout)
  float* d_tval32 = nullptr;      // st_nvals FP32 values (lattice-implicit SELL layout)
  double* d_idiag = nullptr;      // nfree inverse diagonal (FP64, slot order)
  float* d_idiag32 = nullptr;     // nfree inverse diagonal (FP32, slot order)
  // mixed solves with Jacobi: FP32 copy of D^-1/2 A D^-1/2 in the solver layout and D^-1/2
  float* d_val32s = nullptr;      // st_nvals (lattice-implicit) or sell_nnz (SELL) values
  double* d_sdiag = nullptr;      // nvec
  bool scaled_valid = false;      // d_val32s matches the current values
  void* d_tcbuf = nullptr;        // scratch of the tensor-core element matrices (fg_assembly.cu)
  size_t tcbuf_bytes = 0;
  // solver work vectors (allocated on first solve)
  double* d_work = nullptr;       // FP64 work area
  float* d_work32 = nullptr;      // FP32 work area
  double* d_red = nullptr;        // reduction partials + scalars
  unsigned int* d_ticket = nullptr;
  int red_blocks = 0;
  fg_integrand integ;             // last integrand (host copy of scalars)
  bool lean = false;              // FG_LEAN_SYSTEM: element matrices and CSR values released
  bool direct = false;            // assembled straight into the lattice-implicit layout: the CSR
                                  // values (d_val) are derived from it only when exported
};

namespace fg {

// fg_refe.cpp: 1D Gauss-Legendre rule (n points on [-1,1], ascending) and the Lagrange basis
// of order p on equispaced nodes of [-1,1] (value and derivative of basis j at x)
void gl_rule(int n, double* x, double* w);
void lagrange_1d(int p, int j, double x, double& v, double& dv);

fg_status dev_alloc(fg_ctx* ctx, void** p, size_t bytes);
void dev_free(fg_ctx* ctx, void* p);
fg_status upload_tables(fg_ctx* ctx, const RefTables& t, DevTables& d);

// fg_space.cu
fg_status space_number_dofs(fg_space* sp);
fg_status space_build_pattern(fg_space* sp);
fg_status space_export_dof_map(fg_space* sp, int32_t* out_host);
fg_status space_dirichlet_coords(fg_space* sp, double* d_xyz);
fg_status space_export_upper(fg_space* sp, const double* d_val, int one_based, int64_t* irp, int32_t* ja,
                             double* val);

// fg_assembly.cu
fg_status system_interpolate_dirichlet(fg_system* sys, int boundary_fn, const double* prm);
fg_status system_assemble(fg_system* sys);
fg_status space_qp_coords(fg_space* sp, double* d_xyz);

fg_status scan_i64(fg_ctx* ctx, int64_t* a, int64_t n, int64_t* total);
fg_status space_count_upper(fg_space* sp);
// fg_quad.cu: 2D structured quadrilateral meshes
fg_status q2_number_dofs(fg_space* sp);
fg_status q2_build_pattern(fg_space* sp);
fg_status q2_export_dof_map(fg_space* sp, int32_t* out_host);
fg_status q2_dirichlet_coords(fg_space* sp, double* d_xyz);
fg_status q2_interpolate_dirichlet(fg_system* sys, int boundary_fn, const double* prm);
fg_status q2_assemble(fg_system* sys);

// fg_unstructured.cu
fg_status umesh_build_topology(fg_mesh* m, int64_t nb, const int64_t* bptr, const int32_t* bverts,
                               const int32_t* bset);
fg_status umesh_export_vefs(fg_mesh* m, int32_t* cell_vefs, int32_t* vef_sets);
fg_status uspace_number_dofs(fg_space* sp);
fg_status uspace_build_adjacency(fg_space* sp);
fg_status uspace_build_pattern(fg_space* sp);
fg_status uspace_export_dof_map(fg_space* sp, int32_t* out_host);
fg_status uspace_dirichlet_coords(fg_space* sp, double* d_xyz);
fg_status usystem_scatter(fg_system* sys);

// fg_dg.cu
fg_status dg_space_build(fg_space* sp);
fg_status dg_assemble_rows(fg_system* sys);

// fg_sell.cu
fg_status space_build_sell(fg_space* sp);
fg_status system_fill_sell(fg_system* sys);

// fg_stencil.cu
fg_status space_build_stencil(fg_space* sp);
fg_status system_fill_stencil(fg_system* sys);
// true when the row gather can write the lattice-implicit layout directly (3D structured
// continuous spaces whose widest class fits the kernel's shared-memory slice buffer)
bool stencil_direct_ok(const fg_space* sp);
// CSR values (d_val) of a directly assembled system, from its FP64 lattice-implicit values
fg_status system_ensure_csr(fg_system* sys);
// inverse diagonal from the FP64 lattice-implicit values (same numbers as from the CSR)
fg_status system_inv_diag_stencil(fg_system* sys);

// fg_solver.cu
fg_status system_prepare_diag(fg_system* sys);
fg_status system_spmv(fg_system* sys, int precision, const void* x, void* y, cudaStream_t st);
fg_status system_spmv_slot(fg_system* sys, int precision, const void* x, void* y, int reps, cudaStream_t st);
fg_status system_spmv_layout_noalloc(fg_system* sys, int precision, const void* xvec, void* yvec, cudaStream_t st);
fg_status system_solve(fg_system* sys, const fg_solver_params* prm, const double* d_b, const double* d_x0,
                       double* d_x, fg_solve_info* info);

// Dense FP64 product on the bf16 tensor cores (fg_ozaki.cu): C = alpha A B^T + beta C,
// B == nullptr means B = A; work holds ozaki_workspace_bytes(m, n, k, B == nullptr) bytes;
// d_err receives FG_ERR_TIMEOUT if a bounded device wait ran out.
size_t ozaki_workspace_bytes(int64_t m, int64_t n, int64_t k, bool same);
fg_status ozaki_gemm_nt(fg_ctx* ctx, cudaStream_t st, int64_t m, int64_t n, int64_t k, double alpha,
                        const double* A, int64_t a_rs, int64_t a_cs, const double* B, int64_t b_rs, int64_t b_cs,
                        double beta, double* C, int64_t c_rs, int64_t c_cs, bool lower, void* work, int* d_err);
// A batch of lower rank-k updates C_b -= P_b P_b^T (k_b <= 128, column-major with leading
// dimension ld_b), in one launch of each kernel; work holds ozaki_syrk_batch_bytes(b) bytes.
struct OzSyrk {
  const double* p;
  double* c;
  int64_t ld;
  int m, k;
};
size_t ozaki_syrk_batch_bytes(const std::vector<OzSyrk>& b);
fg_status ozaki_syrk_batch(fg_ctx* ctx, cudaStream_t st, const std::vector<OzSyrk>& b, void* work, size_t bytes,
                           int* d_err);

}  // namespace fg

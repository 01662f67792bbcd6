// fg_dg.cu -- discontinuous Galerkin (symmetric interior penalty) Poisson on the device: the
// second formulation of tutorial_01 (tutorial_01_poisson_sharp_circular_wave_modules.f90:146-322).
//
// Space: every dof is a cell-interior dof, numbered cell by cell in local order (id =
// c*nn + a + 1); boundary data enter weakly, so there are no strong Dirichlet dofs.  The row
// of dof (c, a) holds the dofs of c and of its face neighbours, blocks in increasing cell id.
//
// Numeric phase: the volume integrals come from the continuous path's cell kernel (identity
// node table, no lifting).  Then one warp per cell owns the cell's rows: it starts from the
// cell's element matrix and, face by face, integrates the facet terms that land in its rows
//   interior facet, cell side I, other side J (n_1 = n, n_2 = -n, n outward of the smaller
//   cell id, as the reference's first cell around the facet):
//     A(i_I, j_J) += w|J_F| ( -1/2 (grad phi_j^J . n_I) phi_i^I - 1/2 (grad phi_i^I . n_J) phi_j^J
//                             + C_IP/h phi_j^J phi_i^I (n_I . n_J) )
//   boundary facet:  A(i, j) += w|J_F| ( -(grad phi_j . n) phi_i - (grad phi_i . n) phi_j
//                                         + C_IP/h phi_i phi_j ),
//                    b(i) += w|J_F| ( -g (grad phi_i . n) + C_IP/h g phi_i )
// with C_IP = 10 p^2 and h = min over the facet's cells of 2 (prod_i |grad xi_i|^-1)^(1/3)
// (sbm_cell_map.i90:429-461, sbm_facet_integrator.i90:248-264).  Facet geometry per facet
// Gauss point ((p+1)^2 points): the bilinear map of the smaller cell's face vertices gives x,
// dx/ds, dx/dt; n = dx/ds x dx/dt, |n| the area element, n/|n| oriented outward of that
// cell (sbm_facet_map.i90:74-128); each cell evaluates its shapes at its own reference
// point of the facet point (the other cell through the face's shared corners).  Both cells
// of a facet compute it in the same frame, each keeps the rows it owns: deterministic, no
// facet matrices in HBM, no atomics.  The reference sums a diagonal entry's contributions in
// facet id order, this kernel in local face order: entries agree to rounding.
#include <cub/cub.cuh>

#include "fg_internal.h"

namespace fg {

static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// local face lf (0..5) of the hex = n-face 20 + lf in the reference order: xy(z=0), xy(z=1),
// xz(y=0), xz(y=1), yz(x=0), yz(x=1)
__host__ __device__ __forceinline__ void dg_face(int lf, int& d1, int& d2, int& dn, int& anchor) {
  const int dn_of[6] = {2, 2, 1, 1, 0, 0};
  dn = dn_of[lf];
  anchor = (lf & 1) << dn;
  d1 = dn == 0 ? 1 : 0;
  d2 = dn == 2 ? 1 : 2;
}

// ---- space ---------------------------------------------------------------------------
__global__ void k_dg_nbr_struct(int nx, int ny, int nz, int32_t* nbr, int8_t* nbrface) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nc = (int64_t)nx * ny * nz;
  if (idx >= nc * 6) return;
  const int64_t c = idx / 6;
  const int lf = (int)(idx % 6);
  int d1, d2, dn, a;
  dg_face(lf, d1, d2, dn, a);
  const int n[3] = {nx, ny, nz};
  int ijk[3] = {(int)(c % nx), (int)((c / nx) % ny), (int)(c / ((int64_t)nx * ny))};
  const int side = (a >> dn) & 1;
  ijk[dn] += side ? 1 : -1;
  if (ijk[dn] < 0 || ijk[dn] >= n[dn]) {
    nbr[idx] = -1;
    nbrface[idx] = -1;
  } else {
    nbr[idx] = (int32_t)(ijk[0] + (int64_t)nx * (ijk[1] + (int64_t)ny * ijk[2]));
    nbrface[idx] = (int8_t)(lf ^ 1);
  }
}

// unstructured: the face's first cell is known (vowner); the other holder registers itself
__global__ void k_dg_second(int64_t nc, int64_t nv, const int32_t* cellvef, const int64_t* vowner, int64_t* second) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= nc * 6) return;
  const int64_t c = idx / 6;
  const int lf = (int)(idx % 6);
  const int64_t gid = cellvef[c * 26 + 20 + lf];
  if ((vowner[gid - nv] >> 5) != c) second[gid - nv] = c * 32 + 20 + lf;
}
__global__ void k_dg_nbr_unst(int64_t nc, int64_t nv, const int32_t* cellvef, const int64_t* vowner,
                              const int64_t* second, int32_t* nbr, int8_t* nbrface) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= nc * 6) return;
  const int64_t c = idx / 6;
  const int lf = (int)(idx % 6);
  const int64_t gid = cellvef[c * 26 + 20 + lf];
  const int64_t o = vowner[gid - nv];
  const int64_t s = (o >> 5) == c ? second[gid - nv] : o;
  nbr[idx] = s < 0 ? -1 : (int32_t)(s >> 5);
  nbrface[idx] = s < 0 ? (int8_t)-1 : (int8_t)((s & 31) - 20);
}

__global__ void k_dg_ids(int64_t n, int32_t* cellnode, int32_t* latdof, int32_t* free2lat) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  cellnode[i] = (int32_t)i;
  latdof[i] = (int32_t)(i + 1);
  free2lat[i] = (int32_t)i;
}

// blocks of a cell's rows: the cell and its neighbours, ascending
__device__ __forceinline__ int dg_blocks(int64_t c, const int32_t* nbr, int64_t* blk) {
  int nb = 0;
  blk[nb++] = c;
  for (int lf = 0; lf < 6; ++lf)
    if (nbr[c * 6 + lf] >= 0) blk[nb++] = nbr[c * 6 + lf];
  for (int i = 1; i < nb; ++i) {
    int64_t v = blk[i];
    int j = i - 1;
    while (j >= 0 && blk[j] > v) { blk[j + 1] = blk[j]; --j; }
    blk[j + 1] = v;
  }
  return nb;
}

__global__ void k_dg_rowlen(int64_t nc, int nn, const int32_t* nbr, int64_t* rowlen) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nc * nn) return;
  const int64_t c = r / nn;
  int nb = 1;
  for (int lf = 0; lf < 6; ++lf) nb += nbr[c * 6 + lf] >= 0;
  rowlen[r] = (int64_t)nb * nn;
}

__global__ void k_dg_cols(int64_t nc, int nn, const int32_t* nbr, const int64_t* rowptr, int32_t* col) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nc * nn) return;
  const int64_t c = r / nn;
  int64_t blk[7];
  const int nb = dg_blocks(c, nbr, blk);
  int64_t p = rowptr[r];
  for (int k = 0; k < nb; ++k)
    for (int b = 0; b < nn; ++b) col[p++] = (int32_t)(blk[k] * nn + b);
}

fg_status dg_space_build(fg_space* sp) {
  fg_mesh* m = sp->mesh;
  fg_ctx* ctx = m->ctx;
  const int64_t nc = m->ncells, nn = sp->tab.nn, n = nc * nn;
  if (n >= (int64_t)0x7fffffff) {
    set_error("dof count exceeds int32 ids");
    return FG_ERR_UNSUPPORTED;
  }
  sp->nlat = n;
  sp->nfree = n;
  sp->ndir = 0;
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_cellnode, sizeof(int32_t) * n));
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_latdof, sizeof(int32_t) * n));
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_free2lat, sizeof(int32_t) * n));
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_dir2lat, sizeof(int32_t)));
  k_dg_ids<<<nblk(n, 256), 256, 0, ctx->stream>>>(n, sp->d_cellnode, sp->d_latdof, sp->d_free2lat);
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_dgnbr, sizeof(int32_t) * nc * 6));
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_dgnbrface, sizeof(int8_t) * nc * 6));
  if (m->unst) {
    const int64_t nef = m->nedges + m->nfaces;
    int64_t* second = nullptr;
    FG_TRY(dev_alloc(ctx, (void**)&second, sizeof(int64_t) * (nef > 0 ? nef : 1)));
    FG_CUDA_TRY(cudaMemsetAsync(second, 0xff, sizeof(int64_t) * (nef > 0 ? nef : 1), ctx->stream));
    k_dg_second<<<nblk(nc * 6, 256), 256, 0, ctx->stream>>>(nc, m->nverts, m->d_cellvef, m->d_vowner, second);
    k_dg_nbr_unst<<<nblk(nc * 6, 256), 256, 0, ctx->stream>>>(nc, m->nverts, m->d_cellvef, m->d_vowner, second,
                                                               sp->d_dgnbr, sp->d_dgnbrface);
    FG_CUDA_TRY(cudaGetLastError());
    FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    dev_free(ctx, second);
  } else {
    k_dg_nbr_struct<<<nblk(nc * 6, 256), 256, 0, ctx->stream>>>(m->n[0], m->n[1], m->n[2], sp->d_dgnbr,
                                                                 sp->d_dgnbrface);
    FG_CUDA_TRY(cudaGetLastError());
  }
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_rowptr, sizeof(int64_t) * (n + 1)));
  k_dg_rowlen<<<nblk(n, 256), 256, 0, ctx->stream>>>(nc, (int)nn, sp->d_dgnbr, sp->d_rowptr);
  FG_CUDA_TRY(cudaGetLastError());
  int64_t nnz = 0;
  FG_TRY(scan_i64(ctx, sp->d_rowptr, n, &nnz));
  FG_CUDA_TRY(cudaMemcpyAsync(sp->d_rowptr + n, &nnz, sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
  sp->nnz = nnz;
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_col, sizeof(int32_t) * nnz));
  k_dg_cols<<<nblk(n, 256), 256, 0, ctx->stream>>>(nc, (int)nn, sp->d_dgnbr, sp->d_rowptr, sp->d_col);
  FG_CUDA_TRY(cudaGetLastError());
  sp->row_cap = 0;
  FG_TRY(space_count_upper(sp));
  ctx->launches += 6;
  return FG_OK;
}

// ---- numeric phase ------------------------------------------------------------------------
// weak Dirichlet data g at a facet point (the analytic functions of the drivers)
__device__ double dg_boundary_value(int fn, const double* prm, const double* x) {
  switch (fn) {
    case FG_FN_CONST: return prm[0];
    case FG_FN_LINEAR: return x[0] + x[1] + x[2];
    case FG_FN_SHARP_WAVE: {
      const double dx = x[0] - prm[2], dy = x[1] - prm[3], dz = x[2] - prm[4];
      return atan(prm[0] * (sqrt(dx * dx + dy * dy + dz * dz) - prm[1]));
    }
    default: return 0.0;
  }
}

struct DgParams {
  int nx, ny;             // structured lattice (vertex ids); unused on unstructured meshes
  const int32_t* cellvert;  // unstructured meshes (null on the lattice)
  double x1[4], w1[4];    // facet Gauss-Legendre rule, p+1 points
  double cip;             // 10 p^2
  int bfn;                // boundary function (weak Dirichlet data)
  double prm[8];
};

__device__ __forceinline__ int64_t dg_vertex(const DgParams& q, int64_t c, int k) {
  if (q.cellvert) return q.cellvert[c * 8 + k];
  const int64_t nx = q.nx, ny = q.ny;
  const int64_t ci = c % nx, cj = (c / nx) % ny, ck = c / (nx * ny);
  return (ci + (k & 1)) + (nx + 1) * ((cj + ((k >> 1) & 1)) + (ny + 1) * (ck + ((k >> 2) & 1)));
}

// 1D Lagrange basis of order P on equispaced nodes of [-1,1]: values and derivatives at x
template <int P>
__device__ __forceinline__ void lag1d(double x, double* v, double* dv) {
#pragma unroll
  for (int j = 0; j <= P; ++j) {
    const double xj = -1.0 + 2.0 * j / P;
    double val = 1.0, der = 0.0;
#pragma unroll
    for (int k = 0; k <= P; ++k) {
      if (k == j) continue;
      const double xk = -1.0 + 2.0 * k / P;
      const double inv = 1.0 / (xj - xk);
      der = der * ((x - xk) * inv) + val * inv;
      val = val * ((x - xk) * inv);
    }
    v[j] = val;
    dv[j] = der;
  }
}

// Jacobian of the trilinear map of vertices xv (8 x 3) at reference point xi: inverse (column-major,
// b[i + 3j] = d xi_i / d x_j), determinant, and h = 2 (prod_i |grad xi_i|^-1)^(1/3)
__device__ void dg_side_geometry(const double* xv, const double* xi, double* b, double& det, double& h) {
  double J[9];
  for (int j = 0; j < 3; ++j) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int k = 0; k < 8; ++k) {
      double g = 1.0;
      for (int d = 0; d < 3; ++d) {
        const double s = ((k >> d) & 1) ? 1.0 : -1.0;
        g *= d == j ? 0.5 * s : 0.5 * (1.0 + s * xi[d]);
      }
      a0 = a0 + g * xv[k * 3 + 0];
      a1 = a1 + g * xv[k * 3 + 1];
      a2 = a2 + g * xv[k * 3 + 2];
    }
    J[0 + 3 * j] = a0; J[1 + 3 * j] = a1; J[2 + 3 * j] = a2;
  }
  const double t1 = J[4] * J[8] - J[5] * J[7];
  const double t2 = -J[1] * J[8] + J[2] * J[7];
  const double t3 = J[1] * J[5] - J[2] * J[4];
  det = J[0] * t1 + J[3] * t2 + J[6] * t3;
  const double dn = 1.0 / det;
  b[0] = t1 * dn;
  b[1] = t2 * dn;
  b[2] = t3 * dn;
  b[4] = (J[0] * J[8] - J[2] * J[6]) * dn;
  b[5] = (-J[0] * J[5] + J[3] * J[2]) * dn;
  b[8] = (J[0] * J[4] - J[1] * J[3]) * dn;
  b[3] = (-J[3] * J[8] + J[5] * J[6]) * dn;
  b[6] = (J[3] * J[7] - J[4] * J[6]) * dn;
  b[7] = (-J[0] * J[7] + J[1] * J[6]) * dn;
  double ih[3];
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) s = s + b[i + 3 * j] * b[i + 3 * j];
    ih[i] = sqrt(s);
  }
  const double vh = 1.0 / (ih[0] * ih[1] * ih[2]);
  h = 2.0 * pow(vh, 1.0 / 3.0);
}

template <int P>
struct DgShape {
  static constexpr int NP1 = P + 1, NN = NP1 * NP1 * NP1, NQF = NP1 * NP1;
  static constexpr int WARPS = P == 3 ? 1 : (P == 2 ? 4 : 8);
  // per warp: D, O (NN*NN), rv (NN), V[2][NN], A[2][NN], xv[3][24], misc[40], 1D tables[2][3][4][2]
  static constexpr int DOUBLES = 2 * NN * NN + NN + 2 * NN + 2 * NN + 72 + 40 + 48;
  static constexpr size_t BYTES_WARP = (size_t)DOUBLES * 8;
};

template <int P>
__global__ void __launch_bounds__(DgShape<P>::WARPS * 32)
    k_dg_rows(int64_t nc, DgParams q, const double* __restrict__ coords, const int32_t* __restrict__ nbr,
              const int8_t* __restrict__ nbrface, const double* __restrict__ E, const double* __restrict__ EV,
              const int64_t* __restrict__ rowptr, double* __restrict__ val, float* __restrict__ val32,
              double* __restrict__ rhs) {
  using S = DgShape<P>;
  constexpr int NP1 = S::NP1, NN = S::NN, NQF = S::NQF;
  extern __shared__ double sm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  double* D = sm + (size_t)wib * (S::BYTES_WARP / 8);
  double* O = D + NN * NN;
  double* rv = O + NN * NN;
  double* sval = rv + NN;        // [2][NN] shape values of both sides
  double* sA = sval + 2 * NN;    // [2][NN] scaled normal derivatives of both sides
  double* xv = sA + 2 * NN;      // [3][24]: (unused), left cell, right cell
  double* misc = xv + 72;        // n[0..2], factor[3], g[5], b[2][9] at 6, xi[2][3] at 24, h[2] at 30, det at 32,
                                 // B n per side at 33..38
  double* tab = misc + 40;       // [side][dir][j][value, derivative] of the 1D basis
  const int64_t c = (int64_t)blockIdx.x * S::WARPS + wib;
  if (c >= nc) return;
  for (int t = lane; t < NN * NN; t += 32) D[t] = E[(size_t)c * NN * NN + t];
  for (int t = lane; t < NN; t += 32) rv[t] = EV[c * NN + t];
  int64_t blk[7];
  const int nb = dg_blocks(c, nbr, blk);
  __syncwarp();
  for (int lf = 0; lf < 6; ++lf) {
    const int64_t o = nbr[c * 6 + lf];
    const bool boundary = o < 0;
    const int64_t left = boundary ? c : (o < c ? o : c);
    const int64_t right = boundary ? -1 : (o < c ? c : o);
    const int flf = boundary ? lf : (o < c ? nbrface[c * 6 + lf] : lf);  // left cell's local face
    const int I = (left == c) ? 0 : 1;
    int ld1, ld2, ldn, la;
    dg_face(flf, ld1, ld2, ldn, la);
    // vertex coordinates of the left and right cells
    for (int t = lane; t < 48; t += 32) {
      const int side = t / 24, k = (t % 24) / 3, l = t % 3;
      const int64_t cc = side == 0 ? left : right;
      if (cc >= 0) xv[24 + t] = coords[dg_vertex(q, cc, k) * 3 + l];
    }
    // right cell's face axes in the left face's frame, through the shared corners
    int raxis[2] = {0, 1}, rflip[2] = {0, 0}, rd[3] = {0, 0, 0}, ra = 0;
    if (!boundary) {
      const int rlf = (left == c) ? nbrface[c * 6 + lf] : lf;
      dg_face(rlf, rd[0], rd[1], rd[2], ra);
      int M[4];
      for (int bs = 0; bs < 4; ++bs) {
        const int64_t gs = dg_vertex(q, right, ra | ((bs & 1) << rd[0]) | (((bs >> 1) & 1) << rd[1]));
        M[bs] = 0;
        for (int bl = 0; bl < 4; ++bl)
          if (dg_vertex(q, left, la | ((bl & 1) << ld1) | (((bl >> 1) & 1) << ld2)) == gs) M[bs] = bl;
      }
      for (int k = 0; k < 2; ++k) {
        const int diff = M[0] ^ M[1 << k];
        raxis[k] = (diff & 1) ? 0 : 1;
        rflip[k] = (M[0] >> raxis[k]) & 1;
      }
    }
    for (int t = lane; t < NN * NN; t += 32) O[t] = 0.0;
    const double sigma = (ld1 == 0 && ld2 == 2) ? -1.0 : 1.0;
    const double outward = ((la >> ldn) & 1) ? 1.0 : -1.0;
    double orient = 1.0;
    __syncwarp();
    for (int qp = 0; qp < NQF; ++qp) {
      const double s = q.x1[qp % NP1], tt = q.x1[qp / NP1];
      // lanes 0/1: the left/right cell's reference point, Jacobian inverse and h; lane 2: facet map
      if (lane < 2 && (lane == 0 || !boundary)) {
        double xi[3];
        if (lane == 0) {
          xi[ld1] = s; xi[ld2] = tt; xi[ldn] = ((la >> ldn) & 1) ? 1.0 : -1.0;
        } else {
          const double u[2] = {s, tt};
          for (int k = 0; k < 2; ++k) xi[rd[k]] = rflip[k] ? -u[raxis[k]] : u[raxis[k]];
          xi[rd[2]] = ((ra >> rd[2]) & 1) ? 1.0 : -1.0;
        }
        double b[9], det, h;
        dg_side_geometry(xv + 24 + 24 * lane, xi, b, det, h);
        for (int k = 0; k < 9; ++k) misc[6 + 9 * lane + k] = b[k];
        for (int k = 0; k < 3; ++k) misc[24 + 3 * lane + k] = xi[k];
        misc[30 + lane] = h;
        if (lane == 0) misc[32] = det;
      }
      if (lane == 2) {
        double X[4][3];
        for (int k = 0; k < 4; ++k) {
          const int v = la | ((k & 1) << ld1) | (((k >> 1) & 1) << ld2);
          for (int l = 0; l < 3; ++l) X[k][l] = xv[24 + v * 3 + l];
        }
        double xq[3] = {0, 0, 0}, js[3] = {0, 0, 0}, jt[3] = {0, 0, 0};
        for (int k = 0; k < 4; ++k) {
          const double fs = (k & 1) ? 0.5 * (1.0 + s) : 0.5 * (1.0 - s);
          const double ft = (k & 2) ? 0.5 * (1.0 + tt) : 0.5 * (1.0 - tt);
          const double ds = ((k & 1) ? 0.5 : -0.5) * ft, dt = ((k & 2) ? 0.5 : -0.5) * fs;
          for (int l = 0; l < 3; ++l) {
            xq[l] = xq[l] + fs * ft * X[k][l];
            js[l] = js[l] + ds * X[k][l];
            jt[l] = jt[l] + dt * X[k][l];
          }
        }
        double n[3] = {js[1] * jt[2] - js[2] * jt[1], js[2] * jt[0] - js[0] * jt[2], js[0] * jt[1] - js[1] * jt[0]};
        const double det = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int l = 0; l < 3; ++l) misc[l] = det != 0.0 ? n[l] / det : 0.0;
        misc[3] = det * (q.w1[qp % NP1] * q.w1[qp / NP1]);
        misc[5] = boundary ? dg_boundary_value(q.bfn, q.prm, xq) : 0.0;
      }
      __syncwarp();
      if (qp == 0) orient = sigma * outward * (misc[32] > 0.0 ? 1.0 : -1.0);
      const double h = boundary ? misc[30] : fmin(misc[30], misc[31]);
      const double n0 = misc[0] * orient, n1 = misc[1] * orient, n2 = misc[2] * orient;
      const double factor = misc[3];
      const double ch = q.cip / h;
      // 1D basis at both sides' points; J^-1 n per side: grad(phi) . n = grad_ref(phi) . (J^-1 n)
      if (lane < 6 && (lane < 3 || !boundary)) {
        const int side = lane / 3, dir = lane % 3;
        double v[NP1], dv[NP1];
        lag1d<P>(misc[24 + 3 * side + dir], v, dv);
        for (int jj = 0; jj < NP1; ++jj) {
          tab[((side * 3 + dir) * 4 + jj) * 2 + 0] = v[jj];
          tab[((side * 3 + dir) * 4 + jj) * 2 + 1] = dv[jj];
        }
      } else if (lane >= 8 && lane < 14 && (lane < 11 || !boundary)) {
        const int side = (lane - 8) / 3, jr = (lane - 8) % 3;
        const double* b = misc + 6 + 9 * side;
        misc[33 + 3 * side + jr] = b[jr + 0] * n0 + b[jr + 3] * n1 + b[jr + 6] * n2;
      }
      __syncwarp();
      // per node: value and scaled normal derivative (the sign of this cell's side folded in)
      const double sI = I == 0 ? 1.0 : -1.0;
      const double ascale = boundary ? factor : 0.5 * factor * sI;
      for (int t = lane; t < 2 * NN; t += 32) {
        const int side = t / NN, a = t % NN;
        if (side == 1 && boundary) continue;
        const int ai = a % NP1, aj = (a / NP1) % NP1, ak = a / (NP1 * NP1);
        const double* T0 = tab + ((side * 3 + 0) * 4 + ai) * 2;
        const double* T1 = tab + ((side * 3 + 1) * 4 + aj) * 2;
        const double* T2 = tab + ((side * 3 + 2) * 4 + ak) * 2;
        const double* w = misc + 33 + 3 * side;
        const double dn = T0[1] * T1[0] * T2[0] * w[0] + T0[0] * T1[1] * T2[0] * w[1] + T0[0] * T1[0] * T2[1] * w[2];
        sval[side * NN + a] = T0[0] * T1[0] * T2[0];
        sA[side * NN + a] = ascale * dn;
      }
      __syncwarp();
      if (boundary) {
        const double g = misc[5];
        const double pen = factor * ch;
        for (int t = lane; t < NN * NN; t += 32) {
          const int i = t / NN, j = t % NN;
          D[t] = D[t] - (sA[j] * sval[i] + sA[i] * sval[j]) + pen * sval[i] * sval[j];
        }
        for (int i = lane; i < NN; i += 32) rv[i] = rv[i] - g * sA[i] + pen * g * sval[i];
      } else {
        // n_I . n_J = +-|n|^2; with A = sI w|J_F| (grad phi . n)/2:
        //   same side:  -(A_j v_i + A_i v_j) + pen v_j v_i
        //   other side: -A^J_j v_i + A^I_i v^J_j - pen v^J_j v_i
        const double pen = factor * ch * (n0 * n0 + n1 * n1 + n2 * n2);
        const int Jo = 1 - I;
        for (int t = lane; t < NN * NN; t += 32) {
          const int i = t / NN, j = t % NN;
          const double vi = sval[I * NN + i], ai = sA[I * NN + i];
          const double vj = sval[I * NN + j], aj = sA[I * NN + j];
          const double vo = sval[Jo * NN + j], ao = sA[Jo * NN + j];
          D[t] = D[t] - (aj * vi + ai * vj) + pen * vj * vi;
          O[t] = O[t] - ao * vi + ai * vo - pen * vo * vi;
        }
      }
      __syncwarp();
    }
    if (!boundary) {
      int k = 0;
      while (blk[k] != o) ++k;
      for (int t = lane; t < NN * NN; t += 32) {
        const int i = t / NN, j = t % NN;
        const int64_t pos = rowptr[c * NN + i] + (int64_t)k * NN + j;
        val[pos] = O[t];
        if (val32) val32[pos] = (float)O[t];
      }
    }
    __syncwarp();
  }
  int k = 0;
  while (blk[k] != c) ++k;
  for (int t = lane; t < NN * NN; t += 32) {
    const int i = t / NN, j = t % NN;
    const int64_t pos = rowptr[c * NN + i] + (int64_t)k * NN + j;
    val[pos] = D[t];
    if (val32) val32[pos] = (float)D[t];
  }
  for (int i = lane; i < NN; i += 32) rhs[c * NN + i] = rv[i];
  (void)nb;
}

template <int P>
static fg_status launch_dg_rows(fg_system* sys) {
  using S = DgShape<P>;
  fg_space* sp = sys->space;
  fg_mesh* m = sp->mesh;
  fg_ctx* ctx = m->ctx;
  DgParams q;
  q.nx = m->n[0];
  q.ny = m->n[1];
  q.cellvert = m->unst ? m->d_cellvert : nullptr;
  gl_rule(P + 1, q.x1, q.w1);
  q.cip = 10.0 * P * P;
  q.bfn = sys->integ.boundary_fn;
  for (int i = 0; i < 8; ++i) q.prm[i] = sys->integ.fn_param[i];
  const size_t smem = S::BYTES_WARP * S::WARPS;
  FG_CUDA_TRY(cudaFuncSetAttribute((const void*)k_dg_rows<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_dg_rows<P><<<nblk(m->ncells, S::WARPS), S::WARPS * 32, smem, ctx->stream>>>(
      m->ncells, q, m->d_coords, sp->d_dgnbr, sp->d_dgnbrface, sys->d_elmat, sys->d_elvec, sp->d_rowptr, sys->d_val,
      sys->d_val32, sys->d_rhs);
  ctx->launches += 1;
  FG_CUDA_TRY(cudaGetLastError());
  return FG_OK;
}

fg_status dg_assemble_rows(fg_system* sys) {
  switch (sys->space->order) {
    case 1: return launch_dg_rows<1>(sys);
    case 2: return launch_dg_rows<2>(sys);
    case 3: return launch_dg_rows<3>(sys);
    default: set_error("dG order %d not built", sys->space->order); return FG_ERR_UNSUPPORTED;
  }
}

}  // namespace fg

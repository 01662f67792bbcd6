// fg_space.cu -- symbolic phase on the device: global dof numbering, the cell dof map,
// the sparsity pattern of the free-dof matrix and the reference-layout CSR export.
//
// Dof numbering.  The reference numbers dofs by walking the cells in order
// (Sources/Lib/Integration/FESpace/sbm_serial_fe_space.i90:525-716 for the strong
// Dirichlet dofs, :2623-2884 for the free dofs; per-cell work in
// sbm_fe_cell_iterator.i90:352-856):
//   - Dirichlet pass: for each cell, for each vef in polytope n-face order, the first
//     cell that visits a Dirichlet vef numbers its own dofs -1,-2,... (component-major).
//   - free pass: for each cell, its interior dofs, then each vef not yet owned, numbered
//     1,2,...; later cells fetch the owner's ids.
// On a structured mesh the first visitor of a vef is the lexicographically smallest cell
// around it, i.e. the cell whose lower neighbours do not contain it.  So each cell's
// share of new ids is a closed-form count; an exclusive scan over cells gives every
// cell its first id and one thread per cell writes its ids in the reference order.
// Ids live on the global node lattice ((p*n+1)^3 nodes, ncomp slots each).
//
// Sparsity.  The columns of the row of lattice node L are the free dofs of the lattice
// box spanned by the cells around L; one warp gathers the box, sorts it (bitonic, in
// shared memory) and writes the row -- the same set and order as the reference's
// COO -> sort_and_compress (Sources/Lib/LinearAlgebra/SparseMatrix/base_sparse_matrix.f90:4121-4829).
#include <cub/cub.cuh>

#include "fg_internal.h"

namespace fg {

struct Lat {
  int n[3];
  int p;
  int Ln[3];
  int ncomp;
  uint32_t dirmask;
  int codes[27];
  int code2idx[64];
};

static Lat make_lat(const fg_space* sp) {
  Lat g;
  for (int d = 0; d < 3; ++d) { g.n[d] = sp->mesh->n[d]; g.Ln[d] = sp->Ln[d]; }
  g.p = sp->order;
  g.ncomp = sp->ncomp;
  g.dirmask = sp->dirmask;
  for (int i = 0; i < 27; ++i) g.codes[i] = sp->tab.codes[i];
  for (int i = 0; i < 64; ++i) g.code2idx[i] = sp->tab.code2idx[i];
  return g;
}

// Boundary set id of the vef with free directions `type` anchored at lattice vertex v
// (uniform_hex_mesh_generator.f90:600-630).
__device__ __forceinline__ int vef_set_id(const Lat& g, int type, int v0, int v1, int v2) {
  int v[3] = {v0, v1, v2};
  int anchor = 0, t = 0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if ((type >> d) & 1) t |= 1 << d;
    else if (v[d] == 0) {
    } else if (v[d] == g.n[d]) anchor |= 1 << d;
    else t |= 1 << d;
  }
  return g.code2idx[anchor | (t << 3)] + 1;
}

__device__ __forceinline__ void cell_coords(const Lat& g, int64_t c, int& ci, int& cj, int& ck) {
  ci = (int)(c % g.n[0]);
  int64_t r = c / g.n[0];
  cj = (int)(r % g.n[1]);
  ck = (int)(r / g.n[1]);
}

// Is n-face f of cell (ci,cj,ck) first visited by this cell?  Pinned directions at the
// lower side belong to the lower neighbour unless the cell is on the domain boundary.
__device__ __forceinline__ bool owns_vef(int code, int ci, int cj, int ck) {
  int a = code & 7, t = code >> 3;
  int c[3] = {ci, cj, ck};
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (!((t >> d) & 1) && !((a >> d) & 1) && c[d] != 0) return false;
  return true;
}

__global__ void k_count_cell_dofs(Lat g, int64_t ncells, int64_t* cnt_free, int64_t* cnt_dir) {
  int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  int ci, cj, ck;
  cell_coords(g, c, ci, cj, ck);
  const int pm1 = g.p - 1;
  int64_t nf = (int64_t)pm1 * pm1 * pm1 * g.ncomp, nd = 0;
  for (int f = 0; f < 26; ++f) {
    int code = g.codes[f];
    if (!owns_vef(code, ci, cj, ck)) continue;
    int a = code & 7, t = code >> 3;
    int cnt = 1;
    for (int d = 0; d < 3; ++d) if ((t >> d) & 1) cnt *= pm1;
    if (cnt == 0) continue;
    int sid = vef_set_id(g, t, ci + (a & 1), cj + ((a >> 1) & 1), ck + ((a >> 2) & 1));
    if ((g.dirmask >> sid) & 1u) nd += (int64_t)cnt * g.ncomp;
    else nf += (int64_t)cnt * g.ncomp;
  }
  cnt_free[c] = nf;
  cnt_dir[c] = nd;
}

__global__ void k_assign_cell_dofs(Lat g, int64_t ncells, const int64_t* base_free, const int64_t* base_dir,
                                   int32_t* latdof, int32_t* free2lat, int32_t* dir2lat) {
  int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  int ci, cj, ck;
  cell_coords(g, c, ci, cj, ck);
  const int p = g.p;
  int64_t id = base_free[c], did = base_dir[c];
  // cell interior: component-major, nodes lexicographic
  for (int comp = 0; comp < g.ncomp; ++comp)
    for (int k = 1; k < p; ++k)
      for (int j = 1; j < p; ++j)
        for (int i = 1; i < p; ++i) {
          int64_t L = (int64_t)(p * ci + i) + (int64_t)g.Ln[0] * ((p * cj + j) + (int64_t)g.Ln[1] * (p * ck + k));
          int32_t slot = (int32_t)(L * g.ncomp + comp);
          latdof[slot] = (int32_t)(++id);
          free2lat[id - 1] = slot;
        }
  for (int f = 0; f < 26; ++f) {
    int code = g.codes[f];
    if (!owns_vef(code, ci, cj, ck)) continue;
    int a = code & 7, t = code >> 3;
    int lo[3], hi[3];
    int c3[3] = {ci, cj, ck};
    bool empty = false;
    for (int d = 0; d < 3; ++d) {
      if ((t >> d) & 1) { lo[d] = p * c3[d] + 1; hi[d] = p * c3[d] + p - 1; if (hi[d] < lo[d]) empty = true; }
      else { lo[d] = hi[d] = p * c3[d] + ((a >> d) & 1) * p; }
    }
    if (empty) continue;
    int sid = vef_set_id(g, t, ci + (a & 1), cj + ((a >> 1) & 1), ck + ((a >> 2) & 1));
    bool dir = (g.dirmask >> sid) & 1u;
    for (int comp = 0; comp < g.ncomp; ++comp)
      for (int K = lo[2]; K <= hi[2]; ++K)
        for (int J = lo[1]; J <= hi[1]; ++J)
          for (int I = lo[0]; I <= hi[0]; ++I) {
            int64_t L = (int64_t)I + (int64_t)g.Ln[0] * (J + (int64_t)g.Ln[1] * K);
            int32_t slot = (int32_t)(L * g.ncomp + comp);
            if (dir) {
              latdof[slot] = (int32_t)(-(++did));
              dir2lat[did - 1] = slot;
            } else {
              latdof[slot] = (int32_t)(++id);
              free2lat[id - 1] = slot;
            }
          }
  }
}

// lst_dofs_gids of every cell, reference cell-local order: s = node + comp*nn, nodes lexicographic.
__global__ void k_cell_dof_map(Lat g, int64_t ncells, int nn, int nd, const int32_t* latdof, int32_t* out) {
  int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= ncells * nd) return;
  int64_t c = idx / nd;
  int s = (int)(idx % nd);
  int comp = s / nn, a = s % nn;
  int np1 = g.p + 1;
  int ai = a % np1, aj = (a / np1) % np1, ak = a / (np1 * np1);
  int ci, cj, ck;
  cell_coords(g, c, ci, cj, ck);
  int64_t L = (int64_t)(g.p * ci + ai) + (int64_t)g.Ln[0] * ((g.p * cj + aj) + (int64_t)g.Ln[1] * (g.p * ck + ak));
  out[idx] = latdof[L * g.ncomp + comp];
}

// Lattice box of the cells around lattice coordinate I (one direction).
__device__ __forceinline__ void box_range(int I, int p, int n, int& lo, int& hi) {
  int c = I / p;
  int clo, chi;
  if (I % p == 0) { clo = c - 1; chi = c; }
  else { clo = c; chi = c; }
  if (clo < 0) clo = 0;
  if (chi > n - 1) chi = n - 1;
  lo = clo * p;
  hi = (chi + 1) * p;
}

__global__ void k_row_len(Lat g, int64_t nfree, const int32_t* free2lat, const int32_t* latdof, int64_t* row_len) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nfree) return;
  int64_t L = free2lat[r] / g.ncomp;
  int I = (int)(L % g.Ln[0]);
  int J = (int)((L / g.Ln[0]) % g.Ln[1]);
  int K = (int)(L / ((int64_t)g.Ln[0] * g.Ln[1]));
  int lo[3], hi[3];
  box_range(I, g.p, g.n[0], lo[0], hi[0]);
  box_range(J, g.p, g.n[1], lo[1], hi[1]);
  box_range(K, g.p, g.n[2], lo[2], hi[2]);
  int64_t cnt = 0;
  for (int z = lo[2]; z <= hi[2]; ++z)
    for (int y = lo[1]; y <= hi[1]; ++y)
      for (int x = lo[0]; x <= hi[0]; ++x) {
        int64_t M = (int64_t)x + (int64_t)g.Ln[0] * (y + (int64_t)g.Ln[1] * z);
        for (int c = 0; c < g.ncomp; ++c) cnt += latdof[M * g.ncomp + c] > 0;
      }
  row_len[r] = cnt;
}

// One warp per row: gather the box, bitonic-sort it in shared memory, write the row.
template <int CAP>
__global__ void k_row_fill(Lat g, int64_t nfree, const int32_t* free2lat, const int32_t* latdof,
                           const int64_t* rowptr, int32_t* col) {
  extern __shared__ int32_t s_keys[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  int32_t* keys = s_keys + wib * CAP;
  int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (r >= nfree) return;
  int64_t L = free2lat[r] / g.ncomp;
  int I = (int)(L % g.Ln[0]);
  int J = (int)((L / g.Ln[0]) % g.Ln[1]);
  int K = (int)(L / ((int64_t)g.Ln[0] * g.Ln[1]));
  int lo[3], hi[3];
  box_range(I, g.p, g.n[0], lo[0], hi[0]);
  box_range(J, g.p, g.n[1], lo[1], hi[1]);
  box_range(K, g.p, g.n[2], lo[2], hi[2]);
  const int bx = hi[0] - lo[0] + 1, by = hi[1] - lo[1] + 1, bz = hi[2] - lo[2] + 1;
  const int total = bx * by * bz * g.ncomp;
  for (int t = lane; t < CAP; t += 32) {
    int32_t key = 0x7fffffff;
    if (t < total) {
      int comp = t % g.ncomp;
      int q = t / g.ncomp;
      int x = lo[0] + q % bx, y = lo[1] + (q / bx) % by, z = lo[2] + q / (bx * by);
      int64_t M = (int64_t)x + (int64_t)g.Ln[0] * (y + (int64_t)g.Ln[1] * z);
      int32_t id = latdof[M * g.ncomp + comp];
      if (id > 0) key = id - 1;
    }
    keys[t] = key;
  }
  __syncwarp();
  for (int k = 2; k <= CAP; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = lane; t < CAP; t += 32) {
        int u = t ^ j;
        if (u > t) {
          int32_t a = keys[t], b = keys[u];
          bool up = (t & k) == 0;
          if ((a > b) == up) { keys[t] = b; keys[u] = a; }
        }
      }
      __syncwarp();
    }
  }
  const int64_t s = rowptr[r], len = rowptr[r + 1] - s;
  for (int t = lane; t < len; t += 32) col[s + t] = keys[t];
}

__global__ void k_upper_len(int64_t nfree, const int64_t* rowptr, const int32_t* col, int64_t* ulen) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nfree) return;
  int64_t lo = rowptr[r], hi = rowptr[r + 1];
  int64_t a = lo, b = hi;
  while (a < b) {
    int64_t m = (a + b) >> 1;
    if (col[m] < r) a = m + 1;
    else b = m;
  }
  ulen[r] = hi - a;
}

__global__ void k_upper_fill(int64_t nfree, const int64_t* rowptr, const int32_t* col, const double* val,
                             const int64_t* ulen, const int64_t* uptr, int one_based, int32_t* ocol, double* oval) {
  int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (r >= nfree) return;
  int64_t hi = rowptr[r + 1];
  int64_t n = ulen[r];
  int64_t src = hi - n, dst = uptr[r];
  for (int64_t t = lane; t < n; t += 32) {
    ocol[dst + t] = col[src + t] + one_based;
    if (oval) oval[dst + t] = val[src + t];
  }
}

__global__ void k_add_scalar_i64(int64_t n, int64_t* a, int64_t v) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) a[i] += v;
}
__global__ void k_add_scalar_i32(int64_t n, int32_t* a, int32_t v) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) a[i] += v;
}

static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// exclusive scan of n int64 (in may alias out), returns the total
static fg_status exclusive_scan(fg_ctx* ctx, const int64_t* in, int64_t* out, int64_t n, int64_t* total) {
  size_t tmp_bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, in, out, (int64_t)n, ctx->stream);
  void* tmp = nullptr;
  int64_t last_in = 0, last_out = 0;
  FG_CUDA_TRY(cudaMemcpyAsync(&last_in, in + n - 1, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  FG_TRY(dev_alloc(ctx, &tmp, tmp_bytes + 16));
  cudaError_t e = cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, in, out, (int64_t)n, ctx->stream);
  if (e != cudaSuccess) { dev_free(ctx, tmp); set_error("scan: %s", cudaGetErrorString(e)); return FG_ERR_CUDA; }
  FG_CUDA_TRY(cudaMemcpyAsync(&last_out, out + n - 1, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, tmp);
  *total = last_in + last_out;
  return FG_OK;
}

fg_status scan_i64(fg_ctx* ctx, int64_t* a, int64_t n, int64_t* total) { return exclusive_scan(ctx, a, a, n, total); }

// entries of the upper triangle (the reference's symmetric storage), for the CSR export
fg_status space_count_upper(fg_space* sp) {
  fg_ctx* ctx = sp->mesh->ctx;
  const int64_t n = sp->nfree;
  int64_t* ulen = nullptr;
  FG_TRY(dev_alloc(ctx, (void**)&ulen, sizeof(int64_t) * n));
  k_upper_len<<<nblk(n, 256), 256, 0, ctx->stream>>>(n, sp->d_rowptr, sp->d_col, ulen);
  FG_CUDA_TRY(cudaGetLastError());
  int64_t nup = 0;
  FG_TRY(exclusive_scan(ctx, ulen, ulen, n, &nup));
  dev_free(ctx, ulen);
  sp->nnz_upper = nup;
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return FG_OK;
}

fg_status space_number_dofs(fg_space* sp) {
  fg_ctx* ctx = sp->mesh->ctx;
  const int64_t ncells = sp->mesh->ncells;
  Lat g = make_lat(sp);
  int64_t *cf = nullptr, *cd = nullptr;
  FG_TRY(dev_alloc(ctx, (void**)&cf, sizeof(int64_t) * ncells));
  FG_TRY(dev_alloc(ctx, (void**)&cd, sizeof(int64_t) * ncells));
  k_count_cell_dofs<<<nblk(ncells, 256), 256, 0, ctx->stream>>>(g, ncells, cf, cd);
  FG_CUDA_TRY(cudaGetLastError());
  int64_t nfree = 0, ndir = 0;
  FG_TRY(exclusive_scan(ctx, cf, cf, ncells, &nfree));
  FG_TRY(exclusive_scan(ctx, cd, cd, ncells, &ndir));
  if (nfree >= (int64_t)0x7fffffff || sp->nlat * sp->ncomp >= (int64_t)0x7fffffff) {
    set_error("dof count exceeds int32 ids");
    return FG_ERR_UNSUPPORTED;
  }
  sp->nfree = nfree;
  sp->ndir = ndir;
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_latdof, sizeof(int32_t) * sp->nlat * sp->ncomp));
  FG_CUDA_TRY(cudaMemsetAsync(sp->d_latdof, 0, sizeof(int32_t) * sp->nlat * sp->ncomp, ctx->stream));
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_free2lat, sizeof(int32_t) * (nfree > 0 ? nfree : 1)));
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_dir2lat, sizeof(int32_t) * (ndir > 0 ? ndir : 1)));
  k_assign_cell_dofs<<<nblk(ncells, 128), 128, 0, ctx->stream>>>(g, ncells, cf, cd, sp->d_latdof, sp->d_free2lat,
                                                                   sp->d_dir2lat);
  FG_CUDA_TRY(cudaGetLastError());
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, cf);
  dev_free(ctx, cd);
  return FG_OK;
}

fg_status space_build_pattern(fg_space* sp) {
  fg_ctx* ctx = sp->mesh->ctx;
  Lat g = make_lat(sp);
  const int64_t n = sp->nfree;
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_rowptr, sizeof(int64_t) * (n + 1)));
  if (n == 0) {  // no free dofs: an empty pattern (row pointer 0, a one-slot column array)
    FG_CUDA_TRY(cudaMemsetAsync(sp->d_rowptr, 0, sizeof(int64_t), ctx->stream));
    FG_TRY(dev_alloc(ctx, (void**)&sp->d_col, sizeof(int32_t)));
    sp->nnz = 0;
    return FG_OK;
  }
  k_row_len<<<nblk(n, 256), 256, 0, ctx->stream>>>(g, n, sp->d_free2lat, sp->d_latdof, sp->d_rowptr);
  FG_CUDA_TRY(cudaGetLastError());
  int64_t nnz = 0;
  FG_TRY(exclusive_scan(ctx, sp->d_rowptr, sp->d_rowptr, n, &nnz));
  FG_CUDA_TRY(cudaMemcpyAsync(sp->d_rowptr + n, &nnz, sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
  sp->nnz = nnz;
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_col, sizeof(int32_t) * (nnz > 0 ? nnz : 1)));
  int box = 1;
  for (int d = 0; d < 3; ++d) box *= 2 * sp->order + 1;
  box *= sp->ncomp;
  int cap = 32;
  while (cap < box) cap <<= 1;
  sp->box_cap = cap;
  const int warps = cap >= 1024 ? 2 : 4;
  const size_t smem = (size_t)warps * cap * sizeof(int32_t);
  const unsigned grid = nblk(n, warps);
  switch (cap) {
#define FG_CASE(C)                                                                                   \
  case C:                                                                                            \
    k_row_fill<C><<<grid, warps * 32, smem, ctx->stream>>>(g, n, sp->d_free2lat, sp->d_latdof,       \
                                                          sp->d_rowptr, sp->d_col);                 \
    break;
    FG_CASE(32) FG_CASE(64) FG_CASE(128) FG_CASE(256) FG_CASE(512) FG_CASE(1024) FG_CASE(2048)
#undef FG_CASE
    default: set_error("neighbour box too large (%d)", box); return FG_ERR_UNSUPPORTED;
  }
  FG_CUDA_TRY(cudaGetLastError());
  return space_count_upper(sp);
}

fg_status space_export_dof_map(fg_space* sp, int32_t* out_host) {
  if (sp->mesh->unst || sp->dg) return uspace_export_dof_map(sp, out_host);
  if (sp->mesh->dim == 2) return q2_export_dof_map(sp, out_host);
  fg_ctx* ctx = sp->mesh->ctx;
  Lat g = make_lat(sp);
  const int64_t total = sp->mesh->ncells * sp->tab.nd;
  int32_t* d = nullptr;
  FG_TRY(dev_alloc(ctx, (void**)&d, sizeof(int32_t) * total));
  k_cell_dof_map<<<nblk(total, 256), 256, 0, ctx->stream>>>(g, sp->mesh->ncells, sp->tab.nn, sp->tab.nd,
                                                             sp->d_latdof, d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out_host, d, sizeof(int32_t) * total, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  dev_free(ctx, d);
  if (e != cudaSuccess) { set_error("dof map export: %s", cudaGetErrorString(e)); return FG_ERR_CUDA; }
  return FG_OK;
}

// Physical coordinates of a lattice node through the trilinear map of the last cell
// (in cell order) that contains it: the reference's interpolate_dirichlet_values loops
// over the cells in order and the last write wins (sbm_serial_fe_space.i90:1140-1152).
__device__ void lattice_node_xyz(const Lat& g, const double* coords, const double* gnod_unused, int64_t L,
                                 double* x) {
  int I = (int)(L % g.Ln[0]);
  int J = (int)((L / g.Ln[0]) % g.Ln[1]);
  int K = (int)(L / ((int64_t)g.Ln[0] * g.Ln[1]));
  int IJK[3] = {I, J, K};
  int c[3];
  double xi[3];
  for (int d = 0; d < 3; ++d) {
    c[d] = IJK[d] / g.p;
    if (c[d] > g.n[d] - 1) c[d] = g.n[d] - 1;
    int loc = IJK[d] - g.p * c[d];
    xi[d] = (2.0 / g.p) * loc - 1.0;
  }
  x[0] = x[1] = x[2] = 0.0;
  for (int k = 0; k < 8; ++k) {
    int bx = k & 1, by = (k >> 1) & 1, bz = (k >> 2) & 1;
    double fx = bx ? 0.5 * (1 + xi[0]) : 0.5 * (1 - xi[0]);
    double fy = by ? 0.5 * (1 + xi[1]) : 0.5 * (1 - xi[1]);
    double fz = bz ? 0.5 * (1 + xi[2]) : 0.5 * (1 - xi[2]);
    double a = fx * fy * fz;
    int64_t v = (int64_t)(c[0] + bx) + (int64_t)(g.n[0] + 1) * ((c[1] + by) + (int64_t)(g.n[1] + 1) * (c[2] + bz));
    for (int l = 0; l < 3; ++l) x[l] = x[l] + a * coords[v * 3 + l];
  }
}

__global__ void k_dirichlet_coords(Lat g, int64_t ndir, const int32_t* dir2lat, const double* coords, double* xyz) {
  int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (d >= ndir) return;
  int64_t L = dir2lat[d] / g.ncomp;
  double x[3];
  lattice_node_xyz(g, coords, nullptr, L, x);
  xyz[d * 3 + 0] = x[0];
  xyz[d * 3 + 1] = x[1];
  xyz[d * 3 + 2] = x[2];
}

fg_status space_dirichlet_coords(fg_space* sp, double* d_xyz) {
  if (sp->ndir == 0) return FG_OK;
  if (sp->mesh->unst) return uspace_dirichlet_coords(sp, d_xyz);
  if (sp->mesh->dim == 2) return q2_dirichlet_coords(sp, d_xyz);
  Lat g = make_lat(sp);
  k_dirichlet_coords<<<nblk(sp->ndir, 256), 256, 0, sp->mesh->ctx->stream>>>(g, sp->ndir, sp->d_dir2lat,
                                                                              sp->mesh->d_coords, d_xyz);
  FG_CUDA_TRY(cudaGetLastError());
  return FG_OK;
}

fg_status space_export_upper(fg_space* sp, const double* d_val, int one_based, int64_t* irp, int32_t* ja,
                             double* val) {
  fg_ctx* ctx = sp->mesh->ctx;
  const int64_t n = sp->nfree, nup = sp->nnz_upper;
  int64_t *ulen = nullptr, *uptr = nullptr;
  int32_t* ocol = nullptr;
  double* oval = nullptr;
  FG_TRY(dev_alloc(ctx, (void**)&ulen, sizeof(int64_t) * (n + 1)));
  FG_TRY(dev_alloc(ctx, (void**)&uptr, sizeof(int64_t) * (n + 1)));
  FG_TRY(dev_alloc(ctx, (void**)&ocol, sizeof(int32_t) * (nup > 0 ? nup : 1)));
  if (val) FG_TRY(dev_alloc(ctx, (void**)&oval, sizeof(double) * (nup > 0 ? nup : 1)));
  if (n > 0) {
    k_upper_len<<<nblk(n, 256), 256, 0, ctx->stream>>>(n, sp->d_rowptr, sp->d_col, ulen);
    FG_CUDA_TRY(cudaGetLastError());
    int64_t tot = 0;
    FG_TRY(exclusive_scan(ctx, ulen, uptr, n, &tot));
    k_upper_fill<<<nblk(n * 32, 256), 256, 0, ctx->stream>>>(n, sp->d_rowptr, sp->d_col, d_val, ulen, uptr,
                                                              one_based, ocol, oval);
    FG_CUDA_TRY(cudaGetLastError());
    if (one_based) k_add_scalar_i64<<<nblk(n, 256), 256, 0, ctx->stream>>>(n, uptr, 1);
    FG_CUDA_TRY(cudaMemcpyAsync(irp, uptr, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
  }
  if (irp) irp[n] = nup + one_based;
  if (ja && nup) FG_CUDA_TRY(cudaMemcpyAsync(ja, ocol, sizeof(int32_t) * nup, cudaMemcpyDeviceToHost, ctx->stream));
  if (val && nup) FG_CUDA_TRY(cudaMemcpyAsync(val, oval, sizeof(double) * nup, cudaMemcpyDeviceToHost, ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (irp) irp[n] = nup + one_based;
  dev_free(ctx, ulen);
  dev_free(ctx, uptr);
  dev_free(ctx, ocol);
  if (oval) dev_free(ctx, oval);
  return FG_OK;
}

}  // namespace fg

// fg_stencil.cu -- lattice-implicit SELL layout of the free-dof matrix (structured meshes).
//
// On the structured hex mesh the columns of the row of lattice node (I,J,K) are the nodes
// of a box of cells around it, and the box depends only on the node's class
// (I mod p, J mod p, K mod p): per direction [-p,+p] on a vertex plane, [-(I mod p), p -
// (I mod p)] inside a cell.  Rows are grouped by class; each class is cut into slices of
// 32 rows (lane = row, rows in lattice order) and every row of a class stores the same B
// box positions (all components), padded to a multiple of 4 and interleaved 4-wide per
// lane as in the explicit SELL layout, so a warp reads 4 values per lane with one 128-bit
// or 256-bit load.  No column indices are stored: the column of position k is the row's
// node plus a per-class offset from a table of at most 27 x 1029 entries.
//
// The solver vectors live on the node lattice padded by p nodes on every side (ncomp
// entries per node), so every box position is a valid address; entries of Dirichlet,
// halo and padding nodes stay zero.  Box positions outside the domain or on Dirichlet
// nodes hold value 0.  For Q2 Poisson at 128^3 the FP32 matrix is 4 B per stored entry
// instead of 8 B with explicit int32 columns.
#include <algorithm>

#include <cub/cub.cuh>

#include "fg_internal.h"

namespace fg {

static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

__global__ void k_class_keys(int64_t nslots, int ncomp, int p, int Ln0, int Ln1, int ncls, const int32_t* latdof,
                             uint8_t* keys, int32_t* vals, unsigned* counts) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= nslots) return;
  const int64_t L = s / ncomp;
  const int I = (int)(L % Ln0), J = (int)((L / Ln0) % Ln1), K = (int)(L / ((int64_t)Ln0 * Ln1));
  int key = ncls;
  if (latdof[s] > 0) key = (I % p) + p * ((J % p) + p * (K % p));
  keys[s] = (uint8_t)key;
  vals[s] = (int32_t)s;
  if (key < ncls) atomicAdd(counts + key, 1u);
}

__global__ void k_stencil_rows(int64_t nfree, int ncomp, int p, const int Ln[3], int halo, const int Pn[3],
                               const uint8_t* skeys, const int32_t* svals, const int64_t* cls_start,
                               const StencilClass* cls, const int32_t* latdof, const int32_t* slice_perm,
                               int32_t* st_row, int32_t* row2st, int32_t* row2vec, int32_t* slot2row) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nfree) return;
  const int k = skeys[i];
  const int32_t s = svals[i];
  const int64_t L = s / ncomp;
  const int c = (int)(s % ncomp);
  const int I = (int)(L % Ln[0]), J = (int)((L / Ln[0]) % Ln[1]), K = (int)(L / ((int64_t)Ln[0] * Ln[1]));
  // node's index inside its class sub-lattice (padded coordinates divided by p)
  const int S0 = Pn[0] / p, S1 = Pn[1] / p;
  const int64_t sub = (int64_t)((I + halo) / p) + (int64_t)S0 * (((J + halo) / p) + (int64_t)S1 * ((K + halo) / p));
  const int64_t st = sub * ncomp + c;
  // the row's slot in class-by-class numbering, moved to its slice's stored position
  const int64_t slot_c = (int64_t)cls[k].sbase * 32 + (i - cls_start[k]);
  const int64_t slot = (int64_t)slice_perm[slot_c >> 5] * 32 + (slot_c & 31);
  const int32_t r = latdof[s] - 1;
  st_row[slot] = (int32_t)st;
  slot2row[slot] = r;
  row2st[r] = (int32_t)slot;
  row2vec[r] = (int32_t)(st + cls[k].ownoff);
}

// padding lanes of a class's last slice (no row): the bitwise complement of the slice's first
// row, so a kernel reads a valid address there (values are 0) and knows not to store
__global__ void k_stencil_pad(int64_t nslices, const int32_t* slot2row, int32_t* st_row) {
  int64_t sl = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (sl >= nslices) return;
  for (int l = 1; l < 32; ++l)
    if (slot2row[sl * 32 + l] < 0) st_row[sl * 32 + l] = ~st_row[sl * 32];
}

// values: CSR (row order) -> stencil layout, FP64 and FP32 copies (arrays cleared before)
__global__ void k_stencil_vals(int64_t nfree, int ncomp, int p, int Ln0, int Ln1, const int64_t* rowptr,
                               const int32_t* col, const double* val, const int32_t* free2lat, const int32_t* row2st,
                               const uint8_t* scls, const StencilClass* cls, const int64_t* voff, double* sval,
                               float* sval32) {
  const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= nfree) return;
  const int32_t slot = row2st[r];
  const int64_t sl = slot >> 5;
  const int rl = slot & 31;
  const StencilClass& C = cls[scls[sl]];
  const int64_t vb = voff[sl] + 4 * rl;
  const int64_t L = free2lat[r] / ncomp;
  const int I = (int)(L % Ln0), J = (int)((L / Ln0) % Ln1), K = (int)(L / ((int64_t)Ln0 * Ln1));
  const int lox = I + C.lo[0], loy = J + C.lo[1], loz = K + C.lo[2];
  const int64_t s = rowptr[r], e = rowptr[r + 1];
  for (int64_t t = s + lane; t < e; t += 32) {
    const int32_t sl2 = free2lat[col[t]];
    const int64_t L2 = sl2 / ncomp;
    const int c2 = sl2 % ncomp;
    const int mx = (int)(L2 % Ln0) - lox, my = (int)((L2 / Ln0) % Ln1) - loy,
              mz = (int)(L2 / ((int64_t)Ln0 * Ln1)) - loz;
    const int pos = c2 + ncomp * (mx + C.w[0] * (my + C.w[1] * mz));
    const int64_t o = vb + (int64_t)(pos >> 2) * 128 + (pos & 3);
    const double v = val[t];
    sval[o] = v;
    sval32[o] = (float)v;
  }
}

fg_status space_build_stencil(fg_space* sp) {
  fg_ctx* ctx = sp->mesh->ctx;
  const int p = sp->order, ncomp = sp->ncomp;
  const int ncls = p * p * p;
  // Solver vectors: the node lattice padded by p nodes per side (so every box position is
  // an address), rounded up to a multiple of p per direction and split into the p^3 class
  // sub-lattices (residues of the padded coordinates mod p), one after the other.  Rows of
  // a class are consecutive in their sub-lattice, so the 32 lanes of a slice gather 32
  // consecutive entries for every box position.
  sp->halo = p;
  for (int d = 0; d < 3; ++d) sp->Pn[d] = (sp->Ln[d] + 2 * p + p - 1) / p * p;
  const int64_t S0 = sp->Pn[0] / p, S1 = sp->Pn[1] / p, S2 = sp->Pn[2] / p;
  const int64_t ssize = S0 * S1 * S2;
  sp->nvec = (int64_t)ncls * ssize * ncomp;
  if (sp->nvec >= (int64_t)0x7fffffff) { set_error("padded lattice exceeds int32 indices"); return FG_ERR_UNSUPPORTED; }
  // classes: box and offsets
  std::vector<StencilClass> cls(ncls);
  std::vector<int32_t> offs;
  for (int k = 0; k < ncls; ++k) {
    int rr[3] = {k % p, (k / p) % p, k / (p * p)};
    StencilClass& C = cls[k];
    for (int d = 0; d < 3; ++d) {
      if (rr[d] == 0) { C.lo[d] = -p; C.w[d] = 2 * p + 1; }
      else { C.lo[d] = -rr[d]; C.w[d] = p + 1; }
    }
    C.B = C.w[0] * C.w[1] * C.w[2] * ncomp;
    C.Bp = (C.B + 3) / 4 * 4;
    C.offbase = (int)offs.size();
    C.ownoff = (int64_t)k * ssize * ncomp;
    for (int pos = 0; pos < C.Bp; ++pos) {
      if (pos >= C.B) { offs.push_back(0); continue; }
      int c2 = pos % ncomp, q = pos / ncomp;
      int m[3] = {q % C.w[0], (q / C.w[0]) % C.w[1], q / (C.w[0] * C.w[1])};
      // column node = row node + (lo + m); split into its sub-lattice and the index shift
      int res[3], shift[3];
      for (int d = 0; d < 3; ++d) {
        int t = rr[d] + C.lo[d] + m[d];  // residue of the row is rr[d]
        int fl = t >= 0 ? t / p : -((-t + p - 1) / p);
        shift[d] = fl;
        res[d] = t - fl * p;
      }
      const int64_t kk = res[0] + p * (res[1] + p * res[2]);
      const int64_t o = (kk * ssize + shift[0] + S0 * (shift[1] + S1 * shift[2])) * ncomp + c2;
      offs.push_back((int32_t)o);
    }
  }
  // rows grouped by class, lattice order inside a class
  const int64_t nslots = sp->nlat * ncomp;
  uint8_t *keys = nullptr, *skeys = nullptr;
  int32_t *vals = nullptr, *svals = nullptr;
  unsigned* counts = nullptr;
  FG_TRY(dev_alloc(ctx, (void**)&keys, nslots));
  FG_TRY(dev_alloc(ctx, (void**)&skeys, nslots));
  FG_TRY(dev_alloc(ctx, (void**)&vals, sizeof(int32_t) * nslots));
  FG_TRY(dev_alloc(ctx, (void**)&svals, sizeof(int32_t) * nslots));
  FG_TRY(dev_alloc(ctx, (void**)&counts, sizeof(unsigned) * 32));
  FG_CUDA_TRY(cudaMemsetAsync(counts, 0, sizeof(unsigned) * 32, ctx->stream));
  k_class_keys<<<nblk(nslots, 256), 256, 0, ctx->stream>>>(nslots, ncomp, p, sp->Ln[0], sp->Ln[1], ncls, sp->d_latdof,
                                                          keys, vals, counts);
  FG_CUDA_TRY(cudaGetLastError());
  size_t tmp_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, skeys, vals, svals, (int64_t)nslots, 0, 5, ctx->stream);
  void* tmp = nullptr;
  FG_TRY(dev_alloc(ctx, &tmp, tmp_bytes + 16));
  cudaError_t e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, skeys, vals, svals, (int64_t)nslots, 0, 5,
                                                  ctx->stream);
  if (e != cudaSuccess) { set_error("class sort: %s", cudaGetErrorString(e)); return FG_ERR_CUDA; }
  unsigned hcount[32];
  FG_CUDA_TRY(cudaMemcpyAsync(hcount, counts, sizeof(hcount), cudaMemcpyDeviceToHost, ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  ctx->launches += 1;
  std::vector<int64_t> cstart(ncls + 1, 0);
  int64_t nsl = 0, nv = 0;
  for (int k = 0; k < ncls; ++k) {
    StencilClass& C = cls[k];
    C.nrows = hcount[k];
    C.sbase = nsl;
    C.vbase = nv;
    const int64_t s = (C.nrows + 31) / 32;
    nsl += s;
    nv += s * 32 * C.Bp;
    cstart[k + 1] = cstart[k] + C.nrows;
  }
  if (cstart[ncls] != sp->nfree) { set_error("stencil class counts do not add up"); return FG_ERR_CUDA; }
  sp->st_nslices = nsl;
  sp->st_nvals = nv;
  sp->st_ncls = ncls;
  // Slices are stored class by class (a class's slices in lattice order).  The SpMV's warps
  // take slices at a stride of the warp count, so neighbouring warps work on neighbouring rows
  // of one class and share the x entries they gather in L1/L2.  Interleaving the classes by
  // position (runs of 8-4096 slices) read fewer DRAM bytes (x once instead of ~once per
  // class) but ran 7-17 % slower on GB300; the per-slice value offsets keep that choice here.
  std::vector<uint8_t> hscls(nsl > 0 ? nsl : 1);
  std::vector<int64_t> hvoff(nsl > 0 ? nsl : 1, 0);
  std::vector<int32_t> hperm(nsl > 0 ? nsl : 1, 0);  // class-by-class slice id -> stored id
  {
    int64_t t = 0, v = 0;
    for (int k = 0; k < ncls; ++k)
      for (int64_t j = 0; j < (cls[k].nrows + 31) / 32; ++j, ++t) {
        hperm[cls[k].sbase + j] = (int32_t)t;
        hscls[t] = (uint8_t)k;
        hvoff[t] = v;
        v += 32 * (int64_t)cls[k].Bp;
      }
  }
  int32_t* d_perm = nullptr;
  int64_t* d_cstart = nullptr;
  int* d_dims = nullptr;
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_st_cls, sizeof(StencilClass) * ncls));
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_st_off, sizeof(int32_t) * offs.size()));
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_st_scls, hscls.size()));
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_st_voff, sizeof(int64_t) * hvoff.size()));
  FG_TRY(dev_alloc(ctx, (void**)&d_perm, sizeof(int32_t) * hperm.size()));
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_st_row, sizeof(int32_t) * (nsl > 0 ? nsl * 32 : 1)));
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_row2st, sizeof(int32_t) * (sp->nfree > 0 ? sp->nfree : 1)));
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_st_slot2row, sizeof(int32_t) * (nsl > 0 ? nsl * 32 : 1)));
  FG_CUDA_TRY(cudaMemsetAsync(sp->d_st_slot2row, 0xff, sizeof(int32_t) * (nsl > 0 ? nsl * 32 : 1), ctx->stream));
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_row2vec, sizeof(int32_t) * (sp->nfree > 0 ? sp->nfree : 1)));
  FG_TRY(dev_alloc(ctx, (void**)&d_cstart, sizeof(int64_t) * (ncls + 1)));
  FG_TRY(dev_alloc(ctx, (void**)&d_dims, sizeof(int) * 8));
  int hdims[8] = {sp->Ln[0], sp->Ln[1], sp->Ln[2], sp->Pn[0], sp->Pn[1], sp->Pn[2], 0, 0};
  FG_CUDA_TRY(cudaMemcpyAsync(sp->d_st_cls, cls.data(), sizeof(StencilClass) * ncls, cudaMemcpyHostToDevice, ctx->stream));
  FG_CUDA_TRY(cudaMemcpyAsync(sp->d_st_off, offs.data(), sizeof(int32_t) * offs.size(), cudaMemcpyHostToDevice, ctx->stream));
  FG_CUDA_TRY(cudaMemcpyAsync(sp->d_st_scls, hscls.data(), hscls.size(), cudaMemcpyHostToDevice, ctx->stream));
  FG_CUDA_TRY(cudaMemcpyAsync(sp->d_st_voff, hvoff.data(), sizeof(int64_t) * hvoff.size(), cudaMemcpyHostToDevice,
                              ctx->stream));
  FG_CUDA_TRY(cudaMemcpyAsync(d_perm, hperm.data(), sizeof(int32_t) * hperm.size(), cudaMemcpyHostToDevice, ctx->stream));
  FG_CUDA_TRY(cudaMemcpyAsync(d_cstart, cstart.data(), sizeof(int64_t) * (ncls + 1), cudaMemcpyHostToDevice, ctx->stream));
  FG_CUDA_TRY(cudaMemcpyAsync(d_dims, hdims, sizeof(hdims), cudaMemcpyHostToDevice, ctx->stream));
  if (sp->nfree > 0) {
    k_stencil_rows<<<nblk(sp->nfree, 256), 256, 0, ctx->stream>>>(sp->nfree, ncomp, p, d_dims, p, d_dims + 3, skeys,
                                                                   svals, d_cstart, sp->d_st_cls, sp->d_latdof, d_perm,
                                                                   sp->d_st_row, sp->d_row2st, sp->d_row2vec,
                                                                   sp->d_st_slot2row);
    FG_CUDA_TRY(cudaGetLastError());
    k_stencil_pad<<<nblk(nsl, 256), 256, 0, ctx->stream>>>(nsl, sp->d_st_slot2row, sp->d_st_row);
    FG_CUDA_TRY(cudaGetLastError());
    ctx->launches += 2;
  }
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  sp->h_st_cls = cls;
  sp->st_max_bp = 0;
  for (const StencilClass& C : cls) sp->st_max_bp = std::max(sp->st_max_bp, C.Bp);
  dev_free(ctx, keys);
  dev_free(ctx, skeys);
  dev_free(ctx, vals);
  dev_free(ctx, svals);
  dev_free(ctx, counts);
  dev_free(ctx, tmp);
  dev_free(ctx, d_cstart);
  dev_free(ctx, d_dims);
  dev_free(ctx, d_perm);
  return FG_OK;
}

fg_status system_fill_stencil(fg_system* sys) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  if (sp->nfree == 0) return FG_OK;
  FG_CUDA_TRY(cudaMemsetAsync(sys->d_tval, 0, sizeof(double) * sp->st_nvals, ctx->stream));
  FG_CUDA_TRY(cudaMemsetAsync(sys->d_tval32, 0, sizeof(float) * sp->st_nvals, ctx->stream));
  k_stencil_vals<<<nblk(sp->nfree * 32, 256), 256, 0, ctx->stream>>>(
      sp->nfree, sp->ncomp, sp->order, sp->Ln[0], sp->Ln[1], sp->d_rowptr, sp->d_col, sys->d_val, sp->d_free2lat,
      sp->d_row2st, sp->d_st_scls, sp->d_st_cls, sp->d_st_voff, sys->d_tval, sys->d_tval32);
  FG_CUDA_TRY(cudaGetLastError());
  ctx->launches += 1;
  return FG_OK;
}

// CSR values from the lattice-implicit FP64 values (the inverse of k_stencil_vals)
__global__ void k_stencil_to_csr(int64_t nfree, int ncomp, int Ln0, int Ln1, const int64_t* rowptr,
                                 const int32_t* col, const double* sval, const int32_t* free2lat,
                                 const int32_t* row2st, const uint8_t* scls, const StencilClass* cls,
                                 const int64_t* voff, double* val) {
  const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= nfree) return;
  const int32_t slot = row2st[r];
  const int64_t sl = slot >> 5;
  const int rl = slot & 31;
  const StencilClass& C = cls[scls[sl]];
  const int64_t vb = voff[sl] + 4 * rl;
  const int64_t L = free2lat[r] / ncomp;
  const int I = (int)(L % Ln0), J = (int)((L / Ln0) % Ln1), K = (int)(L / ((int64_t)Ln0 * Ln1));
  const int lox = I + C.lo[0], loy = J + C.lo[1], loz = K + C.lo[2];
  const int64_t s = rowptr[r], e = rowptr[r + 1];
  for (int64_t t = s + lane; t < e; t += 32) {
    const int32_t sl2 = free2lat[col[t]];
    const int64_t L2 = sl2 / ncomp;
    const int c2 = sl2 % ncomp;
    const int mx = (int)(L2 % Ln0) - lox, my = (int)((L2 / Ln0) % Ln1) - loy,
              mz = (int)(L2 / ((int64_t)Ln0 * Ln1)) - loz;
    const int pos = c2 + ncomp * (mx + C.w[0] * (my + C.w[1] * mz));
    val[t] = sval[vb + (int64_t)(pos >> 2) * 128 + (pos & 3)];
  }
}

fg_status system_ensure_csr(fg_system* sys) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  if (!sys->direct) return FG_OK;
  if (!sys->d_tval || !sp->d_rowptr || !sp->d_col) {
    set_error("the CSR of this system was released (FG_LEAN_SYSTEM / fg_space_release_pattern)");
    return FG_ERR_UNSUPPORTED;
  }
  if (!sys->d_val) FG_TRY(dev_alloc(ctx, (void**)&sys->d_val, sizeof(double) * (sp->nnz > 0 ? sp->nnz : 1)));
  if (sp->nfree > 0) {
    k_stencil_to_csr<<<nblk(sp->nfree * 32, 256), 256, 0, ctx->stream>>>(
        sp->nfree, sp->ncomp, sp->Ln[0], sp->Ln[1], sp->d_rowptr, sp->d_col, sys->d_tval, sp->d_free2lat,
        sp->d_row2st, sp->d_st_scls, sp->d_st_cls, sp->d_st_voff, sys->d_val);
    FG_CUDA_TRY(cudaGetLastError());
    ctx->launches += 1;
  }
  sys->direct = false;  // d_val now holds the values (until the next direct assembly)
  return FG_OK;
}

// 1/diagonal of every free row, read at the diagonal box position of its class (the node
// itself, component = the row's); entries of non-free vector slots stay 0
__global__ void k_inv_diag_stencil(int64_t nfree, int ncomp, const int32_t* free2lat, const int32_t* row2st,
                                   const int32_t* row2vec, const uint8_t* scls, const StencilClass* cls,
                                   const int64_t* voff, const double* sval, double* d64, float* d32) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nfree) return;
  const int32_t slot = row2st[r];
  const int64_t sl = slot >> 5;
  const int rl = slot & 31;
  const StencilClass& C = cls[scls[sl]];
  const int c = free2lat[r] % ncomp;
  const int pos = c + ncomp * (-C.lo[0] + C.w[0] * (-C.lo[1] + C.w[1] * (-C.lo[2])));
  const double d = sval[voff[sl] + 4 * rl + (int64_t)(pos >> 2) * 128 + (pos & 3)];
  const double inv = 1.0 / d;
  d64[row2vec[r]] = inv;
  d32[row2vec[r]] = (float)inv;
}

fg_status system_inv_diag_stencil(fg_system* sys) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  if (sp->nfree == 0) return FG_OK;
  k_inv_diag_stencil<<<nblk(sp->nfree, 256), 256, 0, ctx->stream>>>(sp->nfree, sp->ncomp, sp->d_free2lat, sp->d_row2st,
                                                                    sp->d_row2vec, sp->d_st_scls, sp->d_st_cls,
                                                                    sp->d_st_voff, sys->d_tval, sys->d_idiag,
                                                                    sys->d_idiag32);
  FG_CUDA_TRY(cudaGetLastError());
  ctx->launches += 1;
  return FG_OK;
}

}  // namespace fg

// fg_sell.cu -- SELL-C-sigma copy of the free-dof matrix for the solver.
//
// Layout: rows are grouped in windows of SIGMA = 256 rows; inside a window they are
// stably sorted by decreasing length, then cut into slices of C = 32 rows.  Slice s has
// width w_s = its longest row rounded up to a multiple of 4, and entry j of the row in
// lane l sits at sptr[s] + 128 (j/4) + 4 l + (j%4): each lane's entries come in runs of
// 4, so a warp that owns a slice (lane = row) reads 4 values per lane with one 128-bit
// (FP32 values, int32 columns) or 256-bit (FP64 values) load -- 512 B to 1 KB per warp
// instruction, fully coalesced -- and needs no cross-lane reduction.  Padding entries
// have value 0 and point at the row itself.
//
// The solver runs in the SELL row order ("slot" order): perm[slot] = row, iperm[row] =
// slot; column indices are stored in slot numbering.  Each row keeps the reference CSR's
// column order (ascending original dof id), so a row's products are summed in that order.
//
// Why SELL on GB300: its FP64 pipe runs about 0.5 Tera-DFMA/s, so the warp-shuffle
// row reductions of a warp-per-row CSR kernel (5 FP64 adds per row) cost more than the
// row's products; here the FP64 work is exactly one DFMA per stored entry, and the FP32
// copy needs no FP64 arithmetic at all.
#include <cub/cub.cuh>

#include "fg_internal.h"

namespace fg {

static constexpr int SELL_C = 32;
static constexpr int SELL_SIGMA = 256;

static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// one block per window: stable rank by decreasing row length
__global__ void __launch_bounds__(SELL_SIGMA) k_sigma_sort(int64_t n, const int64_t* rowptr, int32_t* perm,
                                                           int32_t* iperm) {
  __shared__ int32_t s_len[SELL_SIGMA];
  const int64_t base = (int64_t)blockIdx.x * SELL_SIGMA;
  const int t = threadIdx.x;
  const int64_t r = base + t;
  const int64_t rem = n - base;
  const int cnt = rem < SELL_SIGMA ? (int)rem : SELL_SIGMA;
  int len = -1;
  if (t < cnt) len = (int)(rowptr[r + 1] - rowptr[r]);
  s_len[t] = len;
  __syncthreads();
  if (t >= cnt) return;
  int rank = 0;
  for (int u = 0; u < cnt; ++u) {
    int lu = s_len[u];
    rank += (lu > len) || (lu == len && u < t);
  }
  perm[base + rank] = (int32_t)r;
  iperm[r] = (int32_t)(base + rank);
}

__global__ void k_slice_width(int64_t n, int64_t nslices, const int64_t* rowptr, const int32_t* perm, int64_t* w) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= nslices) return;
  int64_t m = 0;
  for (int l = 0; l < SELL_C; ++l) {
    int64_t slot = s * SELL_C + l;
    if (slot < n) {
      int32_t r = perm[slot];
      int64_t len = rowptr[r + 1] - rowptr[r];
      if (len > m) m = len;
    }
  }
  w[s] = ((m + 3) / 4 * 4) * SELL_C;  // entries of the slice (scanned into slice pointers)
}

// warp per slice: lane = row.  Columns converted to slot numbering.
__global__ void k_sell_cols(int64_t n, int64_t nslices, const int64_t* rowptr, const int32_t* col,
                            const int32_t* perm, const int32_t* iperm, const int64_t* sptr, int32_t* scol) {
  const int64_t s = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (s >= nslices) return;
  const int64_t slot = s * SELL_C + lane;
  const int64_t base = sptr[s];
  const int width = (int)((sptr[s + 1] - base) / SELL_C);
  int64_t rs = 0, len = 0;
  if (slot < n) {
    int32_t r = perm[slot];
    rs = rowptr[r];
    len = rowptr[r + 1] - rs;
  }
  const int32_t self = (int32_t)(slot < n ? slot : 0);
  for (int j = 0; j < width; ++j) {
    int32_t c = j < len ? iperm[col[rs + j]] : self;
    scol[base + (int64_t)(j >> 2) * (4 * SELL_C) + 4 * lane + (j & 3)] = c;
  }
}

// values: CSR (row order) -> SELL (slot order), FP64 and FP32 copies
__global__ void k_sell_vals(int64_t n, int64_t nslices, const int64_t* rowptr, const double* val, const int32_t* perm,
                            const int64_t* sptr, double* sval, float* sval32) {
  const int64_t s = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (s >= nslices) return;
  const int64_t slot = s * SELL_C + lane;
  const int64_t base = sptr[s];
  const int width = (int)((sptr[s + 1] - base) / SELL_C);
  int64_t rs = 0, len = 0;
  if (slot < n) {
    int32_t r = perm[slot];
    rs = rowptr[r];
    len = rowptr[r + 1] - rs;
  }
  for (int j = 0; j < width; ++j) {
    double v = j < len ? val[rs + j] : 0.0;
    const int64_t o = base + (int64_t)(j >> 2) * (4 * SELL_C) + 4 * lane + (j & 3);
    sval[o] = v;
    sval32[o] = (float)v;
  }
}

fg_status space_build_sell(fg_space* sp) {
  fg_ctx* ctx = sp->mesh->ctx;
  const int64_t n = sp->nfree;
  sp->nslices = (n + SELL_C - 1) / SELL_C;
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_perm, sizeof(int32_t) * (n > 0 ? n : 1)));
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_iperm, sizeof(int32_t) * (n > 0 ? n : 1)));
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_sptr, sizeof(int64_t) * (sp->nslices + 1)));
  if (n == 0) {
    sp->sell_nnz = 0;
    FG_CUDA_TRY(cudaMemsetAsync(sp->d_sptr, 0, sizeof(int64_t), ctx->stream));
    return FG_OK;
  }
  const unsigned nwin = (unsigned)((n + SELL_SIGMA - 1) / SELL_SIGMA);
  k_sigma_sort<<<nwin, SELL_SIGMA, 0, ctx->stream>>>(n, sp->d_rowptr, sp->d_perm, sp->d_iperm);
  FG_CUDA_TRY(cudaGetLastError());
  k_slice_width<<<nblk(sp->nslices, 256), 256, 0, ctx->stream>>>(n, sp->nslices, sp->d_rowptr, sp->d_perm, sp->d_sptr);
  FG_CUDA_TRY(cudaGetLastError());
  ctx->launches += 2;
  // exclusive scan of slice sizes
  size_t tmp_bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, sp->d_sptr, sp->d_sptr, (int64_t)(sp->nslices + 1), ctx->stream);
  void* tmp = nullptr;
  FG_TRY(dev_alloc(ctx, &tmp, tmp_bytes + 16));
  // the last element (slot nslices) is uninitialised before the scan: clear it first
  FG_CUDA_TRY(cudaMemsetAsync(sp->d_sptr + sp->nslices, 0, sizeof(int64_t), ctx->stream));
  cudaError_t e = cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, sp->d_sptr, sp->d_sptr, (int64_t)(sp->nslices + 1),
                                                ctx->stream);
  if (e != cudaSuccess) { dev_free(ctx, tmp); set_error("sell scan: %s", cudaGetErrorString(e)); return FG_ERR_CUDA; }
  FG_CUDA_TRY(cudaMemcpyAsync(&sp->sell_nnz, sp->d_sptr + sp->nslices, sizeof(int64_t), cudaMemcpyDeviceToHost,
                              ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, tmp);
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_scol, sizeof(int32_t) * (sp->sell_nnz > 0 ? sp->sell_nnz : 1)));
  k_sell_cols<<<nblk(sp->nslices * 32, 256), 256, 0, ctx->stream>>>(n, sp->nslices, sp->d_rowptr, sp->d_col,
                                                                     sp->d_perm, sp->d_iperm, sp->d_sptr, sp->d_scol);
  FG_CUDA_TRY(cudaGetLastError());
  ctx->launches += 1;
  return FG_OK;
}

fg_status system_fill_sell(fg_system* sys) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  if (sp->nfree == 0) return FG_OK;
  k_sell_vals<<<nblk(sp->nslices * 32, 256), 256, 0, ctx->stream>>>(sp->nfree, sp->nslices, sp->d_rowptr, sys->d_val,
                                                                     sp->d_perm, sp->d_sptr, sys->d_sval,
                                                                     sys->d_sval32);
  FG_CUDA_TRY(cudaGetLastError());
  ctx->launches += 1;
  return FG_OK;
}

}  // namespace fg

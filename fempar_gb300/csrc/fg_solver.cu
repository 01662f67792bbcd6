// fg_solver.cu -- CSR SpMV and the preconditioned CG of the reference, on the device.
//
// FP64 path: the operation sequence of cg_solve_body (Sources/Lib/LinearAlgebra/
// IterativeLinearSolver/cg.f90:101-238) with its stopping criteria (:279-407), Jacobi
// z = D^-1 r (jacobi_preconditioner.f90:356-412):
//   r = b - A x0; z = M r; r_z = <r,z>; p = z
//   loop: Ap = A p; alpha = r_z/<Ap,p>; x += alpha p; r -= alpha Ap; test;
//         z = M r; beta = (1/r_z) * <r,z>; r_z = <r,z>; p = z + beta p
// Each iteration is three kernels: SpMV with the fused <Ap,p>, the x/r update with the
// fused norms, and the p update.  Scalars (alpha, beta, r_z, the iteration counter and
// the done flag) stay on the device; kernels of an iteration that follows convergence
// return at once, so the host polls only every few iterations (CUDA-graph replays of a
// fixed chunk of iterations).  Reductions are deterministic: fixed grid, fixed
// per-thread index sets, block partials summed in index order by the last block.
//
// Mixed path: FP64 outer iterative refinement r = b - A x (FP64 matrix), inner PCG on
// the FP32 copy of the matrix with FP32 vectors and FP32 Jacobi, inner products and
// norms accumulated in FP64, x += correction in FP64.
#include <cmath>
#include <cstring>

#include "fg_internal.h"

namespace fg {

static constexpr int RB = 256;  // threads per block of the vector / SpMV kernels

// device scalar slots
enum { S_RZ = 0, S_ALPHA, S_BETA, S_ERR, S_TOL, S_APP, S_RNRMM, S_RZNEW, S_BNRM, S_R0NRM, S_COUNT = 16 };
enum { I_ITER = 0, I_DONE, I_CONV, I_MAXIT, I_COUNT = 8 };

struct RedBuf {
  double* part;       // [4][nblocks]
  unsigned* ticket;
  int nblocks;
};

template <int NV>
__device__ __forceinline__ bool block_reduce_last(double (&v)[NV], const RedBuf& rb, double (&tot)[NV]) {
  __shared__ double sw[NV][RB / 32];
  __shared__ bool s_last;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) sw[k][w] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = 0.0;
      for (int i = 0; i < RB / 32; ++i) s += sw[k][i];
      rb.part[k * rb.nblocks + blockIdx.x] = s;
    }
    __threadfence();
    unsigned t = atomicAdd(rb.ticket, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double s = 0.0;
    for (int i = threadIdx.x; i < rb.nblocks; i += RB) s += __ldcg(rb.part + k * rb.nblocks + i);
    v[k] = s;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
  }
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) sw[k][w] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = 0.0;
      for (int i = 0; i < RB / 32; ++i) s += sw[k][i];
      tot[k] = s;
    }
    *rb.ticket = 0u;
  }
  return true;
}

// ---------------------------------------------------------------------------
// SpMV, warp per row, rows strided over a fixed grid.  MODE 0: y = A x.
// MODE 1: y = A x and <y,x> reduced; sets alpha = r_z/<Ap,p>.
// MODE 2: r = b - A x and <r,r> reduced (residual of the refinement loop).
template <typename MT, typename VT, int MODE>
__global__ void __launch_bounds__(RB)
    k_spmv(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci, const MT* __restrict__ av,
           const VT* __restrict__ x, VT* __restrict__ y, const double* __restrict__ b, RedBuf rb, double* S,
           const int* I) {
  if (MODE == 1 && I[I_DONE]) return;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * RB + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * RB) >> 5;
  double dsum = 0.0;
  for (int64_t r = warp; r < n; r += nwarps) {
    const int64_t s = rp[r], e = rp[r + 1];
    double acc = 0.0;
    for (int64_t k = s + lane; k < e; k += 32) acc += (double)av[k] * (double)x[ci[k]];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (lane == 0) {
      if (MODE == 2) {
        double rr = b[r] - acc;
        y[r] = (VT)rr;
        dsum += rr * rr;
      } else {
        y[r] = (VT)acc;
        if (MODE == 1) dsum += acc * (double)x[r];
      }
    }
  }
  if (MODE == 0) return;
  double v[1] = {dsum}, tot[1];
  if (block_reduce_last<1>(v, rb, tot) && threadIdx.x == 0) {
    if (MODE == 1) {
      S[S_APP] = tot[0];
      S[S_ALPHA] = tot[0] != 0.0 ? S[S_RZ] / tot[0] : 0.0;
    } else {
      S[S_ERR] = sqrt(tot[0]);
    }
  }
}

// r = b - r (r holds A x0) or r = b; z = M r; p = z; reductions of <r,r>, <r,z>, <b,b>, <b,Mb>.
template <typename VT>
__global__ void __launch_bounds__(RB)
    k_init(int64_t n, const double* __restrict__ b, int have_x0, VT* __restrict__ r, VT* __restrict__ p,
           const VT* __restrict__ idiag, int precond, int criterion, double rtol, double atol, int maxit, RedBuf rb,
           double* S, int* I) {
  double rr = 0.0, rz = 0.0, bb = 0.0, bmb = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)RB + threadIdx.x; i < n; i += (int64_t)gridDim.x * RB) {
    double bi = b[i];
    VT ri = have_x0 ? (VT)(bi - (double)r[i]) : (VT)bi;
    VT zi = precond ? idiag[i] * ri : ri;
    VT mbi = precond ? (VT)((double)idiag[i] * bi) : (VT)bi;
    r[i] = ri;
    p[i] = zi;
    rr += (double)ri * (double)ri;
    rz += (double)ri * (double)zi;
    bb += bi * bi;
    bmb += bi * (double)mbi;
  }
  double v[4] = {rr, rz, bb, bmb}, tot[4];
  if (block_reduce_last<4>(v, rb, tot) && threadIdx.x == 0) {
    S[S_RZ] = tot[1];
    S[S_RNRMM] = sqrt(tot[1]);
    double rn = sqrt(tot[0]), bn = sqrt(tot[2]), bnm = sqrt(tot[3]);
    S[S_R0NRM] = rn;
    S[S_BNRM] = bn;
    double tol = 0.0;
    switch (criterion) {
      case FG_RES_RHS: case FG_DELTA_RHS: tol = rtol * bn + atol; break;
      case FG_RES_RES: tol = rtol * rn + atol; break;
      case FG_RES_NRMGIVEN_RHS_NRMGIVEN: tol = rtol * bnm + atol; break;
      case FG_RES_NRMGIVEN_RES_NRMGIVEN: tol = rtol * S[S_RNRMM] + atol; break;
      default: break;
    }
    S[S_TOL] = tol;
    S[S_ERR] = rn;
    I[I_ITER] = 0;
    I[I_DONE] = 0;
    I[I_CONV] = 0;
    I[I_MAXIT] = maxit;
  }
}

// x += alpha p; r -= alpha Ap; convergence test; beta and r_z for the next iteration.
template <typename VT>
__global__ void __launch_bounds__(RB)
    k_update(int64_t n, VT* __restrict__ x, VT* __restrict__ r, const VT* __restrict__ p, const VT* __restrict__ Ap,
             const VT* __restrict__ idiag, int precond, int criterion, double rtol, double atol, RedBuf rb, double* S,
             int* I) {
  if (I[I_DONE]) return;
  const double alpha = S[S_ALPHA];
  const VT a = (VT)alpha;
  double rr = 0.0, rz = 0.0, pp = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)RB + threadIdx.x; i < n; i += (int64_t)gridDim.x * RB) {
    VT pi = p[i];
    x[i] = a * pi + x[i];
    VT ri = -a * Ap[i] + r[i];
    r[i] = ri;
    VT zi = precond ? idiag[i] * ri : ri;
    rr += (double)ri * (double)ri;
    rz += (double)ri * (double)zi;
    pp += (double)pi * (double)pi;
  }
  double v[3] = {rr, rz, pp}, tot[3];
  if (block_reduce_last<3>(v, rb, tot) && threadIdx.x == 0) {
    const int it = I[I_ITER] + 1;
    I[I_ITER] = it;
    double err = S[S_ERR];
    if (it == 1 && (criterion == FG_DELTA_RHS || criterion == FG_DELTA_DELTA)) {
      err = alpha * sqrt(tot[2]);
      if (criterion == FG_DELTA_DELTA) S[S_TOL] = rtol * err + atol;
    }
    switch (criterion) {
      case FG_RES_RES: case FG_RES_RHS: err = sqrt(tot[0]); break;
      case FG_DELTA_RHS: case FG_DELTA_DELTA: if (it != 1) err = alpha * sqrt(tot[2]); break;
      default: err = S[S_RNRMM]; break;
    }
    S[S_ERR] = err;
    const bool conv = err <= S[S_TOL];
    if (conv || it >= I[I_MAXIT]) {
      I[I_DONE] = 1;
      I[I_CONV] = conv ? 1 : 0;
    } else {
      double beta = 1.0 / S[S_RZ];
      S[S_RZ] = tot[1];
      beta = beta * tot[1];
      S[S_BETA] = beta;
      S[S_RNRMM] = sqrt(tot[1]);
    }
  }
}

// p = z + beta p
template <typename VT>
__global__ void __launch_bounds__(RB)
    k_pupdate(int64_t n, VT* __restrict__ p, const VT* __restrict__ r, const VT* __restrict__ idiag, int precond,
              const double* S, const int* I) {
  if (I[I_DONE]) return;
  const VT beta = (VT)S[S_BETA];
  for (int64_t i = blockIdx.x * (int64_t)RB + threadIdx.x; i < n; i += (int64_t)gridDim.x * RB) {
    VT ri = r[i];
    VT zi = precond ? idiag[i] * ri : ri;
    p[i] = zi + beta * p[i];
  }
}

// inverse diagonal (extract_diagonal by binary search, csr_sparse_matrix.f90:4231-4256)
__global__ void k_inv_diag(int64_t n, const int64_t* rp, const int32_t* ci, const double* av, double* d64, float* d32) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  int64_t lo = rp[r], hi = rp[r + 1];
  while (lo < hi) {
    int64_t m = (lo + hi) >> 1;
    if (ci[m] < r) lo = m + 1;
    else hi = m;
  }
  double d = (lo < rp[r + 1] && ci[lo] == r) ? av[lo] : 0.0;
  double inv = 1.0 / d;
  d64[r] = inv;
  d32[r] = (float)inv;
}

__global__ void k_axpy_f2d(int64_t n, double s, const float* d, double* x) {
  int64_t i = blockIdx.x * (int64_t)RB + threadIdx.x;
  if (i < n) x[i] = x[i] + s * (double)d[i];
}
__global__ void k_scale(int64_t n, const double* a, double s, double* o) {
  int64_t i = blockIdx.x * (int64_t)RB + threadIdx.x;
  if (i < n) o[i] = a[i] * s;
}
__global__ void __launch_bounds__(RB) k_nrm2(int64_t n, const double* a, RedBuf rb, double* S) {
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)RB + threadIdx.x; i < n; i += (int64_t)gridDim.x * RB) s += a[i] * a[i];
  double v[1] = {s}, tot[1];
  if (block_reduce_last<1>(v, rb, tot) && threadIdx.x == 0) S[S_BNRM] = sqrt(tot[0]);
}
template <typename T>
__global__ void k_fill(int64_t n, T* a, T v) {
  int64_t i = blockIdx.x * (int64_t)RB + threadIdx.x;
  if (i < n) a[i] = v;
}

static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

struct Work {
  double *x, *r, *p, *Ap;   // FP64
  float *x32, *r32, *p32, *Ap32;
  double* S;
  int* I;
  RedBuf rb;
  unsigned grid_vec, grid_spmv;
};

static fg_status ensure_work(fg_system* sys, Work& w) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  const int64_t n = sp->nfree > 0 ? sp->nfree : 1;
  const unsigned gv = (unsigned)std::max<int64_t>(1, std::min<int64_t>(nblk(n, RB), (int64_t)ctx->sm_count * 8));
  if (!sys->d_work) {
    FG_TRY(dev_alloc(ctx, (void**)&sys->d_work, sizeof(double) * 4 * n));
    FG_TRY(dev_alloc(ctx, (void**)&sys->d_work32, sizeof(float) * 4 * n));
    sys->red_blocks = (int)std::max<unsigned>(gv, (unsigned)ctx->sm_count * 8);
    FG_TRY(dev_alloc(ctx, (void**)&sys->d_red, sizeof(double) * (4 * sys->red_blocks + S_COUNT) + sizeof(int) * I_COUNT));
    FG_TRY(dev_alloc(ctx, (void**)&sys->d_ticket, sizeof(unsigned) * 4));
    FG_CUDA_TRY(cudaMemsetAsync(sys->d_ticket, 0, sizeof(unsigned) * 4, ctx->stream));
  }
  w.x = sys->d_work; w.r = w.x + n; w.p = w.r + n; w.Ap = w.p + n;
  w.x32 = sys->d_work32; w.r32 = w.x32 + n; w.p32 = w.r32 + n; w.Ap32 = w.p32 + n;
  w.S = sys->d_red + 4 * sys->red_blocks;
  w.I = (int*)(w.S + S_COUNT);
  w.rb.part = sys->d_red;
  w.rb.ticket = sys->d_ticket;
  w.rb.nblocks = sys->red_blocks;
  w.grid_vec = (unsigned)sys->red_blocks;
  w.grid_spmv = (unsigned)sys->red_blocks;
  return FG_OK;
}

fg_status system_prepare_diag(fg_system* sys) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  const int64_t n = sp->nfree;
  if (!sys->d_idiag) {
    FG_TRY(dev_alloc(ctx, (void**)&sys->d_idiag, sizeof(double) * (n > 0 ? n : 1)));
    FG_TRY(dev_alloc(ctx, (void**)&sys->d_idiag32, sizeof(float) * (n > 0 ? n : 1)));
  }
  if (n > 0) {
    ctx->launches += 1;
    k_inv_diag<<<nblk(n, 256), 256, 0, ctx->stream>>>(n, sp->d_rowptr, sp->d_col, sys->d_val, sys->d_idiag,
                                                       sys->d_idiag32);
    FG_CUDA_TRY(cudaGetLastError());
  }
  return FG_OK;
}

fg_status system_spmv(fg_system* sys, int precision, const void* x, void* y, cudaStream_t st) {
  fg_space* sp = sys->space;
  Work w;
  FG_TRY(ensure_work(sys, w));
  const int64_t n = sp->nfree;
  if (n == 0) return FG_OK;
  if (precision == FG_MIXED)
    k_spmv<float, float, 0><<<w.grid_spmv, RB, 0, st>>>(n, sp->d_rowptr, sp->d_col, sys->d_val32, (const float*)x,
                                                         (float*)y, nullptr, w.rb, w.S, w.I);
  else
    k_spmv<double, double, 0><<<w.grid_spmv, RB, 0, st>>>(n, sp->d_rowptr, sp->d_col, sys->d_val, (const double*)x,
                                                           (double*)y, nullptr, w.rb, w.S, w.I);
  FG_CUDA_TRY(cudaGetLastError());
  return FG_OK;
}

// One CG iteration (3 kernels) for matrix type MT / vector type VT.
template <typename MT, typename VT>
static void launch_iteration(fg_system* sys, const Work& w, const MT* av, VT* x, VT* r, VT* p, VT* Ap, const VT* idiag,
                             int precond, int criterion, double rtol, double atol, cudaStream_t st) {
  fg_space* sp = sys->space;
  const int64_t n = sp->nfree;
  k_spmv<MT, VT, 1><<<w.grid_spmv, RB, 0, st>>>(n, sp->d_rowptr, sp->d_col, av, p, Ap, nullptr, w.rb, w.S, w.I);
  k_update<VT><<<w.grid_vec, RB, 0, st>>>(n, x, r, p, Ap, idiag, precond, criterion, rtol, atol, w.rb, w.S, w.I);
  k_pupdate<VT><<<w.grid_vec, RB, 0, st>>>(n, p, r, idiag, precond, w.S, w.I);
}

// Run CG iterations until the device done flag is set.  Returns iterations / converged.
template <typename MT, typename VT>
static fg_status run_cg_loop(fg_system* sys, const Work& w, const MT* av, VT* x, VT* r, VT* p, VT* Ap, const VT* idiag,
                             int precond, int criterion, double rtol, double atol, int check_every, int* h_I,
                             double* h_S) {
  fg_ctx* ctx = sys->space->mesh->ctx;
  cudaStream_t st = ctx->stream;
  // capture a chunk of iterations into a graph, replay until done
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  FG_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < check_every; ++k)
    launch_iteration<MT, VT>(sys, w, av, x, r, p, Ap, idiag, precond, criterion, rtol, atol, st);
  cudaError_t e = cudaStreamEndCapture(st, &graph);
  if (e != cudaSuccess) { set_error("graph capture: %s", cudaGetErrorString(e)); return FG_ERR_CUDA; }
  e = cudaGraphInstantiate(&exec, graph, 0);
  if (e != cudaSuccess) { cudaGraphDestroy(graph); set_error("graph instantiate: %s", cudaGetErrorString(e)); return FG_ERR_CUDA; }
  fg_status st_out = FG_OK;
  for (;;) {
    e = cudaGraphLaunch(exec, st);
    ctx->launches += 3 * check_every;
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_I, w.I, sizeof(int) * I_COUNT, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_S, w.S, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { set_error("cg loop: %s", cudaGetErrorString(e)); st_out = FG_ERR_CUDA; break; }
    if (h_I[I_DONE]) break;
    if (!std::isfinite(h_S[S_ERR])) { st_out = FG_ERR_NUMERIC; set_error("non-finite residual"); break; }
  }
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  return st_out;
}

fg_status system_solve(fg_system* sys, const fg_solver_params* prm, const double* d_b, const double* d_x0,
                       double* d_x, fg_solve_info* info) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  cudaStream_t st = ctx->stream;
  const int64_t n = sp->nfree;
  fg_solve_info out;
  std::memset(&out, 0, sizeof(out));
  if (n == 0) { out.converged = 1; if (info) *info = out; return FG_OK; }
  Work w;
  FG_TRY(ensure_work(sys, w));
  if (!sys->d_idiag) FG_TRY(system_prepare_diag(sys));
  const double* b = d_b ? d_b : sys->d_rhs;
  const int precond = prm->precond == FG_PREC_JACOBI ? 1 : 0;
  int check_every = prm->check_every > 0 ? prm->check_every : (n < 200000 ? 64 : 16);
  int h_I[I_COUNT];
  double h_S[S_COUNT];
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, st);
  const int64_t launches0 = ctx->launches;
  fg_status status = FG_OK;
  if (prm->precision == FG_FP64) {
    if (d_x0) {
      FG_CUDA_TRY(cudaMemcpyAsync(w.x, d_x0, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
      k_spmv<double, double, 0><<<w.grid_spmv, RB, 0, st>>>(n, sp->d_rowptr, sp->d_col, sys->d_val, w.x, w.r, nullptr,
                                                             w.rb, w.S, w.I);
    } else {
      k_fill<double><<<nblk(n, RB), RB, 0, st>>>(n, w.x, 0.0);
    }
    ctx->launches += 2;
    k_init<double><<<w.grid_vec, RB, 0, st>>>(n, b, d_x0 ? 1 : 0, w.r, w.p, sys->d_idiag, precond, prm->criterion,
                                              prm->rtol, prm->atol, prm->max_iters, w.rb, w.S, w.I);
    FG_CUDA_TRY(cudaGetLastError());
    status = run_cg_loop<double, double>(sys, w, sys->d_val, w.x, w.r, w.p, w.Ap, sys->d_idiag, precond, prm->criterion,
                                         prm->rtol, prm->atol, check_every, h_I, h_S);
    out.iterations = h_I[I_ITER];
    out.outer_iterations = 0;
    out.converged = h_I[I_CONV];
    out.error_estimate = h_S[S_ERR];
    out.tolerance = h_S[S_TOL];
    FG_CUDA_TRY(cudaMemcpyAsync(d_x, w.x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  } else {
    // FP64 iterative refinement around FP32 PCG (res_res on the true FP64 residual)
    const double inner_rtol = prm->inner_rtol > 0 ? prm->inner_rtol : 1e-4;
    const int inner_max = prm->inner_max_iters > 0 ? prm->inner_max_iters : prm->max_iters;
    if (d_x0) FG_CUDA_TRY(cudaMemcpyAsync(w.x, d_x0, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    else k_fill<double><<<nblk(n, RB), RB, 0, st>>>(n, w.x, 0.0);
    double tol = -1.0;
    int total_inner = 0, outer = 0;
    for (;;) {
      k_spmv<double, double, 2><<<w.grid_spmv, RB, 0, st>>>(n, sp->d_rowptr, sp->d_col, sys->d_val, w.x, w.r, b, w.rb,
                                                             w.S, w.I);
      ctx->launches += 1;
      FG_CUDA_TRY(cudaGetLastError());
      if (tol < 0 && prm->criterion == FG_RES_RHS) {
        ctx->launches += 1;
        k_nrm2<<<w.grid_vec, RB, 0, st>>>(n, b, w.rb, w.S);
        FG_CUDA_TRY(cudaGetLastError());
      }
      FG_CUDA_TRY(cudaMemcpyAsync(h_S, w.S, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, st));
      FG_CUDA_TRY(cudaStreamSynchronize(st));
      const double rn = h_S[S_ERR];
      if (!std::isfinite(rn)) { status = FG_ERR_NUMERIC; set_error("non-finite residual"); break; }
      if (tol < 0) tol = prm->rtol * (prm->criterion == FG_RES_RHS ? h_S[S_BNRM] : rn) + prm->atol;
      out.error_estimate = rn;
      out.tolerance = tol;
      if (rn <= tol) { out.converged = 1; break; }
      if (total_inner >= prm->max_iters) break;
      ++outer;
      // inner FP32 PCG on A d = r/|r| to a relative reduction inner_rtol
      ctx->launches += 4;  // scale, init, fill, correction
      k_scale<<<nblk(n, RB), RB, 0, st>>>(n, w.r, 1.0 / rn, w.Ap);
      k_init<float><<<w.grid_vec, RB, 0, st>>>(n, w.Ap, 0, w.r32, w.p32, sys->d_idiag32, precond, FG_RES_RES,
                                               inner_rtol, 0.0,
                                               std::max(1, std::min(inner_max, prm->max_iters - total_inner)), w.rb,
                                               w.S, w.I);
      k_fill<float><<<nblk(n, RB), RB, 0, st>>>(n, w.x32, 0.0f);
      FG_CUDA_TRY(cudaGetLastError());
      status = run_cg_loop<float, float>(sys, w, sys->d_val32, w.x32, w.r32, w.p32, w.Ap32, sys->d_idiag32, precond,
                                         FG_RES_RES, inner_rtol, 0.0, check_every, h_I, h_S);
      if (status != FG_OK) break;
      total_inner += h_I[I_ITER];
      k_axpy_f2d<<<nblk(n, RB), RB, 0, st>>>(n, rn, w.x32, w.x);
      FG_CUDA_TRY(cudaGetLastError());
    }
    out.iterations = total_inner;
    out.outer_iterations = outer;
    FG_CUDA_TRY(cudaMemcpyAsync(d_x, w.x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  }
  cudaEventRecord(e1, st);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  out.solve_ms = ms;
  out.kernel_launches = ctx->launches - launches0;
  if (info) *info = out;
  if (status == FG_OK && !out.converged) status = FG_ERR_NOT_CONVERGED;
  return status;
}

}  // namespace fg

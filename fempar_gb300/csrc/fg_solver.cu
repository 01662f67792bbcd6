// fg_solver.cu -- SELL-C-sigma SpMV and the preconditioned CG, on the device.
//
// FP64 path (the drop-in): the operation sequence of cg_solve_body
// (Sources/Lib/LinearAlgebra/IterativeLinearSolver/cg.f90:101-238) and its stopping
// criteria (:279-407), with Jacobi z = D^-1 r (jacobi_preconditioner.f90:356-412):
//   r = b - A x0; z = M r; r_z = <r,z>; p = z
//   loop: Ap = A p; alpha = r_z/<Ap,p>; x += alpha p; r -= alpha Ap; test;
//         z = M r; beta = (1/r_z) * <r,z>; r_z = <r,z>; p = z + beta p
// Three kernels per iteration: SpMV with the fused <Ap,p>, the x/r update with the fused
// norms and the convergence test, and the p update.  Scalars and the done flag stay on
// the device; kernels of iterations after the stop return at once, so the host polls
// only every few iterations, replaying a CUDA graph of a fixed chunk of iterations.
//
// Mixed path: CG on an FP32 copy of the matrix with FP32 vectors, with "reliable updates"
// in FP64: whenever the recursive FP32 residual has dropped by a factor delta (default 0.1)
// since the last update, or the estimate of the true residual reaches the tolerance, the
// FP32 correction is folded into the FP64 solution, the true residual r = b - A x is
// recomputed with the FP64 matrix, the FP32 residual is replaced by it (rescaled) and the
// search direction is kept (rescaled).  The solve stops on the FP64 true residual.  Keeping
// the direction keeps the iteration count close to the FP64 CG's, where restarting an inner
// solve per refinement step would lose the Krylov space each time.  With Jacobi the FP32
// segments run CG on D^-1/2 A D^-1/2 (the same iterates in exact arithmetic, no diagonal
// read per iteration) in two kernels per iteration (see k_update32s).
//
// Inner products.  GB300 runs FP64 FMA and FP32<->FP64 conversion at about 0.5 Tera-op/s,
// some 70x below FP32.  FP64-path dots accumulate in FP64.  FP32-path dots form each
// product exactly as an FP32 pair (p = a*b, e = fma(a,b,-p)) and accumulate it with a
// compensated (double-float) sum; each thread's sum is converted once and the block and
// grid totals are added in FP64.  Reductions are deterministic: fixed grid, fixed
// per-thread index sets, block partials summed in index order by the last block.
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>

#include "fg_internal.h"

namespace fg {

static constexpr int RB = 256;  // threads per block of the vector / SpMV kernels

enum { S_RZ = 0, S_ALPHA, S_BETA, S_ERR, S_TOL, S_APP, S_RNRMM, S_BNRM, S_R0NRM, S_SIGMA, S_RMAX, S_DELTA, S_RNSCALED,
       S_RRH, S_COUNT = 16 };
// I_PEND: a segment end decided by the last x/r/p update, taken at the next iteration;
// I_SKIPP: this iteration's update keeps p (the segment ends after it)
enum { I_ITER = 0, I_DONE, I_CONV, I_MAXIT, I_FLAG, I_PEND, I_SKIPP, I_COUNT = 8 };
// FLAG_BREAK: the FP32 recurrence broke down (non-finite or non-positive r_z, residual grown
// 1e4-fold): the segment's correction is dropped and the solve finishes in FP64
enum { FLAG_NONE = 0, FLAG_UPDATE = 1, FLAG_CHECK = 2, FLAG_MAXIT = 3, FLAG_BREAK = 4 };

struct RedBuf {
  double* part;  // [4][nblocks]
  unsigned* ticket;
  int nblocks;
};

// per-thread dot accumulators
template <typename VT>
struct Acc;
template <>
struct Acc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double a, double b) { s = fma(a, b, s); }
  __device__ __forceinline__ double value() const { return s; }
};
template <>
struct Acc<float> {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float pe = fmaf(a, b, -p);  // exact: a*b = p + pe
    const float s = __fadd_rn(hi, p);
    const float bb = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));  // TwoSum error
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(e, pe));
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// plain FP32 per-thread sum (products rounded): for sums whose terms are all positive
struct AccPlain {
  float s = 0.f;
  __device__ __forceinline__ void add(float a, float b) { s = fmaf(a, b, s); }
  __device__ __forceinline__ double value() const { return (double)s; }
};

// <q,q> of the fused mixed SpMV: compensated (1) or plain per-thread FP32 sums (0).  Measured
// on GB300 at 128^3 Q2: plain sums 1097 iterations and 0.853 ms per iteration, compensated
// 1106 and 0.863 ms (a thread sums ~80 positive terms; the grid total is formed in FP64).
#ifndef FG_MIXED_QQ_COMPENSATED
#define FG_MIXED_QQ_COMPENSATED 0
#endif
// the fused update sums the unscaled residual norm (the stop estimate) every
// FG_MIXED_EXACT_EVERY iterations (a divisor of the graph chunk); 8 vs 4: -2 us per iteration
#ifndef FG_MIXED_EXACT_EVERY
#define FG_MIXED_EXACT_EVERY 8
#endif

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
    for (int i = threadIdx.x; i < (int)gridDim.x; i += RB) s += __ldcg(rb.part + k * rb.nblocks + i);
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

__device__ __forceinline__ double fmaT(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmaT(float a, float b, float c) { return fmaf(a, b, c); }

// 4 consecutive matrix entries of one lane: one 128-bit (FP32) or 256-bit (FP64) streaming load
__device__ __forceinline__ void ld4(const float* p, float (&v)[4]) {
  const float4 t = __ldcs(reinterpret_cast<const float4*>(p));
  v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
__device__ __forceinline__ void ld4(const double* p, double (&v)[4]) {
  asm("ld.global.cs.v4.f64 {%0,%1,%2,%3}, [%4];" : "=d"(v[0]), "=d"(v[1]), "=d"(v[2]), "=d"(v[3]) : "l"(p));
}

// ---------------------------------------------------------------------------
// Mixed path, FP32 segments on the scaled system A^ = S A S, S = D^-1/2 (D = diag A): Jacobi
// PCG on A is CG on A^ with x = S x^ and r = S^-1 r^, so no diagonal is streamed per
// iteration.  Two kernels per iteration:
//   SpMV (MODE 3): q = A^ p, <p,q>, <q,q>; then alpha = |r|^2/<p,q> and, by the recurrence
//     |r - alpha q|^2 = alpha^2 |q|^2 - |r|^2 (as <r,q> = <p,q> in CG), beta = |r_new|^2/|r|^2;
//   update: x += alpha p; r -= alpha q; p = r + beta p; the exact |r_new|^2 for the next alpha,
//     and on every fourth iteration sum r^2 D (the unscaled residual, for the stop estimate).
// A segment end (reliable update, stop check, breakdown, iteration limit) found by an update
// is taken one iteration later: that iteration's update keeps p, so the host can fold x and
// restart the recursion from the true residual with the direction kept.
__device__ __forceinline__ void mixed_alpha_beta(double pap, double qq, double* S, int* I) {
  const double rr = S[S_RRH];
  int skip = I[I_PEND] != FLAG_NONE;
  double a = 0.0, b = 0.0;
  if (!(pap > 0.0 && pap <= 1e300) || !(qq <= 1e300)) {
    I[I_PEND] = FLAG_BREAK;  // alpha = 0: the update leaves x and r as they are
    skip = 1;
  } else {
    a = rr / pap;
    const double rrn = a * a * qq - rr;
    b = rrn / rr;
    if (!(rrn > 0.0)) {  // the recurrence lost its digits: end the segment here
      skip = 1;
      if (I[I_PEND] == FLAG_NONE) I[I_PEND] = FLAG_UPDATE;
    }
  }
  S[S_ALPHA] = a;
  S[S_BETA] = b;
  I[I_SKIPP] = skip;
}

template <bool EXACT>
__global__ void __launch_bounds__(RB)
    k_update32s(int64_t n, float* __restrict__ x, float* __restrict__ r, float* __restrict__ p,
                const float* __restrict__ q, const float* __restrict__ idiag, RedBuf rb, double* S, int* I) {
  if (I[I_DONE]) return;
  const float a = (float)S[S_ALPHA], b = (float)S[S_BETA];
  const bool keep_p = I[I_SKIPP] != 0;
  Acc<float> rr, rt;
  const int64_t t0 = blockIdx.x * (int64_t)RB + threadIdx.x, stride = (int64_t)gridDim.x * RB;
  const int64_t n4 = n >> 2;
  {
    float4* x4 = reinterpret_cast<float4*>(x);
    float4* r4 = reinterpret_cast<float4*>(r);
    float4* p4 = reinterpret_cast<float4*>(p);
    const float4* q4 = reinterpret_cast<const float4*>(q);
    const float4* d4 = reinterpret_cast<const float4*>(idiag);
    for (int64_t i = t0; i < n4; i += stride) {
      float4 xi = x4[i], ri = r4[i], pi = p4[i];
      const float4 qi = q4[i];
      xi.x = fmaf(a, pi.x, xi.x);
      xi.y = fmaf(a, pi.y, xi.y);
      xi.z = fmaf(a, pi.z, xi.z);
      xi.w = fmaf(a, pi.w, xi.w);
      ri.x = fmaf(-a, qi.x, ri.x);
      ri.y = fmaf(-a, qi.y, ri.y);
      ri.z = fmaf(-a, qi.z, ri.z);
      ri.w = fmaf(-a, qi.w, ri.w);
      x4[i] = xi;
      r4[i] = ri;
      if (!keep_p) {
        pi.x = fmaf(b, pi.x, ri.x);
        pi.y = fmaf(b, pi.y, ri.y);
        pi.z = fmaf(b, pi.z, ri.z);
        pi.w = fmaf(b, pi.w, ri.w);
        p4[i] = pi;
      }
      rr.add(ri.x, ri.x);
      rr.add(ri.y, ri.y);
      rr.add(ri.z, ri.z);
      rr.add(ri.w, ri.w);
      if (EXACT) {
        const float4 di = idiag ? d4[i] : make_float4(1.f, 1.f, 1.f, 1.f);
        // unscaled residual entry r^ sqrt(d): r^2 d = r^2 / (1/d); slots that are not free
        // dofs hold r = 0 and 1/d = 0: skipped
        rt.add(ri.x, di.x != 0.f ? ri.x / di.x : 0.f);
        rt.add(ri.y, di.y != 0.f ? ri.y / di.y : 0.f);
        rt.add(ri.z, di.z != 0.f ? ri.z / di.z : 0.f);
        rt.add(ri.w, di.w != 0.f ? ri.w / di.w : 0.f);
      }
    }
  }
  for (int64_t i = (n4 << 2) + t0; i < n; i += stride) {
    x[i] = fmaf(a, p[i], x[i]);
    const float ri = fmaf(-a, q[i], r[i]);
    r[i] = ri;
    if (!keep_p) p[i] = fmaf(b, p[i], ri);
    rr.add(ri, ri);
    if (EXACT) {
      const float di = idiag ? idiag[i] : 1.f;
      rt.add(ri, di != 0.f ? ri / di : 0.f);
    }
  }
  double v[2] = {rr.value(), rt.value()}, tot[2];
  if (block_reduce_last<2>(v, rb, tot) && threadIdx.x == 0) {
    const int it = I[I_ITER] + 1;
    I[I_ITER] = it;
    if (keep_p) {
      // the segment ends: |r|^2 of the new residual for the record; the old one stays in
      // S_RRH for the direction the host keeps
      S[S_APP] = tot[0];
      I[I_FLAG] = I[I_PEND] != FLAG_NONE ? I[I_PEND] : FLAG_UPDATE;
      I[I_DONE] = 1;
      return;
    }
    S[S_RRH] = tot[0];
    const double rn = sqrt(tot[0]);
    int pend = FLAG_NONE;
    if (!(rn <= 1e4 * S[S_RMAX])) pend = FLAG_BREAK;  // NaN fails too
    else if (EXACT && sqrt(tot[1]) * S[S_SIGMA] <= S[S_TOL]) pend = FLAG_CHECK;
    else if (rn < S[S_DELTA] * S[S_RMAX]) pend = FLAG_UPDATE;
    else if (it + 1 >= I[I_MAXIT]) pend = FLAG_MAXIT;
    if (rn > S[S_RMAX]) S[S_RMAX] = rn;
    S[S_RNSCALED] = rn;
    I[I_PEND] = pend;
  }
}

// x64 += sigma * s x^32; x^32 = 0 (s = D^-1/2 per slot; null: 1)
__global__ void k_fold_scaled(int64_t n, double sigma, const double* __restrict__ sd, float* __restrict__ x32,
                              double* __restrict__ x64) {
  for (int64_t i = blockIdx.x * (int64_t)RB + threadIdx.x; i < n; i += (int64_t)gridDim.x * RB) {
    const double si = sd ? sd[i] : 1.0;
    x64[i] = fma(sigma * si, (double)x32[i], x64[i]);
    x32[i] = 0.f;
  }
}

// r^32 = s r64 / sigma_new; |r^|^2; beta for keeping the direction (first: p = r^).
__global__ void __launch_bounds__(RB)
    k_refresh_scaled(int64_t n, const double* __restrict__ r64, const double* __restrict__ sd, float* __restrict__ r32,
                     int first, RedBuf rb, double* S, int* I) {
  const double inv = 1.0 / S[S_ERR];  // S_ERR = ||b - A x64|| from the FP64 residual SpMV
  Acc<float> rr;
  for (int64_t i = blockIdx.x * (int64_t)RB + threadIdx.x; i < n; i += (int64_t)gridDim.x * RB) {
    const float ri = (float)(r64[i] * inv * (sd ? sd[i] : 1.0));
    r32[i] = ri;
    rr.add(ri, ri);
  }
  double v[1] = {rr.value()}, tot[1];
  if (block_reduce_last<1>(v, rb, tot) && threadIdx.x == 0) {
    const double sig_old = S[S_SIGMA], sig_new = S[S_ERR];
    if (first) {
      S[S_BETA] = 0.0;
    } else {
      // old |r^|^2 and direction in the new scale: rr*(s_old/s_new)^2, p*(s_old/s_new)
      const double q = sig_old / sig_new;
      S[S_BETA] = tot[0] / (S[S_RRH] * q * q) * q;
    }
    S[S_RRH] = tot[0];
    S[S_SIGMA] = sig_new;
    S[S_RMAX] = sqrt(tot[0]);
    I[I_DONE] = 0;
    I[I_FLAG] = FLAG_NONE;
    I[I_PEND] = FLAG_NONE;
    I[I_SKIPP] = 0;
  }
}

// s = sqrt(1/d) per solver slot (0 where 1/d is 0: slots that are not free dofs)
__global__ void k_sqrt_idiag(int64_t n, const double* __restrict__ idiag, double* __restrict__ sd) {
  for (int64_t i = blockIdx.x * (int64_t)RB + threadIdx.x; i < n; i += (int64_t)gridDim.x * RB) {
    const double v = idiag[i];
    sd[i] = v > 0.0 ? sqrt(v) : 0.0;
  }
}

// FP32 copy of A^ = S A S in the lattice-implicit layout, from the FP64 values
__global__ void __launch_bounds__(RB)
    k_scale_stencil32(int64_t nslices, const uint8_t* __restrict__ scls, const int64_t* __restrict__ voff,
                      const StencilClass* __restrict__ cls,
                      const int32_t* __restrict__ soff, const int32_t* __restrict__ st_row,
                      const double* __restrict__ tval, const double* __restrict__ sd, int ncomp, float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * RB + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * RB) >> 5;
  for (int64_t s = warp; s < nslices; s += nwarps) {
    const int k = scls[s];
    const int Bp = cls[k].Bp, offbase = cls[k].offbase;
    int32_t st = st_row[s * 32 + lane];
    if (st < 0) st = ~st;  // padding lane: the slice's first row (its values are 0)
    const int32_t base = ncomp == 1 ? st : st - st % ncomp;
    const double srow = sd[st + cls[k].ownoff];
    const int64_t v0 = voff[s] + 4 * lane;
    for (int j = 0; j < (Bp >> 2); ++j) {
      const int4 o = __ldg(reinterpret_cast<const int4*>(soff + offbase) + j);
      const int64_t e = v0 + (int64_t)j * 128;
      // s_i s_j is one product for (i, j) and (j, i): the FP32 copy of an exactly symmetric
      // matrix stays exactly symmetric
      out[e + 0] = (float)(tval[e + 0] * (srow * sd[base + o.x]));
      out[e + 1] = (float)(tval[e + 1] * (srow * sd[base + o.y]));
      out[e + 2] = (float)(tval[e + 2] * (srow * sd[base + o.z]));
      out[e + 3] = (float)(tval[e + 3] * (srow * sd[base + o.w]));
    }
  }
}

// the same in the explicit-column SELL layout
__global__ void __launch_bounds__(RB)
    k_scale_sell32(int64_t nslices, int64_t n, const int64_t* __restrict__ sptr, const int32_t* __restrict__ scol,
                   const double* __restrict__ sval, const double* __restrict__ sd, float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * RB + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * RB) >> 5;
  for (int64_t s = warp; s < nslices; s += nwarps) {
    const int64_t base = sptr[s];
    const int w4 = (int)((sptr[s + 1] - base) >> 7);
    const int64_t slot = s * 32 + lane;
    const double srow = slot < n ? sd[slot] : 0.0;
    for (int j = 0; j < w4; ++j) {
      const int64_t e = base + 4 * lane + (int64_t)j * 128;
#pragma unroll
      for (int t = 0; t < 4; ++t) out[e + t] = (float)(sval[e + t] * (srow * sd[scol[e + t]]));
    }
  }
}

// ---------------------------------------------------------------------------
// SELL SpMV, warp per slice, lane per row, slices strided over a fixed grid.
// MODE 0: y = A x.  MODE 1: y = A x, <y,x> reduced, alpha = r_z/<Ap,p>.
// MODE 2: y = b - A x (b FP64), <y,y> reduced into S_ERR as a norm.
template <typename T, int MODE>
__global__ void __launch_bounds__(RB)
    k_sell_spmv(int64_t nslices, int64_t n, const int64_t* __restrict__ sptr, const int32_t* __restrict__ scol,
                const T* __restrict__ sval, const T* __restrict__ x, T* __restrict__ y, const double* __restrict__ b,
                RedBuf rb, double* S, const int* I) {
  if ((MODE == 1 || MODE == 3) && I[I_DONE]) return;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * RB + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * RB) >> 5;
  Acc<T> dot;
#if FG_MIXED_QQ_COMPENSATED
  Acc<T> dot2;
#else
  AccPlain dot2;
#endif
  for (int64_t s = warp; s < nslices; s += nwarps) {
    const int64_t base = sptr[s];
    const int w4 = (int)((sptr[s + 1] - base) >> 7);  // groups of 4 entries per lane
    const T* vp = sval + base + 4 * lane;
    const int32_t* cp = scol + base + 4 * lane;
    T acc = 0;
#pragma unroll 2
    for (int j = 0; j < w4; ++j) {
      T v[4];
      ld4(vp, v);
      const int4 c = __ldcs(reinterpret_cast<const int4*>(cp));
      const T x0 = __ldg(x + c.x), x1 = __ldg(x + c.y), x2 = __ldg(x + c.z), x3 = __ldg(x + c.w);
      acc = fmaT(v[0], x0, acc);
      acc = fmaT(v[1], x1, acc);
      acc = fmaT(v[2], x2, acc);
      acc = fmaT(v[3], x3, acc);
      vp += 128;
      cp += 128;
    }
    const int64_t slot = s * 32 + lane;
    if (slot < n) {
      if (MODE == 2) {
        const T rr = (T)(b[slot] - (double)acc);
        y[slot] = rr;
        dot.add(rr, rr);
      } else {
        y[slot] = acc;
        if (MODE == 1 || MODE == 3) dot.add(acc, x[slot]);
        if (MODE == 3) dot2.add(acc, acc);
      }
    }
  }
  if (MODE == 0) return;
  if (MODE == 3) {
    double v2[2] = {dot.value(), dot2.value()}, tot2[2];
    if (block_reduce_last<2>(v2, rb, tot2) && threadIdx.x == 0) mixed_alpha_beta(tot2[0], tot2[1], S, const_cast<int*>(I));
    return;
  }
  double v[1] = {dot.value()}, tot[1];
  if (block_reduce_last<1>(v, rb, tot) && threadIdx.x == 0) {
    if (MODE == 1) {
      S[S_APP] = tot[0];
      S[S_ALPHA] = tot[0] != 0.0 ? S[S_RZ] / tot[0] : 0.0;
    } else {
      S[S_ERR] = sqrt(tot[0]);
    }
  }
}

// FP64 path start: r = b - r (r holds A x0) or r = b; z = M r; p = z; <r,r>, <r,z>, <b,b>, <b,Mb>.
__global__ void __launch_bounds__(RB)
    k_init64(int64_t n, const double* __restrict__ b, int have_x0, double* __restrict__ r, double* __restrict__ p,
             const double* __restrict__ idiag, int precond, int criterion, double rtol, double atol, int maxit,
             RedBuf rb, double* S, int* I) {
  Acc<double> rr, rz, bb, bmb;
  for (int64_t i = blockIdx.x * (int64_t)RB + threadIdx.x; i < n; i += (int64_t)gridDim.x * RB) {
    const double bi = b[i];
    const double ri = have_x0 ? bi - r[i] : bi;
    const double zi = precond ? idiag[i] * ri : ri;
    r[i] = ri;
    p[i] = zi;
    rr.add(ri, ri);
    rz.add(ri, zi);
    bb.add(bi, bi);
    bmb.add(bi, precond ? idiag[i] * bi : bi);
  }
  double v[4] = {rr.value(), rz.value(), bb.value(), bmb.value()}, tot[4];
  if (block_reduce_last<4>(v, rb, tot) && threadIdx.x == 0) {
    S[S_RZ] = tot[1];
    S[S_RNRMM] = sqrt(tot[1]);
    const double rn = sqrt(tot[0]), bn = sqrt(tot[2]), bnm = sqrt(tot[3]);
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
    I[I_FLAG] = FLAG_NONE;
  }
}

// FP64 path: x += alpha p; r -= alpha Ap; the reference's convergence test; beta, r_z.
template <bool PRECOND, bool NEED_PP>
__global__ void __launch_bounds__(RB)
    k_update64(int64_t n, double* __restrict__ x, double* __restrict__ r, const double* __restrict__ p,
               const double* __restrict__ Ap, const double* __restrict__ idiag, int criterion, double rtol,
               double atol, RedBuf rb, double* S, int* I) {
  if (I[I_DONE]) return;
  const double a = S[S_ALPHA];
  Acc<double> rr, rz, pp;
  for (int64_t i = blockIdx.x * (int64_t)RB + threadIdx.x; i < n; i += (int64_t)gridDim.x * RB) {
    const double pi = p[i];
    x[i] = fma(a, pi, x[i]);
    const double ri = fma(-a, Ap[i], r[i]);
    r[i] = ri;
    rr.add(ri, ri);
    if (PRECOND) rz.add(ri, idiag[i] * ri);
    if (NEED_PP) pp.add(pi, pi);
  }
  double v[3] = {rr.value(), PRECOND ? rz.value() : rr.value(), pp.value()}, tot[3];
  if (block_reduce_last<3>(v, rb, tot) && threadIdx.x == 0) {
    const int it = I[I_ITER] + 1;
    I[I_ITER] = it;
    double err = S[S_ERR];
    if (it == 1 && (criterion == FG_DELTA_RHS || criterion == FG_DELTA_DELTA)) {
      err = a * sqrt(tot[2]);
      if (criterion == FG_DELTA_DELTA) S[S_TOL] = rtol * err + atol;
    }
    switch (criterion) {
      case FG_RES_RES: case FG_RES_RHS: err = sqrt(tot[0]); break;
      case FG_DELTA_RHS: case FG_DELTA_DELTA: if (it != 1) err = a * sqrt(tot[2]); break;
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

// p = z + beta p (FP32: four entries per thread and load; the vectors are 16-byte aligned)
template <typename T, bool PRECOND>
__global__ void __launch_bounds__(RB)
    k_pupdate(int64_t n, T* __restrict__ p, const T* __restrict__ r, const T* __restrict__ idiag, const double* S,
              const int* I) {
  if (I[I_DONE]) return;
  const T beta = (T)S[S_BETA];
  const int64_t t0 = blockIdx.x * (int64_t)RB + threadIdx.x, stride = (int64_t)gridDim.x * RB;
  int64_t head = 0;
  if (sizeof(T) == 4) {
    const int64_t n4 = n >> 2;
    head = n4 << 2;
    float4* p4 = reinterpret_cast<float4*>(p);
    const float4* r4 = reinterpret_cast<const float4*>(r);
    const float4* d4 = reinterpret_cast<const float4*>(idiag);
    const float b = (float)beta;
    for (int64_t i = t0; i < n4; i += stride) {
      const float4 ri = r4[i];
      float4 pi = p4[i];
      float4 di = make_float4(1.f, 1.f, 1.f, 1.f);
      if (PRECOND) di = d4[i];
      pi.x = fmaf(b, pi.x, PRECOND ? di.x * ri.x : ri.x);
      pi.y = fmaf(b, pi.y, PRECOND ? di.y * ri.y : ri.y);
      pi.z = fmaf(b, pi.z, PRECOND ? di.z * ri.z : ri.z);
      pi.w = fmaf(b, pi.w, PRECOND ? di.w * ri.w : ri.w);
      p4[i] = pi;
    }
  }
  for (int64_t i = head + t0; i < n; i += stride) {
    const T ri = r[i];
    const T zi = PRECOND ? idiag[i] * ri : ri;
    p[i] = fmaT(beta, p[i], zi);
  }
}

// ---------------------------------------------------------------------------
// Lattice-implicit SELL SpMV: warp per slice, lane per row, 4 values per lane per load;
// the column of box position k is the row's node plus the class offset k.
// L2 prefetch distance of the FP32 SpMV's value stream, in groups of 4 entries per lane.
// Swept on GB300 at 128^3 Q2 (unroll 2): 2-4 groups 0.731-0.735 ms per launch, 6 0.747,
// 8 0.757, 16 0.810.
#ifndef FG_SPMV_PREFETCH
#define FG_SPMV_PREFETCH 3
#endif
#ifndef FG_SPMV_UNROLL
#define FG_SPMV_UNROLL 2
#endif
static constexpr int kPrefetch = FG_SPMV_PREFETCH;  // value groups (of 4 entries per lane) prefetched ahead
static constexpr int kUnroll = FG_SPMV_UNROLL;      // value groups per unrolled step
template <typename T, int MODE>
__global__ void __launch_bounds__(RB)
    k_stencil_spmv(int64_t nslices, const uint8_t* __restrict__ scls, const int64_t* __restrict__ voff,
                   const StencilClass* __restrict__ cls, const int32_t* __restrict__ soff,
                   const int32_t* __restrict__ st_row, const T* __restrict__ tval,
                   int ncomp, const T* __restrict__ x, T* __restrict__ y, const double* __restrict__ b, RedBuf rb,
                   double* S, const int* I) {
  if ((MODE == 1 || MODE == 3) && I[I_DONE]) return;
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * RB + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * RB) >> 5;
  Acc<T> dot;
#if FG_MIXED_QQ_COMPENSATED
  Acc<T> dot2;
#else
  AccPlain dot2;
#endif
  for (int64_t s = warp; s < nslices; s += nwarps) {
    const int k = scls[s];
    const int64_t vb = voff[s];
    const int Bp = cls[k].Bp, offbase = cls[k].offbase;
    // st = node index in the class sub-lattice * ncomp + component; the row's own entry is
    // in the class's sub-lattice, its box columns are base + table offsets.  Padding lanes
    // hold the complement of the slice's first row (valid addresses, values 0, no store).
    int32_t st = st_row[s * 32 + lane];
    const bool valid = st >= 0;
    if (!valid) st = ~st;
    const int32_t base = ncomp == 1 ? st : st - st % ncomp;
    const int64_t vec = st + cls[k].ownoff;
    const T* vp = tval + vb + 4 * lane;
    const int4* op = reinterpret_cast<const int4*>(soff + offbase);
    const T* xb = x + base;
    T acc = 0;
    const int w4 = Bp >> 2;
#pragma unroll kUnroll
    for (int j = 0; j < w4; ++j) {
      // FP32: keep the value stream ahead of the gathers by asking L2 for this lane's values
      // kPrefetch groups ahead (no registers held; a hint only, kept inside the slice).  The
      // FP64 variant is bound by the FP64 pipe and runs slower with it.
      if (sizeof(T) == 4 && j + kPrefetch < w4) asm volatile("prefetch.global.L2 [%0];" ::"l"(vp + kPrefetch * 128));
      T v[4];
      ld4(vp, v);
      const int4 o = __ldg(op + j);
      const T x0 = __ldg(xb + o.x), x1 = __ldg(xb + o.y), x2 = __ldg(xb + o.z), x3 = __ldg(xb + o.w);
      acc = fmaT(v[0], x0, acc);
      acc = fmaT(v[1], x1, acc);
      acc = fmaT(v[2], x2, acc);
      acc = fmaT(v[3], x3, acc);
      vp += 128;
    }
    if (valid) {
      if (MODE == 2) {
        const T rr = (T)(b[vec] - (double)acc);
        y[vec] = rr;
        dot.add(rr, rr);
      } else {
        y[vec] = acc;
        if (MODE == 1 || MODE == 3) dot.add(acc, x[vec]);
        if (MODE == 3) dot2.add(acc, acc);
      }
    }
  }
  if (MODE == 0) return;
  if (MODE == 3) {
    double v2[2] = {dot.value(), dot2.value()}, tot2[2];
    if (block_reduce_last<2>(v2, rb, tot2) && threadIdx.x == 0) mixed_alpha_beta(tot2[0], tot2[1], S, const_cast<int*>(I));
    return;
  }
  double v[1] = {dot.value()}, tot[1];
  if (block_reduce_last<1>(v, rb, tot) && threadIdx.x == 0) {
    if (MODE == 1) {
      S[S_APP] = tot[0];
      S[S_ALPHA] = tot[0] != 0.0 ? S[S_RZ] / tot[0] : 0.0;
    } else {
      S[S_ERR] = sqrt(tot[0]);
    }
  }
}

// inverse diagonal in the solver layout (extract_diagonal by binary search,
// csr_sparse_matrix.f90:4231-4256); entries of non-free vector slots stay 0
__global__ void k_inv_diag(int64_t n, const int64_t* rp, const int32_t* ci, const double* av, const int32_t* row2vec,
                           double* d64, float* d32) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  int64_t lo = rp[r], hi = rp[r + 1];
  while (lo < hi) {
    int64_t m = (lo + hi) >> 1;
    if (ci[m] < r) lo = m + 1;
    else hi = m;
  }
  const double d = (lo < rp[r + 1] && ci[lo] == r) ? av[lo] : 0.0;
  const double inv = 1.0 / d;
  const int32_t v = row2vec[r];
  d64[v] = inv;
  d32[v] = (float)inv;
}

// row order <-> solver layout
template <typename TS, typename TD>
__global__ void k_rows_to_vec(int64_t n, const int32_t* __restrict__ row2vec, const TS* __restrict__ src,
                              TD* __restrict__ dst) {
  int64_t r = blockIdx.x * (int64_t)RB + threadIdx.x;
  if (r < n) dst[row2vec[r]] = (TD)src[r];
}
template <typename TS, typename TD>
__global__ void k_vec_to_rows(int64_t n, const int32_t* __restrict__ row2vec, const TS* __restrict__ src,
                              TD* __restrict__ dst) {
  int64_t r = blockIdx.x * (int64_t)RB + threadIdx.x;
  if (r < n) dst[r] = (TD)src[row2vec[r]];
}
template <typename T>
__global__ void k_fill(int64_t n, T* a, T v) {
  int64_t i = blockIdx.x * (int64_t)RB + threadIdx.x;
  if (i < n) a[i] = v;
}
__global__ void k_set_scalar(double* S, int slot, double v) { S[slot] = v; }

static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

struct Work {
  double *x, *r, *p, *Ap, *b, *t;  // FP64, solver layout
  float *x32, *r32, *p32, *Ap32;
  double *io;                       // FP64 row-order staging (x0 of spmv)
  double* S;
  int* I;
  RedBuf rb;
  int sms;
};

// Grid of a grid-stride kernel: exactly the blocks that are co-resident (one wave), from
// the occupancy of that kernel.  Every block does the same share of the work, so a
// second wave would double the kernel's time; the grid is fixed per kernel, which keeps
// the block-partial reductions deterministic.
static unsigned grid_for(const void* k, int sms) {
  static std::mutex mu;
  static std::map<const void*, unsigned> cache;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(k);
  if (it != cache.end()) return it->second;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, RB, 0) != cudaSuccess) { cudaGetLastError(); nb = 1; }
  if (nb < 1) nb = 1;
  if (nb > 8) nb = 8;
  const unsigned g = (unsigned)(nb * sms);
  cache[k] = g;
  return g;
}

template <typename... KA, typename... A>
static inline void launch_k(void (*k)(KA...), const Work& w, cudaStream_t st, A... args) {
  k<<<grid_for((const void*)k, w.sms), RB, 0, st>>>(args...);
}

static fg_status ensure_work(fg_system* sys, Work& w) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  // vector stride a multiple of 4 entries: every FP32 vector starts on a 16-byte boundary
  // (the FP32 update kernels load float4)
  const int64_t n = ((sp->nvec > 0 ? sp->nvec : 1) + 3) & ~(int64_t)3;
  if (!sys->d_work) {
    FG_TRY(dev_alloc(ctx, (void**)&sys->d_work, sizeof(double) * 6 * n));
    FG_TRY(dev_alloc(ctx, (void**)&sys->d_work32, sizeof(float) * 4 * n));
    // entries of non-free vector slots must read zero for the whole life of the buffers
    FG_CUDA_TRY(cudaMemsetAsync(sys->d_work, 0, sizeof(double) * 6 * n, ctx->stream));
    FG_CUDA_TRY(cudaMemsetAsync(sys->d_work32, 0, sizeof(float) * 4 * n, ctx->stream));
    sys->red_blocks = ctx->sm_count * 8;
    FG_TRY(dev_alloc(ctx, (void**)&sys->d_red, sizeof(double) * (4 * sys->red_blocks + S_COUNT) + sizeof(int) * I_COUNT));
    FG_TRY(dev_alloc(ctx, (void**)&sys->d_ticket, sizeof(unsigned) * 4));
    FG_CUDA_TRY(cudaMemsetAsync(sys->d_ticket, 0, sizeof(unsigned) * 4, ctx->stream));
  }
  w.x = sys->d_work; w.r = w.x + n; w.p = w.r + n; w.Ap = w.p + n; w.b = w.Ap + n; w.t = w.b + n;
  w.x32 = sys->d_work32; w.r32 = w.x32 + n; w.p32 = w.r32 + n; w.Ap32 = w.p32 + n;
  w.io = nullptr;
  w.S = sys->d_red + 4 * sys->red_blocks;
  w.I = (int*)(w.S + S_COUNT);
  w.rb.part = sys->d_red;
  w.rb.ticket = sys->d_ticket;
  w.rb.nblocks = sys->red_blocks;
  w.sms = ctx->sm_count;
  return FG_OK;
}

fg_status system_prepare_diag(fg_system* sys) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  const int64_t n = sp->nfree, nv = sp->nvec > 0 ? sp->nvec : 1;
  if (!sys->d_idiag) {
    FG_TRY(dev_alloc(ctx, (void**)&sys->d_idiag, sizeof(double) * nv));
    FG_TRY(dev_alloc(ctx, (void**)&sys->d_idiag32, sizeof(float) * nv));
    FG_CUDA_TRY(cudaMemsetAsync(sys->d_idiag, 0, sizeof(double) * nv, ctx->stream));
    FG_CUDA_TRY(cudaMemsetAsync(sys->d_idiag32, 0, sizeof(float) * nv, ctx->stream));
  }
  if (sp->layout == FG_LAYOUT_STENCIL && sys->d_tval) return system_inv_diag_stencil(sys);
  if (n > 0) {
    ctx->launches += 1;
    k_inv_diag<<<nblk(n, 256), 256, 0, ctx->stream>>>(n, sp->d_rowptr, sp->d_col, sys->d_val, sp->d_row2vec,
                                                       sys->d_idiag, sys->d_idiag32);
    FG_CUDA_TRY(cudaGetLastError());
  }
  return FG_OK;
}

// SpMV of the active solver layout on solver-layout vectors
template <typename T, int MODE>
static void spmv_k(fg_system* sys, const Work& w, const T* x, T* y, const double* b, cudaStream_t st);

#define FG_SPMV_IMPL(T, MODE, VALS, TVALS)                                                                          \
  template <>                                                                                                       \
  void spmv_k<T, MODE>(fg_system * sys, const Work& w, const T* x, T* y, const double* b, cudaStream_t st) {       \
    fg_space* sp = sys->space;                                                                                      \
    if (sp->layout == FG_LAYOUT_STENCIL)                                                                            \
      launch_k(k_stencil_spmv<T, MODE>, w, st, sp->st_nslices, (const uint8_t*)sp->d_st_scls,                       \
               (const int64_t*)sp->d_st_voff, (const StencilClass*)sp->d_st_cls, (const int32_t*)sp->d_st_off, (const int32_t*)sp->d_st_row,       \
               (const T*)sys->TVALS, sp->ncomp, x, y, b, w.rb, w.S, (const int*)w.I);                               \
    else                                                                                                            \
      launch_k(k_sell_spmv<T, MODE>, w, st, sp->nslices, sp->nfree, (const int64_t*)sp->d_sptr,                     \
               (const int32_t*)sp->d_scol, (const T*)sys->VALS, x, y, b, w.rb, w.S, (const int*)w.I);              \
    sp->mesh->ctx->launches += 1;                                                                                   \
  }
FG_SPMV_IMPL(double, 0, d_sval, d_tval)
FG_SPMV_IMPL(double, 1, d_sval, d_tval)
FG_SPMV_IMPL(double, 2, d_sval, d_tval)
FG_SPMV_IMPL(float, 0, d_sval32, d_tval32)
FG_SPMV_IMPL(float, 1, d_sval32, d_tval32)
#undef FG_SPMV_IMPL

// FP32 SpMV of the fused mixed iteration on the given values (the scaled copy with Jacobi,
// the plain FP32 copy without a preconditioner)
static void spmv_fused32(fg_system* sys, const Work& w, const float* vals, const float* x, float* y, cudaStream_t st) {
  fg_space* sp = sys->space;
  if (sp->layout == FG_LAYOUT_STENCIL)
    launch_k(k_stencil_spmv<float, 3>, w, st, sp->st_nslices, (const uint8_t*)sp->d_st_scls,
             (const int64_t*)sp->d_st_voff, (const StencilClass*)sp->d_st_cls, (const int32_t*)sp->d_st_off, (const int32_t*)sp->d_st_row, vals,
             sp->ncomp, x, y, (const double*)nullptr, w.rb, w.S, (const int*)w.I);
  else
    launch_k(k_sell_spmv<float, 3>, w, st, sp->nslices, sp->nfree, (const int64_t*)sp->d_sptr,
             (const int32_t*)sp->d_scol, vals, x, y, (const double*)nullptr, w.rb, w.S, (const int*)w.I);
  sp->mesh->ctx->launches += 1;
}

// D^-1/2 and the FP32 copy of D^-1/2 A D^-1/2 (once per numeric assembly)
static fg_status ensure_scaled(fg_system* sys, const Work& w) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  if (sys->scaled_valid) return FG_OK;
  const bool stencil = sp->layout == FG_LAYOUT_STENCIL;
  const int64_t nvals = stencil ? sp->st_nvals : sp->sell_nnz;
  const double* v64 = stencil ? sys->d_tval : sys->d_sval;
  if (!v64) { set_error("the FP64 solver-layout values are not available"); return FG_ERR_UNSUPPORTED; }
  const int64_t nv = sp->nvec > 0 ? sp->nvec : 1;
  if (!sys->d_sdiag) FG_TRY(dev_alloc(ctx, (void**)&sys->d_sdiag, sizeof(double) * nv));
  if (!sys->d_val32s) FG_TRY(dev_alloc(ctx, (void**)&sys->d_val32s, sizeof(float) * (nvals > 0 ? nvals : 1)));
  cudaStream_t st = ctx->stream;
  launch_k(k_sqrt_idiag, w, st, nv, (const double*)sys->d_idiag, sys->d_sdiag);
  if (stencil)
    launch_k(k_scale_stencil32, w, st, sp->st_nslices, (const uint8_t*)sp->d_st_scls, (const int64_t*)sp->d_st_voff,
             (const StencilClass*)sp->d_st_cls,
             (const int32_t*)sp->d_st_off, (const int32_t*)sp->d_st_row, v64, (const double*)sys->d_sdiag, sp->ncomp,
             sys->d_val32s);
  else
    launch_k(k_scale_sell32, w, st, sp->nslices, sp->nfree, (const int64_t*)sp->d_sptr, (const int32_t*)sp->d_scol, v64,
             (const double*)sys->d_sdiag, sys->d_val32s);
  ctx->launches += 2;
  FG_CUDA_TRY(cudaGetLastError());
  sys->scaled_valid = true;
  return FG_OK;
}

// y = A x in row order (device pointers): into the solver layout, SpMV, back.
fg_status system_spmv(fg_system* sys, int precision, const void* x, void* y, cudaStream_t st) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  Work w;
  FG_TRY(ensure_work(sys, w));
  const int64_t n = sp->nfree;
  if (n == 0) return FG_OK;
  if (precision == FG_MIXED) {
    k_rows_to_vec<float, float><<<nblk(n, RB), RB, 0, st>>>(n, sp->d_row2vec, (const float*)x, w.p32);
    spmv_k<float, 0>(sys, w, w.p32, w.Ap32, nullptr, st);
    k_vec_to_rows<float, float><<<nblk(n, RB), RB, 0, st>>>(n, sp->d_row2vec, w.Ap32, (float*)y);
  } else {
    k_rows_to_vec<double, double><<<nblk(n, RB), RB, 0, st>>>(n, sp->d_row2vec, (const double*)x, w.p);
    spmv_k<double, 0>(sys, w, w.p, w.Ap, nullptr, st);
    k_vec_to_rows<double, double><<<nblk(n, RB), RB, 0, st>>>(n, sp->d_row2vec, w.Ap, (double*)y);
  }
  ctx->launches += 2;
  FG_CUDA_TRY(cudaGetLastError());
  return FG_OK;
}

// reps launches of the solver-layout SpMV alone on solver-layout vectors (timing)
fg_status system_spmv_slot(fg_system* sys, int precision, const void* x, void* y, int reps, cudaStream_t st) {
  Work w;
  FG_TRY(ensure_work(sys, w));
  if (sys->space->nfree == 0) return FG_OK;
  for (int k = 0; k < reps; ++k) {
    if (precision == FG_MIXED) spmv_k<float, 0>(sys, w, (const float*)x, (float*)y, nullptr, st);
    else spmv_k<double, 0>(sys, w, (const double*)x, (double*)y, nullptr, st);
  }
  FG_CUDA_TRY(cudaGetLastError());
  return FG_OK;
}

int64_t system_vec_len(fg_system* sys) { return sys->space->nvec; }

// One SpMV of the active solver layout on caller-provided solver-layout vectors, without
// touching the system's work buffers (no allocation).  The MODE 0 kernels take no
// reduction buffers.
fg_status system_spmv_layout_noalloc(fg_system* sys, int precision, const void* xvec, void* yvec, cudaStream_t st) {
  Work w;
  std::memset(&w, 0, sizeof(w));
  w.sms = sys->space->mesh->ctx->sm_count;
  if (sys->space->nfree == 0) return FG_OK;
  if (precision == FG_MIXED) spmv_k<float, 0>(sys, w, (const float*)xvec, (float*)yvec, nullptr, st);
  else spmv_k<double, 0>(sys, w, (const double*)xvec, (double*)yvec, nullptr, st);
  FG_CUDA_TRY(cudaGetLastError());
  return FG_OK;
}

// Launch one FP64 CG iteration (3 kernels).
static void iter64(fg_system* sys, const Work& w, int precond, bool need_pp, int criterion, double rtol, double atol,
                   cudaStream_t st) {
  fg_space* sp = sys->space;
  const int64_t n = sp->nvec;
  spmv_k<double, 1>(sys, w, w.p, w.Ap, nullptr, st);
#define FG_UPD(P, Q) \
  launch_k(k_update64<P, Q>, w, st, n, w.x, w.r, (const double*)w.p, (const double*)w.Ap, (const double*)sys->d_idiag, criterion, rtol, atol, w.rb, w.S, w.I)
  if (precond) { if (need_pp) FG_UPD(true, true); else FG_UPD(true, false); }
  else { if (need_pp) FG_UPD(false, true); else FG_UPD(false, false); }
#undef FG_UPD
  if (precond) launch_k(k_pupdate<double, true>, w, st, n, w.p, (const double*)w.r, (const double*)sys->d_idiag, (const double*)w.S, (const int*)w.I);
  else launch_k(k_pupdate<double, false>, w, st, n, w.p, (const double*)w.r, (const double*)sys->d_idiag, (const double*)w.S, (const int*)w.I);
}

// Launch one fused FP32 iteration of the mixed path (2 kernels); `exact`: this update also
// sums the unscaled residual norm for the stop estimate.
static void iter32s(fg_system* sys, const Work& w, const float* vals, const float* idiag32, bool exact, cudaStream_t st) {
  const int64_t n = sys->space->nvec;
  spmv_fused32(sys, w, vals, w.p32, w.Ap32, st);
  if (exact) launch_k(k_update32s<true>, w, st, n, w.x32, w.r32, w.p32, (const float*)w.Ap32, idiag32, w.rb, w.S, w.I);
  else launch_k(k_update32s<false>, w, st, n, w.x32, w.r32, w.p32, (const float*)w.Ap32, idiag32, w.rb, w.S, w.I);
}

// Capture `chunk` iterations into a graph and replay it until the device done flag is set.
template <typename F>
static fg_status run_chunks(fg_ctx* ctx, const Work& w, int chunk, F launch_iter, int* h_I, double* h_S) {
  cudaStream_t st = ctx->stream;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  FG_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < chunk; ++k) launch_iter();
  cudaError_t e = cudaStreamEndCapture(st, &graph);
  if (e != cudaSuccess) { set_error("graph capture: %s", cudaGetErrorString(e)); return FG_ERR_CUDA; }
  e = cudaGraphInstantiate(&exec, graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    set_error("graph instantiate: %s", cudaGetErrorString(e));
    return FG_ERR_CUDA;
  }
  fg_status out = FG_OK;
  for (;;) {
    e = cudaGraphLaunch(exec, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_I, w.I, sizeof(int) * I_COUNT, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_S, w.S, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { set_error("cg loop: %s", cudaGetErrorString(e)); out = FG_ERR_CUDA; break; }
    if (h_I[I_DONE]) break;
    if (!std::isfinite(h_S[S_ALPHA]) || !std::isfinite(h_S[S_RZ])) {
      out = FG_ERR_NUMERIC;
      set_error("non-finite CG scalars");
      break;
    }
  }
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  return out;
}

fg_status system_solve(fg_system* sys, const fg_solver_params* prm, const double* d_b, const double* d_x0,
                       double* d_x, fg_solve_info* info) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  cudaStream_t st = ctx->stream;
  const int64_t n = sp->nfree, nv = sp->nvec;
  fg_solve_info out;
  std::memset(&out, 0, sizeof(out));
  if (n == 0) {
    out.converged = 1;
    if (info) *info = out;
    return FG_OK;
  }
  Work w;
  FG_TRY(ensure_work(sys, w));
  if (!sys->d_idiag) FG_TRY(system_prepare_diag(sys));
  const double* b_row = d_b ? d_b : sys->d_rhs;
  const int precond = prm->precond == FG_PREC_JACOBI ? 1 : 0;
  const int chunk = prm->check_every > 0 ? prm->check_every : (n < 200000 ? 64 : 16);
  int h_I[I_COUNT];
  double h_S[S_COUNT];
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, st);
  const int64_t launches0 = ctx->launches;
  fg_status status = FG_OK;
  // right-hand side and initial guess into the solver layout (other entries are zero)
  k_rows_to_vec<double, double><<<nblk(n, RB), RB, 0, st>>>(n, sp->d_row2vec, b_row, w.b);
  if (d_x0) k_rows_to_vec<double, double><<<nblk(n, RB), RB, 0, st>>>(n, sp->d_row2vec, d_x0, w.x);
  else k_fill<double><<<nblk(nv, RB), RB, 0, st>>>(nv, w.x, 0.0);
  ctx->launches += 2;
  FG_CUDA_TRY(cudaGetLastError());
  if (prm->precision == FG_FP64) {
    if (d_x0) spmv_k<double, 0>(sys, w, w.x, w.r, nullptr, st);
    launch_k(k_init64, w, st, nv, (const double*)w.b, d_x0 ? 1 : 0, w.r, w.p, (const double*)sys->d_idiag, precond,
             prm->criterion, prm->rtol, prm->atol, prm->max_iters, w.rb, w.S, w.I);
    ctx->launches += 1;
    FG_CUDA_TRY(cudaGetLastError());
    const bool need_pp = prm->criterion == FG_DELTA_RHS || prm->criterion == FG_DELTA_DELTA;
    status = run_chunks(ctx, w, chunk,
                        [&]() { iter64(sys, w, precond, need_pp, prm->criterion, prm->rtol, prm->atol, st); }, h_I, h_S);
    ctx->launches += (int64_t)3 * chunk * (((int64_t)h_I[I_ITER] + chunk - 1) / chunk + 0);
    out.iterations = h_I[I_ITER];
    out.converged = h_I[I_CONV];
    out.error_estimate = h_S[S_ERR];
    out.tolerance = h_S[S_TOL];
  } else {
    const double delta = prm->inner_rtol > 0 ? prm->inner_rtol : 0.1;
    // true residual of the initial guess and the tolerance
    spmv_k<double, 2>(sys, w, w.x, w.r, w.b, st);
    FG_CUDA_TRY(cudaMemcpyAsync(h_S, w.S, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, st));
    FG_CUDA_TRY(cudaStreamSynchronize(st));
    double rn = h_S[S_ERR];
    double tol;
    if (prm->criterion == FG_RES_RHS) {
      launch_k(k_init64, w, st, nv, (const double*)w.b, 0, w.t, w.Ap, (const double*)sys->d_idiag, 0, (int)FG_RES_RHS,
               prm->rtol, prm->atol, 1, w.rb, w.S, w.I);
      ctx->launches += 1;
      FG_CUDA_TRY(cudaMemcpyAsync(h_S, w.S, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, st));
      FG_CUDA_TRY(cudaStreamSynchronize(st));
      tol = prm->rtol * h_S[S_BNRM] + prm->atol;
      spmv_k<double, 2>(sys, w, w.x, w.r, w.b, st);
    } else {
      tol = prm->rtol * rn + prm->atol;
    }
    int outer = 0, stalls = 0, polish_its = 0;
    bool polish = false;
    double rn_prev = rn;
    int64_t graph_launches = 0;
    if (!std::isfinite(rn)) {
      status = FG_ERR_NUMERIC;
      set_error("non-finite initial residual");
    } else if (rn <= tol) {
      out.converged = 1;
    } else {
      k_set_scalar<<<1, 1, 0, st>>>(w.S, S_TOL, tol);
      k_set_scalar<<<1, 1, 0, st>>>(w.S, S_DELTA, delta);
      k_set_scalar<<<1, 1, 0, st>>>(w.S, S_SIGMA, rn);
      k_fill<float><<<nblk(nv, RB), RB, 0, st>>>(nv, w.x32, 0.0f);
      k_fill<float><<<nblk(nv, RB), RB, 0, st>>>(nv, w.p32, 0.0f);
      ctx->launches += 5;
      int hI0[I_COUNT] = {0};
      hI0[I_MAXIT] = prm->max_iters;
      FG_CUDA_TRY(cudaMemcpyAsync(w.I, hI0, sizeof(hI0), cudaMemcpyHostToDevice, st));
      // FP32 segments on D^-1/2 A D^-1/2 (Jacobi) or A (no preconditioner), fused iterations
      const double* sd = nullptr;
      const float* vals32 = sp->layout == FG_LAYOUT_STENCIL ? sys->d_tval32 : sys->d_sval32;
      const float* id32 = nullptr;
      if (precond) {
        FG_TRY(ensure_scaled(sys, w));
        sd = sys->d_sdiag;
        vals32 = sys->d_val32s;
        id32 = sys->d_idiag32;
      }
      auto refresh = [&](int first) {
        launch_k(k_refresh_scaled, w, st, nv, (const double*)w.r, sd, w.r32, first, w.rb, w.S, w.I);
        launch_k(k_pupdate<float, false>, w, st, nv, w.p32, (const float*)w.r32, (const float*)nullptr,
                 (const double*)w.S, (const int*)w.I);
        ctx->launches += 2;
      };
      refresh(1);
      FG_CUDA_TRY(cudaGetLastError());
      // graph of `chunk` FP32 iterations, replayed; reliable updates on the host's cue
      cudaGraph_t graph = nullptr;
      cudaGraphExec_t exec = nullptr;
      FG_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      for (int k = 0; k < chunk; ++k)  // at least the last iteration of a chunk sums the stop estimate
        iter32s(sys, w, vals32, id32, k % FG_MIXED_EXACT_EVERY == FG_MIXED_EXACT_EVERY - 1 || k == chunk - 1, st);
      cudaError_t e = cudaStreamEndCapture(st, &graph);
      if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
      if (e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        set_error("graph: %s", cudaGetErrorString(e));
        return FG_ERR_CUDA;
      }
      for (;;) {
        e = cudaGraphLaunch(exec, st);
        ++graph_launches;
        if (e == cudaSuccess) e = cudaMemcpyAsync(h_I, w.I, sizeof(int) * I_COUNT, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) { set_error("mixed loop: %s", cudaGetErrorString(e)); status = FG_ERR_CUDA; break; }
        if (!h_I[I_DONE]) continue;
        // reliable update: fold the FP32 correction into x64 and recompute the true residual
        // (after a breakdown the segment's correction is dropped instead)
        FG_CUDA_TRY(cudaMemcpyAsync(h_S, w.S, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, st));
        FG_CUDA_TRY(cudaStreamSynchronize(st));
        const bool broke = h_I[I_FLAG] == FLAG_BREAK;
        if (broke) k_fill<float><<<nblk(nv, RB), RB, 0, st>>>(nv, w.x32, 0.0f);
        else launch_k(k_fold_scaled, w, st, nv, h_S[S_SIGMA], sd, w.x32, w.x);
        ctx->launches += 1;
        spmv_k<double, 2>(sys, w, w.x, w.r, w.b, st);
        ++outer;
        FG_CUDA_TRY(cudaMemcpyAsync(h_S, w.S, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, st));
        FG_CUDA_TRY(cudaStreamSynchronize(st));
        rn = h_S[S_ERR];
        if (!std::isfinite(rn)) { status = FG_ERR_NUMERIC; set_error("non-finite residual"); break; }
        if (rn <= tol) { out.converged = 1; break; }
        if (h_I[I_ITER] >= prm->max_iters) break;
        // FP32 segments aim at a 10x reduction of the true residual; a breakdown, or two
        // segments in a row that gain less than 2x (FP32 rounding of an ill-conditioned
        // matrix near a tight tolerance), hand the rest of the solve to the FP64 PCG
        stalls = rn > 0.5 * rn_prev ? stalls + 1 : 0;
        rn_prev = rn;
        if (broke || stalls >= 2) { polish = true; break; }
        refresh(0);
        FG_CUDA_TRY(cudaGetLastError());
      }
      cudaGraphExecDestroy(exec);
      cudaGraphDestroy(graph);
      FG_CUDA_TRY(cudaMemcpyAsync(h_I, w.I, sizeof(int) * I_COUNT, cudaMemcpyDeviceToHost, st));
      FG_CUDA_TRY(cudaStreamSynchronize(st));
      ctx->launches += graph_launches * 2 * chunk;
      if (polish && status == FG_OK) {
        // FP64 PCG from x64 to the same absolute tolerance, with the iterations left
        const int mixed_its = h_I[I_ITER];
        spmv_k<double, 0>(sys, w, w.x, w.r, nullptr, st);
        launch_k(k_init64, w, st, nv, (const double*)w.b, 1, w.r, w.p, (const double*)sys->d_idiag, precond,
                 (int)FG_RES_RES, 0.0, tol, std::max(prm->max_iters - mixed_its, 1), w.rb, w.S, w.I);
        ctx->launches += 1;
        FG_CUDA_TRY(cudaGetLastError());
        status = run_chunks(ctx, w, chunk,
                            [&]() { iter64(sys, w, precond, false, (int)FG_RES_RES, 0.0, tol, st); }, h_I, h_S);
        ctx->launches += (int64_t)3 * chunk * (((int64_t)h_I[I_ITER] + chunk - 1) / chunk);
        polish_its = h_I[I_ITER];
        out.converged = h_I[I_CONV];
        rn = h_S[S_ERR];
        h_I[I_ITER] = mixed_its;
      }
    }
    out.iterations = h_I[I_ITER] + polish_its;
    out.outer_iterations = outer;
    out.error_estimate = rn;
    out.tolerance = tol;
  }
  // solution back to row order
  k_vec_to_rows<double, double><<<nblk(n, RB), RB, 0, st>>>(n, sp->d_row2vec, w.x, d_x);
  ctx->launches += 1;
  FG_CUDA_TRY(cudaGetLastError());
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

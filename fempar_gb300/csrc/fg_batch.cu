// fg_batch.cu -- many independent Poisson problems assembled and solved in one persistent launch.
//
// Each problem: -div(k grad u) = f on the unit cube, n^3 uniform hexahedra, Lagrangian Q_p
// (p = 1..3), constant k, f given at the Gauss points, u = 0 on the whole boundary; Jacobi-PCG
// to ||b - A x|| <= rtol ||b||.  Per problem this is the reference's tutorial / test_poisson
// path (integration of the tutorial integrand, strong Dirichlet, CG with the Jacobi
// preconditioner: Sources/Lib/LinearAlgebra/IterativeLinearSolver/cg.f90:101-238,
// Sources/Lib/LinearAlgebra/Preconditioner/jacobi_preconditioner.f90:356-412); FEMPAR runs
// one problem per program, the batch form has no counterpart there.
//
// Design (GB300):
//  * Matrix-free operator.  On a uniform mesh with one coefficient the cell matrix is
//    (h/2) k (s x m x m + m x s x m + m x m x s) for the 1D Gauss-integrated mass m and
//    stiffness s of the reference element (the reference's structured-mesh path reuses the
//    first cell's Jacobian the same way, sbm_cell_map.i90:272-320), so the assembled
//    operator is a stencil per node class (I mod p, J mod p, K mod p) built from the 1D
//    assembled matrices: nothing is stored per nonzero.
//  * Right-hand side assembled in the kernel: each cell's load vector by sum factorisation
//    in FP64, gathered per node over its cells in increasing cell order.
//  * Mixed precision without the FP64 pipe in the loop: the inner CG runs in FP32; the
//    solution, the right-hand side and the true residual b - A x are kept in float-float
//    (pairs of FP32, ~2^-48 relative), the stencil applied with error-free FP32 products.
//    Every time the FP32 recursive residual has dropped 10x the float-float true residual
//    replaces it (reliable update, the direction is kept).
//  * One persistent cooperative launch.  A host planner orders the problems by estimated
//    work and gives each a team of co-resident CTAs (one CTA for most problems); team
//    members synchronise through a counter in global memory with a bounded spin, and sum
//    their per-CTA partials in rank order (deterministic for a given plan).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include "fg_internal.h"

namespace fg {

static constexpr int kBatchMaxP = 3;
// coefficient table: per class, wy*wz rows of the x box padded to a multiple of 4 floats
// (128-bit shared-memory loads); p = 3: (8 + 4 + 4) * 15 * 15 = 3600 floats
static constexpr int kMaxBox = 16 * 15 * 15;
static constexpr int kMaxCls = 27;

struct BatchProb {
  int n, p, L, F;        // cells per direction, order, lattice nodes, interior nodes per direction
  float kh_hi, kh_lo;    // stencil scale k h / 2 as float-float
  double h3;             // (h/2)^3, load-vector scale
  const double* f;       // Gauss-point source, n^3 (p+1)^3
  double* x;             // output, F^3 interior nodes
  int64_t voff;          // 8 float vectors of L^3 in the float pool
  int64_t eoff;          // load vectors, n^3 (p+1)^3 doubles
  int64_t roff;          // partials: 3 slots x team x 4 doubles
  int team;              // CTAs in the team
};

struct BatchJob {
  int prob, rank;
};

struct OrderTables {    // unit stencil per order (sum over classes of the boxes)
  int ncls;
  int base[kMaxCls], cnt[kMaxCls];
  int lo[kMaxCls][3], w[kMaxCls][3];
  float sh[kMaxBox], sl[kMaxBox];
  float dg[kMaxCls];     // centre coefficient (unit) per class
  double mw[(kBatchMaxP + 1) * (kBatchMaxP + 1)];  // w_q phi_a(xi_q), [a][q]
};

struct BatchArgs {
  const BatchProb* probs;
  const int* job_ptr;     // per CTA: first job
  const BatchJob* jobs;
  const OrderTables* tabs;  // index p-1
  float* vpool;
  double* epool;
  double* rpool;
  unsigned* bar;          // per problem barrier counter
  int* status;            // per problem
  int* iters;
  int* refines;
  double* relres;
  double rtol, atol;
  int max_iters;
  float delta;            // reliable-update factor
  unsigned long long timeout_ns;  // a team wait gives up after this long (globaltimer)
  int* abort_all;         // set by the first wait that gives up: every CTA stops
  int drop_arrival;       // test of the bounded wait: rank 1 of a team skips its first arrival
};

// ---- float-float helpers (error-free transformations; no reassociation in this file)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void quick_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}
// (sh, sl) += (ch, cl) * (xh, xl)
__device__ __forceinline__ void ff_fma_acc(float ch, float cl, float xh, float xl, float& sh, float& sl) {
  float p = ch * xh;
  float e = fmaf(ch, xh, -p);
  e = fmaf(ch, xl, fmaf(cl, xh, e));
  float s, t;
  two_sum(sh, p, s, t);
  sh = s;
  sl += t + e;
}
__device__ __forceinline__ void ff_mul(float ah, float al, float bh, float bl, float& h, float& l) {
  float p = ah * bh;
  float e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, fmaf(al, bh, e));
  quick_two_sum(p, e, h, l);
}
__device__ __forceinline__ void ff_add(float ah, float al, float bh, float bl, float& h, float& l) {
  float s, e;
  two_sum(ah, bh, s, e);
  e += al + bl;
  quick_two_sum(s, e, h, l);
}

// Kahan-compensated FP32 accumulator
struct Kf {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double val() const { return (double)s - (double)c; }
};

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

struct BatchSmem {
  __align__(16) float sh[kMaxBox];
  __align__(16) float sl[kMaxBox];
  int base[kMaxCls], cnt[kMaxCls];
  int blo[kMaxCls][3], bw[kMaxCls][3];
  float dinv[kMaxCls];
  double mw[(kBatchMaxP + 1) * (kBatchMaxP + 1)];
  double red[32][4];
  double tot[4];
  int abort_flag;
};

// Block sum of nv doubles; result in sm.tot (all threads, after the call).
__device__ void block_sum(double* v, int nv, BatchSmem& sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = 0; k < nv; ++k) {
    double a = warp_sum_d(v[k]);
    if (lane == 0) sm.red[warp][k] = a;
  }
  __syncthreads();
  if (threadIdx.x < nv) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += sm.red[w][threadIdx.x];
    sm.tot[threadIdx.x] = s;
  }
  __syncthreads();
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Team reduction of nv values: CTA partials into slot, barrier, ranks summed in order.
// Returns false if the barrier gave up (status set).
__device__ bool team_sum(const BatchArgs& a, const BatchProb& P, int prob, int rank, int& phase, double* v, int nv,
                         BatchSmem& sm, double* out) {
  block_sum(v, nv, sm);
  if (P.team == 1) {
    for (int k = 0; k < nv; ++k) out[k] = sm.tot[k];
    return true;
  }
  double* slot = a.rpool + P.roff + (int64_t)(phase % 3) * P.team * 4;
  if (threadIdx.x < nv) slot[rank * 4 + threadIdx.x] = sm.tot[threadIdx.x];
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (!(a.drop_arrival && rank == 1 && phase == 0)) atomicAdd(a.bar + prob, 1u);
    const unsigned target = (unsigned)(phase + 1) * (unsigned)P.team;
    const unsigned long long t0 = global_ns();
    int ok = 1;
    while (ld_acquire(a.bar + prob) < target) {
      if (*(volatile int*)a.abort_all || global_ns() - t0 > a.timeout_ns) { ok = 0; break; }
      __nanosleep(256);
    }
    __threadfence();
    sm.abort_flag = ok ? 0 : 1;
    if (!ok) {
      atomicExch(a.status + prob, (int)FG_ERR_TIMEOUT);
      atomicExch(a.abort_all, 1);
    }
  }
  __syncthreads();
  ++phase;
  if (sm.abort_flag) return false;
  for (int k = 0; k < nv; ++k) {
    double s = 0.0;
    for (int r = 0; r < P.team; ++r) s += ((volatile double*)slot)[r * 4 + k];
    out[k] = s;
  }
  return true;
}

// Barrier without values (phases shared with team_sum).
__device__ bool team_sync(const BatchArgs& a, const BatchProb& P, int prob, int rank, int& phase, BatchSmem& sm) {
  double dummy[1] = {0.0}, o[1];
  return team_sum(a, P, prob, rank, phase, dummy, 1, sm, o);
}

// Cell load vectors E_c[a] = (h/2)^3 sum_q w_q f_q phi_a(q) by sum factorisation, FP64, cells [c0, c1).
// Interior nodes u = u0 + threadIdx.x + k blockDim.x of the F^3 block (x fastest), with the
// lattice coordinates advanced incrementally: no integer division inside the loops.
struct NodeWalk {
  int u, u1, I, J, K, g, dI, dJ, dK, F, L, step;
  __device__ __forceinline__ NodeWalk(int u0_, int u1_, int F_, int L_) : u1(u1_), F(F_), L(L_) {
    step = blockDim.x;
    u = u0_ + threadIdx.x;
    if (F > 0) {
      I = 1 + u % F;
      J = 1 + (u / F) % F;
      K = 1 + u / (F * F);
      dI = step % F;
      dJ = (step / F) % F;
      dK = step / (F * F);
    } else {
      I = J = K = 1;
      dI = dJ = dK = 0;
    }
    g = I + L * (J + L * K);
  }
  __device__ __forceinline__ bool ok() const { return u < u1; }
  __device__ __forceinline__ void next() {
    u += step;
    I += dI;
    int c = I > F ? 1 : 0;
    I -= c * F;
    J += dJ + c;
    c = J > F ? 1 : 0;
    J -= c * F;
    K += dK + c;
    g = I + L * (J + L * K);
  }
};

// x-periods of the interior: period (m, J, K) holds the nodes I = p m + k, k = 1..p (x classes
// 1..p-1, then class 0); the class-0 node of the last period of a row is on the boundary.
// v = m + n ((J-1) + F (K-1)), advanced incrementally.
struct PeriodWalk {
  int v, v1, m, J, K, n, F, step, dm, dJ, dK;
  __device__ __forceinline__ PeriodWalk(int v0_, int v1_, int n_, int F_) : v1(v1_), n(n_), F(F_) {
    step = blockDim.x;
    v = v0_ + threadIdx.x;
    if (F > 0) {
      m = v % n;
      J = 1 + (v / n) % F;
      K = 1 + v / (n * F);
      dm = step % n;
      dJ = (step / n) % F;
      dK = step / (n * F);
    } else {
      m = 0;
      J = K = 1;
      dm = dJ = dK = 0;
    }
  }
  __device__ __forceinline__ bool ok() const { return v < v1; }
  __device__ __forceinline__ void next() {
    v += step;
    m += dm;
    int c = m >= n ? 1 : 0;
    m -= c * n;
    J += dJ + c;
    c = J > F ? 1 : 0;
    J -= c * F;
    K += dK + c;
  }
};

// FP32 stencil on one period: acc[0] for the class-0 node I0+p, acc[k] for I0+k.  Each (y,z)
// box row loads the window x = I0..I0+2p once and serves all p nodes.
template <int PO>
__device__ __forceinline__ void period_apply32(const BatchSmem& sm, const float* __restrict__ v, int L, int I0,
                                               int J, int K, bool full, float (&acc)[PO]) {
  const int cy = J % PO, cz = K % PO;
  const int c0 = PO * (cy + PO * cz);
  const int ly = sm.blo[c0][1], wy = sm.bw[c0][1], lz = sm.blo[c0][2], wz = sm.bw[c0][2];
#pragma unroll
  for (int k = 0; k < PO; ++k) acc[k] = 0.f;
  for (int zz = 0; zz < wz; ++zz)
    for (int yy = 0; yy < wy; ++yy) {
      const int base = I0 + L * ((J + ly + yy) + L * (K + lz + zz));
      float win[2 * PO + 1];
#pragma unroll
      for (int t = 0; t <= PO; ++t) win[t] = v[base + t];
#pragma unroll
      for (int t = PO + 1; t <= 2 * PO; ++t) win[t] = full ? v[base + t] : 0.f;
      const int row = yy + wy * zz;
      constexpr int R0 = (2 * PO + 1 + 3) & ~3, RK = (PO + 1 + 3) & ~3;
      {
        const float4* S0 = reinterpret_cast<const float4*>(sm.sh + sm.base[c0] + R0 * row);
#pragma unroll
        for (int v4 = 0; v4 < R0 / 4; ++v4) {
          const float4 c = S0[v4];
          const float cc[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (4 * v4 + e <= 2 * PO) acc[0] = fmaf(cc[e], win[4 * v4 + e], acc[0]);
        }
      }
#pragma unroll
      for (int k = 1; k < PO; ++k) {
        const float4* Sk = reinterpret_cast<const float4*>(sm.sh + sm.base[c0 + k] + RK * row);
#pragma unroll
        for (int v4 = 0; v4 < RK / 4; ++v4) {
          const float4 c = Sk[v4];
          const float cc[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (4 * v4 + e <= PO) acc[k] = fmaf(cc[e], win[4 * v4 + e], acc[k]);
        }
      }
    }
}

// Float-float stencil on one period (error-free products, float-float sums).
template <int PO>
__device__ __forceinline__ void period_apply_ff(const BatchSmem& sm, const float* __restrict__ vh,
                                                const float* __restrict__ vl, int L, int I0, int J, int K, bool full,
                                                float (&ah)[PO], float (&al)[PO]) {
  const int cy = J % PO, cz = K % PO;
  const int c0 = PO * (cy + PO * cz);
  const int ly = sm.blo[c0][1], wy = sm.bw[c0][1], lz = sm.blo[c0][2], wz = sm.bw[c0][2];
#pragma unroll
  for (int k = 0; k < PO; ++k) {
    ah[k] = 0.f;
    al[k] = 0.f;
  }
  for (int zz = 0; zz < wz; ++zz)
    for (int yy = 0; yy < wy; ++yy) {
      const int base = I0 + L * ((J + ly + yy) + L * (K + lz + zz));
      float wh[2 * PO + 1], wl[2 * PO + 1];
#pragma unroll
      for (int t = 0; t <= PO; ++t) {
        wh[t] = vh[base + t];
        wl[t] = vl[base + t];
      }
#pragma unroll
      for (int t = PO + 1; t <= 2 * PO; ++t) {
        wh[t] = full ? vh[base + t] : 0.f;
        wl[t] = full ? vl[base + t] : 0.f;
      }
      const int row = yy + wy * zz;
      constexpr int R0 = (2 * PO + 1 + 3) & ~3, RK = (PO + 1 + 3) & ~3;
      const int b0 = sm.base[c0] + R0 * row;
#pragma unroll
      for (int t = 0; t <= 2 * PO; ++t) ff_fma_acc(sm.sh[b0 + t], sm.sl[b0 + t], wh[t], wl[t], ah[0], al[0]);
#pragma unroll
      for (int k = 1; k < PO; ++k) {
        const int bk = sm.base[c0 + k] + RK * row;
#pragma unroll
        for (int t = 0; t <= PO; ++t) ff_fma_acc(sm.sh[bk + t], sm.sl[bk + t], wh[t], wl[t], ah[k], al[k]);
      }
    }
}

template <int PO>
__device__ __noinline__ void load_vectors(const BatchProb& P, double* E, int64_t c0, int64_t c1, const BatchSmem& sm) {
  constexpr int NP1 = PO + 1, NQ = NP1 * NP1 * NP1;
  for (int64_t c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
    const double* f = P.f + c * NQ;
    double t1[NQ], t2[NQ];
#pragma unroll
    for (int qz = 0; qz < NP1; ++qz)
#pragma unroll
      for (int qy = 0; qy < NP1; ++qy)
#pragma unroll
        for (int ax = 0; ax < NP1; ++ax) {
          double s = 0.0;
#pragma unroll
          for (int qx = 0; qx < NP1; ++qx) s += sm.mw[ax * NP1 + qx] * f[qx + NP1 * (qy + NP1 * qz)];
          t1[ax + NP1 * (qy + NP1 * qz)] = s;
        }
#pragma unroll
    for (int qz = 0; qz < NP1; ++qz)
#pragma unroll
      for (int ay = 0; ay < NP1; ++ay)
#pragma unroll
        for (int ax = 0; ax < NP1; ++ax) {
          double s = 0.0;
#pragma unroll
          for (int qy = 0; qy < NP1; ++qy) s += sm.mw[ay * NP1 + qy] * t1[ax + NP1 * (qy + NP1 * qz)];
          t2[ax + NP1 * (ay + NP1 * qz)] = s;
        }
#pragma unroll
    for (int az = 0; az < NP1; ++az)
#pragma unroll
      for (int ay = 0; ay < NP1; ++ay)
#pragma unroll
        for (int ax = 0; ax < NP1; ++ax) {
          double s = 0.0;
#pragma unroll
          for (int qz = 0; qz < NP1; ++qz) s += sm.mw[az * NP1 + qz] * t2[ax + NP1 * (ay + NP1 * qz)];
          E[c * NQ + ax + NP1 * (ay + NP1 * az)] = s * P.h3;
        }
  }
}

template <int PO>
__device__ void solve_problem(const BatchArgs& a, int prob, int rank, BatchSmem& sm) {
  const BatchProb P = a.probs[prob];
  const OrderTables& T = a.tabs[PO - 1];
  constexpr int NP1 = PO + 1, NQ = NP1 * NP1 * NP1;
  const int L = P.L, F = P.F, n = P.n;
  const int64_t L2 = (int64_t)L * L;
  // tables into shared memory (offsets depend on L)
  for (int c = threadIdx.x; c < T.ncls; c += blockDim.x) {
    sm.base[c] = T.base[c];
    sm.cnt[c] = T.cnt[c];
    for (int d = 0; d < 3; ++d) {
      sm.blo[c][d] = T.lo[c][d];
      sm.bw[c][d] = T.w[c][d];
    }
    float d = T.dg[c] * P.kh_hi;
    sm.dinv[c] = 1.0f / d;
  }
  const int tot = T.base[T.ncls - 1] + T.cnt[T.ncls - 1];
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    sm.sh[t] = T.sh[t];
    sm.sl[t] = T.sl[t];
  }
  for (int t = threadIdx.x; t < NP1 * NP1; t += blockDim.x) sm.mw[t] = T.mw[t];
  __syncthreads();
  float* bh = a.vpool + P.voff;
  float* bl = bh + L * L2;
  float* xh = bl + L * L2;
  float* xl = xh + L * L2;
  float* xc = xl + L * L2;
  float* r = xc + L * L2;
  float* pp = r + L * L2;
  float* q = pp + L * L2;
  double* E = a.epool + P.eoff;
  int phase = 0;
  // team ranges: cells and interior nodes
  const int64_t ncells = (int64_t)n * n * n, nint = (int64_t)F * F * F;
  const int64_t c0 = ncells * rank / P.team, c1 = ncells * (rank + 1) / P.team;
  const int64_t u0 = nint * rank / P.team, u1 = nint * (rank + 1) / P.team;
  const int64_t nper = (int64_t)n * F * F;
  const int v0 = (int)(nper * rank / P.team), v1 = (int)(nper * (rank + 1) / P.team);
  // 1. load vectors by sum factorisation (FP64)
  load_vectors<PO>(P, E, c0, c1, sm);
  if (!team_sync(a, P, prob, rank, phase, sm)) return;
  // 2. gather b per node (cells in increasing order), initial state
  double loc[4] = {0.0, 0.0, 0.0, 0.0};
  {
    Kf rz;
    double bb = 0.0;
    for (NodeWalk w((int)u0, (int)u1, F, L); w.ok(); w.next()) {
      const int I = w.I, J = w.J, K = w.K;
      int cx[2], lx[2], nx = 0, cy[2], ly[2], ny = 0, cz[2], lz[2], nz = 0;
      if (I % PO == 0) { cx[0] = I / PO - 1; lx[0] = PO; cx[1] = I / PO; lx[1] = 0; nx = 2; }
      else { cx[0] = I / PO; lx[0] = I % PO; nx = 1; }
      if (J % PO == 0) { cy[0] = J / PO - 1; ly[0] = PO; cy[1] = J / PO; ly[1] = 0; ny = 2; }
      else { cy[0] = J / PO; ly[0] = J % PO; ny = 1; }
      if (K % PO == 0) { cz[0] = K / PO - 1; lz[0] = PO; cz[1] = K / PO; lz[1] = 0; nz = 2; }
      else { cz[0] = K / PO; lz[0] = K % PO; nz = 1; }
      double b = 0.0;
      for (int kz = 0; kz < nz; ++kz)
        for (int ky = 0; ky < ny; ++ky)
          for (int kx = 0; kx < nx; ++kx) {
            int64_t c = cx[kx] + (int64_t)n * (cy[ky] + (int64_t)n * cz[kz]);
            b += E[c * NQ + lx[kx] + NP1 * (ly[ky] + NP1 * lz[kz])];
          }
      const int64_t g = w.g;
      float h = (float)b;
      float l = (float)(b - (double)h);
      bh[g] = h;
      bl[g] = l;
      xh[g] = 0.f;
      xl[g] = 0.f;
      xc[g] = 0.f;
      r[g] = h;
      const int cls = (I % PO) + PO * ((J % PO) + PO * (K % PO));
      float z = sm.dinv[cls] * h;
      pp[g] = z;
      rz.add(h * z);
      bb = fma(b, b, bb);
    }
    loc[0] = bb;
    loc[1] = rz.val();
  }
  double red[4];
  if (!team_sum(a, P, prob, rank, phase, loc, 2, sm, red)) return;
  const double bnorm = sqrt(red[0]);
  double rzv = red[1];
  double rtrue2 = red[0];
  const double tol = a.rtol * bnorm + a.atol;
  int it = 0, nref = 0, conv = bnorm <= a.atol ? 1 : 0;
  double relres = 1.0;
  const float khf = P.kh_hi;
  while (!conv && it < a.max_iters) {
    ++it;
    // q = A p (FP32), <p, q>
    {
      Kf pq;
      for (PeriodWalk w(v0, v1, n, F); w.ok(); w.next()) {
        const int I0 = PO * w.m;
        const bool full = I0 + PO <= F;
        float acc[PO];
        period_apply32<PO>(sm, pp, L, I0, w.J, w.K, full, acc);
        const int g0 = I0 + L * (w.J + L * w.K);
#pragma unroll
        for (int k = 1; k < PO; ++k) {
          const float y = acc[k] * khf;
          q[g0 + k] = y;
          pq.add(y * pp[g0 + k]);
        }
        if (full) {
          const float y = acc[0] * khf;
          q[g0 + PO] = y;
          pq.add(y * pp[g0 + PO]);
        }
      }
      loc[0] = pq.val();
    }
    if (!team_sum(a, P, prob, rank, phase, loc, 1, sm, red)) return;
    if (!(red[0] > 0.0)) {
      if (threadIdx.x == 0 && rank == 0) atomicExch(a.status + prob, (int)FG_ERR_NUMERIC);
      break;
    }
    const float alpha = (float)(rzv / red[0]);
    {
      Kf rr, rzn;
      for (NodeWalk w((int)u0, (int)u1, F, L); w.ok(); w.next()) {
        const int I = w.I, J = w.J, K = w.K;
        const int64_t g = w.g;
        const int cls = (I % PO) + PO * ((J % PO) + PO * (K % PO));
        xc[g] = fmaf(alpha, pp[g], xc[g]);
        float ri = fmaf(-alpha, q[g], r[g]);
        r[g] = ri;
        rr.add(ri * ri);
        rzn.add(ri * (sm.dinv[cls] * ri));
      }
      loc[0] = rr.val();
      loc[1] = rzn.val();
    }
    if (!team_sum(a, P, prob, rank, phase, loc, 2, sm, red)) return;
    double rzn = red[1];
    const double rr = red[0];
    const bool near = rr <= 0.25 * tol * tol;
    if (rr <= (double)a.delta * (double)a.delta * rtrue2 || near || it >= a.max_iters) {
      // reliable update: x += xc (float-float), then r = b - A x in float-float
      for (NodeWalk w((int)u0, (int)u1, F, L); w.ok(); w.next()) {
        const int64_t g = w.g;
        float h, l;
        ff_add(xh[g], xl[g], xc[g], 0.f, h, l);
        xh[g] = h;
        xl[g] = l;
        xc[g] = 0.f;
      }
      if (!team_sync(a, P, prob, rank, phase, sm)) return;
      Kf rr2, rz2;
      for (PeriodWalk w(v0, v1, n, F); w.ok(); w.next()) {
        const int I0 = PO * w.m;
        const bool full = I0 + PO <= F;
        float sh[PO], sl[PO];
        period_apply_ff<PO>(sm, xh, xl, L, I0, w.J, w.K, full, sh, sl);
        const int g0 = I0 + L * (w.J + L * w.K);
        const int cyz = PO * ((w.J % PO) + PO * (w.K % PO));
#pragma unroll
        for (int k = 0; k < PO; ++k) {
          const int xo = k == 0 ? PO : k;  // acc[0]: class-0 node at I0 + PO
          if (k == 0 && !full) continue;
          const int g = g0 + xo;
          float h, l, ah, al;
          quick_two_sum(sh[k], sl[k], h, l);
          ff_mul(P.kh_hi, P.kh_lo, h, l, ah, al);
          float rh, rl;
          ff_add(bh[g], bl[g], -ah, -al, rh, rl);
          const float ri = rh + rl;
          r[g] = ri;
          rr2.add(ri * ri);
          rz2.add(ri * (sm.dinv[cyz + (xo % PO)] * ri));
        }
      }
      loc[0] = rr2.val();
      loc[1] = rz2.val();
      if (!team_sum(a, P, prob, rank, phase, loc, 2, sm, red)) return;
      ++nref;
      rtrue2 = red[0];
      rzn = red[1];
      relres = bnorm > 0.0 ? sqrt(rtrue2) / bnorm : 0.0;
      if (sqrt(rtrue2) <= tol) {
        conv = 1;
        break;
      }
    }
    const float beta = (float)(rzn / rzv);
    rzv = rzn;
    for (NodeWalk w((int)u0, (int)u1, F, L); w.ok(); w.next()) {
      const int I = w.I, J = w.J, K = w.K;
      const int64_t g = w.g;
      const int cls = (I % PO) + PO * ((J % PO) + PO * (K % PO));
      pp[g] = fmaf(beta, pp[g], sm.dinv[cls] * r[g]);
    }
    if (!team_sync(a, P, prob, rank, phase, sm)) return;
  }
  // solution: x = xh + xl at the interior nodes, x fastest
  for (NodeWalk w((int)u0, (int)u1, F, L); w.ok(); w.next()) {
    const int64_t g = w.g;
    P.x[w.u] = (double)xh[g] + (double)xl[g];
  }
  if (rank == 0 && threadIdx.x == 0) {
    a.iters[prob] = it;
    a.refines[prob] = nref;
    a.relres[prob] = relres;
    if (!conv) atomicCAS(a.status + prob, 0, (int)FG_ERR_NOT_CONVERGED);
  }
}

__global__ void __launch_bounds__(512, 2) k_batch_solve(BatchArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  BatchSmem& sm = *reinterpret_cast<BatchSmem*>(smraw);
  for (int j = a.job_ptr[blockIdx.x]; j < a.job_ptr[blockIdx.x + 1]; ++j) {
    if (threadIdx.x == 0) sm.abort_flag = *(volatile int*)a.abort_all;
    __syncthreads();
    const int stop = sm.abort_flag;  // one value for the whole CTA
    __syncthreads();
    if (stop) {
      // the problems this CTA leads and has not started are reported, not silently skipped
      if (threadIdx.x == 0)
        for (int k = j; k < a.job_ptr[blockIdx.x + 1]; ++k)
          if (a.jobs[k].rank == 0) atomicCAS(a.status + a.jobs[k].prob, 0, (int)FG_ERR_TIMEOUT);
      break;
    }
    const BatchJob J = a.jobs[j];
    const int p = a.probs[J.prob].p;
    if (p == 1) solve_problem<1>(a, J.prob, J.rank, sm);
    else if (p == 2) solve_problem<2>(a, J.prob, J.rank, sm);
    else solve_problem<3>(a, J.prob, J.rank, sm);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------------
// Host

static void build_order_tables(int p, OrderTables& T) {
  std::memset(&T, 0, sizeof(T));
  const int np1 = p + 1;
  double xq[kBatchMaxP + 1], wq[kBatchMaxP + 1];
  gl_rule(np1, xq, wq);
  double phi[kBatchMaxP + 1][kBatchMaxP + 1], dphi[kBatchMaxP + 1][kBatchMaxP + 1];
  for (int a = 0; a < np1; ++a)
    for (int q = 0; q < np1; ++q) lagrange_1d(p, a, xq[q], phi[a][q], dphi[a][q]);
  double m[kBatchMaxP + 1][kBatchMaxP + 1], s[kBatchMaxP + 1][kBatchMaxP + 1];
  for (int a = 0; a < np1; ++a)
    for (int b = 0; b < np1; ++b) {
      double sm = 0.0, ss = 0.0;
      for (int q = 0; q < np1; ++q) {
        sm += wq[q] * phi[a][q] * phi[b][q];
        ss += wq[q] * dphi[a][q] * dphi[b][q];
      }
      m[a][b] = sm;
      s[a][b] = ss;
    }
  for (int a = 0; a < np1; ++a)
    for (int q = 0; q < np1; ++q) T.mw[a * np1 + q] = wq[q] * phi[a][q];
  // 1D assembled rows per class: offsets [lo, lo + w)
  int lo1[kBatchMaxP], w1[kBatchMaxP];
  double M1[kBatchMaxP][2 * kBatchMaxP + 1], S1[kBatchMaxP][2 * kBatchMaxP + 1];
  for (int c = 0; c < p; ++c) {
    if (c == 0) {
      lo1[c] = -p;
      w1[c] = 2 * p + 1;
      for (int o = -p; o <= p; ++o) {
        double mm = 0.0, ss = 0.0;
        if (o <= 0) { mm += m[p][p + o]; ss += s[p][p + o]; }
        if (o >= 0) { mm += m[0][o]; ss += s[0][o]; }
        M1[c][o + p] = mm;
        S1[c][o + p] = ss;
      }
    } else {
      lo1[c] = -c;
      w1[c] = p + 1;
      for (int o = -c; o <= p - c; ++o) {
        M1[c][o + c] = m[c][c + o];
        S1[c][o + c] = s[c][c + o];
      }
    }
  }
  T.ncls = p * p * p;
  int base = 0;
  for (int cz = 0; cz < p; ++cz)
    for (int cy = 0; cy < p; ++cy)
      for (int cx = 0; cx < p; ++cx) {
        const int c = cx + p * (cy + p * cz);
        T.base[c] = base;
        T.lo[c][0] = lo1[cx];
        T.lo[c][1] = lo1[cy];
        T.lo[c][2] = lo1[cz];
        T.w[c][0] = w1[cx];
        T.w[c][1] = w1[cy];
        T.w[c][2] = w1[cz];
        const int rw = (w1[cx] + 3) & ~3;  // padded row
        T.cnt[c] = rw * w1[cy] * w1[cz];
        for (int k = 0; k < w1[cz]; ++k)
          for (int j = 0; j < w1[cy]; ++j)
            for (int i = 0; i < w1[cx]; ++i) {
              double v = S1[cx][i] * M1[cy][j] * M1[cz][k] + M1[cx][i] * S1[cy][j] * M1[cz][k] +
                         M1[cx][i] * M1[cy][j] * S1[cz][k];
              float h = (float)v;
              int t = base + i + rw * (j + w1[cy] * k);
              T.sh[t] = h;
              T.sl[t] = (float)(v - (double)h);
              if (lo1[cx] + i == 0 && lo1[cy] + j == 0 && lo1[cz] + k == 0) T.dg[c] = h;
            }
        base += T.cnt[c];
      }
}

static double avg_nnz(int p) {
  double w = (2.0 * p + 1.0 + (p - 1) * (p + 1.0)) / p;
  return w * w * w;
}

}  // namespace fg

struct fg_batch {
  fg_ctx* ctx = nullptr;
  int nprob = 0, flags = 0;
  fg_solver_params prm;
  std::vector<fg::BatchProb> probs;       // device-facing descriptors
  std::vector<const double*> user_f;      // caller's source pointers
  std::vector<double*> user_x;            // caller's output pointers
  std::vector<int64_t> nf, nx;            // source / output lengths
  int threads = 0, ctas = 0, max_team = 0, teams_gt1 = 0;
  // team sizing: a problem gets ceil(work / (team_share * per-CTA share)) CTAs
  // (0.5, or FG_BATCH_TEAM_SHARE when set > 0)
  double team_share = 0.5;
  double predicted_balance = 0.0, autotune_ms = 0.0, run_ms = 0.0;
  int64_t total_dofs = 0;
  fg::BatchProb* d_probs = nullptr;
  int* d_job_ptr = nullptr;
  fg::BatchJob* d_jobs = nullptr;
  fg::OrderTables* d_tabs = nullptr;
  float* vpool = nullptr;
  double* epool = nullptr;
  double* rpool = nullptr;
  unsigned* bar = nullptr;
  int* abort_all = nullptr;
  int* status = nullptr;
  int* iters = nullptr;
  int* refines = nullptr;
  double* relres = nullptr;
  double* fstage = nullptr;  // host-input mode: staged sources and outputs
  double* xstage = nullptr;
  int64_t nrp = 0;
  std::vector<void*> owned;
  cudaGraphExec_t graph = nullptr;
  bool use_graph = false;
};

namespace fg {

static fg_status ba(fg_batch* B, void** p, size_t bytes) {
  FG_TRY(dev_alloc(B->ctx, p, bytes));
  B->owned.push_back(*p);
  return FG_OK;
}

static size_t batch_smem() { return sizeof(BatchSmem); }

// Team sizes and the per-CTA job lists (greedy list scheduling, problems by decreasing work).
static void batch_schedule(fg_batch* B, int G, std::vector<int>& job_ptr, std::vector<BatchJob>& jobs) {
  const int np = B->nprob;
  std::vector<double> w(np);
  double W = 0.0;
  for (int i = 0; i < np; ++i) {
    const BatchProb& P = B->probs[i];
    double F3 = (double)P.F * P.F * P.F;
    w[i] = std::max(1.0, F3) * avg_nnz(P.p) * (3.0 * P.p * P.n + 20.0);
    W += w[i];
  }
  std::vector<int> order(np);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return w[x] > w[y]; });
  const double target = W / G;
  std::vector<double> avail(G, 0.0);
  std::vector<std::vector<BatchJob>> per(G);
  B->max_team = 1;
  B->teams_gt1 = 0;
  std::vector<int> idx(G);
  for (int i : order) {
    BatchProb& P = B->probs[i];
    const int64_t F3 = (int64_t)P.F * P.F * P.F;
    int t = (int)std::ceil(w[i] / (B->team_share * target));
    t = std::max(1, std::min(t, G));
    t = (int)std::min<int64_t>(t, std::max<int64_t>(1, F3 / (4 * B->threads)));
    P.team = t;
    B->max_team = std::max(B->max_team, t);
    if (t > 1) B->teams_gt1++;
    std::iota(idx.begin(), idx.end(), 0);
    std::partial_sort(idx.begin(), idx.begin() + t, idx.end(),
                      [&](int x, int y) { return avail[x] < avail[y] || (avail[x] == avail[y] && x < y); });
    std::sort(idx.begin(), idx.begin() + t);
    double start = 0.0;
    for (int k = 0; k < t; ++k) start = std::max(start, avail[idx[k]]);
    const double end = start + w[i] / t;
    for (int k = 0; k < t; ++k) {
      avail[idx[k]] = end;
      per[idx[k]].push_back({i, k});
    }
  }
  double mk = *std::max_element(avail.begin(), avail.end());
  B->predicted_balance = mk > 0 ? (W / G) / mk : 1.0;
  job_ptr.assign(G + 1, 0);
  jobs.clear();
  for (int g = 0; g < G; ++g) {
    job_ptr[g] = (int)jobs.size();
    for (auto& j : per[g]) jobs.push_back(j);
  }
  job_ptr[G] = (int)jobs.size();
}

static fg_status batch_launch(fg_batch* B, cudaStream_t st) {
  BatchArgs a;
  a.probs = B->d_probs;
  a.job_ptr = B->d_job_ptr;
  a.jobs = B->d_jobs;
  a.tabs = B->d_tabs;
  a.vpool = B->vpool;
  a.epool = B->epool;
  a.rpool = B->rpool;
  a.bar = B->bar;
  a.status = B->status;
  a.iters = B->iters;
  a.refines = B->refines;
  a.relres = B->relres;
  a.rtol = B->prm.rtol;
  a.atol = B->prm.atol;
  a.max_iters = B->prm.max_iters;
  a.delta = B->prm.inner_rtol > 0.0 ? (float)B->prm.inner_rtol : 0.1f;
  // team waits give up after 60 s (FG_BATCH_BARRIER_TIMEOUT_MS overrides); the test switch
  // FG_BATCH_TEST_DROP_ARRIVAL=1 makes one team member skip an arrival so that the wait runs out
  a.timeout_ns = 60ull * 1000000000ull;
  if (const char* e = std::getenv("FG_BATCH_BARRIER_TIMEOUT_MS")) {
    const long long ms = std::atoll(e);
    if (ms > 0) a.timeout_ns = (unsigned long long)ms * 1000000ull;
  }
  {
    const char* e = std::getenv("FG_BATCH_TEST_DROP_ARRIVAL");
    a.drop_arrival = (e && e[0] == '1') ? 1 : 0;
  }
  a.abort_all = B->abort_all;
  FG_CUDA_TRY(cudaMemsetAsync(B->bar, 0, sizeof(unsigned) * B->nprob, st));
  FG_CUDA_TRY(cudaMemsetAsync(B->abort_all, 0, sizeof(int), st));
  FG_CUDA_TRY(cudaMemsetAsync(B->status, 0, sizeof(int) * B->nprob, st));
  void* args[] = {&a};
  FG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_batch_solve, dim3(B->ctas), dim3(B->threads), args,
                                          batch_smem(), st));
  B->ctx->launches += 1;
  return FG_OK;
}

// Co-resident CTAs for a block size, the schedule and its device copy.
static fg_status batch_plan(fg_batch* B, int threads) {
  fg_ctx* ctx = B->ctx;
  B->threads = threads;
  int per_sm = 0;
  FG_CUDA_TRY(cudaFuncSetAttribute((const void*)k_batch_solve, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)batch_smem()));
  FG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)k_batch_solve, threads,
                                                            batch_smem()));
  if (per_sm < 1) {
    set_error("batch kernel does not fit an SM with %d threads", threads);
    return FG_ERR_UNSUPPORTED;
  }
  B->ctas = per_sm * ctx->sm_count;
  std::vector<int> job_ptr;
  std::vector<BatchJob> jobs;
  batch_schedule(B, B->ctas, job_ptr, jobs);
  // partial slots per problem: 3 x team x 4 doubles
  int64_t roff = 0;
  for (auto& P : B->probs) {
    P.roff = roff;
    roff += 3 * (int64_t)P.team * 4;
  }
  if (roff > B->nrp) {
    if (B->rpool) {
      dev_free(ctx, B->rpool);
      B->owned.erase(std::find(B->owned.begin(), B->owned.end(), (void*)B->rpool));
    }
    FG_TRY(ba(B, (void**)&B->rpool, sizeof(double) * roff));
    B->nrp = roff;
  }
  if (B->d_job_ptr) {
    dev_free(ctx, B->d_job_ptr);
    B->owned.erase(std::find(B->owned.begin(), B->owned.end(), (void*)B->d_job_ptr));
  }
  if (B->d_jobs) {
    dev_free(ctx, B->d_jobs);
    B->owned.erase(std::find(B->owned.begin(), B->owned.end(), (void*)B->d_jobs));
  }
  FG_TRY(ba(B, (void**)&B->d_job_ptr, sizeof(int) * job_ptr.size()));
  FG_TRY(ba(B, (void**)&B->d_jobs, sizeof(BatchJob) * std::max<size_t>(1, jobs.size())));
  FG_CUDA_TRY(cudaMemcpyAsync(B->d_job_ptr, job_ptr.data(), sizeof(int) * job_ptr.size(), cudaMemcpyHostToDevice,
                              ctx->stream));
  if (!jobs.empty())
    FG_CUDA_TRY(cudaMemcpyAsync(B->d_jobs, jobs.data(), sizeof(BatchJob) * jobs.size(), cudaMemcpyHostToDevice,
                                ctx->stream));
  FG_CUDA_TRY(cudaMemcpyAsync(B->d_probs, B->probs.data(), sizeof(BatchProb) * B->nprob, cudaMemcpyHostToDevice,
                              ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return FG_OK;
}

static fg_status batch_time(fg_batch* B, float* ms) {
  cudaStream_t st = B->ctx->stream;
  cudaEvent_t e0, e1;
  FG_CUDA_TRY(cudaEventCreate(&e0));
  FG_CUDA_TRY(cudaEventCreate(&e1));
  FG_CUDA_TRY(cudaEventRecord(e0, st));
  fg_status s = batch_launch(B, st);
  FG_CUDA_TRY(cudaEventRecord(e1, st));
  FG_CUDA_TRY(cudaEventSynchronize(e1));
  cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return s;
}

static void batch_free(fg_batch* B) {
  if (!B) return;
  cudaSetDevice(B->ctx->device);
  cudaStreamSynchronize(B->ctx->stream);
  if (B->graph) cudaGraphExecDestroy(B->graph);
  for (void* p : B->owned) dev_free(B->ctx, p);
  delete B;
}

}  // namespace fg

using namespace fg;

extern "C" {

fg_status fg_batch_create(fg_ctx* ctx, int32_t nprob, const fg_batch_problem* probs, int32_t flags,
                          const fg_solver_params* params, int32_t threads, fg_batch** out) {
  if (!ctx || !probs || !params || !out || nprob < 1) {
    set_error("bad argument: ctx/probs/params/out/nprob");
    return FG_ERR_BADARG;
  }
  *out = nullptr;
  if (threads != 0 && threads != 128 && threads != 256 && threads != 512) {
    set_error("bad argument: threads must be 0 (autotune), 128, 256 or 512");
    return FG_ERR_BADARG;
  }
  if (!(params->rtol >= 0.0) || !(params->atol >= 0.0) || params->max_iters < 1) {
    set_error("bad argument: rtol/atol/max_iters");
    return FG_ERR_BADARG;
  }
  FG_CUDA_TRY(cudaSetDevice(ctx->device));
  fg_batch* B = new fg_batch();
  B->ctx = ctx;
  if (const char* env = std::getenv("FG_BATCH_TEAM_SHARE"))
    if (std::atof(env) > 0.0) B->team_share = std::atof(env);
  B->nprob = nprob;
  B->flags = flags;
  B->prm = *params;
  const bool dev = (flags & FG_INPUTS_ON_DEVICE) != 0;
  int64_t voff = 0, eoff = 0, fstage = 0, xstage = 0;
  for (int i = 0; i < nprob; ++i) {
    const fg_batch_problem& q = probs[i];
    const bool no_interior = q.order * q.n - 1 <= 0;
    if (q.n < 1 || q.order < 1 || q.order > kBatchMaxP || !(q.coef > 0.0) || !q.qp_source || (!q.x && !no_interior)) {
      delete B;
      set_error("bad argument: problem %d (n >= 1, order 1..3, coef > 0, qp_source and x required)", i);
      return FG_ERR_BADARG;
    }
    if ((int64_t)(q.order * q.n + 1) * (q.order * q.n + 1) * (q.order * q.n + 1) >= (1ll << 31)) {
      delete B;
      set_error("problem %d: (order n + 1)^3 lattice nodes exceed the 32-bit index range", i);
      return FG_ERR_UNSUPPORTED;
    }
    BatchProb P;
    std::memset(&P, 0, sizeof(P));
    P.n = q.n;
    P.p = q.order;
    P.L = q.order * q.n + 1;
    P.F = q.order * q.n - 1;
    const double kh = q.coef * (0.5 / q.n);
    P.kh_hi = (float)kh;
    P.kh_lo = (float)(kh - (double)P.kh_hi);
    const double hh = 0.5 / q.n;
    P.h3 = hh * hh * hh;
    P.voff = voff;
    voff += 8 * (int64_t)P.L * P.L * P.L;
    const int64_t nq = (int64_t)(q.order + 1) * (q.order + 1) * (q.order + 1);
    const int64_t ncells = (int64_t)q.n * q.n * q.n;
    P.eoff = eoff;
    eoff += ncells * nq;
    B->nf.push_back(ncells * nq);
    const int64_t F3 = P.F > 0 ? (int64_t)P.F * P.F * P.F : 0;
    B->nx.push_back(F3);
    B->total_dofs += F3;
    B->user_f.push_back(q.qp_source);
    B->user_x.push_back(q.x);
    P.f = dev ? q.qp_source : nullptr;
    P.x = dev ? q.x : nullptr;
    fstage += ncells * nq;
    xstage += F3;
    B->probs.push_back(P);
  }
  fg_status s = FG_OK;
  auto A = [&](void** p, size_t b) { if (s == FG_OK) s = ba(B, p, b); };
  A((void**)&B->vpool, sizeof(float) * std::max<int64_t>(1, voff));
  A((void**)&B->epool, sizeof(double) * std::max<int64_t>(1, eoff));
  A((void**)&B->d_probs, sizeof(BatchProb) * nprob);
  A((void**)&B->d_tabs, sizeof(OrderTables) * kBatchMaxP);
  A((void**)&B->bar, sizeof(unsigned) * nprob);
  A((void**)&B->abort_all, sizeof(int));
  A((void**)&B->status, sizeof(int) * nprob);
  A((void**)&B->iters, sizeof(int) * nprob);
  A((void**)&B->refines, sizeof(int) * nprob);
  A((void**)&B->relres, sizeof(double) * nprob);
  if (!dev) {
    A((void**)&B->fstage, sizeof(double) * std::max<int64_t>(1, fstage));
    A((void**)&B->xstage, sizeof(double) * std::max<int64_t>(1, xstage));
  }
  if (s != FG_OK) {
    batch_free(B);
    return s;
  }
  if (!dev) {
    int64_t fo = 0, xo = 0;
    for (int i = 0; i < nprob; ++i) {
      B->probs[i].f = B->fstage + fo;
      B->probs[i].x = B->xstage + xo;
      fo += B->nf[i];
      xo += B->nx[i];
    }
  }
  // vectors: boundary nodes stay zero for the life of the plan
  cudaError_t e = cudaMemsetAsync(B->vpool, 0, sizeof(float) * std::max<int64_t>(1, voff), ctx->stream);
  OrderTables tabs[kBatchMaxP];
  for (int p = 1; p <= kBatchMaxP; ++p) build_order_tables(p, tabs[p - 1]);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(B->d_tabs, tabs, sizeof(tabs), cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) {
    set_error("batch setup: %s", cudaGetErrorString(e));
    batch_free(B);
    return FG_ERR_CUDA;
  }
  // block size: given, or the fastest of 128/256/512 on this batch (inputs must be valid);
  // large batches are timed on a stratified sample of at most 256 problems.  Team sizing is
  // not timed (a sample run with the full plan's team sizes lasts as long as its largest
  // problem, about half a full run): 0.5, or FG_BATCH_TEAM_SHARE
  if (threads == 0 && nprob > 256) {
    std::vector<int> order(nprob);
    std::iota(order.begin(), order.end(), 0);
    std::vector<double> w(nprob);
    for (int i = 0; i < nprob; ++i) w[i] = (double)B->nx[i] * avg_nnz(probs[i].order);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return w[x] > w[y]; });
    std::vector<fg_batch_problem> sub;
    const int stride = (nprob + 255) / 256;
    for (int k = 0; k < nprob; k += stride) sub.push_back(probs[order[k]]);
    auto t0 = std::chrono::steady_clock::now();
    fg_batch* S = nullptr;
    s = fg_batch_create(ctx, (int32_t)sub.size(), sub.data(), flags, params, 0, &S);
    if (s != FG_OK) {
      batch_free(B);
      return s;
    }
    threads = S->threads;
    batch_free(S);
    B->autotune_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  if (threads == 0) {
    auto t0 = std::chrono::steady_clock::now();
    if (!dev) {
      for (int i = 0; i < nprob; ++i) {
        e = cudaMemcpyAsync((void*)B->probs[i].f, B->user_f[i], sizeof(double) * B->nf[i], cudaMemcpyHostToDevice,
                            ctx->stream);
        if (e != cudaSuccess) break;
      }
    }
    float best = 0.f;
    int best_t = 256;
    for (int t : {128, 256, 512}) {
      s = batch_plan(B, t);
      if (s != FG_OK) break;
      float ms = 0.f;
      s = batch_time(B, &ms);
      if (s != FG_OK) break;
      if (best == 0.f || ms < best) {
        best = ms;
        best_t = t;
      }
    }
    B->autotune_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    threads = best_t;
    if (s != FG_OK) {
      batch_free(B);
      return s;
    }
  }
  s = batch_plan(B, threads);
  if (s != FG_OK) {
    batch_free(B);
    return s;
  }
  // capture the launch (counter resets + the cooperative kernel) in a CUDA graph
  {
    cudaGraph_t g = nullptr;
    cudaStream_t st = ctx->stream;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      fg_status ls = batch_launch(B, st);
      cudaError_t ce = cudaStreamEndCapture(st, &g);
      if (ls == FG_OK && ce == cudaSuccess && g && cudaGraphInstantiate(&B->graph, g, 0) == cudaSuccess)
        B->use_graph = true;
      if (g) cudaGraphDestroy(g);
      ctx->launches -= 1;  // the captured launch did not run
    }
    cudaGetLastError();
  }
  *out = B;
  return FG_OK;
}

fg_status fg_batch_run(fg_batch* B, fg_batch_result* results) {
  if (!B) {
    set_error("bad argument: batch");
    return FG_ERR_BADARG;
  }
  fg_ctx* ctx = B->ctx;
  FG_CUDA_TRY(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  const bool dev = (B->flags & FG_INPUTS_ON_DEVICE) != 0;
  cudaEvent_t e0, e1;
  FG_CUDA_TRY(cudaEventCreate(&e0));
  FG_CUDA_TRY(cudaEventCreate(&e1));
  FG_CUDA_TRY(cudaEventRecord(e0, st));
  if (!dev)
    for (int i = 0; i < B->nprob; ++i)
      FG_CUDA_TRY(cudaMemcpyAsync((void*)B->probs[i].f, B->user_f[i], sizeof(double) * B->nf[i],
                                  cudaMemcpyHostToDevice, st));
  if (B->use_graph) {
    FG_CUDA_TRY(cudaGraphLaunch(B->graph, st));
    ctx->launches += 1;
  } else {
    FG_TRY(batch_launch(B, st));
  }
  if (!dev)
    for (int i = 0; i < B->nprob; ++i)
      FG_CUDA_TRY(cudaMemcpyAsync(B->user_x[i], B->probs[i].x, sizeof(double) * B->nx[i], cudaMemcpyDeviceToHost, st));
  FG_CUDA_TRY(cudaEventRecord(e1, st));
  FG_CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  B->run_ms = ms;
  std::vector<int> stt(B->nprob), it(B->nprob), rf(B->nprob);
  std::vector<double> rr(B->nprob);
  FG_CUDA_TRY(cudaMemcpy(stt.data(), B->status, sizeof(int) * B->nprob, cudaMemcpyDeviceToHost));
  FG_CUDA_TRY(cudaMemcpy(it.data(), B->iters, sizeof(int) * B->nprob, cudaMemcpyDeviceToHost));
  FG_CUDA_TRY(cudaMemcpy(rf.data(), B->refines, sizeof(int) * B->nprob, cudaMemcpyDeviceToHost));
  FG_CUDA_TRY(cudaMemcpy(rr.data(), B->relres, sizeof(double) * B->nprob, cudaMemcpyDeviceToHost));
  fg_status worst = FG_OK;
  for (int i = 0; i < B->nprob; ++i) {
    if (results) {
      results[i].status = stt[i];
      results[i].iterations = it[i];
      results[i].refinements = rf[i];
      results[i].team = B->probs[i].team;
      results[i].rel_residual = rr[i];
    }
    if (stt[i] != 0 && (worst == FG_OK || stt[i] == FG_ERR_TIMEOUT)) worst = stt[i];
  }
  if (worst == FG_ERR_TIMEOUT) set_error("batch: a team barrier gave up");
  else if (worst == FG_ERR_NOT_CONVERGED) set_error("batch: some problems did not converge");
  return worst;
}

fg_status fg_batch_get_info(fg_batch* B, fg_batch_info* info) {
  if (!B || !info) {
    set_error("bad argument: batch/info");
    return FG_ERR_BADARG;
  }
  info->threads = B->threads;
  info->ctas = B->ctas;
  info->max_team = B->max_team;
  info->teams_gt1 = B->teams_gt1;
  info->graph = B->use_graph ? 1 : 0;
  info->total_dofs = B->total_dofs;
  info->predicted_balance = B->predicted_balance;
  info->run_ms = B->run_ms;
  info->autotune_ms = B->autotune_ms;
  info->team_share = B->team_share;
  return FG_OK;
}

fg_status fg_batch_destroy(fg_batch* B) {
  batch_free(B);
  return FG_OK;
}

}  // extern "C"

// fg_bddc.cu -- two-level BDDC preconditioner on box subdomains, and the PCG that uses it.
//
// Reference: FEMPAR's mlbddc_t (Sources/Lib/LinearAlgebra/Preconditioner/sbm_base_mlbddc.i90)
// with the standard coarse FE handler (Sources/Lib/Integration/FESpace/
// sbm_standard_coarse_fe_handler.i90), one level of subdomains and a directly solved coarse
// problem.  The apply is the reference's five steps (sbm_base_mlbddc.i90:909-1009):
//   1. delta_I = A_II^-1 r_I per subdomain; y_I = delta_I
//   2.-3. r_G -= (A delta)_G (one global SpMV: interior dofs belong to one subdomain)
//   4. r_i = W_i R_i r on the interface; coarse correction Phi_i K_c^-1 sum_j Phi_j^T r_j plus
//      the constrained Neumann correction; y_G = sum_i R_i^T W_i (both)
//   5. y_I -= A_II^-1 (A y_G)_I (second global SpMV)
//
// How the constrained Neumann problem is solved (our design, not the reference's
// augmented-matrix direct solve): local dofs are ordered [I | E | V] (interior, interface
// non-vertex, vertex).  Vertex dofs are primal variables and are eliminated outright; the
// remaining constraints (edge / face functionals, rows [C_e C_eV] over the E and V dofs)
// are appended as extra rows.  One partial FP64 Cholesky of the first nr = nI + nE columns of
//        [ K_rr   .    .  ]
//        [ K_Vr  K_VV  .  ]          (lower triangle, N = m + ne rows)
//        [ C_e   C_eV  0  ]
// gives the factor L of K_rr, the rows L_V = K_Vr L^-T and L_e = C_e L^-T, and in the
// trailing block the Schur complements K_VV - K_Vr K_rr^-1 K_rV, -T = C_eV - C_e K_rr^-1 K_rV
// and -S_e = -C_e K_rr^-1 C_e^T.  The local coarse matrix Phi^T K Phi follows from those
// without forming Phi, and the apply needs one forward solve before the coarse solve and
// one backward solve after it:
//   z = L^-1 g_r,  f_Pi = [g_V - L_V z + H^T L_e z ; S_e^-1 L_e z]     (H = S_e^-1 T)
//   s = z - L_V^T u_V,  mu = S_e^-1 (L_e s - u_e + C_eV u_V),  w_r = L^-T (s - L_e^T mu),  w_V = u_V
// (C_eV, the constraint weights on vertex dofs, is zero for the standard handler's averages
// and nonzero for the elasticity handler's face functionals.)
// Without primal vertices (use_vertices = 0, nV = 0) the constraints are added to the local
// matrix as an augmented Lagrangian, K + C^T R C (k_bddc_augment): same constrained
// solutions, an SPD leading block for floating subdomains; K_Pi = S~^-1 - R and the backward
// solve gains L_e^T R u_e.
// (u = the coarse solution restricted to the subdomain).  The coarse matrix is inverted
// by the same partial Cholesky on [[K_c, I], [I, 0]] whose trailing block is -K_c^-1.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <numeric>
#include <type_traits>
#include <utility>
#include <vector>

#include "fg_internal.h"

namespace fg {

struct BSub {
  int64_t aoff;  // FP64 matrix N x N, column-major (lda N)
  int64_t foff;  // FP32 factor nr x nr, column-major (lda nr)
  int64_t roff;  // rows V|e of the factor, row-major nP x nr
  int64_t loff;  // local dofs (m): solver-vector index, order I | E | V
  int64_t woff;  // interface positions (nE + nV): weights, contributions
  int64_t eoff;  // E dofs (nE): z_E
  int64_t poff;  // local coarse dofs (nP = nV + ne): global coarse index, f_Pi
  int64_t koff;  // local coarse matrix nP x nP
  int64_t goff;  // S_e^-1 (ne x ne) then H (ne x nV)
  int64_t boff;  // box map: box lattice nodes x ncomp -> local index (-1 not free)
  int64_t qoff;  // constraint entries (nq): row e, local column (E or V dof), weight
  int64_t cvoff; // C_eV, ne x nV row-major
  int N, m, nI, nE, nV, ne, nr, nP, nq;
  int c0[3], c1[3];
};

static constexpr int kMaxNe = 64;   // edge / face constraints per subdomain (box: 18 objects x 3)
static constexpr int kMaxNv = 32;   // vertex dofs per subdomain (box: 8 vertices x 3)
static constexpr int kMaxLocal = 16384;
static constexpr int kMaxCoarse = 16384;
static constexpr size_t kCoarseLocalSmem = sizeof(double) * (2 * kMaxNe * (kMaxNe + 1) + 2 * kMaxNe * kMaxNv);

}  // namespace fg

struct fg_bddc {
  fg_system* sys = nullptr;
  fg_bddc_params prm;
  std::vector<int32_t> cuts[3];
  int nsub = 0;
  std::vector<fg::BSub> subs;
  fg::BSub* d_subs = nullptr;
  int maxN = 0, maxnr = 0, maxnI = 0, maxnd = 0;
  int64_t nA = 0, nF = 0, nR = 0, nL = 0, nW = 0, nE = 0, nP = 0, nK = 0, nG = 0, nB = 0;
  int64_t nIface = 0, nC = 0, nKpair = 0;
  double* dA = nullptr;
  float* dF = nullptr;
  double* dR = nullptr;
  float* dR32 = nullptr;
  int32_t* dLoc = nullptr;
  double* dW = nullptr;
  double* dDiag = nullptr;
  double* dC = nullptr;
  float* dC32 = nullptr;
  int32_t* dQrow = nullptr;  // constraint entries of all subdomains
  int32_t* dQcol = nullptr;
  double* dQw = nullptr;
  double* dCv = nullptr;     // C_eV of all subdomains
  float* dCv32 = nullptr;
  double* dZ = nullptr;
  float* dZ32 = nullptr;
  int32_t* dPc = nullptr;
  double* dFp = nullptr;
  float* dFp32 = nullptr;
  double* dKp = nullptr;
  double* dG = nullptr;
  float* dG32 = nullptr;
  int32_t* dBox = nullptr;
  int32_t* dOrder = nullptr;  // subdomains by decreasing factorisation work
  bool stepped = false;        // factorise panel step by panel step over all subdomains
  bool coarse_emulated = false; // coarse trailing updates on the tensor cores (last setup)
  bool local_emulated = false;  // subdomain trailing updates on the tensor cores (last setup)
  double* dRho = nullptr;       // use_vertices = 0: augmentation weights R_e at poff + nV + e
  int64_t* dIptr = nullptr;
  int64_t* dIsrc = nullptr;
  int32_t* dIvec = nullptr;
  int64_t* dCptr = nullptr;
  int64_t* dCsrc = nullptr;
  int64_t* dKdst = nullptr;
  int64_t* dKptr = nullptr;
  int64_t* dKsrc = nullptr;
  double* dKc = nullptr;     // 2nC x 2nC, column-major
  double* dKinv = nullptr;   // nC x nC row-major
  float* dKinv32 = nullptr;
  double *dU0 = nullptr, *dV = nullptr, *dQ = nullptr, *dT = nullptr, *dFc = nullptr, *dUc = nullptr;
  float *dU032 = nullptr, *dV32 = nullptr, *dQ32 = nullptr, *dT32 = nullptr, *dFc32 = nullptr, *dUc32 = nullptr;
  double *dRv = nullptr, *dZv = nullptr;                      // row-order apply staging
  double *dX = nullptr, *dRr = nullptr, *dP = nullptr, *dAp = nullptr, *dZz = nullptr;  // PCG (solver layout)
  double* dPart = nullptr;                                     // reduction partials
  int* dErr = nullptr;
  int nred = 0;
  double symbolic_ms = 0.0, numeric_ms = 0.0, factor_flops = 0.0, factor_ms = 0.0, coarse_ms = 0.0;
  uint64_t bytes = 0;
  std::vector<void*> owned;
};

namespace fg {

static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// ---------------------------------------------------------------------------------------
// Dense partial Cholesky building blocks (lower triangle, column-major, lda).
// Block columns of 32; trailing updates in 64 x 64 tiles, 256 threads.

struct CholSmem {
  double D[32][33];
  double Pi[32][64 + 1];
  double Pj[32][64 + 1];
  int fail;
};

// Load the nb x nb diagonal block at j0, factor it in shared memory (warp 0), write it
// back.  Returns false (to every thread) on a non-positive pivot.
__device__ bool chol_diag(double* A, int64_t lda, int j0, int nb, CholSmem& sm) {
  const int tid = threadIdx.x;
  for (int t = tid; t < 32 * 32; t += blockDim.x) {
    int i = t & 31, j = t >> 5;
    sm.D[i][j] = (i < nb && j < nb && i >= j) ? A[(j0 + i) + (int64_t)(j0 + j) * lda] : 0.0;
  }
  if (tid == 0) sm.fail = 0;
  __syncthreads();
  if (tid < 32) {
    const int lane = tid;
    for (int k = 0; k < nb; ++k) {
      double piv = sm.D[k][k];
      if (!(piv > 0.0)) {
        if (lane == 0) sm.fail = 1;
        break;
      }
      double d = sqrt(piv);
      __syncwarp();
      if (lane > k && lane < nb) sm.D[lane][k] /= d;
      __syncwarp();
      if (lane == k) sm.D[k][k] = d;
      for (int j = k + 1; j < nb; ++j)
        if (lane >= j && lane < nb) sm.D[lane][j] -= sm.D[lane][k] * sm.D[j][k];
      __syncwarp();
    }
  }
  __syncthreads();
  if (sm.fail) return false;
  for (int t = tid; t < 32 * 32; t += blockDim.x) {
    int i = t & 31, j = t >> 5;
    if (i < nb && j < nb && i >= j) A[(j0 + i) + (int64_t)(j0 + j) * lda] = sm.D[i][j];
  }
  return true;
}

// Row i (>= j0+nb): A[i, j0:j0+nb] <- A[i, j0:j0+nb] D^-T  (D in shared memory)
__device__ __forceinline__ void chol_trsm_row(double* A, int64_t lda, int j0, int nb, int64_t i, const double (&D)[32][33]) {
  double x[32];
#pragma unroll
  for (int k = 0; k < 32; ++k) x[k] = k < nb ? A[i + (int64_t)(j0 + k) * lda] : 0.0;
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    if (k < nb) {
      double s = x[k];
#pragma unroll
      for (int l = 0; l < k; ++l) s -= x[l] * D[k][l];
      x[k] = s / D[k][k];
    }
  }
#pragma unroll
  for (int k = 0; k < 32; ++k)
    if (k < nb) A[i + (int64_t)(j0 + k) * lda] = x[k];
}

// Trailing tile (ti, tj) of 64 x 64 at rows/cols starting t0: A[r, c] -= sum_k A[r, j0+k] A[c, j0+k]
// for r >= c, r < N, c < cN (cN < 0: N).
__device__ void chol_syrk_tile(double* A, int64_t lda, int N, int j0, int nb, int t0, int ti, int tj, CholSmem& sm,
                               int cN = -1) {
  const int cn = cN < 0 ? N : cN;
  const int tid = threadIdx.x;
  const int r0 = t0 + ti * 64, q0 = t0 + tj * 64;
  for (int t = tid; t < 32 * 64; t += blockDim.x) {
    int r = t & 63, k = t >> 6;
    sm.Pi[k][r] = (k < nb && r0 + r < N) ? A[(r0 + r) + (int64_t)(j0 + k) * lda] : 0.0;
    sm.Pj[k][r] = (k < nb && q0 + r < N) ? A[(q0 + r) + (int64_t)(j0 + k) * lda] : 0.0;
  }
  __syncthreads();
  const int tr = tid & 15, tc = tid >> 4;
  double acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = 0.0;
  for (int k = 0; k < nb; ++k) {
    double a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) a[u] = sm.Pi[k][tr + 16 * u];
#pragma unroll
    for (int v = 0; v < 4; ++v) b[v] = sm.Pj[k][tc + 16 * v];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const int c = q0 + tc + 16 * v;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int r = r0 + tr + 16 * u;
      if (r < N && c < cn && r >= c) A[r + (int64_t)c * lda] -= acc[u][v];
    }
  }
  __syncthreads();
}

// One CTA factors the first ncols columns of an N x N matrix and updates the trailing block.
__device__ bool chol_partial_cta(double* A, int64_t lda, int N, int ncols, CholSmem& sm) {
  for (int j0 = 0; j0 < ncols; j0 += 32) {
    const int nb = min(32, ncols - j0);
    if (!chol_diag(A, lda, j0, nb, sm)) return false;
    __syncthreads();
    for (int64_t i = j0 + nb + threadIdx.x; i < N; i += blockDim.x) chol_trsm_row(A, lda, j0, nb, i, sm.D);
    __syncthreads();
    const int t0 = j0 + nb, tn = N - t0;
    if (tn <= 0) continue;
    const int nt = (tn + 63) / 64;
    for (int ti = 0; ti < nt; ++ti)
      for (int tj = 0; tj <= ti; ++tj) chol_syrk_tile(A, lda, N, j0, nb, t0, ti, tj, sm);
  }
  return true;
}

// ---------------------------------------------------------------------------------------
// Setup kernels

// Dense local matrix from the element matrices (cells in increasing index, each entry's
// sum in that order), constraint rows, and the interface diagonal.  One CTA per subdomain.
__global__ void __launch_bounds__(256)
    k_bddc_assemble(const BSub* __restrict__ subs, const double* __restrict__ E, int nx, int ny, int p, int nn, int nd,
                    int ncomp, const int32_t* __restrict__ box, const int32_t* __restrict__ qrow,
                    const int32_t* __restrict__ qcol, const double* __restrict__ qw, double* __restrict__ A,
                    double* __restrict__ diag) {
  const BSub S = subs[blockIdx.x];
  double* As = A + S.aoff;
  const int64_t N = S.N;
  const int32_t* bm = box + S.boff;
  const int bn0 = p * (S.c1[0] - S.c0[0]) + 1, bn1 = p * (S.c1[1] - S.c0[1]) + 1;
  __shared__ int li[3 * FG_MAX_NN];
  for (int ck = S.c0[2]; ck < S.c1[2]; ++ck)
    for (int cj = S.c0[1]; cj < S.c1[1]; ++cj)
      for (int ci = S.c0[0]; ci < S.c1[0]; ++ci) {
        const int64_t c = ci + (int64_t)nx * (cj + (int64_t)ny * ck);
        for (int t = threadIdx.x; t < nd; t += blockDim.x) {
          int comp = t / nn, a = t - comp * nn;
          int ai = a % (p + 1), aj = (a / (p + 1)) % (p + 1), ak = a / ((p + 1) * (p + 1));
          int bx = p * (ci - S.c0[0]) + ai, by = p * (cj - S.c0[1]) + aj, bz = p * (ck - S.c0[2]) + ak;
          li[t] = bm[(((int64_t)bz * bn1 + by) * bn0 + bx) * ncomp + comp];
        }
        __syncthreads();
        const double* Ec = E + c * nd * nd;
        for (int idx = threadIdx.x; idx < nd * nd; idx += blockDim.x) {
          int a = idx / nd, b = idx - a * nd;
          int ia = li[a], ib = li[b];
          if (ia >= 0 && ib >= 0 && ia >= ib) As[ia + (int64_t)ib * N] += Ec[idx];
        }
        __syncthreads();
      }
  for (int t = threadIdx.x; t < S.nq; t += blockDim.x)
    As[(S.m + qrow[S.qoff + t]) + (int64_t)qcol[S.qoff + t] * N] = qw[S.qoff + t];
  for (int k = threadIdx.x; k < S.nE + S.nV; k += blockDim.x) {
    int i = S.nI + k;
    diag[S.woff + k] = As[i + (int64_t)i * N];
  }
}

// Without primal vertices (use_vertices = 0) a floating subdomain's K_rr is singular.  The
// constrained Neumann problem [K C^T; C 0][w; mu] = [g; h] has the same solution as
// [K + C^T R C, C^T; C 0][w; mu] = [g + C^T R h; h] for any diagonal R > 0, and K + C^T R C
// is SPD once the constraints fix K's kernel.  R_e = mean(diag K_EE) / |c_e|^2 (the scale of
// K on the constraint's direction).  The local coarse matrix becomes S~^-1 - R and the
// backward apply adds L_e^T R u_e (k_bddc_coarse_local, k_bddc_neumann_bwd).  Entries are
// grouped by row; rows are added one after another (each (i, j) once per row): deterministic.
__global__ void __launch_bounds__(256)
    k_bddc_augment(const BSub* __restrict__ subs, const int32_t* __restrict__ qrow, const int32_t* __restrict__ qcol,
                   const double* __restrict__ qw, double* __restrict__ A, double* __restrict__ rho) {
  const BSub S = subs[blockIdx.x];
  double* As = A + S.aoff;
  const int64_t N = S.N;
  __shared__ double red[256];
  __shared__ int rs[kMaxNe + 1];
  double d = 0.0;
  for (int k = threadIdx.x; k < S.nE; k += blockDim.x) d += As[(S.nI + k) + (int64_t)(S.nI + k) * N];
  red[threadIdx.x] = d;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  const double dbar = S.nE > 0 ? red[0] / S.nE : 1.0;
  if (threadIdx.x == 0) {
    int t = 0;
    for (int e = 0; e <= S.ne; ++e) {
      while (t < S.nq && qrow[S.qoff + t] < e) ++t;
      rs[e] = t;
    }
  }
  __syncthreads();
  for (int e = 0; e < S.ne; ++e) {
    const int t0 = rs[e], len = rs[e + 1] - rs[e];
    double nrm = 0.0;
    for (int t = 0; t < len; ++t) nrm += qw[S.qoff + t0 + t] * qw[S.qoff + t0 + t];
    const double re = nrm > 0.0 ? dbar / nrm : 0.0;
    if (threadIdx.x == 0) rho[S.poff + S.nV + e] = re;
    for (int64_t pq = threadIdx.x; pq < (int64_t)len * len; pq += blockDim.x) {
      const int a = (int)(pq / len), b = (int)(pq - (int64_t)a * len);
      const int ca = qcol[S.qoff + t0 + a], cb = qcol[S.qoff + t0 + b];
      if (ca >= cb) As[ca + (int64_t)cb * N] += re * qw[S.qoff + t0 + a] * qw[S.qoff + t0 + b];
    }
    __syncthreads();
  }
}

// Interface weights: multiplicity (1 / subdomains around) or diag(A_i) / sum_j diag(A_j);
// one thread per global interface dof, contributions in subdomain order.
__global__ void k_bddc_weights(int64_t nG, const int64_t* __restrict__ iptr, const int64_t* __restrict__ isrc,
                               const double* __restrict__ diag, int stiffness, double* __restrict__ w) {
  int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= nG) return;
  const int64_t b = iptr[g], e = iptr[g + 1];
  double s = 0.0;
  for (int64_t t = b; t < e; ++t) s += diag[isrc[t]];
  for (int64_t t = b; t < e; ++t) w[isrc[t]] = stiffness ? diag[isrc[t]] / s : 1.0 / (double)(e - b);
}

// Subdomains in order of decreasing size (order[]), so the largest start first and the
// smaller ones fill the tail; two CTAs per SM share its FP64 pipe.
__global__ void __launch_bounds__(256, 2)
    k_bddc_potrf(const BSub* __restrict__ subs, const int32_t* __restrict__ order, double* __restrict__ A, int* err) {
  __shared__ CholSmem sm;
  const int sid = order[blockIdx.x];
  const BSub S = subs[sid];
  if (!chol_partial_cta(A + S.aoff, S.N, S.N, S.nr, sm)) {
    if (threadIdx.x == 0) atomicCAS(err, 0, 1 + sid);
  }
}

// The same partial Cholesky stepped by panel over all subdomains at once: per step j0 one
// launch for the diagonal blocks, one for the row solves, one for the trailing 64 x 64 tiles of
// every subdomain (grid.y = subdomain).  Work of uneven subdomains is then spread over all SMs
// at every step instead of one CTA carrying the largest subdomain to the end.
__global__ void k_bstep_diag(const BSub* __restrict__ subs, double* __restrict__ A, int j0, int* err) {
  __shared__ CholSmem sm;
  const BSub S = subs[blockIdx.x];
  if (j0 >= S.nr) return;
  const int nb = min(32, S.nr - j0);
  if (!chol_diag(A + S.aoff, S.N, j0, nb, sm)) {
    if (threadIdx.x == 0) atomicCAS(err, 0, 1 + (int)blockIdx.x);
  }
}

__global__ void __launch_bounds__(256) k_bstep_trsm(const BSub* __restrict__ subs, double* __restrict__ A, int j0) {
  __shared__ double Dsh[32][33];
  const BSub S = subs[blockIdx.y];
  if (j0 >= S.nr) return;
  const int nb = min(32, S.nr - j0);
  const int64_t i = j0 + nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j0 + nb + (int64_t)blockIdx.x * blockDim.x >= S.N) return;  // whole block past the matrix
  double* As = A + S.aoff;
  for (int t = threadIdx.x; t < 32 * 32; t += blockDim.x) {
    int r = t & 31, c = t >> 5;
    Dsh[r][c] = (r < nb && c < nb && r >= c) ? As[(j0 + r) + (int64_t)(j0 + c) * S.N] : 0.0;
  }
  __syncthreads();
  if (i < S.N) chol_trsm_row(As, S.N, j0, nb, i, Dsh);
}

__global__ void __launch_bounds__(256) k_bstep_syrk(const BSub* __restrict__ subs, double* __restrict__ A, int j0) {
  __shared__ CholSmem sm;
  const BSub S = subs[blockIdx.y];
  if (j0 >= S.nr) return;
  const int nb = min(32, S.nr - j0);
  const int t0 = j0 + nb, tn = S.N - t0;
  if (tn <= 0) return;
  const int nt = (tn + 63) / 64;
  const int64_t b = blockIdx.x;
  if (b >= (int64_t)nt * (nt + 1) / 2) return;
  int ti = (int)((sqrt(8.0 * (double)b + 1.0) - 1.0) * 0.5);
  while ((int64_t)(ti + 1) * (ti + 2) / 2 <= b) ++ti;
  while ((int64_t)ti * (ti + 1) / 2 > b) --ti;
  const int tj = (int)(b - (int64_t)ti * (ti + 1) / 2);
  chol_syrk_tile(A + S.aoff, S.N, S.N, j0, nb, t0, ti, tj, sm);
}

// k_bstep_syrk restricted to the columns [j0 + nb, min(cend, nr)) of a wider panel: tiles
// (ti, tj, subdomain) = blockIdx (x, y, z), ti >= tj.
__global__ void __launch_bounds__(256) k_bstep_syrk_panel(const BSub* __restrict__ subs, double* __restrict__ A,
                                                          int j0, int cend) {
  __shared__ CholSmem sm;
  const BSub S = subs[blockIdx.z];
  if (j0 >= S.nr) return;
  const int nb = min(32, S.nr - j0);
  const int t0 = j0 + nb, cN = min(cend, S.nr);
  const int ti = blockIdx.x, tj = blockIdx.y;
  if (ti < tj || t0 + tj * 64 >= cN || t0 + ti * 64 >= S.N) return;
  chol_syrk_tile(A + S.aoff, S.N, S.N, j0, nb, t0, ti, tj, sm, cN);
}

// Local coarse matrix K_Pi (order [V | e]), S_e^-1 and H = S_e^-1 T from the trailing block.
__global__ void __launch_bounds__(128)
    k_bddc_coarse_local(const BSub* __restrict__ subs, const double* __restrict__ A, double* __restrict__ Kp,
                        double* __restrict__ G, float* __restrict__ G32, const double* __restrict__ rho, int* err) {
  // dynamic shared memory: Se, Gi (kMaxNe x (kMaxNe+1)), T, H (kMaxNe x kMaxNv)
  extern __shared__ __align__(16) unsigned char smraw[];
  auto Se = reinterpret_cast<double(*)[kMaxNe + 1]>(smraw);
  auto Gi = reinterpret_cast<double(*)[kMaxNe + 1]>(smraw + sizeof(double) * kMaxNe * (kMaxNe + 1));
  auto T = reinterpret_cast<double(*)[kMaxNv]>(smraw + 2 * sizeof(double) * kMaxNe * (kMaxNe + 1));
  auto H = reinterpret_cast<double(*)[kMaxNv]>(smraw + 2 * sizeof(double) * kMaxNe * (kMaxNe + 1) +
                                               sizeof(double) * kMaxNe * kMaxNv);
  __shared__ int fail;
  const BSub S = subs[blockIdx.x];
  const double* As = A + S.aoff;
  const int64_t N = S.N;
  const int nr = S.nr, nV = S.nV, ne = S.ne, nP = S.nP;
  const int tid = threadIdx.x;
  auto tr = [&](int i, int j) -> double {  // trailing block, symmetric access
    int a = i >= j ? i : j, b = i >= j ? j : i;
    return As[(nr + a) + (int64_t)(nr + b) * N];
  };
  for (int t = tid; t < ne * ne; t += blockDim.x) {
    int i = t / ne, j = t - i * ne;
    Se[i][j] = -tr(nV + i, nV + j);
  }
  for (int t = tid; t < ne * nV; t += blockDim.x) {
    int i = t / nV, v = t - i * nV;
    T[i][v] = -tr(nV + i, v);
  }
  if (tid == 0) fail = 0;
  __syncthreads();
  // Cholesky of S_e (thread 0; ne <= 64)
  if (tid == 0) {
    for (int k = 0; k < ne && !fail; ++k) {
      double piv = Se[k][k];
      for (int l = 0; l < k; ++l) piv -= Se[k][l] * Se[k][l];
      if (!(piv > 0.0)) { fail = 1; break; }
      Se[k][k] = sqrt(piv);
      for (int i = k + 1; i < ne; ++i) {
        double s = Se[i][k];
        for (int l = 0; l < k; ++l) s -= Se[i][l] * Se[k][l];
        Se[i][k] = s / Se[k][k];
      }
    }
  }
  __syncthreads();
  if (fail) {
    if (tid == 0) atomicCAS(err, 0, 1 + (int)blockIdx.x);
    return;
  }
  // S_e^-1: column j solved by thread j
  for (int j = tid; j < ne; j += blockDim.x) {
    double y[kMaxNe];
    for (int i = 0; i < ne; ++i) {
      double s = (i == j) ? 1.0 : 0.0;
      for (int l = 0; l < i; ++l) s -= Se[i][l] * y[l];
      y[i] = s / Se[i][i];
    }
    for (int i = ne - 1; i >= 0; --i) {
      double s = y[i];
      for (int l = i + 1; l < ne; ++l) s -= Se[l][i] * y[l];
      y[i] = s / Se[i][i];
    }
    for (int i = 0; i < ne; ++i) Gi[i][j] = y[i];
  }
  __syncthreads();
  for (int t = tid; t < ne * nV; t += blockDim.x) {
    int i = t / nV, v = t - i * nV;
    double s = 0.0;
    for (int l = 0; l < ne; ++l) s += Gi[i][l] * T[l][v];
    H[i][v] = s;
  }
  __syncthreads();
  double* K = Kp + S.koff;
  for (int t = tid; t < nP * nP; t += blockDim.x) {
    int i = t / nP, j = t - i * nP;
    double v;
    if (i < nV && j < nV) {
      double s = tr(i, j);
      for (int l = 0; l < ne; ++l) s += T[l][i] * H[l][j];
      v = s;
    } else if (i >= nV && j < nV) {
      v = H[i - nV][j];
    } else if (i < nV && j >= nV) {
      v = H[j - nV][i];
    } else {
      v = Gi[i - nV][j - nV];
      if (rho && i == j) v -= rho[S.poff + i];  // augmented: Phi^T K Phi = S~^-1 - R
    }
    K[t] = v;
  }
  for (int t = tid; t < ne * ne; t += blockDim.x) {
    int i = t / ne, j = t - i * ne;
    G[S.goff + t] = Gi[i][j];
    G32[S.goff + t] = (float)Gi[i][j];
  }
  for (int t = tid; t < ne * nV; t += blockDim.x) {
    int i = t / nV, v = t - i * nV;
    G[S.goff + ne * ne + t] = H[i][v];
    G32[S.goff + ne * ne + t] = (float)H[i][v];
  }
}

// FP32 copy of the factor (nr x nr, lda nr) and the rows V|e of the factor, row-major.
__global__ void __launch_bounds__(256)
    k_bddc_panels(const BSub* __restrict__ subs, const double* __restrict__ A, float* __restrict__ F,
                  double* __restrict__ R, float* __restrict__ R32) {
  const BSub S = subs[blockIdx.x];
  const double* As = A + S.aoff;
  const int64_t N = S.N;
  const int nr = S.nr;
  float* Fs = F + S.foff;
  for (int j = 0; j < nr; ++j)
    for (int i = j + threadIdx.x; i < nr; i += blockDim.x) Fs[i + (int64_t)j * nr] = (float)As[i + (int64_t)j * N];
  for (int k = 0; k < S.nP; ++k)
    for (int i = threadIdx.x; i < nr; i += blockDim.x) {
      double v = As[(nr + k) + (int64_t)i * N];
      R[S.roff + (int64_t)k * nr + i] = v;
      R32[S.roff + (int64_t)k * nr + i] = (float)v;
    }
}

// Deterministic segmented sums: out[dst[u]] = sum_{t in [ptr[u], ptr[u+1])} src[sidx[t]].
__global__ void k_seg_sum(int64_t nseg, const int64_t* __restrict__ ptr, const int64_t* __restrict__ sidx,
                          const int64_t* __restrict__ dst, const double* __restrict__ src, double* __restrict__ out) {
  int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= nseg) return;
  double s = 0.0;
  for (int64_t t = ptr[u]; t < ptr[u + 1]; ++t) s += src[sidx[t]];
  out[dst ? dst[u] : u] = s;
}

__global__ void k_coarse_identity(int64_t nC, double* __restrict__ Kc) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < nC) Kc[(nC + i) + i * 2 * nC] = 1.0;
}

__global__ void k_chol_diag1(double* A, int64_t lda, int j0, int nb, int* err) {
  __shared__ CholSmem sm;
  if (!chol_diag(A, lda, j0, nb, sm)) {
    if (threadIdx.x == 0) atomicCAS(err, 0, 1);
  }
}

__global__ void __launch_bounds__(256) k_chol_trsm1(double* A, int64_t lda, int N, int j0, int nb) {
  __shared__ double Dsh[32][33];
  for (int t = threadIdx.x; t < 32 * 32; t += blockDim.x) {
    int i = t & 31, j = t >> 5;
    Dsh[i][j] = (i < nb && j < nb && i >= j) ? A[(j0 + i) + (int64_t)(j0 + j) * lda] : 0.0;
  }
  __syncthreads();
  int64_t i = j0 + nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= N) return;
  chol_trsm_row(A, lda, j0, nb, i, Dsh);
}

__global__ void __launch_bounds__(256) k_chol_syrk1(double* A, int64_t lda, int N, int j0, int nb, int nt) {
  __shared__ CholSmem sm;
  // blockIdx.x -> lower tile (ti, tj)
  int64_t b = blockIdx.x;
  int ti = (int)((sqrt(8.0 * (double)b + 1.0) - 1.0) * 0.5);
  while ((int64_t)(ti + 1) * (ti + 2) / 2 <= b) ++ti;
  while ((int64_t)ti * (ti + 1) / 2 > b) --ti;
  int tj = (int)(b - (int64_t)ti * (ti + 1) / 2);
  if (ti >= nt) return;
  chol_syrk_tile(A, lda, N, j0, nb, j0 + nb, ti, tj, sm);
}

// The same update restricted to the columns [j0 + nb, cN) of a wider panel: tiles (ti, tj) =
// blockIdx (x, y), ti >= tj.
__global__ void __launch_bounds__(256) k_chol_syrk_panel(double* A, int64_t lda, int N, int j0, int nb, int cN) {
  __shared__ CholSmem sm;
  const int ti = blockIdx.x, tj = blockIdx.y;
  if (ti < tj) return;
  chol_syrk_tile(A, lda, N, j0, nb, j0 + nb, ti, tj, sm, cN);
}

__global__ void k_coarse_extract(int64_t nC, const double* __restrict__ Kc, double* __restrict__ Kinv,
                                 float* __restrict__ Kinv32) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nC * nC) return;
  int64_t i = t / nC, j = t - i * nC;
  int64_t a = i >= j ? i : j, b = i >= j ? j : i;
  double v = -Kc[(nC + a) + (nC + b) * 2 * nC];
  Kinv[t] = v;
  Kinv32[t] = (float)v;
}

// ---------------------------------------------------------------------------------------
// Apply kernels (T = double: FP64 factor in A with lda N; T = float: FP32 copy, lda nr)

template <typename T>
struct Fac;
template <>
struct Fac<double> {
  static __device__ __forceinline__ const double* L(const double* A, const float*, const BSub& S) { return A + S.aoff; }
  static __device__ __forceinline__ int64_t lda(const BSub& S) { return S.N; }
};
template <>
struct Fac<float> {
  static __device__ __forceinline__ const float* L(const double*, const float* F, const BSub& S) { return F + S.foff; }
  static __device__ __forceinline__ int64_t lda(const BSub& S) { return S.nr; }
};

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Solve L x = x in place for rows [start, n); x[0:start) must be zero on entry.
template <typename T>
__device__ void trsv_lower(const T* __restrict__ L, int64_t lda, int n, int start, T* x) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int j0 = (start / 32) * 32; j0 < n; j0 += 32) {
    const int nb = min(32, n - j0);
    if (warp == 0) {
      T row[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) row[k] = (lane < nb && k < nb) ? L[(j0 + lane) + (int64_t)(j0 + k) * lda] : T(0);
      T xv = lane < nb ? x[j0 + lane] : T(0);
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        if (k < nb) {
          T xk = __shfl_sync(0xffffffffu, xv, k);
          xk = xk / __shfl_sync(0xffffffffu, row[k], k);
          if (lane == k) xv = xk;
          if (lane > k) xv -= row[k] * xk;
        }
      }
      if (lane < nb) x[j0 + lane] = xv;
    }
    __syncthreads();
    for (int i = j0 + nb + tid; i < n; i += blockDim.x) {
      T acc = T(0);
#pragma unroll 8
      for (int k = 0; k < nb; ++k) acc += L[i + (int64_t)(j0 + k) * lda] * x[j0 + k];
      x[i] -= acc;
    }
    __syncthreads();
  }
}

// Solve L^T x = x in place for rows [0, n).
template <typename T>
__device__ void trsv_upper_t(const T* __restrict__ L, int64_t lda, int n, T* x) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  if (n <= 0) return;
  for (int j0 = ((n - 1) / 32) * 32; j0 >= 0; j0 -= 32) {
    const int nb = min(32, n - j0);
    const int below = j0 + nb;
    for (int c = warp; c < nb; c += nw) {
      const T* col = L + (int64_t)(j0 + c) * lda;
      T acc = T(0);
      for (int i = below + lane; i < n; i += 32) acc += col[i] * x[i];
      acc = warp_sum(acc);
      if (lane == 0) x[j0 + c] -= acc;
    }
    __syncthreads();
    if (warp == 0) {
      T colv[32];  // lane i holds L[j0+k, j0+i] for k = 0..31
#pragma unroll
      for (int k = 0; k < 32; ++k) colv[k] = (lane < nb && k < nb) ? L[(j0 + k) + (int64_t)(j0 + lane) * lda] : T(0);
      T xv = lane < nb ? x[j0 + lane] : T(0);
#pragma unroll
      for (int k = 31; k >= 0; --k) {
        if (k < nb) {
          T xk = __shfl_sync(0xffffffffu, xv, k);
          xk = xk / __shfl_sync(0xffffffffu, colv[k], k);
          if (lane == k) xv = xk;
          if (lane < k) xv -= colv[k] * xk;
        }
      }
      if (lane < nb) x[j0 + lane] = xv;
    }
    __syncthreads();
  }
}

// Steps 1 (PHASE 1) and 5 (PHASE 2): interior Dirichlet solves.
template <typename T, int PHASE>
__global__ void __launch_bounds__(256)
    k_bddc_dirichlet(const BSub* __restrict__ subs, const double* __restrict__ A, const float* __restrict__ F,
                     const int32_t* __restrict__ loc, const double* __restrict__ r, const T* __restrict__ t,
                     T* __restrict__ u0, double* __restrict__ z) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* x = reinterpret_cast<T*>(smraw);
  const BSub S = subs[blockIdx.x];
  const int nI = S.nI;
  if (nI == 0) return;
  const T* L = Fac<T>::L(A, F, S);
  const int64_t lda = Fac<T>::lda(S);
  const int32_t* lv = loc + S.loff;
  for (int i = threadIdx.x; i < nI; i += blockDim.x) x[i] = PHASE == 1 ? (T)r[lv[i]] : t[lv[i]];
  __syncthreads();
  trsv_lower<T>(L, lda, nI, 0, x);
  trsv_upper_t<T>(L, lda, nI, x);
  for (int i = threadIdx.x; i < nI; i += blockDim.x) {
    int v = lv[i];
    if (PHASE == 1) {
      u0[v] = x[i];
      z[v] = (double)x[i];
    } else {
      z[v] -= (double)x[i];
    }
  }
}

// Step 4, before the coarse solve: z = L^-1 [0; g_E], coarse residual f_Pi.
template <typename T>
__global__ void __launch_bounds__(256)
    k_bddc_neumann_fwd(const BSub* __restrict__ subs, const double* __restrict__ A, const float* __restrict__ F,
                       const T* __restrict__ R, const T* __restrict__ G, const int32_t* __restrict__ loc,
                       const double* __restrict__ w, const double* __restrict__ r, const T* __restrict__ q,
                       T* __restrict__ zE, T* __restrict__ fP) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* x = reinterpret_cast<T*>(smraw);
  __shared__ T gV[kMaxNv], ab[kMaxNv + kMaxNe];
  const BSub S = subs[blockIdx.x];
  const int nI = S.nI, nE = S.nE, nV = S.nV, ne = S.ne, nr = S.nr, nP = S.nP;
  const T* L = Fac<T>::L(A, F, S);
  const int64_t lda = Fac<T>::lda(S);
  const int32_t* lv = loc + S.loff;
  for (int i = threadIdx.x; i < nI; i += blockDim.x) x[i] = T(0);
  for (int k = threadIdx.x; k < nE + nV; k += blockDim.x) {
    int v = lv[nI + k];
    T g = (T)(w[S.woff + k] * (r[v] - (double)q[v]));
    if (k < nE) x[nI + k] = g;
    else gV[k - nE] = g;
  }
  __syncthreads();
  trsv_lower<T>(L, lda, nr, nI, x);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const T* Rs = R + S.roff;
  for (int k = warp; k < nP; k += nw) {
    const T* row = Rs + (int64_t)k * nr;
    T acc = T(0);
    for (int i = nI + lane; i < nr; i += 32) acc += row[i] * x[i];
    acc = warp_sum(acc);
    if (lane == 0) ab[k] = acc;
  }
  __syncthreads();
  const T* Gi = G + S.goff;
  const T* H = Gi + ne * ne;
  for (int j = threadIdx.x; j < nP; j += blockDim.x) {
    T f;
    if (j < nV) {
      f = gV[j] - ab[j];
      for (int l = 0; l < ne; ++l) f += H[l * nV + j] * ab[nV + l];
    } else {
      f = T(0);
      for (int l = 0; l < ne; ++l) f += Gi[(j - nV) * ne + l] * ab[nV + l];
    }
    fP[S.poff + j] = f;
  }
  for (int k = threadIdx.x; k < nE; k += blockDim.x) zE[S.eoff + k] = x[nI + k];
}

// Step 4, after the coarse solve: constrained local solution, weighted interface values.
template <typename T>
__global__ void __launch_bounds__(256)
    k_bddc_neumann_bwd(const BSub* __restrict__ subs, const double* __restrict__ A, const float* __restrict__ F,
                       const T* __restrict__ R, const T* __restrict__ G, const T* __restrict__ Cv,
                       const int32_t* __restrict__ pc, const T* __restrict__ uc, const T* __restrict__ zE,
                       const double* __restrict__ w, const double* __restrict__ rho, T* __restrict__ contrib) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* x = reinterpret_cast<T*>(smraw);
  __shared__ T uP[kMaxNv + kMaxNe], cm[kMaxNe], mu[kMaxNe];
  const BSub S = subs[blockIdx.x];
  const int nI = S.nI, nE = S.nE, nV = S.nV, ne = S.ne, nr = S.nr, nP = S.nP;
  const T* L = Fac<T>::L(A, F, S);
  const int64_t lda = Fac<T>::lda(S);
  const T* Rs = R + S.roff;
  for (int j = threadIdx.x; j < nP; j += blockDim.x) uP[j] = uc[pc[S.poff + j]];
  __syncthreads();
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
    T s = i < nI ? T(0) : zE[S.eoff + (i - nI)];
    for (int v = 0; v < nV; ++v) s -= Rs[(int64_t)v * nr + i] * uP[v];
    if (rho)  // augmented: the right-hand side gains C^T R u_e, i.e. s gains L_e^T R u_e
      for (int k = 0; k < ne; ++k) s += Rs[(int64_t)(nV + k) * nr + i] * (T)rho[S.poff + nV + k] * uP[nV + k];
    x[i] = s;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = warp; k < ne; k += nw) {
    const T* row = Rs + (int64_t)(nV + k) * nr;
    T acc = T(0);
    for (int i = lane; i < nr; i += 32) acc += row[i] * x[i];
    acc = warp_sum(acc);
    if (lane == 0) {
      const T* cv = Cv + S.cvoff + (int64_t)k * nV;
      for (int v = 0; v < nV; ++v) acc += cv[v] * uP[v];
      cm[k] = acc - uP[nV + k];
    }
  }
  __syncthreads();
  const T* Gi = G + S.goff;
  for (int k = threadIdx.x; k < ne; k += blockDim.x) {
    T s = T(0);
    for (int l = 0; l < ne; ++l) s += Gi[k * ne + l] * cm[l];
    mu[k] = s;
  }
  __syncthreads();
  if (ne > 0) {
    for (int i = threadIdx.x; i < nr; i += blockDim.x) {
      T s = x[i];
      for (int k = 0; k < ne; ++k) s -= Rs[(int64_t)(nV + k) * nr + i] * mu[k];
      x[i] = s;
    }
    __syncthreads();
  }
  trsv_upper_t<T>(L, lda, nr, x);
  for (int k = threadIdx.x; k < nE + nV; k += blockDim.x) {
    T v = k < nE ? x[nI + k] : uP[k - nE];
    contrib[S.woff + k] = (T)(w[S.woff + k] * (double)v);
  }
}

template <typename T>
__global__ void k_coarse_gather(int64_t nC, const int64_t* __restrict__ ptr, const int64_t* __restrict__ src,
                                const T* __restrict__ fP, T* __restrict__ fc) {
  int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (I >= nC) return;
  double s = 0.0;
  for (int64_t t = ptr[I]; t < ptr[I + 1]; ++t) s += (double)fP[src[t]];
  fc[I] = (T)s;
}

template <typename T>
__global__ void __launch_bounds__(256) k_coarse_gemv(int64_t nC, const T* __restrict__ K, const T* __restrict__ f,
                                                     T* __restrict__ u) {
  const int lane = threadIdx.x & 31;
  int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (row >= nC) return;
  const T* k = K + row * nC;
  double acc = 0.0;
  if constexpr (std::is_same<T, float>::value) {
    // FP32 factors: compensated FP32 sums per lane (a conversion and an FP64 FMA per element
    // would make this FP64-pipe bound), the 32 lane sums in FP64
    float s = 0.f, c = 0.f;
    for (int64_t j = lane; j < nC; j += 32) {
      const float y = fmaf(k[j], f[j], -c);
      const float t = s + y;
      c = (t - s) - y;
      s = t;
    }
    acc = (double)s - (double)c;
  } else {
    for (int64_t j = lane; j < nC; j += 32) acc += (double)k[j] * (double)f[j];
  }
  acc = warp_sum(acc);
  if (lane == 0) u[row] = (T)acc;
}

template <typename T>
__global__ void k_iface_sum(int64_t nG, const int64_t* __restrict__ ptr, const int64_t* __restrict__ src,
                            const int32_t* __restrict__ ivec, const T* __restrict__ contrib, T* __restrict__ v,
                            double* __restrict__ z) {
  int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g >= nG) return;
  double s = 0.0;
  for (int64_t t = ptr[g]; t < ptr[g + 1]; ++t) s += (double)contrib[src[t]];
  v[ivec[g]] = (T)s;
  z[ivec[g]] = s;
}

// ---------------------------------------------------------------------------------------
// PCG vector kernels (solver-layout FP64 vectors; padding entries stay zero)

static constexpr int VB = 256;

template <int NV>
__device__ void block_partials(double (&v)[NV], double* part) {
  __shared__ double sh[NV][VB / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double a = warp_sum(v[k]);
    if (lane == 0) sh[k][warp] = a;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double s = 0.0;
    for (int w = 0; w < VB / 32; ++w) s += sh[threadIdx.x][w];
    part[(int64_t)threadIdx.x * gridDim.x + blockIdx.x] = s;
  }
}

__global__ void __launch_bounds__(VB) k_dot2(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                                             const double* __restrict__ c, double* part) {
  double v[2] = {0.0, 0.0};
  for (int64_t i = blockIdx.x * (int64_t)VB + threadIdx.x; i < n; i += (int64_t)gridDim.x * VB) {
    v[0] = fma(a[i], b[i], v[0]);
    if (c) v[1] = fma(c[i], c[i], v[1]);
  }
  block_partials<2>(v, part);
}

__global__ void __launch_bounds__(VB) k_axpy_res(int64_t n, double alpha, const double* __restrict__ p,
                                                 const double* __restrict__ ap, double* __restrict__ x,
                                                 double* __restrict__ r, double* part) {
  double v[1] = {0.0};
  for (int64_t i = blockIdx.x * (int64_t)VB + threadIdx.x; i < n; i += (int64_t)gridDim.x * VB) {
    x[i] = fma(alpha, p[i], x[i]);
    double ri = fma(-alpha, ap[i], r[i]);
    r[i] = ri;
    v[0] = fma(ri, ri, v[0]);
  }
  block_partials<1>(v, part);
}

__global__ void k_xpby(int64_t n, const double* __restrict__ z, double beta, double* __restrict__ p) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) p[i] = fma(beta, p[i], z[i]);
}

__global__ void k_sub(int64_t n, const double* __restrict__ a, double* __restrict__ r) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) r[i] -= a[i];
}

__global__ void k_rows_in(int64_t n, const int32_t* __restrict__ row2vec, const double* __restrict__ src,
                          double* __restrict__ dst) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) dst[row2vec[i]] = src[i];
}

__global__ void k_rows_out(int64_t n, const int32_t* __restrict__ row2vec, const double* __restrict__ src,
                           double* __restrict__ dst) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[row2vec[i]];
}

// ---------------------------------------------------------------------------------------
// Host side

static fg_status balloc(fg_bddc* B, void** p, size_t bytes) {
  fg_ctx* ctx = B->sys->space->mesh->ctx;
  FG_TRY(dev_alloc(ctx, p, bytes));
  B->owned.push_back(*p);
  B->bytes += bytes;
  return FG_OK;
}

template <typename T>
static fg_status balloc_n(fg_bddc* B, T** p, int64_t n, bool zero = false) {
  FG_TRY(balloc(B, (void**)p, sizeof(T) * (size_t)(n > 0 ? n : 1)));
  if (zero) FG_CUDA_TRY(cudaMemsetAsync(*p, 0, sizeof(T) * (size_t)(n > 0 ? n : 1), B->sys->space->mesh->ctx->stream));
  return FG_OK;
}

template <typename T>
static fg_status upload(fg_bddc* B, T** p, const std::vector<T>& h) {
  FG_TRY(balloc_n(B, p, (int64_t)h.size()));
  if (!h.empty())
    FG_CUDA_TRY(cudaMemcpyAsync(*p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice,
                                B->sys->space->mesh->ctx->stream));
  return FG_OK;
}

// Counting sort of (key, value) pairs by key, stable: CSR pointer over nkeys + values.
static void pairs_to_csr(int64_t nkeys, const std::vector<std::pair<int64_t, int64_t>>& pr, std::vector<int64_t>& ptr,
                         std::vector<int64_t>& val) {
  ptr.assign(nkeys + 1, 0);
  for (auto& kv : pr) ptr[kv.first + 1]++;
  for (int64_t k = 0; k < nkeys; ++k) ptr[k + 1] += ptr[k];
  val.resize(pr.size());
  std::vector<int64_t> pos(ptr.begin(), ptr.end() - 1);
  for (auto& kv : pr) val[pos[kv.first]++] = kv.second;
}

struct AxisInfo {
  std::vector<char> on_cut, plane;
  std::vector<int> idx;   // plane index on slab planes, else the slab that contains the position
  std::vector<int> slab;  // the slab that contains the position (domain-boundary planes included)
};

// Face functionals of the elasticity coarse handler (sbm_elasticity_coarse_fe_handler.i90:
// 180-381, strategy CI): for the face object `key` of a subdomain and rigid-body mode r_m
// (translations e_1..e_3, rotations r4 = (y,-x,0), r5 = (-z,0,x), r6 = (0,z,-y) in the
// coordinates themselves, :37-73), the constraint row of the local dof (node a, component c)
// is (1/|F|) sum over the face's facets and their Gauss points of N_a r_m[c] w |J_F|, |F| the
// face measure by the same rule.  Facets are the subdomain's own cell faces on the plane;
// (p+1)^2 Gauss-Legendre points per facet on the bilinear map of its four vertices,
// |J_F| = |dx/ds x dx/dt|.  Entries of dofs that are not free are dropped.
// One change of basis: the rotations are taken about the face's centroid x_F and divided by
// sqrt(|F|) (r4 = ((y - y_F), -(x - x_F), 0) / sqrt(|F|), ...).  Each is the reference's rotation
// plus translations, scaled, so the six rows span the same space and the BDDC operator (which
// depends on the constraints' span only) is the same; in the reference's coordinates the
// rotation rows are nearly combinations of the translation rows far from the origin, and
// S_e = C K^-1 C^T is too ill-conditioned for the FP32 factors.
// The facets: the subdomain's cell faces on the plane normal to axis a at side `side` of its
// cells ca (0: the low face, 1: the high face) for which facet(cb, cc) holds.
template <typename Facet>
static void face_functionals_on(int a, int ca, int side, Facet facet, int row0, const int* c0, const int* c1,
                                const int* lo, const int* bn, const int* ncell, int p, int nc,
                                const std::vector<double>& xyz, const int32_t* box, std::vector<int32_t>& qrow,
                                std::vector<int32_t>& qcol, std::vector<double>& qw) {
  const int b = a == 0 ? 1 : 0, c = a == 2 ? 1 : 2;  // the face's axes, b < c
  const int nq = p + 1;
  std::vector<double> gx(nq), gw(nq);
  gl_rule(nq, gx.data(), gw.data());
  const int64_t nvx = ncell[0] + 1, nvy = ncell[1] + 1;
  std::map<int, std::array<double, 6>> acc;  // local dof -> six integrals
  double meas = 0.0, xF[3] = {0.0, 0.0, 0.0}, scale = 1.0;
  // pass 0: the face measure and centroid; pass 1: the integrals
  auto sweep = [&](int pass) {
    for (int cc = c0[c]; cc < c1[c]; ++cc)
      for (int cb = c0[b]; cb < c1[b]; ++cb) {
        if (!facet(cb, cc)) continue;
        double V[2][2][3];
        for (int v = 0; v < 2; ++v)
          for (int u = 0; u < 2; ++u) {
            int I3[3];
            I3[a] = ca + side;
            I3[b] = cb + u;
            I3[c] = cc + v;
            const int64_t vid = I3[0] + nvx * (I3[1] + nvy * I3[2]);
            for (int d = 0; d < 3; ++d) V[u][v][d] = xyz[3 * vid + d];
          }
        for (int jt = 0; jt < nq; ++jt)
          for (int is = 0; is < nq; ++is) {
            const double s = gx[is], t = gx[jt];
            const double fs[2] = {0.5 * (1 - s), 0.5 * (1 + s)}, ft[2] = {0.5 * (1 - t), 0.5 * (1 + t)};
            double x[3], ds[3], dt[3];
            for (int d = 0; d < 3; ++d) {
              x[d] = ds[d] = dt[d] = 0.0;
              for (int v = 0; v < 2; ++v)
                for (int u = 0; u < 2; ++u) {
                  x[d] += fs[u] * ft[v] * V[u][v][d];
                  ds[d] += (u ? 0.5 : -0.5) * ft[v] * V[u][v][d];
                  dt[d] += fs[u] * (v ? 0.5 : -0.5) * V[u][v][d];
                }
            }
            const double nx = ds[1] * dt[2] - ds[2] * dt[1], ny = ds[2] * dt[0] - ds[0] * dt[2],
                         nz = ds[0] * dt[1] - ds[1] * dt[0];
            const double f = gw[is] * gw[jt] * std::sqrt(nx * nx + ny * ny + nz * nz);
            if (pass == 0) {
              meas += f;
              for (int d = 0; d < 3; ++d) xF[d] += f * x[d];
              continue;
            }
            // r_m[comp] at x (rotations about the centroid, scaled)
            const double X = (x[0] - xF[0]) * scale, Y = (x[1] - xF[1]) * scale, Z = (x[2] - xF[2]) * scale;
            const double r[6][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {Y, -X, 0}, {-Z, 0, X}, {0, Z, -Y}};
            for (int j = 0; j <= p; ++j)
              for (int i = 0; i <= p; ++i) {
                double li, lj, dl;
                lagrange_1d(p, i, s, li, dl);
                lagrange_1d(p, j, t, lj, dl);
                const double Nv = li * lj;
                if (Nv == 0.0) continue;
                int P3[3];
                P3[a] = p * (ca + side);
                P3[b] = p * cb + i;
                P3[c] = p * cc + j;
                const int64_t nb = (((int64_t)(P3[2] - lo[2]) * bn[1] + (P3[1] - lo[1])) * bn[0] + (P3[0] - lo[0])) * nc;
                for (int comp = 0; comp < nc; ++comp) {
                  const int ld = box[nb + comp];
                  if (ld < 0) continue;
                  auto& e = acc[ld];
                  for (int m = 0; m < 6; ++m) e[m] += Nv * r[m][comp] * f;
                }
              }
          }
      }
  };
  sweep(0);
  if (!(meas > 0.0)) return;
  for (int d = 0; d < 3; ++d) xF[d] /= meas;
  scale = 1.0 / std::sqrt(meas);
  sweep(1);
  for (int m = 0; m < 6; ++m)
    for (auto& kv : acc)
      if (kv.second[m] != 0.0) {
        qrow.push_back(row0 + m);
        qcol.push_back(kv.first);
        qw.push_back(kv.second[m] / meas);
      }
}

// The face object `key` of the box grid: all of the subdomain's cell faces on that plane.
static void face_functionals(uint64_t key, int row0, const std::vector<int32_t>* cuts, const int* c0, const int* c1,
                             const int* lo, const int* bn, const int* ncell, int p, int nc, const std::vector<double>& xyz,
                             const int32_t* box, std::vector<int32_t>& qrow, std::vector<int32_t>& qcol,
                             std::vector<double>& qw) {
  const int a = (int)((key >> 60) & 3);
  const int ia[3] = {(int)((key >> 40) & 0xFFFFF), (int)((key >> 20) & 0xFFFFF), (int)(key & 0xFFFFF)};
  const int plane = cuts[a][ia[a]];                  // cell index of the plane along a
  const int ca = plane == c0[a] ? c0[a] : c1[a] - 1;  // this subdomain's cells along a
  const int side = plane == c0[a] ? 0 : 1;
  face_functionals_on(a, ca, side, [](int, int) { return true; }, row0, c0, c1, lo, bn, ncell, p, nc, xyz, box, qrow,
                      qcol, qw);
}

static fg_status bddc_symbolic(fg_bddc* B) {
  fg_space* sp = B->sys->space;
  fg_mesh* me = sp->mesh;
  fg_ctx* ctx = me->ctx;
  const int p = sp->order, nc = sp->ncomp;
  const int64_t nlat = sp->nlat, nfree = sp->nfree;
  std::vector<int32_t> latdof(nlat * nc), row2vec(nfree > 0 ? nfree : 1);
  FG_CUDA_TRY(cudaMemcpyAsync(latdof.data(), sp->d_latdof, sizeof(int32_t) * latdof.size(), cudaMemcpyDeviceToHost,
                              ctx->stream));
  if (nfree > 0)
    FG_CUDA_TRY(cudaMemcpyAsync(row2vec.data(), sp->d_row2vec, sizeof(int32_t) * nfree, cudaMemcpyDeviceToHost,
                                ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  int ns[3];
  AxisInfo ax[3];
  for (int d = 0; d < 3; ++d) {
    ns[d] = (int)B->cuts[d].size() - 1;
    const int Ln = sp->Ln[d];
    ax[d].on_cut.assign(Ln, 0);
    ax[d].plane.assign(Ln, 0);
    ax[d].idx.assign(Ln, 0);
    ax[d].slab.assign(Ln, 0);
    for (int k = 0; k <= ns[d]; ++k) {
      int X = p * B->cuts[d][k];
      ax[d].plane[X] = 1;
      if (k > 0 && k < ns[d]) ax[d].on_cut[X] = 1;
    }
    int k = 0;
    for (int X = 0; X < Ln; ++X) {
      while (k + 1 < ns[d] && X >= p * B->cuts[d][k + 1]) ++k;
      // plane positions take the plane index, others the slab that contains them
      int pk = k;
      if (ax[d].plane[X]) {
        for (int q = 0; q <= ns[d]; ++q)
          if (p * B->cuts[d][q] == X) pk = q;
      }
      ax[d].idx[X] = pk;
      ax[d].slab[X] = k;
    }
  }
  B->nsub = ns[0] * ns[1] * ns[2];
  B->subs.assign(B->nsub, BSub());
  // physics-based partition: the subparts are the face-connected components of equal cell
  // coefficient within each subdomain, numbered in order of their first cell
  const bool pb = B->prm.use_subparts != 0;
  const int ncx = me->n[0], ncy = me->n[1], ncz = me->n[2];
  std::vector<int32_t> csub, sub_part;
  std::vector<double> subE;
  auto cell_part = [&](int i, int j, int k) {
    int q[3] = {i, j, k}, s3[3];
    for (int d = 0; d < 3; ++d) {
      s3[d] = 0;
      while (s3[d] + 1 < ns[d] && q[d] >= B->cuts[d][s3[d] + 1]) ++s3[d];
    }
    return s3[0] + ns[0] * (s3[1] + ns[1] * s3[2]);
  };
  if (pb) {
    const int64_t ncell = (int64_t)ncx * ncy * ncz;
    std::vector<double> coef(ncell, B->sys->integ.coef_const);
    if (B->sys->d_coef) {
      FG_CUDA_TRY(cudaMemcpyAsync(coef.data(), B->sys->d_coef, sizeof(double) * ncell, cudaMemcpyDeviceToHost,
                                  ctx->stream));
      FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    }
    std::vector<int32_t> cpart(ncell);
    for (int k = 0; k < ncz; ++k)
      for (int j = 0; j < ncy; ++j)
        for (int i = 0; i < ncx; ++i) cpart[i + (int64_t)ncx * (j + (int64_t)ncy * k)] = cell_part(i, j, k);
    csub.assign(ncell, -1);
    std::vector<int64_t> stack;
    for (int64_t c0 = 0; c0 < ncell; ++c0) {
      if (csub[c0] >= 0) continue;
      const int32_t id = (int32_t)subE.size();
      subE.push_back(coef[c0]);
      sub_part.push_back(cpart[c0]);
      csub[c0] = id;
      stack.assign(1, c0);
      while (!stack.empty()) {
        const int64_t c = stack.back();
        stack.pop_back();
        const int i = (int)(c % ncx), j = (int)((c / ncx) % ncy), k = (int)(c / ((int64_t)ncx * ncy));
        const int nbr[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j - 1, k}, {i, j + 1, k}, {i, j, k - 1}, {i, j, k + 1}};
        for (auto& q : nbr) {
          if (q[0] < 0 || q[0] >= ncx || q[1] < 0 || q[1] >= ncy || q[2] < 0 || q[2] >= ncz) continue;
          const int64_t cq = q[0] + (int64_t)ncx * (q[1] + (int64_t)ncy * q[2]);
          if (csub[cq] < 0 && cpart[cq] == cpart[c0] && coef[cq] == coef[c0]) {
            csub[cq] = id;
            stack.push_back(cq);
          }
        }
      }
    }
  }
  // subparts of the cells around lattice node (X, Y, Z), sorted and unique
  auto node_subparts = [&](int X, int Y, int Z, int* out) {
    int lo3[3], hi3[3];
    const int P3[3] = {X, Y, Z}, nn3[3] = {ncx, ncy, ncz};
    for (int d = 0; d < 3; ++d) {
      if (P3[d] % p == 0) {
        lo3[d] = std::max(0, P3[d] / p - 1);
        hi3[d] = std::min(nn3[d] - 1, P3[d] / p);
      } else {
        lo3[d] = hi3[d] = P3[d] / p;
      }
    }
    int cnt = 0;
    for (int k = lo3[2]; k <= hi3[2]; ++k)
      for (int j = lo3[1]; j <= hi3[1]; ++j)
        for (int i = lo3[0]; i <= hi3[0]; ++i) {
          const int32_t sid = csub[i + (int64_t)ncx * (j + (int64_t)ncy * k)];
          bool seen = false;
          for (int t = 0; t < cnt; ++t) seen |= out[t] == sid;
          if (!seen) out[cnt++] = sid;
        }
    std::sort(out, out + cnt);
    return cnt;
  };
  std::vector<double> h_w;  // FG_BDDC_WEIGHT_SUBPART: interface weights, computed here
  std::map<std::pair<uint64_t, int>, int32_t> coarse_id;
  std::vector<int64_t> iface_of(nfree > 0 ? nfree : 1, -1);
  std::vector<int32_t> ivec;
  std::vector<std::pair<int64_t, int64_t>> ipairs, cpairs;
  std::vector<std::pair<int32_t, int32_t>> kpairs_ij;  // (I, J) per K_Pi entry in pool order
  std::vector<int32_t> h_loc, h_pc, h_box, h_qrow, h_qcol;
  std::vector<double> h_qw, h_cv;
  int64_t aoff = 0, foff = 0, roff = 0, loff = 0, woff = 0, eoff = 0, poff = 0, koff = 0, goff = 0, boff = 0,
          cvoff = 0;
  const bool rigid = B->prm.coarse_handler == FG_BDDC_HANDLER_ELASTICITY;
  std::vector<double> xyz;  // vertex coordinates (elasticity handler's face integrals)
  if (rigid) {
    const int64_t nv = (int64_t)(me->n[0] + 1) * (me->n[1] + 1) * (me->n[2] + 1);
    xyz.resize(3 * nv);
    FG_CUDA_TRY(cudaMemcpyAsync(xyz.data(), me->d_coords, sizeof(double) * xyz.size(), cudaMemcpyDeviceToHost,
                                ctx->stream));
    FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  }
  auto enc = [](int type, int a, int i0, int i1, int i2) -> uint64_t {
    return ((uint64_t)type << 62) | ((uint64_t)a << 60) | ((uint64_t)i0 << 40) | ((uint64_t)i1 << 20) | (uint64_t)i2;
  };
  struct LD {
    int64_t L;
    int comp;
    int32_t gid;
    int cls;  // 0 I, 1 E, 2 V
    uint64_t key;
    double w;  // subpart weight (FG_BDDC_WEIGHT_SUBPART)
  };
  std::vector<LD> dofs;
  for (int sk = 0; sk < ns[2]; ++sk)
    for (int sj = 0; sj < ns[1]; ++sj)
      for (int si = 0; si < ns[0]; ++si) {
        const int s = si + ns[0] * (sj + ns[1] * sk);
        BSub& S = B->subs[s];
        const int sc[3] = {si, sj, sk};
        int lo[3], hi[3], bn[3];
        for (int d = 0; d < 3; ++d) {
          S.c0[d] = B->cuts[d][sc[d]];
          S.c1[d] = B->cuts[d][sc[d] + 1];
          lo[d] = p * S.c0[d];
          hi[d] = p * S.c1[d];
          bn[d] = hi[d] - lo[d] + 1;
        }
        dofs.clear();
        for (int Z = lo[2]; Z <= hi[2]; ++Z)
          for (int Y = lo[1]; Y <= hi[1]; ++Y)
            for (int X = lo[0]; X <= hi[0]; ++X) {
              const int P3[3] = {X, Y, Z};
              const int64_t L = X + (int64_t)sp->Ln[0] * (Y + (int64_t)sp->Ln[1] * Z);
              int ncut = 0, npl = 0;
              for (int d = 0; d < 3; ++d) {
                ncut += ax[d].on_cut[P3[d]];
                npl += ax[d].plane[P3[d]];
              }
              int cls = 0;
              uint64_t key = 0;
              double wsub = 0.0;
              if (ncut > 0 && pb) {
                // objects by the subparts around: a face object holds the dofs whose cells
                // belong to exactly two subparts (one per side of one cut plane); the rest
                // are edge or vertex objects, primal vertices only as asked
                int sg[8];
                const int nsg = node_subparts(X, Y, Z, sg);
                double tot = 0.0, own = 0.0;
                for (int t = 0; t < nsg; ++t) {
                  tot += subE[sg[t]];
                  if (sub_part[sg[t]] == s) own += subE[sg[t]];
                }
                wsub = tot > 0.0 ? own / tot : 0.0;
                if (npl == 3 && B->prm.use_vertices) {
                  cls = 2;
                  key = enc(0, 0, X, Y, Z);
                } else if (ncut == 1 && nsg == 2) {
                  cls = 1;
                  int a = 0;
                  for (int d = 0; d < 3; ++d)
                    if (ax[d].on_cut[P3[d]]) a = d;
                  key = enc(2, a, sg[0], sg[1], 0);
                } else {
                  cls = 1;
                  key = enc(1, 0, 0, 0, 0);  // no constraint (edges are off with subparts)
                }
              } else if (ncut > 0) {
                if (npl == 3) {
                  // a vertex: primal (V), or with use_vertices = 0 an interface dof without a
                  // coarse dof of its own
                  cls = B->prm.use_vertices ? 2 : 1;
                  key = enc(0, 0, X, Y, Z);
                } else if (ncut == 2) {
                  cls = 1;
                  int a = 0;
                  for (int d = 0; d < 3; ++d)
                    if (!ax[d].plane[P3[d]]) a = d;
                  key = enc(1, a, ax[0].idx[X], ax[1].idx[Y], ax[2].idx[Z]);
                } else {
                  // a face: the cut plane and the slabs along the other two axes; points on the
                  // domain boundary join the face (the same two subdomains share them)
                  cls = 1;
                  int a = 0;
                  for (int d = 0; d < 3; ++d)
                    if (ax[d].on_cut[P3[d]]) a = d;
                  int id3[3];
                  for (int d = 0; d < 3; ++d) id3[d] = d == a ? ax[d].idx[P3[d]] : ax[d].slab[P3[d]];
                  key = enc(2, a, id3[0], id3[1], id3[2]);
                }
              }
              for (int c = 0; c < nc; ++c) {
                int32_t ld = latdof[L * nc + c];
                if (ld <= 0) continue;
                dofs.push_back({L, c, ld - 1, cls, key, wsub});
              }
            }
        // local order I | E | V (stable)
        std::stable_sort(dofs.begin(), dofs.end(), [](const LD& a, const LD& b) { return a.cls < b.cls; });
        int nI = 0, nE = 0, nV = 0;
        for (auto& d : dofs) (d.cls == 0 ? nI : d.cls == 1 ? nE : nV)++;
        const int m = nI + nE + nV;
        // box map
        const int64_t nbox = (int64_t)bn[0] * bn[1] * bn[2] * nc;
        const size_t b0 = h_box.size();
        h_box.resize(b0 + nbox, -1);
        for (int i = 0; i < m; ++i) {
          const LD& d = dofs[i];
          int X = (int)(d.L % sp->Ln[0]), Y = (int)((d.L / sp->Ln[0]) % sp->Ln[1]),
              Z = (int)(d.L / ((int64_t)sp->Ln[0] * sp->Ln[1]));
          int64_t bidx = (((int64_t)(Z - lo[2]) * bn[1] + (Y - lo[1])) * bn[0] + (X - lo[0])) * nc + d.comp;
          h_box[b0 + bidx] = i;
          h_loc.push_back(row2vec[d.gid]);
        }
        // constraints over E dofs
        std::map<std::pair<uint64_t, int>, int> lcon;
        std::vector<int> lcnt;
        std::vector<std::pair<uint64_t, int>> lkeys;
        std::vector<int> econ(nE, -1);
        std::vector<uint64_t> rfaces;  // elasticity handler: faces in order of first E dof
        for (int k = 0; k < nE; ++k) {
          const LD& d = dofs[nI + k];
          int type = (int)(d.key >> 62);
          bool use = (type == 1 && B->prm.use_edges) || (type == 2 && B->prm.use_faces);
          if (!use) continue;
          if (rigid) {  // faces only (edges rejected at creation): six functionals, in mode order
            if (lcon.find(std::make_pair(d.key, 0)) == lcon.end()) {
              for (int mode = 0; mode < 6; ++mode) {
                lcon[std::make_pair(d.key, mode)] = (int)lcnt.size();
                lcnt.push_back(0);
                lkeys.push_back(std::make_pair(d.key, mode));
              }
              rfaces.push_back(d.key);
            }
            continue;
          }
          auto kc = std::make_pair(d.key, d.comp);
          auto it = lcon.find(kc);
          int ci;
          if (it == lcon.end()) {
            ci = (int)lcnt.size();
            lcon[kc] = ci;
            lcnt.push_back(0);
            lkeys.push_back(kc);
          } else {
            ci = it->second;
          }
          econ[k] = ci;
          lcnt[ci]++;
        }
        const int ne = (int)lcnt.size();
        if (ne > kMaxNe || nV > kMaxNv) {
          set_error("BDDC: subdomain %d has %d edge/face constraints and %d vertex dofs (limits %d, %d)", s, ne, nV,
                    kMaxNe, kMaxNv);
          return FG_ERR_UNSUPPORTED;
        }
        // constraint entries (row, local column, weight) and C_eV
        const int64_t q0 = (int64_t)h_qrow.size();
        if (!rigid) {
          for (int k = 0; k < nE; ++k)
            if (econ[k] >= 0) {
              h_qrow.push_back(econ[k]);
              h_qcol.push_back(nI + k);
              h_qw.push_back(1.0 / (double)lcnt[econ[k]]);
            }
        } else {
          for (size_t f = 0; f < rfaces.size(); ++f) {
            if (!pb) {
              face_functionals(rfaces[f], (int)(6 * f), B->cuts, S.c0, S.c1, lo, bn, me->n, p, nc, xyz,
                               h_box.data() + b0, h_qrow, h_qcol, h_qw);
              continue;
            }
            // a subpart face object: the facets between its two subparts
            const uint64_t key = rfaces[f];
            const int a = (int)((key >> 60) & 3);
            const int s1 = (int)((key >> 40) & 0xFFFFF), s2 = (int)((key >> 20) & 0xFFFFF);
            const int other = sub_part[s1] == s ? sub_part[s2] : sub_part[s1];
            const int o3[3] = {other % ns[0], (other / ns[0]) % ns[1], other / (ns[0] * ns[1])};
            const int side = o3[a] < sc[a] ? 0 : 1;
            const int ca = side == 0 ? S.c0[a] : S.c1[a] - 1;
            const int b = a == 0 ? 1 : 0, c = a == 2 ? 1 : 2;
            auto facet = [&](int cb, int cc) {
              int q[3], r3[3];
              q[a] = ca;
              q[b] = cb;
              q[c] = cc;
              r3[0] = q[0];
              r3[1] = q[1];
              r3[2] = q[2];
              r3[a] = side == 0 ? ca - 1 : ca + 1;
              const int32_t u = csub[q[0] + (int64_t)ncx * (q[1] + (int64_t)ncy * q[2])];
              const int32_t v = csub[r3[0] + (int64_t)ncx * (r3[1] + (int64_t)ncy * r3[2])];
              return (u == s1 && v == s2) || (u == s2 && v == s1);
            };
            face_functionals_on(a, ca, side, facet, (int)(6 * f), S.c0, S.c1, lo, bn, me->n, p, nc, xyz,
                                h_box.data() + b0, h_qrow, h_qcol, h_qw);
          }
        }
        {  // entries grouped by constraint row (the augmentation takes them row by row)
          std::vector<int64_t> ord((int64_t)h_qrow.size() - q0);
          std::iota(ord.begin(), ord.end(), q0);
          std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return h_qrow[a] < h_qrow[b]; });
          std::vector<int32_t> r2(ord.size()), c2(ord.size());
          std::vector<double> w2(ord.size());
          for (size_t t = 0; t < ord.size(); ++t) {
            r2[t] = h_qrow[ord[t]];
            c2[t] = h_qcol[ord[t]];
            w2[t] = h_qw[ord[t]];
          }
          std::copy(r2.begin(), r2.end(), h_qrow.begin() + q0);
          std::copy(c2.begin(), c2.end(), h_qcol.begin() + q0);
          std::copy(w2.begin(), w2.end(), h_qw.begin() + q0);
        }
        S.qoff = q0;
        S.nq = (int)((int64_t)h_qrow.size() - q0);
        S.cvoff = cvoff;
        h_cv.resize(cvoff + (int64_t)ne * nV, 0.0);
        for (int64_t t = q0; t < (int64_t)h_qrow.size(); ++t)
          if (h_qcol[t] >= nI + nE) h_cv[cvoff + (int64_t)h_qrow[t] * nV + (h_qcol[t] - nI - nE)] = h_qw[t];
        cvoff += (int64_t)ne * nV;
        // local coarse dofs [V | e] -> global coarse ids
        std::vector<int32_t> cg;
        for (int k = 0; k < nV; ++k) {
          const LD& d = dofs[nI + nE + k];
          auto kc = std::make_pair(d.key, d.comp);
          auto it = coarse_id.find(kc);
          int32_t id;
          if (it == coarse_id.end()) {
            id = (int32_t)coarse_id.size();
            coarse_id[kc] = id;
          } else {
            id = it->second;
          }
          cg.push_back(id);
        }
        for (int e = 0; e < ne; ++e) {
          auto it = coarse_id.find(lkeys[e]);
          int32_t id;
          if (it == coarse_id.end()) {
            id = (int32_t)coarse_id.size();
            coarse_id[lkeys[e]] = id;
          } else {
            id = it->second;
          }
          cg.push_back(id);
        }
        const int nP = nV + ne;
        // interface contributions in subdomain order
        for (int k = 0; k < nE + nV; ++k) {
          h_w.push_back(dofs[nI + k].w);
          int32_t gid = dofs[nI + k].gid;
          if (iface_of[gid] < 0) {
            iface_of[gid] = (int64_t)ivec.size();
            ivec.push_back(row2vec[gid]);
          }
          ipairs.push_back({iface_of[gid], woff + k});
        }
        for (int j = 0; j < nP; ++j) {
          h_pc.push_back(cg[j]);
          cpairs.push_back({cg[j], poff + j});
        }
        for (int i = 0; i < nP; ++i)
          for (int j = 0; j < nP; ++j) kpairs_ij.push_back({cg[i], cg[j]});
        S.N = m + ne;
        S.m = m;
        S.nI = nI;
        S.nE = nE;
        S.nV = nV;
        S.ne = ne;
        S.nr = nI + nE;
        S.nP = nP;
        if (S.N > kMaxLocal) {
          set_error("BDDC: subdomain %d has %d local dofs (dense limit %d)", s, S.N, kMaxLocal);
          return FG_ERR_UNSUPPORTED;
        }
        S.aoff = aoff;
        aoff += (int64_t)S.N * S.N;
        S.foff = foff;
        foff += (int64_t)S.nr * S.nr;
        S.roff = roff;
        roff += (int64_t)nP * S.nr;
        S.loff = loff;
        loff += m;
        S.woff = woff;
        woff += nE + nV;
        S.eoff = eoff;
        eoff += nE;
        S.poff = poff;
        poff += nP;
        S.koff = koff;
        koff += (int64_t)nP * nP;
        S.goff = goff;
        goff += (int64_t)ne * ne + (int64_t)ne * nV;
        S.boff = boff;
        boff += nbox;
        B->factor_flops += ((double)S.N * S.N * S.N - (double)(S.N - S.nr) * (S.N - S.nr) * (S.N - S.nr)) / 3.0;
        B->maxN = std::max(B->maxN, S.N);
        B->maxnr = std::max(B->maxnr, S.nr);
        B->maxnI = std::max(B->maxnI, S.nI);
      }
  B->nA = aoff;
  B->nF = foff;
  B->nR = roff;
  B->nL = loff;
  B->nW = woff;
  B->nE = eoff;
  B->nP = poff;
  B->nK = koff;
  B->nG = goff;
  B->nB = boff;
  B->nIface = (int64_t)ivec.size();
  B->nC = (int64_t)coarse_id.size();
  if (B->nC > kMaxCoarse) {
    set_error("BDDC: %lld coarse dofs (dense coarse solver limit %d)", (long long)B->nC, kMaxCoarse);
    return FG_ERR_UNSUPPORTED;
  }
  // memory check before the large pools
  const int64_t nvec = sp->nvec;
  const uint64_t need = 8ull * B->nA + 4ull * B->nF + 12ull * B->nR + 8ull * (uint64_t)(2 * B->nC) * (2 * B->nC) +
                        12ull * B->nC * B->nC + 12ull * 4 * nvec + 8ull * 7 * nvec;
  if (ctx->budget && ctx->in_use + need > ctx->budget) {
    set_error("BDDC: dense local and coarse matrices need %.2f GB, %.2f GB left in the HBM budget", need / 1e9,
              (ctx->budget - ctx->in_use) / 1e9);
    return FG_ERR_OOM;
  }
  // CSR of the gathers
  std::vector<int64_t> iptr, isrc, cptr, csrc;
  pairs_to_csr(B->nIface, ipairs, iptr, isrc);
  pairs_to_csr(B->nC, cpairs, cptr, csrc);
  // coarse matrix: unique (I, J) pairs (I >= J, lower of the 2nC column-major block), sources in subdomain order
  std::vector<std::pair<int64_t, int64_t>> kp;
  kp.reserve(kpairs_ij.size());
  for (size_t t = 0; t < kpairs_ij.size(); ++t) {
    int64_t I = kpairs_ij[t].first, J = kpairs_ij[t].second;
    if (I >= J) kp.push_back({I * B->nC + J, (int64_t)t});
  }
  std::stable_sort(kp.begin(), kp.end(),
                   [](const std::pair<int64_t, int64_t>& a, const std::pair<int64_t, int64_t>& b) { return a.first < b.first; });
  std::vector<int64_t> kdst, kptr, ksrc;
  for (size_t t = 0; t < kp.size(); ++t) {
    if (t == 0 || kp[t].first != kp[t - 1].first) {
      kptr.push_back((int64_t)t);
      int64_t I = kp[t].first / B->nC, J = kp[t].first % B->nC;
      kdst.push_back(I + J * 2 * B->nC);
    }
    ksrc.push_back(kp[t].second);
  }
  kptr.push_back((int64_t)kp.size());
  B->nKpair = (int64_t)kdst.size();
  // uploads
  FG_TRY(upload(B, &B->d_subs, B->subs));
  {
    std::vector<int32_t> ord(B->nsub);
    for (int i = 0; i < B->nsub; ++i) ord[i] = i;
    auto work = [&](int i) {
      const double N = B->subs[i].N, r = N - B->subs[i].nr;
      return N * N * N - r * r * r;
    };
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return work(a) > work(b); });
    FG_TRY(upload(B, &B->dOrder, ord));
    // stepped over all subdomains by default (measured on GB300 at 32^3 Q2 elasticity, 512
    // subdomains: 1.71 s vs 1.93 s for one CTA per subdomain with even sizes, 2.18 s vs 4.03 s
    // with +-30 % sizes, where the largest subdomain alone sets the one-CTA finishing time);
    // FG_BDDC_STEPPED=0 selects the single launch with one CTA per subdomain
    const char* e = std::getenv("FG_BDDC_STEPPED");
    B->stepped = !(e && e[0] == '0');
  }
  FG_TRY(upload(B, &B->dLoc, h_loc));
  FG_TRY(upload(B, &B->dQrow, h_qrow));
  FG_TRY(upload(B, &B->dQcol, h_qcol));
  FG_TRY(upload(B, &B->dQw, h_qw));
  FG_TRY(upload(B, &B->dCv, h_cv));
  {
    std::vector<float> cv32(h_cv.begin(), h_cv.end());
    FG_TRY(upload(B, &B->dCv32, cv32));
  }
  FG_TRY(upload(B, &B->dPc, h_pc));
  FG_TRY(upload(B, &B->dBox, h_box));
  FG_TRY(upload(B, &B->dIptr, iptr));
  FG_TRY(upload(B, &B->dIsrc, isrc));
  FG_TRY(upload(B, &B->dIvec, ivec));
  FG_TRY(upload(B, &B->dCptr, cptr));
  FG_TRY(upload(B, &B->dCsrc, csrc));
  FG_TRY(upload(B, &B->dKdst, kdst));
  FG_TRY(upload(B, &B->dKptr, kptr));
  FG_TRY(upload(B, &B->dKsrc, ksrc));
  // pools
  FG_TRY(balloc_n(B, &B->dA, B->nA));
  FG_TRY(balloc_n(B, &B->dF, B->nF));
  FG_TRY(balloc_n(B, &B->dR, B->nR));
  FG_TRY(balloc_n(B, &B->dR32, B->nR));
  if (B->prm.weighting == FG_BDDC_WEIGHT_SUBPART) FG_TRY(upload(B, &B->dW, h_w));
  else FG_TRY(balloc_n(B, &B->dW, B->nW));
  FG_TRY(balloc_n(B, &B->dDiag, B->nW));
  FG_TRY(balloc_n(B, &B->dC, B->nW));
  FG_TRY(balloc_n(B, &B->dC32, B->nW));
  FG_TRY(balloc_n(B, &B->dZ, B->nE));
  FG_TRY(balloc_n(B, &B->dZ32, B->nE));
  FG_TRY(balloc_n(B, &B->dFp, B->nP));
  FG_TRY(balloc_n(B, &B->dFp32, B->nP));
  FG_TRY(balloc_n(B, &B->dKp, B->nK));
  if (!B->prm.use_vertices) FG_TRY(balloc_n(B, &B->dRho, std::max<int64_t>(B->nP, 1), true));
  FG_TRY(balloc_n(B, &B->dG, B->nG));
  FG_TRY(balloc_n(B, &B->dG32, B->nG));
  FG_TRY(balloc_n(B, &B->dKc, 4 * B->nC * B->nC));
  FG_TRY(balloc_n(B, &B->dKinv, B->nC * B->nC));
  FG_TRY(balloc_n(B, &B->dKinv32, B->nC * B->nC));
  FG_TRY(balloc_n(B, &B->dFc, B->nC));
  FG_TRY(balloc_n(B, &B->dUc, B->nC));
  FG_TRY(balloc_n(B, &B->dFc32, B->nC));
  FG_TRY(balloc_n(B, &B->dUc32, B->nC));
  FG_TRY(balloc_n(B, &B->dU0, nvec, true));
  FG_TRY(balloc_n(B, &B->dV, nvec, true));
  FG_TRY(balloc_n(B, &B->dQ, nvec, true));
  FG_TRY(balloc_n(B, &B->dT, nvec, true));
  FG_TRY(balloc_n(B, &B->dU032, nvec, true));
  FG_TRY(balloc_n(B, &B->dV32, nvec, true));
  FG_TRY(balloc_n(B, &B->dQ32, nvec, true));
  FG_TRY(balloc_n(B, &B->dT32, nvec, true));
  FG_TRY(balloc_n(B, &B->dErr, 1, true));
  B->nred = std::max(1, 2 * ctx->sm_count);
  FG_TRY(balloc_n(B, &B->dPart, 2 * B->nred));
  // largest number of cell dofs for the assembly kernel's shared map
  B->maxnd = sp->tab.nd;
  if (B->maxnd > 3 * FG_MAX_NN) {
    set_error("BDDC: %d dofs per cell", B->maxnd);
    return FG_ERR_UNSUPPORTED;
  }
  return FG_OK;
}

static fg_status check_err(fg_bddc* B, const char* what) {
  fg_ctx* ctx = B->sys->space->mesh->ctx;
  int h = 0;
  FG_CUDA_TRY(cudaMemcpyAsync(&h, B->dErr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (h) {
    FG_CUDA_TRY(cudaMemsetAsync(B->dErr, 0, sizeof(int), ctx->stream));
    set_error("BDDC: %s is not positive definite (subdomain %d)", what, h - 1);
    return FG_ERR_NUMERIC;
  }
  return FG_OK;
}

// Partial Cholesky of the first ncols columns of one N x N matrix, many CTAs per step.
// Rows from zrow on may be a unit block (row zrow + i holds a 1 in column i and zeros before
// it, as in [[K, I], [I, 0]]): such a row's panel entries stay zero until the panel reaches
// column i, so at panel j0 the rows from zrow + j0 + nb on are skipped by the solve and the
// trailing update (exactly: their contributions are zero).  zrow = N: no unit block.
// With work (ozaki_workspace_bytes(N, N, 128, true) bytes + an int), the factorisation is
// blocked by 128 columns: each 128-column panel is factored by 32-column steps whose
// updates stay inside the panel, and the trailing matrix gets one rank-128 update on the
// tensor cores (FP64 emulated by digit slicing, fg_ozaki.cu) instead of four rank-32
// updates on the FP64 pipe.
static fg_status chol_partial_grid(fg_ctx* ctx, double* A, int64_t lda, int N, int ncols, int zrow, int* err,
                                   void* work = nullptr) {
  cudaStream_t st = ctx->stream;
  const int NB = work ? 128 : ncols;
  for (int J0 = 0; J0 < ncols; J0 += NB) {
    const int J1 = std::min(J0 + NB, ncols);
    for (int j0 = J0; j0 < J1; j0 += 32) {
      const int nb = std::min(32, J1 - j0);
      k_chol_diag1<<<1, 32, 0, st>>>(A, lda, j0, nb, err);
      const int Neff = (int)std::min<int64_t>(N, (int64_t)zrow + j0 + nb);
      const int rows = Neff - j0 - nb;
      if (rows > 0) {
        k_chol_trsm1<<<nblk(rows, 256), 256, 0, st>>>(A, lda, Neff, j0, nb);
        const int nt = (rows + 63) / 64;
        if (work) {
          const int ntc = (J1 - (j0 + nb) + 63) / 64;  // columns left inside the panel
          if (ntc > 0) {
            k_chol_syrk_panel<<<dim3((unsigned)nt, (unsigned)ntc), 256, 0, st>>>(A, lda, Neff, j0, nb, J1);
            ctx->launches += 1;
          }
        } else {
          k_chol_syrk1<<<(unsigned)((int64_t)nt * (nt + 1) / 2), 256, 0, st>>>(A, lda, Neff, j0, nb, nt);
          ctx->launches += 1;
        }
        ctx->launches += 1;
      }
      ctx->launches += 1;
    }
    if (work) {
      // A[J1:Ne, J1:Ne] -= P P^T (lower), P = A[J1:Ne, J0:J1]
      const int Ne = (int)std::min<int64_t>(N, (int64_t)zrow + J1);
      const int rows = Ne - J1;
      if (rows > 0) {
        double* P = A + J1 + (int64_t)J0 * lda;
        double* Ct = A + J1 + (int64_t)J1 * lda;
        int* oz_err = (int*)((uint8_t*)work + ozaki_workspace_bytes(N, N, 128, true));
        FG_TRY(ozaki_gemm_nt(ctx, st, rows, rows, J1 - J0, -1.0, P, 1, lda, nullptr, 0, 0, 1.0, Ct, 1, lda, true,
                             work, oz_err));
      }
    }
  }
  FG_CUDA_TRY(cudaGetLastError());
  return FG_OK;
}

static fg_status bddc_numeric(fg_bddc* B) {
  fg_system* sys = B->sys;
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  cudaStream_t st = ctx->stream;
  const int ns = B->nsub;
  FG_CUDA_TRY(cudaMemsetAsync(B->dA, 0, sizeof(double) * (size_t)std::max<int64_t>(B->nA, 1), st));
  k_bddc_assemble<<<ns, 256, 0, st>>>(B->d_subs, sys->d_elmat, sp->mesh->n[0], sp->mesh->n[1], sp->order, sp->tab.nn,
                                      sp->tab.nd, sp->ncomp, B->dBox, B->dQrow, B->dQcol, B->dQw, B->dA,
                                      B->dDiag);
  if (B->dRho) {
    k_bddc_augment<<<ns, 256, 0, st>>>(B->d_subs, B->dQrow, B->dQcol, B->dQw, B->dA, B->dRho);
    ctx->launches += 1;
  }
  if (B->nIface > 0 && B->prm.weighting != FG_BDDC_WEIGHT_SUBPART)
    k_bddc_weights<<<nblk(B->nIface, 256), 256, 0, st>>>(B->nIface, B->dIptr, B->dIsrc, B->dDiag,
                                                         B->prm.weighting == FG_BDDC_WEIGHT_STIFFNESS, B->dW);
  cudaEvent_t ev[4];
  for (auto& e : ev) FG_CUDA_TRY(cudaEventCreate(&e));
  FG_CUDA_TRY(cudaEventRecord(ev[0], st));
  // subdomain trailing updates on the tensor cores (FP64 emulated, fg_ozaki.cu), blocked by
  // 128 columns, unless FG_BDDC_EMULATED_FP64=0
  const char* ee = std::getenv("FG_BDDC_EMULATED_FP64");
  const bool emulate = !(ee && ee[0] == '0');
  B->local_emulated = false;
  if (B->stepped && emulate) {
    auto panel_items = [&](int J0) {
      std::vector<OzSyrk> items;
      for (const BSub& S : B->subs) {
        if (J0 >= S.nr) continue;
        const int J1 = std::min(J0 + 128, S.nr);
        if (S.N - J1 <= 0) continue;
        double* As = B->dA + S.aoff;
        items.push_back(OzSyrk{As + J1 + (int64_t)J0 * S.N, As + J1 + (int64_t)J1 * S.N, (int64_t)S.N, S.N - J1,
                               J1 - J0});
      }
      return items;
    };
    const size_t wbytes = ozaki_syrk_batch_bytes(panel_items(0));
    void* work = nullptr;
    FG_TRY(dev_alloc(ctx, &work, wbytes + sizeof(int)));
    int* oz_err = (int*)((uint8_t*)work + wbytes);
    fg_status ls = FG_OK;
    cudaError_t ce = cudaMemsetAsync(oz_err, 0, sizeof(int), st);
    for (int J0 = 0; J0 < B->maxnr && ls == FG_OK && ce == cudaSuccess; J0 += 128) {
      for (int j0 = J0; j0 < std::min(J0 + 128, B->maxnr); j0 += 32) {
        k_bstep_diag<<<ns, 32, 0, st>>>(B->d_subs, B->dA, j0, B->dErr);
        const int rem = B->maxN - j0 - 1;
        if (rem > 0) {
          k_bstep_trsm<<<dim3(nblk(rem, 256), ns), 256, 0, st>>>(B->d_subs, B->dA, j0);
          const int nt = (rem + 63) / 64;
          const int ntc = std::max(0, (J0 + 128 - (j0 + 32) + 63) / 64);  // column tiles left in the panel
          if (ntc > 0) {
            k_bstep_syrk_panel<<<dim3((unsigned)nt, (unsigned)ntc, ns), 256, 0, st>>>(B->d_subs, B->dA, j0, J0 + 128);
            ctx->launches += 1;
          }
          ctx->launches += 1;
        }
        ctx->launches += 1;
      }
      ls = ozaki_syrk_batch(ctx, st, panel_items(J0), work, wbytes, oz_err);
    }
    int h_oz = 0;
    if (ls == FG_OK && ce == cudaSuccess) ce = cudaMemcpyAsync(&h_oz, oz_err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (ls == FG_OK && ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    dev_free(ctx, work);
    if (ls != FG_OK) {
      for (auto& e : ev) cudaEventDestroy(e);
      return ls;
    }
    if (ce != cudaSuccess) {
      for (auto& e : ev) cudaEventDestroy(e);
      set_error("BDDC factorisation: %s", cudaGetErrorString(ce));
      return FG_ERR_CUDA;
    }
    if (h_oz) {
      for (auto& e : ev) cudaEventDestroy(e);
      set_error("BDDC: a bounded tensor-core wait ran out in the subdomain factorisation");
      return (fg_status)h_oz;
    }
    B->local_emulated = true;
  } else if (B->stepped) {
    for (int j0 = 0; j0 < B->maxnr; j0 += 32) {
      k_bstep_diag<<<ns, 32, 0, st>>>(B->d_subs, B->dA, j0, B->dErr);
      const int rem = B->maxN - j0 - 1;
      if (rem > 0) {
        k_bstep_trsm<<<dim3(nblk(rem, 256), ns), 256, 0, st>>>(B->d_subs, B->dA, j0);
        const int nt = (rem + 63) / 64;
        k_bstep_syrk<<<dim3((unsigned)((int64_t)nt * (nt + 1) / 2), ns), 256, 0, st>>>(B->d_subs, B->dA, j0);
        ctx->launches += 2;
      }
      ctx->launches += 1;
    }
  } else {
    k_bddc_potrf<<<ns, 256, 0, st>>>(B->d_subs, B->dOrder, B->dA, B->dErr);
  }
  FG_CUDA_TRY(cudaEventRecord(ev[1], st));
  ctx->launches += 3;
  FG_CUDA_TRY(cudaGetLastError());
  fg_status sf = check_err(B, "a subdomain matrix with its vertex dofs removed");
  if (sf != FG_OK) {
    for (auto& e : ev) cudaEventDestroy(e);
    return sf;
  }
  float fms = 0.f;
  cudaEventElapsedTime(&fms, ev[0], ev[1]);
  B->factor_ms = fms;
  FG_CUDA_TRY(cudaFuncSetAttribute((const void*)k_bddc_coarse_local, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)kCoarseLocalSmem));
  k_bddc_coarse_local<<<ns, 128, kCoarseLocalSmem, st>>>(B->d_subs, B->dA, B->dKp, B->dG, B->dG32, B->dRho,
                                                          B->dErr);
  k_bddc_panels<<<ns, 256, 0, st>>>(B->d_subs, B->dA, B->dF, B->dR, B->dR32);
  ctx->launches += 2;
  FG_CUDA_TRY(cudaGetLastError());
  FG_TRY(check_err(B, "an edge/face constraint block"));
  const int64_t nC = B->nC;
  FG_CUDA_TRY(cudaEventRecord(ev[2], st));
  if (nC > 0) {
    FG_CUDA_TRY(cudaMemsetAsync(B->dKc, 0, sizeof(double) * 4 * nC * nC, st));
    k_seg_sum<<<nblk(B->nKpair, 256), 256, 0, st>>>(B->nKpair, B->dKptr, B->dKsrc, B->dKdst, B->dKp, B->dKc);
    k_coarse_identity<<<nblk(nC, 256), 256, 0, st>>>(nC, B->dKc);
    ctx->launches += 2;
    // coarse matrices of 1024 dofs and more: trailing updates on the tensor cores (FP64
    // emulated), unless FG_BDDC_EMULATED_FP64=0
    void* work = nullptr;
    const size_t wbytes = ozaki_workspace_bytes(2 * nC, 2 * nC, 128, true);
    if (nC >= 1024 && emulate) {
      FG_TRY(dev_alloc(ctx, &work, wbytes + sizeof(int)));
      FG_CUDA_TRY(cudaMemsetAsync((uint8_t*)work + wbytes, 0, sizeof(int), st));
    }
    fg_status cs = chol_partial_grid(ctx, B->dKc, 2 * nC, (int)(2 * nC), (int)nC, (int)nC, B->dErr, work);
    int oz_err = 0;
    if (cs == FG_OK && work) {
      cudaError_t ce = cudaMemcpyAsync(&oz_err, (uint8_t*)work + wbytes, sizeof(int), cudaMemcpyDeviceToHost, st);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
      if (ce != cudaSuccess) cs = FG_ERR_CUDA;
    }
    B->coarse_emulated = work != nullptr;
    if (work) dev_free(ctx, work);
    FG_TRY(cs);
    if (oz_err) {
      set_error("BDDC: a bounded tensor-core wait ran out in the coarse factorisation");
      return (fg_status)oz_err;
    }
    FG_TRY(check_err(B, "the coarse matrix"));
    k_coarse_extract<<<nblk(nC * nC, 256), 256, 0, st>>>(nC, B->dKc, B->dKinv, B->dKinv32);
    ctx->launches += 1;
  }
  FG_CUDA_TRY(cudaEventRecord(ev[3], st));
  FG_CUDA_TRY(cudaGetLastError());
  FG_CUDA_TRY(cudaStreamSynchronize(st));
  float cms = 0.f;
  cudaEventElapsedTime(&cms, ev[2], ev[3]);
  B->coarse_ms = cms;
  for (auto& e : ev) cudaEventDestroy(e);
  return FG_OK;
}

static size_t smem_for(int n, size_t elem) { return std::max<size_t>(16, (size_t)n * elem); }

template <typename T>
static fg_status set_smem(const void* k, size_t bytes) {
  if (bytes > 48 * 1024) FG_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return FG_OK;
}

// z = M^-1 r on solver-layout FP64 vectors (r: nvec, z: nvec; padding of z untouched).
template <typename T>
static fg_status bddc_apply_layout(fg_bddc* B, const double* r, double* z) {
  fg_system* sys = B->sys;
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  cudaStream_t st = ctx->stream;
  const bool f32 = sizeof(T) == 4;
  const int ns = B->nsub;
  T* u0 = f32 ? (T*)B->dU032 : (T*)B->dU0;
  T* v = f32 ? (T*)B->dV32 : (T*)B->dV;
  T* q = f32 ? (T*)B->dQ32 : (T*)B->dQ;
  T* t = f32 ? (T*)B->dT32 : (T*)B->dT;
  const T* R = f32 ? (const T*)B->dR32 : (const T*)B->dR;
  const T* G = f32 ? (const T*)B->dG32 : (const T*)B->dG;
  T* zE = f32 ? (T*)B->dZ32 : (T*)B->dZ;
  T* fP = f32 ? (T*)B->dFp32 : (T*)B->dFp;
  T* contrib = f32 ? (T*)B->dC32 : (T*)B->dC;
  T* fc = f32 ? (T*)B->dFc32 : (T*)B->dFc;
  T* uc = f32 ? (T*)B->dUc32 : (T*)B->dUc;
  const T* Kinv = f32 ? (const T*)B->dKinv32 : (const T*)B->dKinv;
  const int prec = f32 ? FG_MIXED : FG_FP64;
  const size_t smI = smem_for(B->maxnI, sizeof(T)), smR = smem_for(B->maxnr, sizeof(T));
  FG_TRY(set_smem<T>((const void*)k_bddc_dirichlet<T, 1>, smI));
  FG_TRY(set_smem<T>((const void*)k_bddc_dirichlet<T, 2>, smI));
  FG_TRY(set_smem<T>((const void*)k_bddc_neumann_fwd<T>, smR));
  FG_TRY(set_smem<T>((const void*)k_bddc_neumann_bwd<T>, smR));
  // 1. interior correction
  k_bddc_dirichlet<T, 1><<<ns, 256, smI, st>>>(B->d_subs, B->dA, B->dF, B->dLoc, r, (const T*)nullptr, u0, z);
  // 2-3. (A u0) on the interface
  FG_TRY(system_spmv_layout_noalloc(sys, prec, u0, q, st));
  // 4. constrained Neumann (forward), coarse residual, coarse solve, Neumann (backward)
  k_bddc_neumann_fwd<T><<<ns, 256, smR, st>>>(B->d_subs, B->dA, B->dF, R, G, B->dLoc, B->dW, r, q, zE, fP);
  if (B->nC > 0) {
    k_coarse_gather<T><<<nblk(B->nC, 256), 256, 0, st>>>(B->nC, B->dCptr, B->dCsrc, fP, fc);
    k_coarse_gemv<T><<<nblk(B->nC * 32, 256), 256, 0, st>>>(B->nC, Kinv, fc, uc);
    ctx->launches += 2;
  }
  const T* Cv = f32 ? (const T*)B->dCv32 : (const T*)B->dCv;
  k_bddc_neumann_bwd<T><<<ns, 256, smR, st>>>(B->d_subs, B->dA, B->dF, R, G, Cv, B->dPc, uc, zE, B->dW, B->dRho,
                                              contrib);
  if (B->nIface > 0)
    k_iface_sum<T><<<nblk(B->nIface, 256), 256, 0, st>>>(B->nIface, B->dIptr, B->dIsrc, B->dIvec, contrib, v, z);
  // 5. harmonic extension
  FG_TRY(system_spmv_layout_noalloc(sys, prec, v, t, st));
  k_bddc_dirichlet<T, 2><<<ns, 256, smI, st>>>(B->d_subs, B->dA, B->dF, B->dLoc, r, t, u0, z);
  ctx->launches += 7;
  FG_CUDA_TRY(cudaGetLastError());
  return FG_OK;
}

static fg_status bddc_apply(fg_bddc* B, int precision, const double* r, double* z) {
  return precision == FG_MIXED ? bddc_apply_layout<float>(B, r, z) : bddc_apply_layout<double>(B, r, z);
}

static fg_status ensure_pcg(fg_bddc* B) {
  if (B->dX) return FG_OK;
  const int64_t nvec = B->sys->space->nvec;
  FG_TRY(balloc_n(B, &B->dX, nvec, true));
  FG_TRY(balloc_n(B, &B->dRr, nvec, true));
  FG_TRY(balloc_n(B, &B->dP, nvec, true));
  FG_TRY(balloc_n(B, &B->dAp, nvec, true));
  FG_TRY(balloc_n(B, &B->dZz, nvec, true));
  FG_TRY(balloc_n(B, &B->dRv, nvec, true));
  FG_TRY(balloc_n(B, &B->dZv, nvec, true));
  return FG_OK;
}

// Host sums of the per-block partials (fixed order).
static fg_status read_partials(fg_bddc* B, int nv, double* out) {
  fg_ctx* ctx = B->sys->space->mesh->ctx;
  std::vector<double> h((size_t)nv * B->nred);
  FG_CUDA_TRY(cudaMemcpyAsync(h.data(), B->dPart, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  for (int k = 0; k < nv; ++k) {
    double s = 0.0;
    for (int b = 0; b < B->nred; ++b) s += h[(size_t)k * B->nred + b];
    out[k] = s;
  }
  return FG_OK;
}

static fg_status bddc_pcg(fg_bddc* B, const fg_solver_params* prm, const double* d_b, const double* d_x0, double* d_x,
                          fg_solve_info* info) {
  fg_system* sys = B->sys;
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  cudaStream_t st = ctx->stream;
  FG_TRY(ensure_pcg(B));
  const int64_t n = sp->nfree, nvec = sp->nvec;
  const int64_t launches0 = ctx->launches;
  cudaEvent_t e0, e1;
  FG_CUDA_TRY(cudaEventCreate(&e0));
  FG_CUDA_TRY(cudaEventCreate(&e1));
  FG_CUDA_TRY(cudaEventRecord(e0, st));
  double *x = B->dX, *r = B->dRr, *p = B->dP, *ap = B->dAp, *z = B->dZz;
  const int prec = prm->precision;
  const unsigned G = (unsigned)B->nred;
  const int crit = prm->criterion;
  FG_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(double) * nvec, st));
  FG_CUDA_TRY(cudaMemsetAsync(r, 0, sizeof(double) * nvec, st));
  if (n > 0) {
    k_rows_in<<<nblk(n, 256), 256, 0, st>>>(n, sp->d_row2vec, d_b ? d_b : sys->d_rhs, r);
    ctx->launches += 1;
  }
  if (d_x0 && n > 0) {
    k_rows_in<<<nblk(n, 256), 256, 0, st>>>(n, sp->d_row2vec, d_x0, x);
    FG_TRY(system_spmv_layout_noalloc(sys, FG_FP64, x, ap, st));
    k_sub<<<nblk(nvec, 256), 256, 0, st>>>(nvec, ap, r);
    ctx->launches += 3;
  }
  double h[2];
  // b norms for the criteria that need them
  double b_nrm = 0.0, bMb = 0.0;
  if (crit == FG_RES_RHS || crit == FG_DELTA_RHS || crit == FG_RES_NRMGIVEN_RHS_NRMGIVEN) {
    double* bv = B->dRv;
    FG_CUDA_TRY(cudaMemsetAsync(bv, 0, sizeof(double) * nvec, st));
    if (n > 0) k_rows_in<<<nblk(n, 256), 256, 0, st>>>(n, sp->d_row2vec, d_b ? d_b : sys->d_rhs, bv);
    if (crit == FG_RES_NRMGIVEN_RHS_NRMGIVEN) {
      FG_TRY(bddc_apply(B, prec, bv, z));
      k_dot2<<<G, VB, 0, st>>>(nvec, bv, z, nullptr, B->dPart);
      FG_TRY(read_partials(B, 1, h));
      bMb = std::sqrt(h[0]);
    } else {
      k_dot2<<<G, VB, 0, st>>>(nvec, bv, bv, nullptr, B->dPart);
      FG_TRY(read_partials(B, 1, h));
      b_nrm = std::sqrt(h[0]);
    }
    ctx->launches += 2;
  }
  FG_TRY(bddc_apply(B, prec, r, z));
  k_dot2<<<G, VB, 0, st>>>(nvec, r, z, r, B->dPart);
  FG_TRY(read_partials(B, 2, h));
  double r_z = h[0], r_nrm = std::sqrt(h[1]), r_nrm_M = std::sqrt(std::max(r_z, 0.0));
  FG_CUDA_TRY(cudaMemcpyAsync(p, z, sizeof(double) * nvec, cudaMemcpyDeviceToDevice, st));
  const double rtol = prm->rtol, atol = prm->atol;
  double rhs_test = 0.0;
  switch (crit) {
    case FG_RES_RHS: case FG_DELTA_RHS: rhs_test = rtol * b_nrm + atol; break;
    case FG_RES_RES: rhs_test = rtol * r_nrm + atol; break;
    case FG_RES_NRMGIVEN_RHS_NRMGIVEN: rhs_test = rtol * bMb + atol; break;
    case FG_RES_NRMGIVEN_RES_NRMGIVEN: rhs_test = rtol * r_nrm_M + atol; break;
    default: break;
  }
  int it = 0;
  bool conv = false;
  double err = 0.0;
  fg_status status = FG_OK;
  while (true) {
    ++it;
    FG_TRY(system_spmv_layout_noalloc(sys, FG_FP64, p, ap, st));
    const bool need_pp = crit == FG_DELTA_RHS || crit == FG_DELTA_DELTA;
    k_dot2<<<G, VB, 0, st>>>(nvec, ap, p, need_pp ? p : nullptr, B->dPart);
    FG_TRY(read_partials(B, 2, h));
    const double pAp = h[0], p_nrm = std::sqrt(h[1]);
    const double alpha = pAp != 0.0 ? r_z / pAp : 0.0;
    k_axpy_res<<<G, VB, 0, st>>>(nvec, alpha, p, ap, x, r, B->dPart);
    FG_TRY(read_partials(B, 1, h));
    const double rr = std::sqrt(h[0]);
    if (it == 1 && need_pp) {
      err = alpha * p_nrm;
      if (crit == FG_DELTA_DELTA) rhs_test = rtol * err + atol;
    }
    switch (crit) {
      case FG_RES_RES: case FG_RES_RHS: err = rr; break;
      case FG_DELTA_RHS: case FG_DELTA_DELTA: if (it != 1) err = alpha * p_nrm; break;
      default: err = r_nrm_M; break;
    }
    ctx->launches += 2;
    if (!std::isfinite(err) || !std::isfinite(alpha)) {
      status = FG_ERR_NUMERIC;
      set_error("BDDC-PCG breakdown at iteration %d", it);
      break;
    }
    conv = err <= rhs_test;
    if (conv || it >= prm->max_iters) break;
    FG_TRY(bddc_apply(B, prec, r, z));
    k_dot2<<<G, VB, 0, st>>>(nvec, r, z, nullptr, B->dPart);
    FG_TRY(read_partials(B, 1, h));
    const double beta = h[0] / r_z;
    r_z = h[0];
    r_nrm_M = std::sqrt(std::max(r_z, 0.0));
    k_xpby<<<nblk(nvec, 256), 256, 0, st>>>(nvec, z, beta, p);
    ctx->launches += 2;
  }
  if (n > 0) {
    k_rows_out<<<nblk(n, 256), 256, 0, st>>>(n, sp->d_row2vec, x, d_x);
    ctx->launches += 1;
  }
  FG_CUDA_TRY(cudaEventRecord(e1, st));
  FG_CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (info) {
    info->iterations = it;
    info->outer_iterations = 0;
    info->converged = conv ? 1 : 0;
    info->error_estimate = err;
    info->tolerance = rhs_test;
    info->solve_ms = ms;
    info->kernel_launches = ctx->launches - launches0;
  }
  if (status != FG_OK) return status;
  return conv ? FG_OK : FG_ERR_NOT_CONVERGED;
}

}  // namespace fg

using namespace fg;

static double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static fg_status bddc_bad(const char* msg) {
  set_error("bad argument: %s", msg);
  return FG_ERR_BADARG;
}

static void bddc_free(fg_bddc* B) {
  if (!B) return;
  fg_ctx* ctx = B->sys->space->mesh->ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (void* p : B->owned) dev_free(ctx, p);
  delete B;
}

extern "C" {

void fg_bddc_params_default(fg_bddc_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->nsub[0] = p->nsub[1] = p->nsub[2] = 2;
  p->use_vertices = 1;
  p->use_edges = 1;
  p->use_faces = 0;
  p->weighting = FG_BDDC_WEIGHT_MULTIPLICITY;
}

fg_status fg_bddc_create(fg_system* sys, const fg_bddc_params* prm, fg_bddc** out) {
  if (!sys || !prm || !out) return bddc_bad("system/params/out");
  *out = nullptr;
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  FG_CUDA_TRY(cudaSetDevice(ctx->device));
  if (sp->mesh->unst || sp->dg || sp->mesh->dim != 3) {
    set_error("BDDC: box subdomains are built for continuous spaces on structured meshes only");
    return FG_ERR_UNSUPPORTED;
  }
  if (!prm->use_vertices && !prm->use_edges && !prm->use_faces) {
    set_error("BDDC: no coarse constraints (use_vertices, use_edges and use_faces all 0)");
    return FG_ERR_UNSUPPORTED;
  }
  if (prm->weighting != FG_BDDC_WEIGHT_MULTIPLICITY && prm->weighting != FG_BDDC_WEIGHT_STIFFNESS &&
      prm->weighting != FG_BDDC_WEIGHT_SUBPART)
    return bddc_bad("weighting");
  if ((prm->weighting == FG_BDDC_WEIGHT_SUBPART || prm->use_subparts) && (!prm->use_subparts || prm->use_edges)) {
    set_error("BDDC: subpart weights need use_subparts = 1, and subparts need use_edges = 0");
    return FG_ERR_UNSUPPORTED;
  }
  if (prm->coarse_handler != FG_BDDC_HANDLER_STANDARD && prm->coarse_handler != FG_BDDC_HANDLER_ELASTICITY)
    return bddc_bad("coarse_handler");
  if (prm->coarse_handler == FG_BDDC_HANDLER_ELASTICITY && (sp->ncomp != 3 || prm->use_edges)) {
    // the reference's elasticity handler asserts .not.use_edges (sbm_elasticity_coarse_fe_handler.i90:110-111)
    set_error("BDDC: the elasticity coarse handler needs a 3-component space and use_edges = 0");
    return FG_ERR_UNSUPPORTED;
  }
  if (!sys->d_elmat) return bddc_bad("system without element matrices");
  fg_bddc* B = new fg_bddc();
  B->sys = sys;
  B->prm = *prm;
  B->prm.cuts = nullptr;
  for (int d = 0; d < 3; ++d) {
    const int nd = prm->nsub[d], nc = sp->mesh->n[d];
    if (nd < 1 || nd > nc) {
      delete B;
      return bddc_bad("nsub must be in [1, cells per direction]");
    }
    B->cuts[d].resize(nd + 1);
    int off = 0;
    for (int e = 0; e < d; ++e) off += prm->nsub[e] + 1;
    for (int k = 0; k <= nd; ++k)
      B->cuts[d][k] = prm->cuts ? prm->cuts[off + k] : (int32_t)(((int64_t)k * nc) / nd);
    bool ok = B->cuts[d][0] == 0 && B->cuts[d][nd] == nc;
    for (int k = 0; k < nd; ++k) ok = ok && B->cuts[d][k + 1] > B->cuts[d][k];
    if (!ok) {
      delete B;
      return bddc_bad("cuts must increase from 0 to the cells per direction");
    }
  }
  double t0 = now_ms();
  fg_status s = bddc_symbolic(B);
  if (s == FG_OK) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
      set_error("BDDC symbolic: %s", cudaGetErrorString(e));
      s = FG_ERR_CUDA;
    }
  }
  double t1 = now_ms();
  if (s == FG_OK) s = bddc_numeric(B);
  double t2 = now_ms();
  if (s != FG_OK) {
    bddc_free(B);
    return s;
  }
  B->symbolic_ms = t1 - t0;
  B->numeric_ms = t2 - t1;
  *out = B;
  return FG_OK;
}

fg_status fg_bddc_numerical_setup(fg_bddc* B) {
  if (!B) return bddc_bad("bddc");
  FG_CUDA_TRY(cudaSetDevice(B->sys->space->mesh->ctx->device));
  double t0 = now_ms();
  FG_TRY(bddc_numeric(B));
  B->numeric_ms = now_ms() - t0;
  return FG_OK;
}

fg_status fg_bddc_get_info(fg_bddc* B, fg_bddc_info* info) {
  if (!B || !info) return bddc_bad("bddc/info");
  info->num_subdomains = B->nsub;
  int mx = 0;
  for (auto& S : B->subs) mx = std::max(mx, S.m);
  info->max_local_dofs = mx;
  info->num_interface_dofs = B->nIface;
  info->num_coarse_dofs = B->nC;
  info->symbolic_ms = B->symbolic_ms;
  info->numeric_ms = B->numeric_ms;
  info->device_bytes = B->bytes;
  info->factor_flops = B->factor_flops;
  info->factor_ms = B->factor_ms;
  info->coarse_ms = B->coarse_ms;
  return FG_OK;
}

fg_status fg_bddc_apply_device(fg_bddc* B, int precision, const double* r_dev, double* z_dev) {
  if (!B || !r_dev || !z_dev) return bddc_bad("bddc/r/z");
  if (precision != FG_FP64 && precision != FG_MIXED) return bddc_bad("precision");
  fg_space* sp = B->sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  FG_CUDA_TRY(cudaSetDevice(ctx->device));
  FG_TRY(ensure_pcg(B));
  const int64_t n = sp->nfree;
  cudaStream_t st = ctx->stream;
  if (n > 0) {
    k_rows_in<<<nblk(n, 256), 256, 0, st>>>(n, sp->d_row2vec, r_dev, B->dRv);
    FG_TRY(bddc_apply(B, precision, B->dRv, B->dZv));
    k_rows_out<<<nblk(n, 256), 256, 0, st>>>(n, sp->d_row2vec, B->dZv, z_dev);
    ctx->launches += 2;
  }
  FG_CUDA_TRY(cudaGetLastError());
  FG_CUDA_TRY(cudaStreamSynchronize(st));
  return FG_OK;
}

static fg_status check_solve(const fg_solver_params* p) {
  if (!p) return bddc_bad("params");
  if (p->precision != FG_FP64 && p->precision != FG_MIXED) return bddc_bad("precision");
  if (p->criterion < FG_RES_RES || p->criterion > FG_RES_NRMGIVEN_RES_NRMGIVEN) return bddc_bad("criterion");
  if (!(p->rtol >= 0.0) || !(p->atol >= 0.0) || p->max_iters < 1) return bddc_bad("rtol/atol/max_iters");
  return FG_OK;
}

fg_status fg_bddc_solve_device(fg_bddc* B, const fg_solver_params* prm, const double* b_dev, const double* x0_dev,
                               double* x_dev, fg_solve_info* info) {
  if (!B || !x_dev) return bddc_bad("bddc/x");
  FG_TRY(check_solve(prm));
  FG_CUDA_TRY(cudaSetDevice(B->sys->space->mesh->ctx->device));
  return bddc_pcg(B, prm, b_dev, x0_dev, x_dev, info);
}

fg_status fg_bddc_solve(fg_bddc* B, const fg_solver_params* prm, const double* b, const double* x0, double* x,
                        fg_solve_info* info) {
  if (!B || !x) return bddc_bad("bddc/x");
  FG_TRY(check_solve(prm));
  fg_space* sp = B->sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  FG_CUDA_TRY(cudaSetDevice(ctx->device));
  const int64_t n = sp->nfree;
  const size_t bytes = sizeof(double) * (size_t)(n > 0 ? n : 1);
  double *db = nullptr, *dx0 = nullptr, *dx = nullptr;
  fg_status s = FG_OK;
  if (b) s = dev_alloc(ctx, (void**)&db, bytes);
  if (s == FG_OK && x0) s = dev_alloc(ctx, (void**)&dx0, bytes);
  if (s == FG_OK) s = dev_alloc(ctx, (void**)&dx, bytes);
  if (s == FG_OK && b && cudaMemcpyAsync(db, b, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
    s = FG_ERR_CUDA;
  if (s == FG_OK && x0 && cudaMemcpyAsync(dx0, x0, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
    s = FG_ERR_CUDA;
  fg_status ss = s;
  if (s == FG_OK) ss = bddc_pcg(B, prm, db, dx0, dx, info);
  if (ss == FG_OK || ss == FG_ERR_NOT_CONVERGED) {
    cudaError_t e = cudaMemcpyAsync(x, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
      set_error("%s", cudaGetErrorString(e));
      ss = FG_ERR_CUDA;
    }
  }
  dev_free(ctx, db);
  dev_free(ctx, dx0);
  dev_free(ctx, dx);
  return ss;
}

fg_status fg_bddc_destroy(fg_bddc* B) {
  bddc_free(B);
  return FG_OK;
}

}  // extern "C"

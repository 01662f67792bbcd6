// fg_assembly.cu -- numeric phase: cell-batch integration and the deterministic,
// atomic-free assembly of the global CSR matrix and right-hand side.
//
// Stage 1, k_integrate_poisson<P>: one warp per cell.  The warp computes the
// trilinear Jacobian, its inverse and |det| at every Gauss point (reference:
// sbm_cell_map.i90:245-369, invmtx in sbm_cell_integrator.i90:448-500), the physical
// shape gradients grad(phi_a) = J^-T grad_ref(phi_a) (sbm_lagrangian_reference_fe.i90:
// 1330-1342), the upper triangle of the element matrix (lanes own (a,b) pairs and
// accumulate over the Gauss points; the lower triangle is its mirror, as the
// reference's element matrix is exactly symmetric), the element vector, and the
// strong-Dirichlet lifting elvec -= elmat(:,j) g_j in column order
// (sbm_fe_cell_iterator.i90:1610-1637).  Element matrices go to an HBM buffer.
// GB300's FP64 rate (about 1 TFLOP/s) makes this stage FP64-bound; the buffer's
// extra HBM traffic costs a few milliseconds at the 128^3 Q2 size.
//
// Stage 1 by default for Poisson (structured and unstructured, not dG): the element
// matrices of all cells as one emulated-FP64 tensor-core product of the cells' geometric
// factors with a table shared by all cells (k_poisson_geom or k_poisson_geom_ff, then
// ozaki_gemm_nt, then k_poisson_unpack with the lifting; see the comment at PoissonTC).
//
// Stage 2, k_scatter_rows<P>: one warp per free row.  The row's node sits in at most
// 8 cells; they are visited in increasing cell index, so every entry is summed in the
// reference's order (COO appended cell by cell, stable sort, duplicates summed in
// order -- base_sparse_matrix.f90:3469-3513,4121-4829), and the right-hand side entry
// likewise (serial_scalar_array.f90:247-262).  Lanes own the row's (cell, column)
// contributions of one cell at a time; the column position comes from a binary search
// in the row's sorted columns staged in shared memory.  No atomics: the result is
// identical run to run.  The FP32 copy of the values is written in the same pass.
#include "fg_internal.h"

namespace fg {

struct AsmGeom {
  int n[3];
  int p;
  int Ln[3];
  int ncomp;
  // unstructured meshes: cell vertices (8 per cell) and cell nodes ((p+1)^3 per cell);
  // null on the structured lattice
  const int32_t* cellvert;
  const int32_t* cellnode;
};

static AsmGeom make_geom(const fg_space* sp) {
  AsmGeom g;
  for (int d = 0; d < 3; ++d) { g.n[d] = sp->mesh->n[d]; g.Ln[d] = sp->Ln[d]; }
  g.p = sp->order;
  g.ncomp = sp->ncomp;
  g.cellvert = sp->mesh->unst ? sp->mesh->d_cellvert : nullptr;
  g.cellnode = sp->d_cellnode;  // unstructured meshes and dG spaces
  return g;
}

// vertex k of cell c (lattice or explicit)
__device__ __forceinline__ int64_t asm_vertex(const AsmGeom& g, int64_t c, int ci, int cj, int ck, int k) {
  if (g.cellvert) return g.cellvert[c * 8 + k];
  return (int64_t)(ci + (k & 1)) + (int64_t)(g.n[0] + 1) * ((cj + ((k >> 1) & 1)) + (int64_t)(g.n[1] + 1) * (ck + ((k >> 2) & 1)));
}
// node of local node a (lexicographic) of cell c
template <int P>
__device__ __forceinline__ int64_t asm_node(const AsmGeom& g, int64_t c, int ci, int cj, int ck, int a) {
  constexpr int NP1 = P + 1;
  if (g.cellnode) return g.cellnode[c * (NP1 * NP1 * NP1) + a];
  const int ai = a % NP1, aj = (a / NP1) % NP1, ak = a / (NP1 * NP1);
  return (int64_t)(P * ci + ai) + (int64_t)g.Ln[0] * ((P * cj + aj) + (int64_t)g.Ln[1] * (P * ck + ak));
}

struct SourceSpec {
  int fn;
  double prm[8];
  const double* qp;  // per-qp values
};

// tutorial_01 source f = -lap(atan(alpha(|x-c|-r))) (tutorial modules :395-458)
__device__ double sharp_wave_source(const double* prm, const double* x) {
  double alpha = prm[0], r = prm[1];
  double alpha_2 = alpha * alpha, alpha_3 = alpha_2 * alpha;
  double x_minus_xc_2 = (x[0] - prm[2]) * (x[0] - prm[2]);
  double y_minus_yc_2 = (x[1] - prm[3]) * (x[1] - prm[3]);
  double z_minus_zc_2 = (x[2] - prm[4]) * (x[2] - prm[4]);
  double term1 = x_minus_xc_2 + y_minus_yc_2 + z_minus_zc_2;
  double sqrt_term1 = sqrt(term1);
  double term2 = sqrt_term1 - r;
  double term2_2 = term2 * term2;
  double a2t = alpha_2 * term2_2 + 1.0;
  double denom1 = sqrt_term1 * a2t;
  double denom2 = pow(term1, 1.5) * a2t;
  double denom3 = term1 * a2t * a2t;
  double dx2 = alpha / denom1 - (alpha * x_minus_xc_2) / denom2 - (2.0 * alpha_3 * x_minus_xc_2 * term2) / denom3;
  double dy2 = alpha / denom1 - (alpha * y_minus_yc_2) / denom2 - (2.0 * alpha_3 * y_minus_yc_2 * term2) / denom3;
  double dz2 = alpha / denom1 - (alpha * z_minus_zc_2) / denom2 - (2.0 * alpha_3 * z_minus_zc_2 * term2) / denom3;
  return -dx2 - dy2 - dz2;
}

__device__ double boundary_value(int fn, const double* prm, const double* x) {
  switch (fn) {
    case FG_FN_CONST: return prm[0];
    case FG_FN_LINEAR: return x[0] + x[1] + x[2];
    case FG_FN_SHARP_WAVE: {
      double dx = x[0] - prm[2], dy = x[1] - prm[3], dz = x[2] - prm[4];
      return atan(prm[0] * (sqrt(dx * dx + dy * dy + dz * dz) - prm[1]));
    }
    default: return 0.0;
  }
}

template <int P>
struct PoissonShape {
  static constexpr int NP1 = P + 1;
  static constexpr int NN = NP1 * NP1 * NP1;
  static constexpr int NQ = NN;
  static constexpr int ND = NN;
  static constexpr int NPAIR = ND * (ND + 1) / 2;
  static constexpr int CH = P == 1 ? 2 : (P == 2 ? 12 : 16);  // pairs per lane per pass
  static constexpr int WARPS = P == 1 ? 8 : (P == 2 ? 4 : 1);
  // shared doubles per warp: xv, invj, fac, xq, fsrc, sqrt(fac*k), grads, elmat
  static constexpr int SM_XV = 24, SM_INVJ = NQ * 9, SM_FAC = NQ, SM_XQ = NQ * 3, SM_F = NQ, SM_SQ = NQ,
                       SM_G = NQ * NN * 3, SM_EL = ND * ND;
  static constexpr int SM_DOUBLES = SM_XV + SM_INVJ + SM_FAC + SM_XQ + SM_F + SM_SQ + SM_G + SM_EL;
  static constexpr int SM_INTS = ND;  // cell gids
  // per-warp stride, rounded to 16 bytes so that the next warp's doubles stay aligned
  // and the int tail of one warp never reaches into the next warp's region
  static constexpr size_t SM_BYTES_WARP = ((size_t)SM_DOUBLES * 8 + SM_INTS * 4 + 15) / 16 * 16;
};

// Float-float variant for Q1/Q2: the scaled gradients are computed one Gauss point at a time
// into a slice of NN x 3 (hi, lo) floats and every pair accumulates that point at once (the
// pairs of a lane fit in registers), so a warp needs ~9 KB of shared memory instead of ~26 KB.
template <int P>
struct PoissonShapeFF : PoissonShape<P> {
  using B = PoissonShape<P>;
  static constexpr int WARPS = 8;
  static constexpr int SM_G = B::NN * 3;  // one slice: NN x 3 hi + NN x 3 lo floats
  static constexpr int SM_DOUBLES = B::SM_XV + B::SM_INVJ + B::SM_FAC + B::SM_XQ + B::SM_F + B::SM_SQ + SM_G + B::SM_EL;
  static constexpr size_t SM_BYTES_WARP = ((size_t)SM_DOUBLES * 8 + B::SM_INTS * 4 + 15) / 16 * 16;
};
template <int P, bool FF>
struct PoissonShapeSel {
  using type = PoissonShape<P>;
};
template <>
struct PoissonShapeSel<1, true> {
  using type = PoissonShapeFF<1>;
};
template <>
struct PoissonShapeSel<2, true> {
  using type = PoissonShapeFF<2>;
};

// upper-triangle pair index -> (a,b), row-packed
__device__ __forceinline__ void pair_ab(int p, int nd, int& a, int& b) {
  int row = 0, off = 0;
  while (off + (nd - row) <= p) { off += nd - row; ++row; }
  a = row;
  b = row + (p - off);
}

// float-float helpers: values carried as hi + lo (FP32 pair), products error-free via fmaf
__device__ __forceinline__ void ff_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void ff_renorm(float& h, float& l) {
  float s = h + l;
  l = l - (s - h);
  h = s;
}
// (sh, sl) += (ah, al) * (bh, bl)
__device__ __forceinline__ void ff_fma(float ah, float al, float bh, float bl, float& sh, float& sl) {
  float p = ah * bh;
  float e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, fmaf(al, bh, e));
  float s, t;
  ff_two_sum(sh, p, s, t);
  sh = s;
  sl += t + e;
}
__device__ __forceinline__ void ff_split(double v, float& h, float& l) {
  h = (float)v;
  l = (float)(v - (double)h);
}
// (h, l) = a * b
__device__ __forceinline__ void ff_mul(float ah, float al, float bh, float bl, float& h, float& l) {
  const float p = ah * bh;
  float e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, fmaf(al, bh, e));
  h = p + e;
  l = e - (h - p);
}
// (h, l) = a + b
__device__ __forceinline__ void ff_add(float ah, float al, float bh, float bl, float& h, float& l) {
  float sh, e;
  ff_two_sum(ah, bh, sh, e);
  e += al + bl;
  h = sh + e;
  l = e - (h - sh);
}
// (h, l) = 1 / a: FP32 reciprocal and one Newton step in float-float
__device__ __forceinline__ void ff_recip(float ah, float al, float& h, float& l) {
  const float r = 1.0f / ah;
  float ph, pl, eh, el, ch, cl;
  ff_mul(ah, al, r, 0.f, ph, pl);
  ff_add(1.0f, 0.f, -ph, -pl, eh, el);  // 1 - a r
  ff_mul(r, 0.f, eh, el, ch, cl);
  ff_add(r, 0.f, ch, cl, h, l);
}

// Per cell: vertex coordinates, the dofs' global ids (negative: Dirichlet), and per Gauss
// point J^-1 (invmtx order), |det J| w_q and the source value.  Reference: sbm_cell_map.i90:
// 245-369, invmtx in sbm_cell_integrator.i90:448-500; |det| everywhere if the first det is
// negative.
template <int P>
__device__ __forceinline__ void poisson_cell_geometry(const AsmGeom& g, int64_t c, int ci, int cj, int ck,
                                                      const double* __restrict__ coords, const DevTables& tb,
                                                      const int32_t* __restrict__ latdof, const SourceSpec& src,
                                                      int lane, double* xv, double* invj, double* fac, double* xq,
                                                      double* fsrc, int32_t* gid) {
  constexpr int NQ = PoissonShape<P>::NQ, ND = PoissonShape<P>::ND;
  if (lane < 24) {
    int k = lane / 3, l = lane % 3;
    xv[lane] = coords[asm_vertex(g, c, ci, cj, ck, k) * 3 + l];
  }
  for (int s = lane; s < ND; s += 32) gid[s] = latdof[asm_node<P>(g, c, ci, cj, ck, s)];
  __syncwarp();
  // Jacobian, inverse, det and physical coordinates per Gauss point
  for (int q = lane; q < NQ; q += 32) {
    double J[9];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double a0 = 0.0, a1 = 0.0, a2 = 0.0;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        double alpha = tb.gshg[(k * NQ + q) * 3 + j];
        a0 = a0 + alpha * xv[k * 3 + 0];
        a1 = a1 + alpha * xv[k * 3 + 1];
        a2 = a2 + alpha * xv[k * 3 + 2];
      }
      J[0 + 3 * j] = a0; J[1 + 3 * j] = a1; J[2 + 3 * j] = a2;
    }
    // invmtx, 3x3 cofactors (column-major, A(i,j) = J[(i-1)+3(j-1)])
    double t1 = J[4] * J[8] - J[5] * J[7];
    double t2 = -J[1] * J[8] + J[2] * J[7];
    double t3 = J[1] * J[5] - J[2] * J[4];
    double det = J[0] * t1 + J[3] * t2 + J[6] * t3;
    double denom = 1.0 / det;
    double* b = invj + q * 9;
    b[0] = t1 * denom;
    b[1] = t2 * denom;
    b[2] = t3 * denom;
    b[4] = (J[0] * J[8] - J[2] * J[6]) * denom;
    b[5] = (-J[0] * J[5] + J[3] * J[2]) * denom;
    b[8] = (J[0] * J[4] - J[1] * J[3]) * denom;
    b[3] = (-J[3] * J[8] + J[5] * J[6]) * denom;
    b[6] = (J[3] * J[7] - J[4] * J[6]) * denom;
    b[7] = (-J[0] * J[7] + J[1] * J[6]) * denom;
    fac[q] = det;
    if (src.fn == FG_FN_SHARP_WAVE) {  // the only source that reads the physical coordinates
      double x0 = 0.0, x1 = 0.0, x2 = 0.0;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        double a = tb.gshp[k * NQ + q];
        x0 = x0 + a * xv[k * 3 + 0];
        x1 = x1 + a * xv[k * 3 + 1];
        x2 = x2 + a * xv[k * 3 + 2];
      }
      xq[q * 3 + 0] = x0; xq[q * 3 + 1] = x1; xq[q * 3 + 2] = x2;
    }
  }
  __syncwarp();
  const bool neg = fac[0] < 0.0;  // reference: |det| everywhere if the first one is negative
  __syncwarp();
  for (int q = lane; q < NQ; q += 32) {
    double d = neg ? fabs(fac[q]) : fac[q];
    fac[q] = d * tb.qw[q];
    double f;
    if (src.fn == FG_FN_SHARP_WAVE) f = sharp_wave_source(src.prm, xq + q * 3);
    else if (src.fn == FG_FN_QP_VALUES) f = src.qp[c * NQ + q];
    else if (src.fn == FG_FN_CONST) f = src.prm[0];
    else f = 0.0;
    fsrc[q] = f;
  }
  __syncwarp();
}

template <int P, bool FF>
__global__ void __launch_bounds__(PoissonShapeSel<P, FF>::type::WARPS * 32)
    k_integrate_poisson(AsmGeom g, int64_t ncells, const double* __restrict__ coords, DevTables tb,
                        const int32_t* __restrict__ latdof, const double* __restrict__ gvals,
                        const double* __restrict__ coef, double coef_const, SourceSpec src,
                        double* __restrict__ E, double* __restrict__ EV) {
  using S = typename PoissonShapeSel<P, FF>::type;
  constexpr bool STREAM = FF && P <= 2;
  constexpr int NN = S::NN, NQ = S::NQ, ND = S::ND;
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  double* base = smem + (size_t)wib * (S::SM_BYTES_WARP / 8);
  double* xv = base;
  double* invj = xv + S::SM_XV;
  double* fac = invj + S::SM_INVJ;
  double* xq = fac + S::SM_FAC;
  double* fsrc = xq + S::SM_XQ;
  double* sq = fsrc + S::SM_F;
  double* sg = sq + S::SM_SQ;
  double* el = sg + S::SM_G;
  int32_t* gid = (int32_t*)(el + S::SM_EL);

  const int64_t c = (int64_t)blockIdx.x * S::WARPS + wib;
  if (c >= ncells) return;
  const int ci = (int)(c % g.n[0]);
  const int cj = (int)((c / g.n[0]) % g.n[1]);
  const int ck = (int)(c / ((int64_t)g.n[0] * g.n[1]));
  const double kc = coef ? coef[c] : coef_const;

  poisson_cell_geometry<P>(g, c, ci, cj, ck, coords, tb, latdof, src, lane, xv, invj, fac, xq, fsrc, gid);
  for (int q = lane; q < NQ; q += 32) sq[q] = sqrt(fac[q] * kc);  // |det J| w k > 0
  __syncwarp();
  if constexpr (FF) {
    // float-float variant: J^-1 and sqrt(fk) as FP32 pairs (converted in place: the pairs
    // take half the bytes of the doubles they replace), scaled gradients and the element
    // matrix accumulated with error-free FP32 products
    constexpr int NI = (NQ * 9 + 31) / 32, NS = (NQ + 31) / 32;
    double tv[NI], ts[NS];
#pragma unroll
    for (int k = 0; k < NI; ++k) tv[k] = (lane + 32 * k < NQ * 9) ? invj[lane + 32 * k] : 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) ts[k] = (lane + 32 * k < NQ) ? sq[lane + 32 * k] : 0.0;
    __syncwarp();
    float* ivh = reinterpret_cast<float*>(invj);
    float* ivl = ivh + NQ * 9;
    float* sqh = reinterpret_cast<float*>(sq);
    float* sql = sqh + NQ;
#pragma unroll
    for (int k = 0; k < NI; ++k)
      if (lane + 32 * k < NQ * 9) ff_split(tv[k], ivh[lane + 32 * k], ivl[lane + 32 * k]);
#pragma unroll
    for (int k = 0; k < NS; ++k)
      if (lane + 32 * k < NQ) ff_split(ts[k], sqh[lane + 32 * k], sql[lane + 32 * k]);
    __syncwarp();
    if constexpr (STREAM) {
      // one Gauss point at a time: slice of scaled gradients, all pairs of the lane accumulate it
      float* qh = reinterpret_cast<float*>(sg);
      float* ql = qh + NN * 3;
      float ah[S::CH], al[S::CH];
      int pa[S::CH], pb[S::CH];
#pragma unroll
      for (int t = 0; t < S::CH; ++t) {
        ah[t] = 0.f;
        al[t] = 0.f;
        int p = lane + 32 * t;
        if (p < S::NPAIR) pair_ab(p, ND, pa[t], pb[t]);
        else { pa[t] = 0; pb[t] = 0; }
      }
      static_assert(32 * S::CH >= S::NPAIR, "one pass over the pairs");
      for (int q = 0; q < NQ; ++q) {
        for (int idx = lane; idx < NN * 3; idx += 32) {
          const int a = idx / 3, i = idx - 3 * a;
          const int r = (a * NQ + q) * 3;
          float th = 0.f, tl = 0.f;
#pragma unroll
          for (int j = 0; j < 3; ++j) ff_fma(ivh[q * 9 + j + 3 * i], ivl[q * 9 + j + 3 * i], tb.shgh[r + j], tb.shgl[r + j], th, tl);
          ff_renorm(th, tl);
          float gh = 0.f, gl = 0.f;
          ff_fma(sqh[q], sql[q], th, tl, gh, gl);
          ff_renorm(gh, gl);
          qh[idx] = gh;
          ql[idx] = gl;
        }
        __syncwarp();
#pragma unroll
        for (int t = 0; t < S::CH; ++t) {
#pragma unroll
          for (int i = 0; i < 3; ++i)
            ff_fma(qh[pb[t] * 3 + i], ql[pb[t] * 3 + i], qh[pa[t] * 3 + i], ql[pa[t] * 3 + i], ah[t], al[t]);
        }
        __syncwarp();
      }
#pragma unroll
      for (int t = 0; t < S::CH; ++t) {
        int p = lane + 32 * t;
        if (p < S::NPAIR) {
          ff_renorm(ah[t], al[t]);
          const double v = (double)ah[t] + (double)al[t];
          el[pa[t] * ND + pb[t]] = v;
          el[pb[t] * ND + pa[t]] = v;
        }
      }
      __syncwarp();
    } else {
    float* sgh = reinterpret_cast<float*>(sg);
    float* sgl = sgh + NQ * NN * 3;
    for (int idx = lane; idx < NQ * NN; idx += 32) {
      const int q = idx / NN, a = idx % NN;
      const int r = (a * NQ + q) * 3;
      const float rh[3] = {tb.shgh[r], tb.shgh[r + 1], tb.shgh[r + 2]};
      const float rl[3] = {tb.shgl[r], tb.shgl[r + 1], tb.shgl[r + 2]};
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        float th = 0.f, tl = 0.f;
#pragma unroll
        for (int j = 0; j < 3; ++j) ff_fma(ivh[q * 9 + j + 3 * i], ivl[q * 9 + j + 3 * i], rh[j], rl[j], th, tl);
        ff_renorm(th, tl);
        float gh = 0.f, gl = 0.f;
        ff_fma(sqh[q], sql[q], th, tl, gh, gl);
        ff_renorm(gh, gl);
        sgh[idx * 3 + i] = gh;
        sgl[idx * 3 + i] = gl;
      }
    }
    __syncwarp();
    for (int pbase = 0; pbase < S::NPAIR; pbase += 32 * S::CH) {
      float ah[S::CH], al[S::CH];
      int pa[S::CH], pb[S::CH];
#pragma unroll
      for (int t = 0; t < S::CH; ++t) {
        ah[t] = 0.f;
        al[t] = 0.f;
        int p = pbase + lane + 32 * t;
        if (p < S::NPAIR) pair_ab(p, ND, pa[t], pb[t]);
        else { pa[t] = 0; pb[t] = 0; }
      }
      for (int q = 0; q < NQ; ++q) {
        const float* gqh = sgh + q * NN * 3;
        const float* gql = sgl + q * NN * 3;
#pragma unroll
        for (int t = 0; t < S::CH; ++t) {
#pragma unroll
          for (int i = 0; i < 3; ++i)
            ff_fma(gqh[pb[t] * 3 + i], gql[pb[t] * 3 + i], gqh[pa[t] * 3 + i], gql[pa[t] * 3 + i], ah[t], al[t]);
        }
      }
#pragma unroll
      for (int t = 0; t < S::CH; ++t) {
        int p = pbase + lane + 32 * t;
        if (p < S::NPAIR) {
          ff_renorm(ah[t], al[t]);
          const double v = (double)ah[t] + (double)al[t];
          el[pa[t] * ND + pb[t]] = v;
          el[pb[t] * ND + pa[t]] = v;
        }
      }
    }
    __syncwarp();
    }
  } else {
  // physical gradients scaled by sqrt(|det J| w k): s_a = sqrt(fk) J^-T grad_ref(phi_a), so an
  // element entry is sum_q s_a . s_b, 3 FP64 FMAs per Gauss point (FP64 is GB300's scarce pipe)
  for (int idx = lane; idx < NQ * NN; idx += 32) {
    int q = idx / NN, a = idx % NN;
    const double* rg = tb.shg + ((size_t)a * NQ + q) * 3;
    const double* b = invj + q * 9;
    const double s = sq[q];
    double r0 = rg[0], r1 = rg[1], r2 = rg[2];
#pragma unroll
    for (int i = 0; i < 3; ++i) sg[idx * 3 + i] = s * (b[0 + 3 * i] * r0 + b[1 + 3 * i] * r1 + b[2 + 3 * i] * r2);
  }
  __syncwarp();
  // element matrix, upper triangle by pairs
  for (int pbase = 0; pbase < S::NPAIR; pbase += 32 * S::CH) {
    double acc[S::CH];
    int pa[S::CH], pb[S::CH];
#pragma unroll
    for (int t = 0; t < S::CH; ++t) {
      acc[t] = 0.0;
      int p = pbase + lane + 32 * t;
      if (p < S::NPAIR) pair_ab(p, ND, pa[t], pb[t]);
      else { pa[t] = 0; pb[t] = 0; }
    }
    for (int q = 0; q < NQ; ++q) {
      const double* gq = sg + q * NN * 3;
#pragma unroll
      for (int t = 0; t < S::CH; ++t) {
        const double* ga = gq + pa[t] * 3;
        const double* gb = gq + pb[t] * 3;
        acc[t] = fma(gb[0], ga[0], acc[t]);
        acc[t] = fma(gb[1], ga[1], acc[t]);
        acc[t] = fma(gb[2], ga[2], acc[t]);
      }
    }
#pragma unroll
    for (int t = 0; t < S::CH; ++t) {
      int p = pbase + lane + 32 * t;
      if (p < S::NPAIR) {
        el[pa[t] * ND + pb[t]] = acc[t];
        el[pb[t] * ND + pa[t]] = acc[t];
      }
    }
  }
  __syncwarp();
  }
  // element vector + Dirichlet lifting
  bool any_dir = false;
  for (int s = lane; s < ND; s += 32) any_dir |= gid[s] < 0;
  any_dir = __any_sync(0xffffffffu, any_dir);
  for (int a = lane; a < ND; a += 32) {
    double ev = 0.0;
    for (int q = 0; q < NQ; ++q) ev = ev + fac[q] * fsrc[q] * tb.shp[(size_t)a * NQ + q];
    if (any_dir)
      for (int b = 0; b < ND; ++b) {
        int32_t gb = gid[b];
        if (gb < 0) ev = ev - el[a * ND + b] * gvals[-gb - 1];
      }
    EV[c * ND + a] = ev;
  }
  // Dirichlet columns are spent on the lifting above: stored as zeros, so the row gathers add
  // nothing there without looking the columns up
  double* Ec = E + (size_t)c * ND * ND;
  for (int idx = lane; idx < ND * ND; idx += 32) Ec[idx] = gid[idx % ND] < 0 ? 0.0 : el[idx];
}

// ---------------------------------------------------------------------------
// Poisson element matrices on the tensor cores.  With r_a(q) the reference gradient of shape
// a at Gauss point q and M_q = |det J_q| w_q k J_q^-1 J_q^-T (symmetric 3 x 3), an element
// entry is E_ab = sum_q r_a(q)^T M_q r_b(q) = sum_{q,m} T[ab][6q + m] G[c][6q + m], m running
// over the six entries of M_q (T holds r_ai r_bj + r_aj r_bi off the diagonal).  T (upper
// pairs x 6 NQ) is the same for every cell, so the element matrices of all cells are one
// product G T^T (cells x pairs, K = 6 NQ) -- the tensor form of the element matrix (Kirby and
// Logg, ACM TOMS 32 (2006)) -- computed in FP64 emulated on the bf16 tensor cores
// (ozaki_gemm_nt, fg_ozaki.cu).  Three kernels around it: the geometric factors G and the
// source part of the element vector (warp per cell, the geometry of k_integrate_poisson), the
// product, and the unpacking of each cell's upper triangle into the staged element matrix
// with the Dirichlet lifting.
template <int P>
struct PoissonTC {
  using S = PoissonShape<P>;
  static constexpr int NQ = S::NQ, ND = S::ND, NPAIR = S::NPAIR, K = 6 * NQ;
  static constexpr int WARPS = 8;
  static constexpr int SM_DOUBLES = S::SM_XV + S::SM_INVJ + S::SM_FAC + S::SM_XQ + S::SM_F;
  static constexpr size_t SM_BYTES_WARP = ((size_t)SM_DOUBLES * 8 + ND * 4 + 15) / 16 * 16;
};

template <int P>
__global__ void __launch_bounds__(PoissonTC<P>::WARPS * 32)
    k_poisson_geom(AsmGeom g, int64_t ncells, const double* __restrict__ coords, DevTables tb,
                   const int32_t* __restrict__ latdof, const double* __restrict__ coef, double coef_const,
                   SourceSpec src, double* __restrict__ G, double* __restrict__ EV) {
  using T = PoissonTC<P>;
  constexpr int NQ = T::NQ, ND = T::ND, K = T::K;
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  double* xv = smem + (size_t)wib * (T::SM_BYTES_WARP / 8);
  double* invj = xv + T::S::SM_XV;
  double* fac = invj + T::S::SM_INVJ;
  double* xq = fac + T::S::SM_FAC;
  double* fsrc = xq + T::S::SM_XQ;
  int32_t* gid = (int32_t*)(fsrc + T::S::SM_F);
  const int64_t c = (int64_t)blockIdx.x * T::WARPS + wib;
  if (c >= ncells) return;
  const int ci = (int)(c % g.n[0]);
  const int cj = (int)((c / g.n[0]) % g.n[1]);
  const int ck = (int)(c / ((int64_t)g.n[0] * g.n[1]));
  const double kc = coef ? coef[c] : coef_const;
  poisson_cell_geometry<P>(g, c, ci, cj, ck, coords, tb, latdof, src, lane, xv, invj, fac, xq, fsrc, gid);
  // per Gauss point: |det J| w k (into xq, free unless the source read it) and |det J| w f
  double* fk = xq;
  for (int q = lane; q < NQ; q += 32) {
    const double fq = fac[q];
    fk[q] = fq * kc;
    fsrc[q] = fq * fsrc[q];
  }
  __syncwarp();
  // M_jk = |det J| w k sum_l B[j + 3l] B[k + 3l], B = J^-1 as stored by invmtx; order 00 11 22 01 02 12
  for (int e = lane; e < K; e += 32) {
    const int q = e / 6, m = e - 6 * q;
    const int j = m < 3 ? m : (m == 5 ? 1 : 0), k = m < 3 ? m : (m == 3 ? 1 : 2);
    const double* b = invj + q * 9;
    G[c * K + e] = fk[q] * (b[j] * b[k] + b[j + 3] * b[k + 3] + b[j + 6] * b[k + 6]);
  }
  // element vector, source part (the lifting follows the product); the same products and
  // order as k_integrate_poisson's (fac f) phi
  for (int a = lane; a < ND; a += 32) {
    double ev = 0.0;
    for (int q = 0; q < NQ; ++q) ev = ev + fsrc[q] * tb.shp[(size_t)a * NQ + q];
    EV[c * ND + a] = ev;
  }
}

// The same in float-float (FP32 pairs, ~2^-44 relative), for fast-integration requests: the
// Jacobian, invmtx, |det J| w k J^-1 J^-T and the source part of the element vector run on the
// FP32 pipe (GB300's FP64 rate is ~1/70 of FP32's).  ff tables: the Q1 geometry gradients
// (8 x NQ x 3), the shape values (ND x NQ) and the weights (NQ), hi then lo.
template <int P>
struct PoissonTCFF {
  static constexpr int NQ = PoissonTC<P>::NQ, ND = PoissonTC<P>::ND;
  static constexpr int WARPS = 8;
  static constexpr int G3 = 8 * NQ * 3, SH = ND * NQ;
  static constexpr int TAB = 2 * (G3 + SH + NQ);  // floats of the table
  // per warp: vertices (24 pairs), J^-1 (9 pairs per point), det, |det| w k, |det| w f (pairs)
  static constexpr int SM_FLOATS = 48 + NQ * 18 + NQ * 2 * 3;
  static constexpr size_t SM_BYTES_WARP = ((size_t)SM_FLOATS * 4 + 15) / 16 * 16;
};

template <int P>
__global__ void __launch_bounds__(PoissonTCFF<P>::WARPS * 32)
    k_poisson_geom_ff(AsmGeom g, int64_t ncells, const double* __restrict__ coords, DevTables tb,
                      const float* __restrict__ tab, const double* __restrict__ coef, double coef_const, SourceSpec src,
                      double* __restrict__ G, double* __restrict__ EV) {
  using T = PoissonTCFF<P>;
  constexpr int NQ = T::NQ, ND = T::ND, K = PoissonTC<P>::K;
  extern __shared__ float fsm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  float* xvh = fsm + (size_t)wib * (T::SM_BYTES_WARP / 4);
  float* xvl = xvh + 24;
  float* bh = xvl + 24;      // NQ x 9
  float* bl = bh + NQ * 9;
  float* dh = bl + NQ * 9;   // det
  float* dl = dh + NQ;
  float* kh = dl + NQ;       // |det| w k
  float* kl = kh + NQ;
  float* wh = kl + NQ;       // |det| w f
  float* wl = wh + NQ;
  const float* gh = tab;
  const float* gl = gh + T::G3;
  const float* shh = gl + T::G3;
  const float* shl = shh + T::SH;
  const float* qwh = shl + T::SH;
  const float* qwl = qwh + NQ;
  const int64_t c = (int64_t)blockIdx.x * T::WARPS + wib;
  if (c >= ncells) return;
  const int ci = (int)(c % g.n[0]);
  const int cj = (int)((c / g.n[0]) % g.n[1]);
  const int ck = (int)(c / ((int64_t)g.n[0] * g.n[1]));
  float kch, kcl;
  ff_split(coef ? coef[c] : coef_const, kch, kcl);
  // vertex coordinates relative to vertex 0, taken in FP64: J = sum_k grad N_k x_k = sum_k
  // grad N_k (x_k - x_0) (the gradients sum to zero), so the O(h) Jacobian is not a
  // cancellation of O(1) coordinates in float-float
  const int64_t v0 = asm_vertex(g, c, ci, cj, ck, 0);
  if (lane < 24)
    ff_split(coords[asm_vertex(g, c, ci, cj, ck, lane / 3) * 3 + lane % 3] - coords[v0 * 3 + lane % 3], xvh[lane],
             xvl[lane]);
  __syncwarp();
  for (int q = lane; q < NQ; q += 32) {
    float Jh[9], Jl[9];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      float ah[3] = {0.f, 0.f, 0.f}, al[3] = {0.f, 0.f, 0.f};
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const float th = gh[(k * NQ + q) * 3 + j], tl = gl[(k * NQ + q) * 3 + j];
#pragma unroll
        for (int i = 0; i < 3; ++i) ff_fma(th, tl, xvh[k * 3 + i], xvl[k * 3 + i], ah[i], al[i]);
      }
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        ff_renorm(ah[i], al[i]);
        Jh[i + 3 * j] = ah[i];
        Jl[i + 3 * j] = al[i];
      }
    }
    // invmtx cofactors: x = a b - c d as two products and a sum
    auto cof = [&](int a, int b, int cc, int d, float& h, float& l) {
      float ph, pl, mh, ml;
      ff_mul(Jh[a], Jl[a], Jh[b], Jl[b], ph, pl);
      ff_mul(Jh[cc], Jl[cc], Jh[d], Jl[d], mh, ml);
      ff_add(ph, pl, -mh, -ml, h, l);
    };
    float c0h, c0l, c1h, c1l, c2h, c2l, c3h, c3l, c4h, c4l, c5h, c5l, c6h, c6l, c7h, c7l, c8h, c8l;
    cof(4, 8, 5, 7, c0h, c0l);  // t1
    cof(2, 7, 1, 8, c1h, c1l);  // t2
    cof(1, 5, 2, 4, c2h, c2l);  // t3
    cof(5, 6, 3, 8, c3h, c3l);
    cof(0, 8, 2, 6, c4h, c4l);
    cof(3, 2, 0, 5, c5h, c5l);
    cof(3, 7, 4, 6, c6h, c6l);
    cof(1, 6, 0, 7, c7h, c7l);
    cof(0, 4, 1, 3, c8h, c8l);
    float deth, detl, th, tl;
    ff_mul(Jh[0], Jl[0], c0h, c0l, deth, detl);
    ff_mul(Jh[3], Jl[3], c1h, c1l, th, tl);
    ff_add(deth, detl, th, tl, deth, detl);
    ff_mul(Jh[6], Jl[6], c2h, c2l, th, tl);
    ff_add(deth, detl, th, tl, deth, detl);
    float rh, rl;
    ff_recip(deth, detl, rh, rl);
    const float ch[9] = {c0h, c1h, c2h, c3h, c4h, c5h, c6h, c7h, c8h};
    const float cl[9] = {c0l, c1l, c2l, c3l, c4l, c5l, c6l, c7l, c8l};
#pragma unroll
    for (int m = 0; m < 9; ++m) ff_mul(ch[m], cl[m], rh, rl, bh[q * 9 + m], bl[q * 9 + m]);
    dh[q] = deth;
    dl[q] = detl;
  }
  __syncwarp();
  const bool neg = dh[0] < 0.f;  // reference: |det| everywhere if the first one is negative
  for (int q = lane; q < NQ; q += 32) {
    float ah = dh[q], al = dl[q];
    if (neg && ah < 0.f) { ah = -ah; al = -al; }
    float fh, fl;
    ff_mul(ah, al, qwh[q], qwl[q], fh, fl);  // |det J| w
    ff_mul(fh, fl, kch, kcl, kh[q], kl[q]);
    double f;
    if (src.fn == FG_FN_SHARP_WAVE) {  // x = x_0 + sum_k N_k (x_k - x_0)
      double x[3] = {coords[v0 * 3], coords[v0 * 3 + 1], coords[v0 * 3 + 2]};
      for (int k = 0; k < 8; ++k)
        for (int i = 0; i < 3; ++i)
          x[i] = x[i] + tb.gshp[k * NQ + q] * ((double)xvh[k * 3 + i] + (double)xvl[k * 3 + i]);
      f = sharp_wave_source(src.prm, x);
    } else if (src.fn == FG_FN_QP_VALUES) f = src.qp[c * NQ + q];
    else if (src.fn == FG_FN_CONST) f = src.prm[0];
    else f = 0.0;
    float sh, sl;
    ff_split(f, sh, sl);
    ff_mul(fh, fl, sh, sl, wh[q], wl[q]);
  }
  __syncwarp();
  for (int e = lane; e < K; e += 32) {
    const int q = e / 6, m = e - 6 * q;
    const int j = m < 3 ? m : (m == 5 ? 1 : 0), k = m < 3 ? m : (m == 3 ? 1 : 2);
    const float* b0 = bh + q * 9;
    const float* b1 = bl + q * 9;
    float sh = 0.f, sl = 0.f;
#pragma unroll
    for (int l = 0; l < 3; ++l) ff_fma(b0[j + 3 * l], b1[j + 3 * l], b0[k + 3 * l], b1[k + 3 * l], sh, sl);
    ff_renorm(sh, sl);
    float vh, vl;
    ff_mul(kh[q], kl[q], sh, sl, vh, vl);
    G[c * K + e] = (double)vh + (double)vl;
  }
  for (int a = lane; a < ND; a += 32) {
    float sh = 0.f, sl = 0.f;
    for (int q = 0; q < NQ; ++q) ff_fma(wh[q], wl[q], shh[a * NQ + q], shl[a * NQ + q], sh, sl);
    EV[c * ND + a] = (double)sh + (double)sl;
  }
}

// upper triangle (row-packed pairs) -> the staged element matrix, Dirichlet columns zero, and
// the strong-Dirichlet lifting elvec -= elmat(:, j) g_j in column order, as k_integrate_poisson
template <int P>
__global__ void __launch_bounds__(256)
    k_poisson_unpack(AsmGeom g, int64_t ncells, const int32_t* __restrict__ latdof, const double* __restrict__ gvals,
                     const double* __restrict__ Cp, double* __restrict__ E, double* __restrict__ EV) {
  using T = PoissonTC<P>;
  constexpr int ND = T::ND, NPAIR = T::NPAIR;
  __shared__ int32_t sgid[8][ND];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t c = (int64_t)blockIdx.x * 8 + wib;
  if (c >= ncells) return;
  const int ci = (int)(c % g.n[0]);
  const int cj = (int)((c / g.n[0]) % g.n[1]);
  const int ck = (int)(c / ((int64_t)g.n[0] * g.n[1]));
  int32_t* gid = sgid[wib];
  for (int s = lane; s < ND; s += 32) gid[s] = latdof[asm_node<P>(g, c, ci, cj, ck, s)];
  __syncwarp();
  const double* cp = Cp + c * NPAIR;
  double* Ec = E + (size_t)c * ND * ND;
  for (int idx = lane; idx < ND * ND; idx += 32) {
    const int a = idx / ND, b = idx - a * ND;
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    Ec[idx] = gid[b] < 0 ? 0.0 : cp[lo * ND - lo * (lo - 1) / 2 + (hi - lo)];
  }
  bool any_dir = false;
  for (int s = lane; s < ND; s += 32) any_dir |= gid[s] < 0;
  if (!__any_sync(0xffffffffu, any_dir)) return;
  for (int a = lane; a < ND; a += 32) {
    double ev = EV[c * ND + a];
    for (int b = 0; b < ND; ++b) {
      const int32_t gb = gid[b];
      const int lo = a < b ? a : b, hi = a < b ? b : a;
      if (gb < 0) ev = ev - cp[lo * ND - lo * (lo - 1) / 2 + (hi - lo)] * gvals[-gb - 1];
    }
    EV[c * ND + a] = ev;
  }
}

// warp per free row; CAP = power-of-two box capacity
template <int P, int CAP, int W = 8>
__global__ void __launch_bounds__(W * 32)
    k_scatter_rows(AsmGeom g, int64_t nfree, const int32_t* __restrict__ free2lat, const int32_t* __restrict__ latdof,
                   const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                   const double* __restrict__ E, const double* __restrict__ EV, double* __restrict__ val,
                   float* __restrict__ val32, double* __restrict__ rhs) {
  constexpr int NP1 = P + 1, NN = NP1 * NP1 * NP1;
  __shared__ int32_t s_col[W][CAP];
  __shared__ double s_acc[W][CAP];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t r = (int64_t)blockIdx.x * W + wib;
  if (r >= nfree) return;
  const int ncomp = g.ncomp, ND = NN * ncomp;
  const int32_t slot = free2lat[r];
  const int64_t L = slot / ncomp;
  const int comp = slot % ncomp;
  const int I = (int)(L % g.Ln[0]);
  const int J = (int)((L / g.Ln[0]) % g.Ln[1]);
  const int K = (int)(L / ((int64_t)g.Ln[0] * g.Ln[1]));
  const int64_t s = rowptr[r];
  const int len = (int)(rowptr[r + 1] - s);
  int32_t* cols = s_col[wib];
  double* acc = s_acc[wib];
  for (int t = lane; t < CAP; t += 32) {
    cols[t] = t < len ? col[s + t] : 0x7fffffff;
    acc[t] = 0.0;
  }
  __syncwarp();
  int clo[3], chi[3];
  const int IJK[3] = {I, J, K};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    int cc = IJK[d] / P;
    clo[d] = (IJK[d] % P == 0) ? cc - 1 : cc;
    chi[d] = cc;
    if (clo[d] < 0) clo[d] = 0;
    if (chi[d] > g.n[d] - 1) chi[d] = g.n[d] - 1;
  }
  double rsum = 0.0;
  for (int ck = clo[2]; ck <= chi[2]; ++ck)
    for (int cj = clo[1]; cj <= chi[1]; ++cj)
      for (int ci = clo[0]; ci <= chi[0]; ++ci) {
        const int64_t c = (int64_t)ci + (int64_t)g.n[0] * (cj + (int64_t)g.n[1] * ck);
        const int anode = (I - P * ci) + NP1 * ((J - P * cj) + NP1 * (K - P * ck));
        const int a = anode + comp * NN;
        const double* Erow = E + ((size_t)c * ND + a) * ND;
        for (int b = lane; b < ND; b += 32) {
          const int bnode = b % NN, bcomp = b / NN;
          const int bi = bnode % NP1, bj = (bnode / NP1) % NP1, bk = bnode / (NP1 * NP1);
          const int64_t M = (int64_t)(P * ci + bi) + (int64_t)g.Ln[0] * ((P * cj + bj) + (int64_t)g.Ln[1] * (P * ck + bk));
          const int32_t id = latdof[M * ncomp + bcomp];
          if (id > 0) {
            const int32_t key = id - 1;
            int lo = 0, hi = len;
            while (lo < hi) {
              int m = (lo + hi) >> 1;
              if (cols[m] < key) lo = m + 1;
              else hi = m;
            }
            acc[lo] = acc[lo] + Erow[b];
          }
        }
        if (lane == 0) rsum = rsum + EV[c * ND + a];
        __syncwarp();
      }
  for (int t = lane; t < len; t += 32) {
    double v = acc[t];
    val[s + t] = v;
    if (val32) val32[s + t] = (float)v;
  }
  if (lane == 0) rhs[r] = rsum;
}

// Row gather straight into the lattice-implicit layout: one block per slice (32 rows of one
// class).  Each warp assembles rows of the slice in shared memory, in box-position order
// (the column of position k is fixed by the class, so no search): the row's node sits in at
// most 8 cells, visited in increasing cell index, and every position sums its contributions
// in that order -- the reference's duplicate-summation order, so the values equal
// k_scatter_rows' CSR values bit for bit.  A lane loads its column of every cell first
// (streaming loads: each element-matrix entry is read once), then the sums run cell by cell.
// Dirichlet columns of the element matrices are stored as zeros by the integration kernels,
// so they add exact zeros to positions that stay zero.  The slice's 32 x Bp
// block is then written out with consecutive threads on consecutive addresses, FP64 and
// FP32, padding included: no clearing pass and no CSR in between.
template <int P, int NC, int W, int MINB>
__global__ void __launch_bounds__(W * 32, MINB)
    k_scatter_stencil(AsmGeom g, const uint8_t* __restrict__ scls, const int64_t* __restrict__ voff,
                      const StencilClass* __restrict__ cls,
                      const int32_t* __restrict__ slot2row, const int32_t* __restrict__ free2lat,
                      const int32_t* __restrict__ latdof, const double* __restrict__ E, const double* __restrict__ EV,
                      double* __restrict__ tval, float* __restrict__ tval32, double* __restrict__ rhs) {
  constexpr int NP1 = P + 1, NN = NP1 * NP1 * NP1;
  extern __shared__ double s_slice[];
  const int64_t sl = blockIdx.x;
  const StencilClass C = cls[scls[sl]];
  const int Bp = C.Bp, stride = C.Bp + 4;  // +4 doubles: rows of the buffer start on shifted banks
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  for (int k = threadIdx.x; k < 32 * stride; k += W * 32) s_slice[k] = 0.0;
  __syncthreads();
  constexpr int ncomp = NC, ND = NN * NC;
  constexpr int BCH = (ND + 31) / 32;  // column chunks per lane and cell
  for (int rl = wib; rl < 32; rl += W) {
    const int32_t r = slot2row[sl * 32 + rl];
    if (r < 0) continue;  // padding row of the class's last slice: zeros
    double* acc = s_slice + rl * stride;
    const int32_t slot = free2lat[r];
    const int64_t L = slot / ncomp;
    const int comp = slot % ncomp;
    const int I = (int)(L % g.Ln[0]);
    const int J = (int)((L / g.Ln[0]) % g.Ln[1]);
    const int K = (int)(L / ((int64_t)g.Ln[0] * g.Ln[1]));
    int clo[3], chi[3];
    const int IJK[3] = {I, J, K};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int cc = IJK[d] / P;
      clo[d] = (IJK[d] % P == 0) ? cc - 1 : cc;
      chi[d] = cc;
      if (clo[d] < 0) clo[d] = 0;
      if (chi[d] > g.n[d] - 1) chi[d] = g.n[d] - 1;
    }
    const int nci = chi[0] - clo[0] + 1, ncj = chi[1] - clo[1] + 1, nck = chi[2] - clo[2] + 1;
    const int ncell = nci * ncj * nck;
    double v[8][BCH];
    int pos[8][BCH];
    double evl = 0.0;  // lane q: the element-vector entry of cell q
    // loads first (up to 8 cells x BCH columns per lane in flight), in increasing cell order
#pragma unroll
    for (int q = 0; q < 8; ++q) {
#pragma unroll
      for (int h = 0; h < BCH; ++h) pos[q][h] = -1;
      if (q < ncell) {
        const int ci = clo[0] + q % nci, cj = clo[1] + (q / nci) % ncj, ck = clo[2] + q / (nci * ncj);
        const int64_t c = (int64_t)ci + (int64_t)g.n[0] * (cj + (int64_t)g.n[1] * ck);
        const int a = (I - P * ci) + NP1 * ((J - P * cj) + NP1 * (K - P * ck)) + comp * NN;
        const double* Erow = E + ((size_t)c * ND + a) * ND;
#pragma unroll
        for (int h = 0; h < BCH; ++h) {
          const int b = lane + 32 * h;
          if (b < ND) {
            const int bnode = b % NN, bcomp = b / NN;
            const int bi = bnode % NP1, bj = (bnode / NP1) % NP1, bk = bnode / (NP1 * NP1);
            const int Mi = P * ci + bi, Mj = P * cj + bj, Mk = P * ck + bk;
            // Dirichlet columns hold zeros (the integration stores them so): no lookup needed
            pos[q][h] = bcomp + ncomp * ((Mi - I - C.lo[0]) + C.w[0] * ((Mj - J - C.lo[1]) + C.w[1] * (Mk - K - C.lo[2])));
            v[q][h] = __ldcs(Erow + b);
          }
        }
        if (lane == q) evl = EV[c * ND + a];
      }
    }
    double rsum = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      if (q < ncell) {
        // the columns of one cell are distinct positions: lanes never collide within a cell
#pragma unroll
        for (int h = 0; h < BCH; ++h)
          if (pos[q][h] >= 0) acc[pos[q][h]] = acc[pos[q][h]] + v[q][h];
        rsum = rsum + __shfl_sync(0xffffffffu, evl, q);
        __syncwarp();
      }
    }
    if (lane == 0) rhs[r] = rsum;
  }
  __syncthreads();
  const int64_t vb = voff[sl];
  for (int k = threadIdx.x; k < 32 * Bp; k += W * 32) {
    const int grp = k >> 7, w = k & 127;
    const double x = s_slice[(w >> 2) * stride + grp * 4 + (w & 3)];
    tval[vb + k] = x;
    tval32[vb + k] = (float)x;
  }
}

// shared memory of k_scatter_stencil for the widest class (bytes)
static size_t scatter_stencil_smem(const fg_space* sp) { return sizeof(double) * 32 * (size_t)(sp->st_max_bp + 4); }

bool stencil_direct_ok(const fg_space* sp) {
  return sp->layout == FG_LAYOUT_STENCIL && !sp->dg && !sp->explicit_nodes && sp->mesh->dim == 3 &&
         sp->st_max_bp > 0 && scatter_stencil_smem(sp) <= 110 * 1024;
}

template <int P, int NC>
static fg_status launch_scatter_stencil(fg_system* sys, const AsmGeom& g) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  constexpr int W = 8;
  const size_t smem = scatter_stencil_smem(sp);
  // scalar Q1/Q2 rows: four blocks per SM (64 registers, a 4-byte spill; the shared slices
  // take 4 x 34 KB).  The gather is latency-bound: at 128^3 Q2 the row gather takes ~22.5 ms
  // at two blocks, 17.9 ms at three, ~14.5 ms at four (identical results: only the register
  // allocation changes).  Q3 and vector rows would spill heavily.
  constexpr int MINB = (NC == 1 && P <= 2) ? 4 : 1;
  auto kern = k_scatter_stencil<P, NC, W, MINB>;
  FG_CUDA_TRY(cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (sp->st_nslices > 0) {
    ctx->launches += 1;
    kern<<<(unsigned)sp->st_nslices, W * 32, smem, ctx->stream>>>(
        g, sp->d_st_scls, sp->d_st_voff, sp->d_st_cls, sp->d_st_slot2row, sp->d_free2lat, sp->d_latdof, sys->d_elmat, sys->d_elvec,
        sys->d_tval, sys->d_tval32, sys->d_rhs);
    FG_CUDA_TRY(cudaGetLastError());
  }
  sys->direct = true;
  return FG_OK;
}

// Physical coordinates of every cell's quadrature points: x_q = sum_k N_k(xi_q) x_k with the
// trilinear geometry, in the integration kernels' summation order (cell_map quadrature-point
// coordinates, sbm_cell_map.i90:673-686).  Thread per (cell, point); xyz[(c*nq + q)*3 + l].
__global__ void k_qp_coords(AsmGeom g, int64_t ncells, int nq, const double* __restrict__ coords,
                            const double* __restrict__ gshp, double* __restrict__ xyz) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= ncells * nq) return;
  const int64_t c = t / nq;
  const int q = (int)(t % nq);
  int ci = 0, cj = 0, ck = 0;
  if (!g.cellvert) {
    ci = (int)(c % g.n[0]);
    cj = (int)((c / g.n[0]) % g.n[1]);
    ck = (int)(c / ((int64_t)g.n[0] * g.n[1]));
  }
  double x0 = 0.0, x1 = 0.0, x2 = 0.0;
  for (int k = 0; k < 8; ++k) {
    const int64_t v = asm_vertex(g, c, ci, cj, ck, k);
    const double a = gshp[k * nq + q];
    x0 = x0 + a * coords[v * 3 + 0];
    x1 = x1 + a * coords[v * 3 + 1];
    x2 = x2 + a * coords[v * 3 + 2];
  }
  xyz[t * 3 + 0] = x0;
  xyz[t * 3 + 1] = x1;
  xyz[t * 3 + 2] = x2;
}

fg_status space_qp_coords(fg_space* sp, double* d_xyz) {
  if (sp->mesh->dim != 3) {
    set_error("quadrature-point coordinates are exported for 3D hexahedral meshes");
    return FG_ERR_UNSUPPORTED;
  }
  const int64_t total = sp->mesh->ncells * sp->tab.nq;
  if (total == 0) return FG_OK;
  AsmGeom g = make_geom(sp);
  k_qp_coords<<<(unsigned)((total + 255) / 256), 256, 0, sp->mesh->ctx->stream>>>(
      g, sp->mesh->ncells, sp->tab.nq, sp->mesh->d_coords, sp->dtab.gshp, d_xyz);
  FG_CUDA_TRY(cudaGetLastError());
  sp->mesh->ctx->launches += 1;
  return FG_OK;
}

__global__ void k_dirichlet_values(int64_t ndir, const double* xyz, int fn, SourceSpec prm, double* gv) {
  int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (d >= ndir) return;
  gv[d] = boundary_value(fn, prm.prm, xyz + d * 3);
}

static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

fg_status system_interpolate_dirichlet(fg_system* sys, int boundary_fn, const double* prm) {
  fg_space* sp = sys->space;
  if (sp->mesh->dim == 2) return q2_interpolate_dirichlet(sys, boundary_fn, prm);
  fg_ctx* ctx = sp->mesh->ctx;
  if (sp->ndir == 0) return FG_OK;
  double* xyz = nullptr;
  FG_TRY(dev_alloc(ctx, (void**)&xyz, sizeof(double) * 3 * sp->ndir));
  fg_status st = space_dirichlet_coords(sp, xyz);
  if (st == FG_OK) {
    SourceSpec s;
    s.fn = boundary_fn;
    for (int i = 0; i < 8; ++i) s.prm[i] = prm[i];
    s.qp = nullptr;
    k_dirichlet_values<<<nblk(sp->ndir, 256), 256, 0, ctx->stream>>>(sp->ndir, xyz, boundary_fn, s, sys->d_gvals);
    ctx->launches += 2;  // coordinates + values
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { set_error("dirichlet values: %s", cudaGetErrorString(e)); st = FG_ERR_CUDA; }
  }
  cudaStreamSynchronize(ctx->stream);
  dev_free(ctx, xyz);
  return st;
}

template <int P>
static fg_status poisson_scatter(fg_system* sys, const AsmGeom& g) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  const int64_t n = sp->nfree;
  if (sp->dg) return dg_assemble_rows(sys);
  if (sp->explicit_nodes) return usystem_scatter(sys);
  sys->direct = false;
  if (!sys->lean && stencil_direct_ok(sp) && sys->d_tval && sys->d_tval32) return launch_scatter_stencil<P, 1>(sys, g);
  if (n > 0) {
    constexpr int CAP = P == 1 ? 32 : (P == 2 ? 128 : 512);
    ctx->launches += 1;
    k_scatter_rows<P, CAP><<<nblk(n, 8), 256, 0, ctx->stream>>>(g, n, sp->d_free2lat, sp->d_latdof, sp->d_rowptr,
                                                                 sp->d_col, sys->d_elmat, sys->d_elvec, sys->d_val,
                                                                 sys->d_val32, sys->d_rhs);
    FG_CUDA_TRY(cudaGetLastError());
  }
  return FG_OK;
}

// FG_TC_INTEGRATION: 0 the FP64-pipe and float-float kernels only; 1 Poisson element
// matrices on the tensor cores where FP64 integration is asked for; 2 (default) also where
// float-float is (FG_FAST_INTEGRATION): the tensor-core matrices are FP64-accurate and, on
// GB300, faster than both (128^3 Q2: 61 / 48 ms per assembly against 186 ms FP64, 84 ms
// float-float)
static int tc_integration_mode() {
  const char* e = getenv("FG_TC_INTEGRATION");
  const int v = e ? atoi(e) : 2;
  return v < 0 ? 0 : (v > 2 ? 2 : v);
}

// scratch of the tensor-core path: G (cells x K), the packed upper triangles (cells x pairs),
// the product's workspace and its error flag, 256-byte aligned pieces
static size_t tc_align(size_t b) { return (b + 255) / 256 * 256; }

template <int P>
static fg_status launch_poisson_tc(fg_system* sys) {
  using T = PoissonTC<P>;
  constexpr int NQ = T::NQ, ND = T::ND, NPAIR = T::NPAIR, K = T::K;
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  cudaStream_t st = ctx->stream;
  const int64_t ncells = sp->mesh->ncells;
  if (!sp->d_tcT) {
    // T[p][6q + m] for the row-packed upper pairs p = (a, b), b >= a
    std::vector<double> hT((size_t)NPAIR * K);
    const std::vector<double>& r = sp->tab.shg;  // (a NQ + q) 3 + j
    size_t p = 0;
    for (int a = 0; a < ND; ++a)
      for (int b = a; b < ND; ++b, ++p)
        for (int q = 0; q < NQ; ++q) {
          const double* ra = &r[((size_t)a * NQ + q) * 3];
          const double* rb = &r[((size_t)b * NQ + q) * 3];
          double* t = &hT[p * K + 6 * q];
          t[0] = ra[0] * rb[0];
          t[1] = ra[1] * rb[1];
          t[2] = ra[2] * rb[2];
          t[3] = ra[0] * rb[1] + ra[1] * rb[0];
          t[4] = ra[0] * rb[2] + ra[2] * rb[0];
          t[5] = ra[1] * rb[2] + ra[2] * rb[1];
        }
    FG_TRY(dev_alloc(ctx, (void**)&sp->d_tcT, sizeof(double) * hT.size()));
    FG_CUDA_TRY(cudaMemcpyAsync(sp->d_tcT, hT.data(), sizeof(double) * hT.size(), cudaMemcpyHostToDevice, st));
    FG_CUDA_TRY(cudaStreamSynchronize(st));
  }
  const size_t gbytes = tc_align(sizeof(double) * ncells * K), cbytes = tc_align(sizeof(double) * ncells * NPAIR);
  const size_t wbytes = tc_align(ozaki_workspace_bytes(ncells, NPAIR, K, false));
  const size_t need = gbytes + cbytes + wbytes + 256;
  if (!sys->d_tcbuf || sys->tcbuf_bytes < need) {
    dev_free(ctx, sys->d_tcbuf);
    sys->d_tcbuf = nullptr;
    sys->tcbuf_bytes = 0;
    FG_TRY(dev_alloc(ctx, &sys->d_tcbuf, need));
    sys->tcbuf_bytes = need;
  }
  const bool ff = (sys->integ.flags & FG_FAST_INTEGRATION) != 0;
  if (ff && !sp->d_tcff) {
    // float-float tables of the geometry kernel: Q1 geometry gradients, shape values, weights
    using F = PoissonTCFF<P>;
    std::vector<float> h(F::TAB);
    auto split = [&](const std::vector<double>& src, size_t n, float* hi, float* lo) {
      for (size_t i = 0; i < n; ++i) {
        hi[i] = (float)src[i];
        lo[i] = (float)(src[i] - (double)hi[i]);
      }
    };
    float* t = h.data();
    split(sp->tab.gshg, F::G3, t, t + F::G3);
    split(sp->tab.shp, F::SH, t + 2 * F::G3, t + 2 * F::G3 + F::SH);
    split(sp->tab.qw, NQ, t + 2 * (F::G3 + F::SH), t + 2 * (F::G3 + F::SH) + NQ);
    FG_TRY(dev_alloc(ctx, (void**)&sp->d_tcff, sizeof(float) * h.size()));
    FG_CUDA_TRY(cudaMemcpyAsync(sp->d_tcff, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice, st));
    FG_CUDA_TRY(cudaStreamSynchronize(st));
  }
  double* G = (double*)sys->d_tcbuf;
  double* Cp = (double*)((uint8_t*)sys->d_tcbuf + gbytes);
  void* work = (uint8_t*)sys->d_tcbuf + gbytes + cbytes;
  int* d_err = (int*)((uint8_t*)work + wbytes);
  AsmGeom g = make_geom(sp);
  SourceSpec src;
  src.fn = sys->integ.source_fn;
  for (int i = 0; i < 8; ++i) src.prm[i] = sys->integ.fn_param[i];
  src.qp = sys->d_qpsrc;
  if (ff) {
    using F = PoissonTCFF<P>;
    const size_t smem = F::SM_BYTES_WARP * F::WARPS;
    FG_CUDA_TRY(cudaFuncSetAttribute((const void*)k_poisson_geom_ff<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
    k_poisson_geom_ff<P><<<nblk(ncells, F::WARPS), F::WARPS * 32, smem, st>>>(
        g, ncells, sp->mesh->d_coords, sp->dtab, sp->d_tcff, sys->d_coef, sys->integ.coef_const, src, G, sys->d_elvec);
  } else {
    const size_t smem = T::SM_BYTES_WARP * T::WARPS;
    FG_CUDA_TRY(cudaFuncSetAttribute((const void*)k_poisson_geom<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
    k_poisson_geom<P><<<nblk(ncells, T::WARPS), T::WARPS * 32, smem, st>>>(g, ncells, sp->mesh->d_coords, sp->dtab,
                                                                         sp->d_latdof, sys->d_coef,
                                                                         sys->integ.coef_const, src, G, sys->d_elvec);
  }
  FG_CUDA_TRY(cudaGetLastError());
  FG_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), st));
  FG_TRY(ozaki_gemm_nt(ctx, st, ncells, NPAIR, K, 1.0, G, K, 1, sp->d_tcT, K, 1, 0.0, Cp, NPAIR, 1, false, work, d_err));
  k_poisson_unpack<P><<<nblk(ncells, 8), 256, 0, st>>>(g, ncells, sp->d_latdof, sys->d_gvals, Cp, sys->d_elmat,
                                                       sys->d_elvec);
  FG_CUDA_TRY(cudaGetLastError());
  ctx->launches += 2;
  int h_err = 0;
  FG_CUDA_TRY(cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  FG_CUDA_TRY(cudaStreamSynchronize(st));
  if (h_err) {
    set_error("element matrices on the tensor cores: a bounded device wait ran out");
    return (fg_status)h_err;
  }
  return poisson_scatter<P>(sys, g);
}

template <int P>
static fg_status launch_poisson(fg_system* sys) {
  using S = PoissonShape<P>;
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  const bool ff = (sys->integ.flags & FG_FAST_INTEGRATION) != 0;
  const int tcm = tc_integration_mode();
  if (!sp->dg && sp->mesh->ncells > 0 && (ff ? tcm == 2 : tcm >= 1)) {
    // the tensor-core path needs scratch (G, packed triangles, digits: ~7 KB per Q2 cell);
    // where the context's HBM budget has no room for it, the direct kernels run instead
    const fg_status s = launch_poisson_tc<P>(sys);
    if (s != FG_ERR_OOM) return s;
  }
  AsmGeom g = make_geom(sp);
  const int64_t ncells = sp->mesh->ncells;
  SourceSpec src;
  src.fn = sys->integ.source_fn;
  for (int i = 0; i < 8; ++i) src.prm[i] = sys->integ.fn_param[i];
  src.qp = sys->d_qpsrc;
  using SF = typename PoissonShapeSel<P, true>::type;
  const int warps = ff ? SF::WARPS : S::WARPS;
  const size_t smem = ff ? SF::SM_BYTES_WARP * SF::WARPS : S::SM_BYTES_WARP * S::WARPS;
  auto kern = ff ? k_integrate_poisson<P, true> : k_integrate_poisson<P, false>;
  FG_CUDA_TRY(cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const unsigned grid = nblk(ncells, warps);
  ctx->launches += 1;
  kern<<<grid, warps * 32, smem, ctx->stream>>>(g, ncells, sp->mesh->d_coords, sp->dtab, sp->d_latdof,
                                                sys->d_gvals, sys->d_coef, sys->integ.coef_const, src,
                                                sys->d_elmat, sys->d_elvec);
  FG_CUDA_TRY(cudaGetLastError());
  return poisson_scatter<P>(sys, g);
}

// ---------------------------------------------------------------------------
// Linear elasticity (vector Q_P, 3 components), one warp per cell.
// Reference integrand (Sources/Tests/Par/par_test_pb_bddc_linear_elasticity/modules/
// sbm_irreducible_heterogeneous_discrete_integration.i90:57-84): per Gauss point and dof
// pair, elmat(i,j) += dV grad(phi_i) : (lambda tr(eps_j) I + 2 mu eps_j), eps_j =
// sym(grad(phi_j)), with lambda = nu E/((1+nu)(1-2nu)), mu = E/(2(1+nu)) per cell.  For
// dofs (node a, component ci) and (node b, component cj) this is
//   dV [lambda g_a[ci] g_b[cj] + mu g_a[cj] g_b[ci] + mu delta_{ci cj} g_a.g_b],
// so with s = sqrt(dV) g and A_ab = sum_q s_a s_b^T (3x3, 9 FP64 FMAs per node pair and
// Gauss point) the 3x3 block of the node pair is lambda A + mu A^T + mu tr(A) I.
// Cell-local dof order: node + component*NN (component-major), as in the reference.
template <int P>
struct ElastShape {
  static constexpr int NP1 = P + 1;
  static constexpr int NN = NP1 * NP1 * NP1;
  static constexpr int NQ = NN;
  static constexpr int ND = 3 * NN;
  static constexpr int NPAIR = NN * (NN + 1) / 2;
  static constexpr int CH = P == 1 ? 2 : 4;  // node pairs per lane per pass
  static constexpr int WARPS = P == 1 ? 8 : P == 2 ? 3 : 2;
  // Q3: the 192 x 192 element matrix (288 KB) does not fit in shared memory; it is written
  // straight to its slot in HBM and read back from there for the Dirichlet lifting
  static constexpr bool EL_GLOBAL = P >= 3;
  static constexpr int SM_XV = 24, SM_INVJ = NQ * 9, SM_FAC = NQ, SM_XQ = NQ * 3, SM_F = NQ * 3, SM_SQ = NQ,
                       SM_G = NQ * NN * 3, SM_EL = EL_GLOBAL ? 0 : ND * ND;
  static constexpr int SM_DOUBLES = SM_XV + SM_INVJ + SM_FAC + SM_XQ + SM_F + SM_SQ + SM_G + SM_EL;
  static constexpr int SM_INTS = ND;
  static constexpr size_t SM_BYTES_WARP = ((size_t)SM_DOUBLES * 8 + SM_INTS * 4 + 15) / 16 * 16;
};

template <int P>
__global__ void __launch_bounds__(ElastShape<P>::WARPS * 32)
    k_integrate_elasticity(AsmGeom g, int64_t ncells, const double* __restrict__ coords, DevTables tb,
                           const int32_t* __restrict__ latdof, const double* __restrict__ gvals,
                           const double* __restrict__ coef, double coef_const, double nu, SourceSpec src,
                           double* __restrict__ E, double* __restrict__ EV) {
  using S = ElastShape<P>;
  constexpr int NN = S::NN, NQ = S::NQ, ND = S::ND;
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  double* base = smem + (size_t)wib * (S::SM_BYTES_WARP / 8);
  double* xv = base;
  double* invj = xv + S::SM_XV;
  double* fac = invj + S::SM_INVJ;
  double* xq = fac + S::SM_FAC;
  double* fsrc = xq + S::SM_XQ;
  double* sq = fsrc + S::SM_F;
  double* sg = sq + S::SM_SQ;
  int32_t* gid = (int32_t*)(sg + S::SM_G + S::SM_EL);

  const int64_t c = (int64_t)blockIdx.x * S::WARPS + wib;
  if (c >= ncells) return;
  double* const Ec = E + (size_t)c * ND * ND;
  double* const el = S::EL_GLOBAL ? Ec : sg + S::SM_G;
  const int ci = (int)(c % g.n[0]);
  const int cj = (int)((c / g.n[0]) % g.n[1]);
  const int ck = (int)(c / ((int64_t)g.n[0] * g.n[1]));
  const double Ev = coef ? coef[c] : coef_const;
  const double lambda = (nu * Ev) / ((1.0 + nu) * (1.0 - 2.0 * nu));
  const double mu = Ev / (2.0 * (1.0 + nu));

  if (lane < 24) {
    int k = lane / 3, l = lane % 3;
    xv[lane] = coords[asm_vertex(g, c, ci, cj, ck, k) * 3 + l];
  }
  for (int s = lane; s < ND; s += 32) {
    const int a = s % NN, comp = s / NN;
    gid[s] = latdof[asm_node<P>(g, c, ci, cj, ck, a) * 3 + comp];
  }
  __syncwarp();
  for (int q = lane; q < NQ; q += 32) {
    double J[9];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double a0 = 0.0, a1 = 0.0, a2 = 0.0;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        double alpha = tb.gshg[(k * NQ + q) * 3 + j];
        a0 = a0 + alpha * xv[k * 3 + 0];
        a1 = a1 + alpha * xv[k * 3 + 1];
        a2 = a2 + alpha * xv[k * 3 + 2];
      }
      J[0 + 3 * j] = a0; J[1 + 3 * j] = a1; J[2 + 3 * j] = a2;
    }
    double t1 = J[4] * J[8] - J[5] * J[7];
    double t2 = -J[1] * J[8] + J[2] * J[7];
    double t3 = J[1] * J[5] - J[2] * J[4];
    double det = J[0] * t1 + J[3] * t2 + J[6] * t3;
    double denom = 1.0 / det;
    double* b = invj + q * 9;
    b[0] = t1 * denom;
    b[1] = t2 * denom;
    b[2] = t3 * denom;
    b[4] = (J[0] * J[8] - J[2] * J[6]) * denom;
    b[5] = (-J[0] * J[5] + J[3] * J[2]) * denom;
    b[8] = (J[0] * J[4] - J[1] * J[3]) * denom;
    b[3] = (-J[3] * J[8] + J[5] * J[6]) * denom;
    b[6] = (J[3] * J[7] - J[4] * J[6]) * denom;
    b[7] = (-J[0] * J[7] + J[1] * J[6]) * denom;
    fac[q] = det;
    double x0 = 0.0, x1 = 0.0, x2 = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      double a = tb.gshp[k * NQ + q];
      x0 = x0 + a * xv[k * 3 + 0];
      x1 = x1 + a * xv[k * 3 + 1];
      x2 = x2 + a * xv[k * 3 + 2];
    }
    xq[q * 3 + 0] = x0; xq[q * 3 + 1] = x1; xq[q * 3 + 2] = x2;
  }
  __syncwarp();
  const bool neg = fac[0] < 0.0;
  __syncwarp();
  for (int q = lane; q < NQ; q += 32) {
    double d = neg ? fabs(fac[q]) : fac[q];
    fac[q] = d * tb.qw[q];
    for (int comp = 0; comp < 3; ++comp) {
      double f;
      if (src.fn == FG_FN_QP_VALUES) f = src.qp[(c * NQ + q) * 3 + comp];
      else if (src.fn == FG_FN_CONST) f = src.prm[comp];
      else f = 0.0;
      fsrc[q * 3 + comp] = f;
    }
    sq[q] = sqrt(fac[q]);
  }
  __syncwarp();
  for (int idx = lane; idx < NQ * NN; idx += 32) {
    int q = idx / NN, a = idx % NN;
    const double* rg = tb.shg + ((size_t)a * NQ + q) * 3;
    const double* b = invj + q * 9;
    const double s = sq[q];
    double r0 = rg[0], r1 = rg[1], r2 = rg[2];
#pragma unroll
    for (int i = 0; i < 3; ++i) sg[idx * 3 + i] = s * (b[0 + 3 * i] * r0 + b[1 + 3 * i] * r1 + b[2 + 3 * i] * r2);
  }
  __syncwarp();
  for (int pbase = 0; pbase < S::NPAIR; pbase += 32 * S::CH) {
    double A[S::CH][9];
    int pa[S::CH], pb[S::CH];
#pragma unroll
    for (int t = 0; t < S::CH; ++t) {
#pragma unroll
      for (int e = 0; e < 9; ++e) A[t][e] = 0.0;
      int p = pbase + lane + 32 * t;
      if (p < S::NPAIR) pair_ab(p, NN, pa[t], pb[t]);
      else { pa[t] = 0; pb[t] = 0; }
    }
    for (int q = 0; q < NQ; ++q) {
      const double* gq = sg + q * NN * 3;
#pragma unroll
      for (int t = 0; t < S::CH; ++t) {
        const double* sa = gq + pa[t] * 3;
        const double* sb = gq + pb[t] * 3;
        const double a0 = sa[0], a1 = sa[1], a2 = sa[2], b0 = sb[0], b1 = sb[1], b2 = sb[2];
        A[t][0] = fma(a0, b0, A[t][0]); A[t][1] = fma(a0, b1, A[t][1]); A[t][2] = fma(a0, b2, A[t][2]);
        A[t][3] = fma(a1, b0, A[t][3]); A[t][4] = fma(a1, b1, A[t][4]); A[t][5] = fma(a1, b2, A[t][5]);
        A[t][6] = fma(a2, b0, A[t][6]); A[t][7] = fma(a2, b1, A[t][7]); A[t][8] = fma(a2, b2, A[t][8]);
      }
    }
#pragma unroll
    for (int t = 0; t < S::CH; ++t) {
      int p = pbase + lane + 32 * t;
      if (p >= S::NPAIR) continue;
      const double tr = A[t][0] + A[t][4] + A[t][8];
#pragma unroll
      for (int u = 0; u < 3; ++u)
#pragma unroll
        for (int v = 0; v < 3; ++v) {
          double m = lambda * A[t][u * 3 + v] + mu * A[t][v * 3 + u];
          if (u == v) m = m + mu * tr;
          const int i = pa[t] + u * NN, j = pb[t] + v * NN;
          el[i * ND + j] = m;
          el[j * ND + i] = m;
        }
    }
  }
  __syncwarp();
  bool any_dir = false;
  for (int s = lane; s < ND; s += 32) any_dir |= gid[s] < 0;
  any_dir = __any_sync(0xffffffffu, any_dir);
  for (int i = lane; i < ND; i += 32) {
    const int a = i % NN, comp = i / NN;
    double ev = 0.0;
    for (int q = 0; q < NQ; ++q) ev = ev + fac[q] * (fsrc[q * 3 + comp] * tb.shp[(size_t)a * NQ + q]);
    if (any_dir)
      for (int j = 0; j < ND; ++j) {
        int32_t gj = gid[j];
        if (gj < 0) ev = ev - el[i * ND + j] * gvals[-gj - 1];
      }
    EV[c * ND + i] = ev;
  }
  // Dirichlet columns are spent on the lifting above: stored as zeros (see k_integrate_poisson)
  if (!S::EL_GLOBAL) {
    for (int idx = lane; idx < ND * ND; idx += 32) Ec[idx] = gid[idx % ND] < 0 ? 0.0 : el[idx];
  } else if (any_dir) {
    __syncwarp();
    for (int idx = lane; idx < ND * ND; idx += 32)
      if (gid[idx % ND] < 0) Ec[idx] = 0.0;
  }
}

template <int P>
static fg_status launch_elasticity(fg_system* sys) {
  using S = ElastShape<P>;
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  AsmGeom g = make_geom(sp);
  const int64_t ncells = sp->mesh->ncells;
  SourceSpec src;
  src.fn = sys->integ.source_fn;
  for (int i = 0; i < 8; ++i) src.prm[i] = sys->integ.fn_param[i];
  src.qp = sys->d_qpsrc;
  const size_t smem = S::SM_BYTES_WARP * S::WARPS;
  // per call: the attribute is per device, and server workers assemble concurrently
  FG_CUDA_TRY(cudaFuncSetAttribute(k_integrate_elasticity<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  ctx->launches += sp->nfree > 0 ? 2 : 1;
  k_integrate_elasticity<P><<<nblk(ncells, S::WARPS), S::WARPS * 32, smem, ctx->stream>>>(
      g, ncells, sp->mesh->d_coords, sp->dtab, sp->d_latdof, sys->d_gvals, sys->d_coef, sys->integ.coef_const,
      sys->integ.nu, src, sys->d_elmat, sys->d_elvec);
  FG_CUDA_TRY(cudaGetLastError());
  const int64_t n = sp->nfree;
  if (sp->explicit_nodes) return usystem_scatter(sys);
  sys->direct = false;
  if (!sys->lean && stencil_direct_ok(sp) && sys->d_tval && sys->d_tval32) return launch_scatter_stencil<P, 3>(sys, g);
  if (n > 0) {
    constexpr int CAP = P == 1 ? 128 : P == 2 ? 512 : 1056;  // (2P+1)^3 * 3 box entries, rounded up to 32
    constexpr int W = P == 3 ? 2 : 8;                         // warps (rows) per block: static smem <= 48 KB
    k_scatter_rows<P, CAP, W><<<nblk(n, W), W * 32, 0, ctx->stream>>>(
        g, n, sp->d_free2lat, sp->d_latdof, sp->d_rowptr, sp->d_col, sys->d_elmat, sys->d_elvec, sys->d_val,
        sys->d_val32, sys->d_rhs);
    FG_CUDA_TRY(cudaGetLastError());
  }
  return FG_OK;
}

fg_status system_assemble(fg_system* sys) {
  fg_space* sp = sys->space;
  if (sp->mesh->dim == 2) return q2_assemble(sys);
  if (sys->integ.kind == FG_ELASTICITY && sp->ncomp == 3) {
    switch (sp->order) {
      case 1: return launch_elasticity<1>(sys);
      case 2: return launch_elasticity<2>(sys);
      case 3: return launch_elasticity<3>(sys);
      default:
        set_error("elasticity of order %d is not built on the device (orders 1-3)", sp->order);
        return FG_ERR_UNSUPPORTED;
    }
  }
  if (sp->dg && (sys->integ.kind != FG_POISSON || sys->integ.cell_coef || sys->integ.coef_const != 1.0)) {
    set_error("the dG formulation is built for the Poisson integrand with k = 1 (tutorial_01)");
    return FG_ERR_UNSUPPORTED;
  }
  if (sys->integ.kind != FG_POISSON || sp->ncomp != 1) {
    set_error("integrand kind %d with %d components is not built", sys->integ.kind, sp->ncomp);
    return FG_ERR_UNSUPPORTED;
  }
  switch (sp->order) {
    case 1: return launch_poisson<1>(sys);
    case 2: return launch_poisson<2>(sys);
    case 3: return launch_poisson<3>(sys);
    default: set_error("order %d not built", sp->order); return FG_ERR_UNSUPPORTED;
  }
}

}  // namespace fg

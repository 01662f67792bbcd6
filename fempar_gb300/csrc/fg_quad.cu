// fg_quad.cu -- 2D structured meshes of quadrilaterals (num_dims = 2): dof numbering, the
// sparsity pattern, cell integration (Poisson and plane-strain elasticity), the row-gather
// assembly and the Dirichlet data.  The solver then runs on the explicit-column SELL layout.
//
// The reference's structured generator and FE space are dimension-generic
// (uniform_hex_mesh_generator.f90:145-647, sbm_serial_fe_space.i90:525-716,2623-2884): cells
// c = i + nx j, the quadrilateral's n-faces are the codes anchor | (free directions << 2) sorted
// by (dimension, code) -- 4 vertices, 4 edges, the interior -- and the boundary set ids are
// 1..8 (9 in the interior).  The numbering rules are those of the hexahedral path: a vef's
// first visitor is the lowest cell around it, so each cell's share of new ids is a
// closed-form count and an exclusive scan gives its first id.  The cell integrand and the
// lifting follow the same reference lines as the hexahedral kernels, with a 2 x 2 Jacobian
// (invmtx for n = 2, sbm_cell_integrator.i90:448-500).
#include "fg_internal.h"

namespace fg {

static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

struct Prm8 {
  double v[8];
};

struct Lat2 {
  int n[2];
  int Ln[2];
  int p, ncomp;
  uint32_t dirmask;
  int codes[9];
  int code2idx[16];
};

static Lat2 make_lat2(const fg_space* sp) {
  Lat2 g;
  for (int d = 0; d < 2; ++d) { g.n[d] = sp->mesh->n[d]; g.Ln[d] = sp->Ln[d]; }
  g.p = sp->order;
  g.ncomp = sp->ncomp;
  g.dirmask = sp->dirmask;
  for (int i = 0; i < 9; ++i) g.codes[i] = sp->tab.codes[i];
  for (int i = 0; i < 16; ++i) g.code2idx[i] = sp->tab.code2idx[i];
  return g;
}

// Boundary set id of the vef with free directions t anchored at lattice vertex (v0, v1).
__device__ __forceinline__ int q_set_id(const Lat2& g, int t, int v0, int v1) {
  const int v[2] = {v0, v1};
  int anchor = 0, tt = 0;
#pragma unroll
  for (int d = 0; d < 2; ++d) {
    if ((t >> d) & 1) tt |= 1 << d;
    else if (v[d] == 0) {
    } else if (v[d] == g.n[d]) anchor |= 1 << d;
    else tt |= 1 << d;
  }
  return g.code2idx[anchor | (tt << 2)] + 1;
}

// Is n-face `code` of cell (ci, cj) first visited by this cell?
__device__ __forceinline__ bool q_owns(int code, int ci, int cj) {
  const int a = code & 3, t = code >> 2;
  const int c[2] = {ci, cj};
#pragma unroll
  for (int d = 0; d < 2; ++d)
    if (!((t >> d) & 1) && !((a >> d) & 1) && c[d] != 0) return false;
  return true;
}

__global__ void k_q_count(Lat2 g, int64_t ncells, int64_t* cnt_free, int64_t* cnt_dir) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  const int ci = (int)(c % g.n[0]), cj = (int)(c / g.n[0]);
  const int pm1 = g.p - 1;
  int64_t nf = (int64_t)pm1 * pm1 * g.ncomp, nd = 0;
  for (int f = 0; f < 8; ++f) {
    const int code = g.codes[f];
    if (!q_owns(code, ci, cj)) continue;
    const int a = code & 3, t = code >> 2;
    int cnt = 1;
    for (int d = 0; d < 2; ++d)
      if ((t >> d) & 1) cnt *= pm1;
    if (cnt == 0) continue;
    const int sid = q_set_id(g, t, ci + (a & 1), cj + ((a >> 1) & 1));
    if ((g.dirmask >> sid) & 1u) nd += (int64_t)cnt * g.ncomp;
    else nf += (int64_t)cnt * g.ncomp;
  }
  cnt_free[c] = nf;
  cnt_dir[c] = nd;
}

__global__ void k_q_assign(Lat2 g, int64_t ncells, const int64_t* base_free, const int64_t* base_dir, int32_t* latdof,
                           int32_t* free2lat, int32_t* dir2lat) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  const int ci = (int)(c % g.n[0]), cj = (int)(c / g.n[0]);
  const int p = g.p;
  int64_t id = base_free[c], did = base_dir[c];
  // cell interior: component-major, nodes lexicographic
  for (int comp = 0; comp < g.ncomp; ++comp)
    for (int j = 1; j < p; ++j)
      for (int i = 1; i < p; ++i) {
        const int64_t L = (int64_t)(p * ci + i) + (int64_t)g.Ln[0] * (p * cj + j);
        const int32_t slot = (int32_t)(L * g.ncomp + comp);
        latdof[slot] = (int32_t)(++id);
        free2lat[id - 1] = slot;
      }
  for (int f = 0; f < 8; ++f) {
    const int code = g.codes[f];
    if (!q_owns(code, ci, cj)) continue;
    const int a = code & 3, t = code >> 2;
    const int c2[2] = {ci, cj};
    int lo[2], hi[2];
    bool empty = false;
    for (int d = 0; d < 2; ++d) {
      if ((t >> d) & 1) {
        lo[d] = p * c2[d] + 1;
        hi[d] = p * c2[d] + p - 1;
        if (hi[d] < lo[d]) empty = true;
      } else {
        lo[d] = hi[d] = p * c2[d] + ((a >> d) & 1) * p;
      }
    }
    if (empty) continue;
    const int sid = q_set_id(g, t, ci + (a & 1), cj + ((a >> 1) & 1));
    const bool dir = (g.dirmask >> sid) & 1u;
    for (int comp = 0; comp < g.ncomp; ++comp)
      for (int J = lo[1]; J <= hi[1]; ++J)
        for (int I = lo[0]; I <= hi[0]; ++I) {
          const int64_t L = (int64_t)I + (int64_t)g.Ln[0] * J;
          const int32_t slot = (int32_t)(L * g.ncomp + comp);
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

// Lattice range of the cells around lattice coordinate I (one direction).
__device__ __forceinline__ void q_box(int I, int p, int n, int& lo, int& hi) {
  const int c = I / p;
  int clo = (I % p == 0) ? c - 1 : c, chi = c;
  if (clo < 0) clo = 0;
  if (chi > n - 1) chi = n - 1;
  lo = clo * p;
  hi = (chi + 1) * p;
}

__global__ void k_q_row_len(Lat2 g, int64_t nfree, const int32_t* free2lat, const int32_t* latdof, int64_t* row_len) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nfree) return;
  const int64_t L = free2lat[r] / g.ncomp;
  const int I = (int)(L % g.Ln[0]), J = (int)(L / g.Ln[0]);
  int lo[2], hi[2];
  q_box(I, g.p, g.n[0], lo[0], hi[0]);
  q_box(J, g.p, g.n[1], lo[1], hi[1]);
  int64_t cnt = 0;
  for (int y = lo[1]; y <= hi[1]; ++y)
    for (int x = lo[0]; x <= hi[0]; ++x) {
      const int64_t M = (int64_t)x + (int64_t)g.Ln[0] * y;
      for (int c = 0; c < g.ncomp; ++c) cnt += latdof[M * g.ncomp + c] > 0;
    }
  row_len[r] = cnt;
}

// One warp per row: the free dofs of the box, sorted (bitonic in shared memory).
constexpr int kQCap = 128;  // (2p+1)^2 * ncomp <= 98 for p <= 3, ncomp <= 2
__global__ void __launch_bounds__(128)
    k_q_row_fill(Lat2 g, int64_t nfree, const int32_t* free2lat, const int32_t* latdof, const int64_t* rowptr,
                 int32_t* col) {
  __shared__ int32_t s_keys[4][kQCap];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  int32_t* keys = s_keys[wib];
  const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (r >= nfree) return;
  const int64_t L = free2lat[r] / g.ncomp;
  const int I = (int)(L % g.Ln[0]), J = (int)(L / g.Ln[0]);
  int lo[2], hi[2];
  q_box(I, g.p, g.n[0], lo[0], hi[0]);
  q_box(J, g.p, g.n[1], lo[1], hi[1]);
  const int bx = hi[0] - lo[0] + 1, by = hi[1] - lo[1] + 1;
  const int total = bx * by * g.ncomp;
  for (int t = lane; t < kQCap; t += 32) {
    int32_t key = 0x7fffffff;
    if (t < total) {
      const int comp = t % g.ncomp, q = t / g.ncomp;
      const int64_t M = (int64_t)(lo[0] + q % bx) + (int64_t)g.Ln[0] * (lo[1] + q / bx);
      const int32_t id = latdof[M * g.ncomp + comp];
      if (id > 0) key = id - 1;
    }
    keys[t] = key;
  }
  __syncwarp();
  for (int k = 2; k <= kQCap; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = lane; t < kQCap; t += 32) {
        const int u = t ^ j;
        if (u > t) {
          const int32_t a = keys[t], b = keys[u];
          const bool up = (t & k) == 0;
          if ((a > b) == up) {
            keys[t] = b;
            keys[u] = a;
          }
        }
      }
      __syncwarp();
    }
  const int64_t s = rowptr[r], len = rowptr[r + 1] - s;
  for (int t = lane; t < len; t += 32) col[s + t] = keys[t];
}

__global__ void k_q_cell_dof_map(Lat2 g, int64_t ncells, int nn, int nd, const int32_t* latdof, int32_t* out) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= ncells * nd) return;
  const int64_t c = idx / nd;
  const int s = (int)(idx % nd), comp = s / nn, a = s % nn, np1 = g.p + 1;
  const int ci = (int)(c % g.n[0]), cj = (int)(c / g.n[0]);
  const int64_t L = (int64_t)(g.p * ci + a % np1) + (int64_t)g.Ln[0] * (g.p * cj + a / np1);
  out[idx] = latdof[L * g.ncomp + comp];
}

// Physical coordinates of a lattice node through the bilinear map of the last cell (in cell
// order) that contains it (sbm_serial_fe_space.i90:1140-1152: the last write wins).
__device__ void q_node_xy(const Lat2& g, const double* coords, int64_t L, double* x) {
  const int IJ[2] = {(int)(L % g.Ln[0]), (int)(L / g.Ln[0])};
  int c[2];
  double xi[2];
  for (int d = 0; d < 2; ++d) {
    c[d] = IJ[d] / g.p;
    if (c[d] > g.n[d] - 1) c[d] = g.n[d] - 1;
    xi[d] = (2.0 / g.p) * (IJ[d] - g.p * c[d]) - 1.0;
  }
  x[0] = x[1] = x[2] = 0.0;
  for (int k = 0; k < 4; ++k) {
    const int bx = k & 1, by = (k >> 1) & 1;
    const double a = (bx ? 0.5 * (1 + xi[0]) : 0.5 * (1 - xi[0])) * (by ? 0.5 * (1 + xi[1]) : 0.5 * (1 - xi[1]));
    const int64_t v = (int64_t)(c[0] + bx) + (int64_t)(g.n[0] + 1) * (c[1] + by);
    for (int l = 0; l < 3; ++l) x[l] = x[l] + a * coords[v * 3 + l];
  }
}

__global__ void k_q_dirichlet_coords(Lat2 g, int64_t ndir, const int32_t* dir2lat, const double* coords, double* xyz) {
  const int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (d >= ndir) return;
  double x[3];
  q_node_xy(g, coords, dir2lat[d] / g.ncomp, x);
  for (int l = 0; l < 3; ++l) xyz[d * 3 + l] = x[l];
}

// The drivers' analytic functions in 2D (tutorial_01 modules :395-533, test_poisson
// poisson_analytical_functions.f90:71-124).
__device__ double q_value(int fn, const double* prm, const double* x) {
  switch (fn) {
    case FG_FN_CONST: return prm[0];
    case FG_FN_LINEAR: return x[0] + x[1];
    case FG_FN_SHARP_WAVE: {
      const double dx = x[0] - prm[2], dy = x[1] - prm[3];
      return atan(prm[0] * (sqrt(dx * dx + dy * dy) - prm[1]));
    }
    default: return 0.0;
  }
}

__device__ double q_sharp_source(const double* prm, const double* x) {
  const double alpha = prm[0], r = prm[1];
  const double alpha_2 = alpha * alpha, alpha_3 = alpha_2 * alpha;
  const double x_minus_xc_2 = (x[0] - prm[2]) * (x[0] - prm[2]);
  const double y_minus_yc_2 = (x[1] - prm[3]) * (x[1] - prm[3]);
  const double term1 = x_minus_xc_2 + y_minus_yc_2;
  const double sqrt_term1 = sqrt(term1);
  const double term2 = sqrt_term1 - r;
  const double a2t = alpha_2 * term2 * term2 + 1.0;
  const double denom1 = sqrt_term1 * a2t, denom2 = pow(term1, 1.5) * a2t, denom3 = term1 * a2t * a2t;
  const double dx2 = alpha / denom1 - (alpha * x_minus_xc_2) / denom2 - (2.0 * alpha_3 * x_minus_xc_2 * term2) / denom3;
  const double dy2 = alpha / denom1 - (alpha * y_minus_yc_2) / denom2 - (2.0 * alpha_3 * y_minus_yc_2 * term2) / denom3;
  return -dx2 - dy2;
}

__global__ void k_q_dirichlet_values(int64_t ndir, const double* xyz, int fn, Prm8 prm, double* gv) {
  const int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (d >= ndir) return;
  gv[d] = q_value(fn, prm.v, xyz + d * 3);
}

// ---------------------------------------------------------------------------------------
// Cell integration, one warp per cell.  Poisson (NC = 1): elmat += |J| w k grad(phi_j).grad(phi_i),
// elvec += |J| w f phi_i (tutorial modules :114-128).  Plane-strain elasticity (NC = 2): for dofs
// (node a, comp ci), (node b, comp cj) the integrand dV grad(phi_i) : (lambda tr(eps_j) I +
// 2 mu eps_j) is dV [lambda g_a[ci] g_b[cj] + mu g_a[cj] g_b[ci] + mu delta_{ci cj} g_a.g_b]
// (sbm_irreducible_discrete_integration.i90:100-121).  Strong Dirichlet lifting
// (sbm_fe_cell_iterator.i90:1610-1637).  Element matrices are written row-major (c, i, j).
template <int P, int NC>
struct QShape {
  static constexpr int NP1 = P + 1, NN = NP1 * NP1, NQ = NN, ND = NN * NC;
  static constexpr int WARPS = 4;
  static constexpr int SM_DOUBLES = 12 + NQ * 4 + NQ + NQ * 2 + NQ * NN * 2 + ND * ND + NQ * NC;
  static constexpr size_t SM_BYTES_WARP = ((size_t)SM_DOUBLES * 8 + ND * 4 + 15) / 16 * 16;
};

template <int P, int NC>
__global__ void __launch_bounds__(128)
    k_q_integrate(Lat2 g, int64_t ncells, const double* __restrict__ coords, DevTables tb,
                  const int32_t* __restrict__ latdof, const double* __restrict__ gvals,
                  const double* __restrict__ coef, double coef_const, double nu, int sfn, Prm8 sprm,
                  const double* __restrict__ qpsrc, double* __restrict__ E, double* __restrict__ EV) {
  using S = QShape<P, NC>;
  constexpr int NN = S::NN, NQ = S::NQ, ND = S::ND, NP1 = S::NP1;
  extern __shared__ double qsm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  double* xv = qsm + (size_t)wib * (S::SM_BYTES_WARP / 8);  // 4 vertices x 3
  double* invj = xv + 12;                                    // per qp: B(1,1) B(2,1) B(1,2) B(2,2)
  double* det = invj + NQ * 4;
  double* xq = det + NQ;
  double* gr = xq + NQ * 2;     // physical gradients (node, qp, 2)
  double* el = gr + NQ * NN * 2;
  double* fq = el + ND * ND;    // source per qp and component
  int32_t* gid = (int32_t*)(fq + NQ * NC);
  const int64_t c = (int64_t)blockIdx.x * S::WARPS + wib;
  if (c >= ncells) return;
  const int ci = (int)(c % g.n[0]), cj = (int)(c / g.n[0]);
  if (lane < 12) {
    const int k = lane / 3, l = lane % 3;
    xv[lane] = coords[((int64_t)(ci + (k & 1)) + (int64_t)(g.n[0] + 1) * (cj + (k >> 1))) * 3 + l];
  }
  for (int s = lane; s < ND; s += 32) {
    const int a = s % NN, comp = s / NN;
    const int64_t L = (int64_t)(P * ci + a % NP1) + (int64_t)g.Ln[0] * (P * cj + a / NP1);
    gid[s] = latdof[L * NC + comp];
  }
  __syncwarp();
  for (int q = lane; q < NQ; q += 32) {
    // J(l, j) = sum_k dN_k/dxi_j x_k(l); invmtx for n = 2
    double J[2][2];
    for (int j = 0; j < 2; ++j)
      for (int l = 0; l < 2; ++l) {
        double acc = 0.0;
        for (int k = 0; k < 4; ++k) acc = acc + tb.gshg[(k * NQ + q) * 3 + j] * xv[k * 3 + l];
        J[l][j] = acc;
      }
    const double dt = J[0][0] * J[1][1] - J[1][0] * J[0][1];
    const double denom = 1.0 / dt;
    invj[q * 4 + 0] = J[1][1] * denom;   // B(1,1)
    invj[q * 4 + 1] = -J[1][0] * denom;  // B(2,1)
    invj[q * 4 + 2] = -J[0][1] * denom;  // B(1,2)
    invj[q * 4 + 3] = J[0][0] * denom;   // B(2,2)
    det[q] = dt;
    double x0 = 0.0, x1 = 0.0;
    for (int k = 0; k < 4; ++k) {
      const double a = tb.gshp[k * NQ + q];
      x0 = x0 + a * xv[k * 3 + 0];
      x1 = x1 + a * xv[k * 3 + 1];
    }
    xq[q * 2 + 0] = x0;
    xq[q * 2 + 1] = x1;
  }
  __syncwarp();
  const bool neg = det[0] < 0.0;
  __syncwarp();
  for (int q = lane; q < NQ; q += 32) {
    const double d = (neg ? fabs(det[q]) : det[q]) * tb.qw[q];
    det[q] = d;
    const double xx[3] = {xq[q * 2], xq[q * 2 + 1], 0.0};
    for (int comp = 0; comp < NC; ++comp) {
      double f = 0.0;
      if (sfn == FG_FN_QP_VALUES) f = NC == 1 ? qpsrc[c * NQ + q] : qpsrc[(c * NQ + q) * NC + comp];
      else if (sfn == FG_FN_CONST) f = sprm.v[NC == 1 ? 0 : comp];
      else if (sfn == FG_FN_SHARP_WAVE && NC == 1) f = q_sharp_source(sprm.v, xx);
      fq[q * NC + comp] = f;
    }
  }
  for (int idx = lane; idx < NQ * NN; idx += 32) {
    const int q = idx / NN, a = idx % NN;
    const double* rg = tb.shg + ((size_t)a * NQ + q) * 3;
    const double* b = invj + q * 4;
    // grad_i = sum_j B(j, i) dphi/dxi_j
    gr[idx * 2 + 0] = b[0] * rg[0] + b[1] * rg[1];
    gr[idx * 2 + 1] = b[2] * rg[0] + b[3] * rg[1];
  }
  __syncwarp();
  const double kc = coef ? coef[c] : coef_const;
  const double lambda = (nu * kc) / ((1.0 + nu) * (1.0 - 2.0 * nu)), mu = kc / (2.0 * (1.0 + nu));
  for (int e = lane; e < ND * ND; e += 32) {
    const int i = e / ND, j = e % ND;
    const int na = i % NN, ca = i / NN, nb = j % NN, cb = j / NN;
    double acc = 0.0;
    for (int q = 0; q < NQ; ++q) {
      const double* ga = gr + (q * NN + na) * 2;
      const double* gb = gr + (q * NN + nb) * 2;
      double v;
      if (NC == 1) {
        v = (det[q] * kc) * (gb[0] * ga[0] + gb[1] * ga[1]);
      } else {
        double m = lambda * ga[ca] * gb[cb] + mu * ga[cb] * gb[ca];
        if (ca == cb) m = m + mu * (ga[0] * gb[0] + ga[1] * gb[1]);
        v = det[q] * m;
      }
      acc = acc + v;
    }
    el[e] = acc;
  }
  __syncwarp();
  bool any_dir = false;
  for (int s = lane; s < ND; s += 32) any_dir |= gid[s] < 0;
  any_dir = __any_sync(0xffffffffu, any_dir);
  for (int i = lane; i < ND; i += 32) {
    const int a = i % NN, comp = i / NN;
    double ev = 0.0;
    for (int q = 0; q < NQ; ++q) ev = ev + det[q] * (fq[q * NC + comp] * tb.shp[(size_t)a * NQ + q]);
    if (any_dir)
      for (int j = 0; j < ND; ++j) {
        const int32_t gj = gid[j];
        if (gj < 0) ev = ev - el[i * ND + j] * gvals[-gj - 1];
      }
    EV[c * ND + i] = ev;
  }
  double* Ec = E + (size_t)c * ND * ND;
  for (int e = lane; e < ND * ND; e += 32) Ec[e] = el[e];
}

// One warp per free row: the row's entries from the element matrices of the cells around its
// node, in increasing cell order (the order of the reference's COO append and sort).
template <int P, int NC>
__global__ void __launch_bounds__(128)
    k_q_scatter(Lat2 g, int64_t nfree, const int32_t* __restrict__ free2lat, const int32_t* __restrict__ latdof,
                const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col, const double* __restrict__ E,
                const double* __restrict__ EV, double* __restrict__ val, double* __restrict__ rhs) {
  constexpr int NP1 = P + 1, NN = NP1 * NP1, ND = NN * NC;
  __shared__ int32_t s_col[4][kQCap];
  __shared__ double s_acc[4][kQCap];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t r = (int64_t)blockIdx.x * 4 + wib;
  if (r >= nfree) return;
  const int32_t slot = free2lat[r];
  const int64_t L = slot / NC;
  const int comp = slot % NC;
  const int I = (int)(L % g.Ln[0]), J = (int)(L / g.Ln[0]);
  const int64_t s = rowptr[r];
  const int len = (int)(rowptr[r + 1] - s);
  int32_t* cols = s_col[wib];
  double* acc = s_acc[wib];
  for (int t = lane; t < kQCap; t += 32) {
    cols[t] = t < len ? col[s + t] : 0x7fffffff;
    acc[t] = 0.0;
  }
  __syncwarp();
  int clo[2], chi[2];
  const int IJ[2] = {I, J};
  for (int d = 0; d < 2; ++d) {
    const int cc = IJ[d] / P;
    clo[d] = (IJ[d] % P == 0) ? cc - 1 : cc;
    chi[d] = cc;
    if (clo[d] < 0) clo[d] = 0;
    if (chi[d] > g.n[d] - 1) chi[d] = g.n[d] - 1;
  }
  double rsum = 0.0;
  for (int cj = clo[1]; cj <= chi[1]; ++cj)
    for (int ci = clo[0]; ci <= chi[0]; ++ci) {
      const int64_t c = (int64_t)ci + (int64_t)g.n[0] * cj;
      const int a = (I - P * ci) + NP1 * (J - P * cj) + comp * NN;
      const double* Erow = E + ((size_t)c * ND + a) * ND;
      for (int b = lane; b < ND; b += 32) {
        const int bn = b % NN, bc = b / NN;
        const int64_t M = (int64_t)(P * ci + bn % NP1) + (int64_t)g.Ln[0] * (P * cj + bn / NP1);
        const int32_t id = latdof[M * NC + bc];
        if (id > 0) {
          const int32_t key = id - 1;
          int lo = 0, hi = len;
          while (lo < hi) {
            const int m = (lo + hi) >> 1;
            if (cols[m] < key) lo = m + 1;
            else hi = m;
          }
          if (lo < len) acc[lo] = acc[lo] + Erow[b];
        }
      }
      if (lane == 0) rsum = rsum + EV[c * ND + a];
      __syncwarp();
    }
  for (int t = lane; t < len; t += 32) val[s + t] = acc[t];
  if (lane == 0) rhs[r] = rsum;
}

// ---------------------------------------------------------------------------------------
// Host side

fg_status q2_number_dofs(fg_space* sp) {
  fg_ctx* ctx = sp->mesh->ctx;
  const Lat2 g = make_lat2(sp);
  const int64_t ncells = sp->mesh->ncells;
  int64_t *cf = nullptr, *cd = nullptr;
  FG_TRY(dev_alloc(ctx, (void**)&cf, sizeof(int64_t) * ncells));
  FG_TRY(dev_alloc(ctx, (void**)&cd, sizeof(int64_t) * ncells));
  k_q_count<<<nblk(ncells, 256), 256, 0, ctx->stream>>>(g, ncells, cf, cd);
  FG_CUDA_TRY(cudaGetLastError());
  int64_t nfree = 0, ndir = 0;
  FG_TRY(scan_i64(ctx, cf, ncells, &nfree));
  FG_TRY(scan_i64(ctx, cd, ncells, &ndir));
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
  k_q_assign<<<nblk(ncells, 128), 128, 0, ctx->stream>>>(g, ncells, cf, cd, sp->d_latdof, sp->d_free2lat,
                                                           sp->d_dir2lat);
  FG_CUDA_TRY(cudaGetLastError());
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, cf);
  dev_free(ctx, cd);
  return FG_OK;
}

fg_status q2_build_pattern(fg_space* sp) {
  fg_ctx* ctx = sp->mesh->ctx;
  const Lat2 g = make_lat2(sp);
  const int64_t n = sp->nfree;
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_rowptr, sizeof(int64_t) * (n + 1)));
  if (n == 0) {  // no free dofs: an empty pattern (row pointer 0, a one-slot column array)
    FG_CUDA_TRY(cudaMemsetAsync(sp->d_rowptr, 0, sizeof(int64_t), ctx->stream));
    FG_TRY(dev_alloc(ctx, (void**)&sp->d_col, sizeof(int32_t)));
    sp->nnz = 0;
    return FG_OK;
  }
  k_q_row_len<<<nblk(n, 256), 256, 0, ctx->stream>>>(g, n, sp->d_free2lat, sp->d_latdof, sp->d_rowptr);
  FG_CUDA_TRY(cudaGetLastError());
  int64_t nnz = 0;
  FG_TRY(scan_i64(ctx, sp->d_rowptr, n, &nnz));
  FG_CUDA_TRY(cudaMemcpyAsync(sp->d_rowptr + n, &nnz, sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
  sp->nnz = nnz;
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_col, sizeof(int32_t) * (nnz > 0 ? nnz : 1)));
  k_q_row_fill<<<nblk(n, 4), 128, 0, ctx->stream>>>(g, n, sp->d_free2lat, sp->d_latdof, sp->d_rowptr, sp->d_col);
  FG_CUDA_TRY(cudaGetLastError());
  sp->box_cap = kQCap;
  return space_count_upper(sp);
}

fg_status q2_export_dof_map(fg_space* sp, int32_t* out_host) {
  fg_ctx* ctx = sp->mesh->ctx;
  const int64_t total = sp->mesh->ncells * sp->tab.nd;
  int32_t* d = nullptr;
  FG_TRY(dev_alloc(ctx, (void**)&d, sizeof(int32_t) * (total > 0 ? total : 1)));
  k_q_cell_dof_map<<<nblk(total, 256), 256, 0, ctx->stream>>>(make_lat2(sp), sp->mesh->ncells, sp->tab.nn,
                                                               sp->tab.nd, sp->d_latdof, d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out_host, d, sizeof(int32_t) * total, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  dev_free(ctx, d);
  if (e != cudaSuccess) {
    set_error("dof map export: %s", cudaGetErrorString(e));
    return FG_ERR_CUDA;
  }
  return FG_OK;
}

fg_status q2_dirichlet_coords(fg_space* sp, double* d_xyz) {
  if (sp->ndir == 0) return FG_OK;
  k_q_dirichlet_coords<<<nblk(sp->ndir, 256), 256, 0, sp->mesh->ctx->stream>>>(make_lat2(sp), sp->ndir,
                                                                                sp->d_dir2lat, sp->mesh->d_coords,
                                                                                d_xyz);
  FG_CUDA_TRY(cudaGetLastError());
  return FG_OK;
}

fg_status q2_interpolate_dirichlet(fg_system* sys, int boundary_fn, const double* prm) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  if (sp->ndir == 0) return FG_OK;
  double* xyz = nullptr;
  FG_TRY(dev_alloc(ctx, (void**)&xyz, sizeof(double) * 3 * sp->ndir));
  fg_status st = q2_dirichlet_coords(sp, xyz);
  if (st == FG_OK) {
    Prm8 p8;
    for (int i = 0; i < 8; ++i) p8.v[i] = prm[i];
    k_q_dirichlet_values<<<nblk(sp->ndir, 256), 256, 0, ctx->stream>>>(sp->ndir, xyz, boundary_fn, p8,
                                                                        sys->d_gvals);
    ctx->launches += 2;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error("dirichlet values: %s", cudaGetErrorString(e));
      st = FG_ERR_CUDA;
    }
  }
  dev_free(ctx, xyz);
  return st;
}

template <int P, int NC>
static fg_status q2_launch(fg_system* sys) {
  using S = QShape<P, NC>;
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  const Lat2 g = make_lat2(sp);
  const int64_t ncells = sp->mesh->ncells;
  Prm8 p8;
  for (int i = 0; i < 8; ++i) p8.v[i] = sys->integ.fn_param[i];
  const size_t smem = S::SM_BYTES_WARP * S::WARPS;
  FG_CUDA_TRY(cudaFuncSetAttribute(k_q_integrate<P, NC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_q_integrate<P, NC><<<nblk(ncells, S::WARPS), S::WARPS * 32, smem, ctx->stream>>>(
      g, ncells, sp->mesh->d_coords, sp->dtab, sp->d_latdof, sys->d_gvals, sys->d_coef, sys->integ.coef_const,
      sys->integ.nu, sys->integ.source_fn, p8, sys->d_qpsrc, sys->d_elmat, sys->d_elvec);
  FG_CUDA_TRY(cudaGetLastError());
  ctx->launches += 1;
  if (sp->nfree > 0) {
    k_q_scatter<P, NC><<<nblk(sp->nfree, 4), 128, 0, ctx->stream>>>(g, sp->nfree, sp->d_free2lat, sp->d_latdof,
                                                                    sp->d_rowptr, sp->d_col, sys->d_elmat,
                                                                    sys->d_elvec, sys->d_val, sys->d_rhs);
    FG_CUDA_TRY(cudaGetLastError());
    ctx->launches += 1;
  }
  return FG_OK;
}

fg_status q2_assemble(fg_system* sys) {
  fg_space* sp = sys->space;
  const int nc = sp->ncomp;
  if (sys->integ.kind == FG_POISSON && nc == 1) {
    switch (sp->order) {
      case 1: return q2_launch<1, 1>(sys);
      case 2: return q2_launch<2, 1>(sys);
      case 3: return q2_launch<3, 1>(sys);
    }
  } else if (sys->integ.kind == FG_ELASTICITY && nc == 2) {
    switch (sp->order) {
      case 1: return q2_launch<1, 2>(sys);
      case 2: return q2_launch<2, 2>(sys);
      case 3: return q2_launch<3, 2>(sys);
    }
  }
  set_error("2D: integrand kind %d with %d components and order %d is not built", sys->integ.kind, nc, sp->order);
  return FG_ERR_UNSUPPORTED;
}

}  // namespace fg

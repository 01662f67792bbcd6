// fempar_oracle.cpp -- CPU restatement of FEMPAR's serial FE assembly + CG path.
//
// TEST INFRASTRUCTURE ONLY (the checker for the GPU path; see fempar_oracle.h for
// the list of reference files and lines each part follows).  The code is written
// to reproduce the reference's results, in its operation order where rounding can
// be affected, on structured hexahedral (3D) and quadrilateral (2D) meshes.
//
// Parity of the dof numbering / sparsity / matrix entries is pinned by this
// restatement of the reference algorithm (the reference's own tests do not pin
// them); quadrature, integration, Dirichlet interpolation and the solve are
// pinned against the reference's own tables (tests/golden).
#include "fempar_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// std::vector allocator that leaves new elements uninitialised, so the large CSR arrays are
// first touched by the threads that fill them instead of being zeroed serially.
template <class T>
struct NoInit : std::allocator<T> {
  template <class U> struct rebind { using other = NoInit<U>; };
  NoInit() = default;
  template <class U> NoInit(const NoInit<U>&) noexcept {}
  template <class U, class... A> void construct(U* q, A&&... a) { ::new ((void*)q) U(std::forward<A>(a)...); }
  template <class U> void construct(U* q) noexcept { ::new ((void*)q) U; }
};

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

int popcount(int x) { int c = 0; while (x) { c += x & 1; x >>= 1; } return c; }

// ---------------------------------------------------------------------------
// Polytope n-faces of the hypercube.  A code holds the anchor vertex in the low
// `dim` bits and the free ("extruded") directions in the next `dim` bits; the
// list is sorted by (n-face dimension, code).
// sbm_polytope.i90:175-269 (polytope_create / sort_n_faces / fill_polytope_chain)
// ---------------------------------------------------------------------------
std::vector<int> polytope_codes(int dim) {
  std::vector<int> codes;
  for (int t = 0; t < (1 << dim); ++t)
    for (int a = 0; a < (1 << dim); ++a)
      if ((a & t) == 0) codes.push_back(a | (t << dim));
  std::sort(codes.begin(), codes.end(), [dim](int x, int y) {
    int dx = popcount(x >> dim), dy = popcount(y >> dim);
    if (dx != dy) return dx < dy;
    return x < y;
  });
  return codes;
}

// ---------------------------------------------------------------------------
// Reference Lagrangian hex FE: nodes (lexicographic, x fastest), own dofs per
// n-face (interior nodes, node-iterator order: lowest free direction fastest),
// vector components appended component-major.
// sbm_polytope.i90:396-433,640-860; sbm_lagrangian_reference_fe.i90:1072-1153,1240-1285,1549-1758
// ---------------------------------------------------------------------------
struct RefFE {
  int dim = 3, order = 1, ncomp = 1;
  int nnodes = 0, nshape = 0, nfaces = 0;
  std::vector<int> codes;
  std::vector<std::vector<int>> own;  // per n-face (0-based, volume last): local shape ids (0-based)
  std::vector<int> node_ijk;          // nnodes*3

  void build(int d, int p, int nc) {
    dim = d; order = p; ncomp = nc;
    int np1 = p + 1;
    nnodes = 1;
    for (int i = 0; i < d; ++i) nnodes *= np1;
    nshape = nnodes * nc;
    node_ijk.assign(nnodes * 3, 0);
    for (int n = 0; n < nnodes; ++n) {
      int r = n;
      for (int i = 0; i < d; ++i) { node_ijk[n * 3 + i] = r % np1; r /= np1; }
    }
    codes = polytope_codes(d);
    nfaces = (int)codes.size();
    own.assign(nfaces, {});
    for (int f = 0; f < nfaces; ++f) {
      int code = codes[f];
      int anchor = code & ((1 << d) - 1), type = code >> d;
      std::vector<int> freed;
      for (int i = 0; i < d; ++i) if ((type >> i) & 1) freed.push_back(i);
      std::vector<int> nodes;
      // odometer over free directions, first free direction fastest, range [1,p-1]
      std::vector<int> disp(freed.size(), 1);
      bool empty = false;
      for (size_t k = 0; k < freed.size(); ++k) if (p - 1 < 1) empty = true;
      if (!empty) {
        while (true) {
          int ijk[3] = {0, 0, 0};
          for (int i = 0; i < d; ++i) if (!((type >> i) & 1)) ijk[i] = ((anchor >> i) & 1) ? p : 0;
          for (size_t k = 0; k < freed.size(); ++k) ijk[freed[k]] = disp[k];
          int lex = 0, mul = 1;
          for (int i = 0; i < d; ++i) { lex += ijk[i] * mul; mul *= np1; }
          nodes.push_back(lex);
          size_t k = 0;
          for (; k < freed.size(); ++k) {
            if (++disp[k] <= p - 1) break;
            disp[k] = 1;
          }
          if (k == freed.size()) break;
        }
      }
      for (int c = 0; c < nc; ++c)
        for (int n : nodes) own[f].push_back(n + c * nnodes);
    }
  }
  int comp_of(int s) const { return s / nnodes; }
  int node_of(int s) const { return s % nnodes; }
};

// ---------------------------------------------------------------------------
// Gauss-Legendre nodes/weights on [-1,1], ascending.  The reference uses the
// Glaser-Liu-Rokhlin method (sbm_quadrature.i90:825-1334); this restatement uses
// Newton iteration on P_n, which converges to the same nodes to machine precision
// (checked against test_quadratures.f90's table in tests/).
// ---------------------------------------------------------------------------
void gauss_legendre(int n, double* x, double* w) {
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    double z = std::cos(pi * (i + 0.75) / (n + 0.5));
    double dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      if (n == 0) p1 = 1.0;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1; p1 = p2;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1; p1 = p2;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
    }
    x[n - 1 - i] = z;
    w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
  if (n == 1) { x[0] = 0.0; w[0] = 2.0; }
  // exact symmetry
  for (int i = 0; i < n / 2; ++i) {
    double a = 0.5 * (x[n - 1 - i] - x[i]);
    x[i] = -a; x[n - 1 - i] = a;
    double b = 0.5 * (w[i] + w[n - 1 - i]);
    w[i] = b; w[n - 1 - i] = b;
  }
  if (n % 2 == 1) x[n / 2] = 0.0;
}

// 1D Lagrange polynomial on equispaced nodes (2/p)i-1, value/1st/2nd derivative
// evaluated with the reference's product recurrence (sbm_polynomial.i90:61-109).
struct Lagrange1D {
  int order;
  std::vector<std::vector<double>> coef;  // per polynomial: order roots + scale
  void build(int p) {
    order = p;
    std::vector<double> nc(p + 1);
    for (int i = 0; i <= p; ++i) nc[i] = i;
    if (p > 0) for (int i = 0; i <= p; ++i) nc[i] = (2.0 / p) * nc[i] - 1.0;
    coef.assign(p + 1, std::vector<double>(p + 1, 0.0));
    for (int i = 0; i <= p; ++i) {
      int c = 0;
      for (int j = 0; j <= p; ++j) if (j != i) coef[i][c++] = nc[j];
      double s = 1.0;
      for (int j = 0; j <= p; ++j) if (j != i) s = s * (nc[i] - nc[j]);
      coef[i][p] = 1.0 / s;
    }
  }
  void values(int i, double x, double* px) const {
    px[0] = 1.0; px[1] = 0.0; px[2] = 0.0;
    for (int k = 0; k < order; ++k) {
      for (int j = 2; j >= 1; --j) px[j] = px[j] * (x - coef[i][k]) + px[j - 1];
      px[0] = px[0] * (x - coef[i][k]);
    }
    px[2] = 2.0 * px[2];
    for (int j = 0; j < 3; ++j) px[j] = px[j] * coef[i][order];
  }
};

// Shape values and reference gradients of the tensor-product space at a set of
// points (sbm_tensor_product_polynomial.i90:28-120, sbm_hex_lagrangian_reference_fe.i90:173-231).
void tensor_shapes(int dim, int order, const std::vector<double>& pts /*npts*3*/, int npts,
                   std::vector<double>& val /*nn*npts*/, std::vector<double>& grad /*nn*npts*3*/) {
  Lagrange1D L; L.build(order);
  int np1 = order + 1, nn = 1;
  for (int i = 0; i < dim; ++i) nn *= np1;
  val.assign((size_t)nn * npts, 0.0);
  grad.assign((size_t)nn * npts * 3, 0.0);
  std::vector<double> w((size_t)3 * np1 * npts * 3);  // [d][j][q][deriv]
  for (int d = 0; d < dim; ++d)
    for (int j = 0; j < np1; ++j)
      for (int q = 0; q < npts; ++q) L.values(j, pts[q * 3 + d], &w[(((size_t)d * np1 + j) * npts + q) * 3]);
  auto W = [&](int d, int j, int q, int k) { return w[(((size_t)d * np1 + j) * npts + q) * 3 + k]; };
  for (int q = 0; q < npts; ++q)
    for (int s = 0; s < nn; ++s) {
      int ijk[3] = {0, 0, 0}, r = s;
      for (int d = 0; d < dim - 1; ++d) { ijk[d] = r % np1; r /= np1; }
      ijk[dim - 1] = r;
      double v = 1.0;
      for (int d = 0; d < dim; ++d) v = v * W(d, ijk[d], q, 0);
      val[(size_t)s * npts + q] = v;
      for (int d = 0; d < dim; ++d) {
        double g = W(d, ijk[d], q, 1);
        for (int e = 0; e < dim; ++e) if (e != d) g = g * W(e, ijk[e], q, 0);
        grad[((size_t)s * npts + q) * 3 + d] = g;
      }
    }
}

// 3x3 (or 2x2) inverse and determinant, sbm_cell_integrator.i90:448-500 (invmtx).
// a and b are column-major 3x3 (a[r + 3c] == a(r+1,c+1)).
void invmtx(int n, const double* a, double* b, double& deter) {
#define A(i, j) a[((i)-1) + 3 * ((j)-1)]
#define B(i, j) b[((i)-1) + 3 * ((j)-1)]
  if (n == 2) {
    deter = A(1, 1) * A(2, 2) - A(2, 1) * A(1, 2);
    if (deter != 0.0) {
      double denom = 1.0 / deter;
      B(1, 1) = A(2, 2) * denom;
      B(2, 2) = A(1, 1) * denom;
      B(2, 1) = -A(2, 1) * denom;
      B(1, 2) = -A(1, 2) * denom;
    }
    return;
  }
  double t1 = A(2, 2) * A(3, 3) - A(3, 2) * A(2, 3);
  double t2 = -A(2, 1) * A(3, 3) + A(3, 1) * A(2, 3);
  double t3 = A(2, 1) * A(3, 2) - A(3, 1) * A(2, 2);
  deter = A(1, 1) * t1 + A(1, 2) * t2 + A(1, 3) * t3;
  if (deter == 0.0) return;
  double denom = 1.0 / deter;
  B(1, 1) = t1 * denom;
  B(2, 1) = t2 * denom;
  B(3, 1) = t3 * denom;
  B(2, 2) = (A(1, 1) * A(3, 3) - A(3, 1) * A(1, 3)) * denom;
  B(3, 2) = (-A(1, 1) * A(3, 2) + A(1, 2) * A(3, 1)) * denom;
  B(3, 3) = (A(1, 1) * A(2, 2) - A(2, 1) * A(1, 2)) * denom;
  B(1, 2) = (-A(1, 2) * A(3, 3) + A(3, 2) * A(1, 3)) * denom;
  B(1, 3) = (A(1, 2) * A(2, 3) - A(2, 2) * A(1, 3)) * denom;
  B(2, 3) = (-A(1, 1) * A(2, 3) + A(2, 1) * A(1, 3)) * denom;
#undef A
#undef B
}

// Analytic functions of the drivers.
// tutorial_01_poisson_sharp_circular_wave_modules.f90:395-533 (sharp circular wave)
// test_poisson/modules/poisson_analytical_functions.f90:71-124 (linear)
double fn_value(int fn, const double* prm, int dim, const double* x) {
  switch (fn) {
    case ORC_FN_ZERO: return 0.0;
    case ORC_FN_CONST: return prm[0];
    case ORC_FN_LINEAR: return dim == 2 ? x[0] + x[1] : x[0] + x[1] + x[2];
    case ORC_FN_SHARP_WAVE: {
      double a = prm[0], r = prm[1];
      double dx = x[0] - prm[2], dy = x[1] - prm[3];
      if (dim == 2) return std::atan(a * (std::sqrt(dx * dx + dy * dy) - r));
      double dz = x[2] - prm[4];
      return std::atan(a * (std::sqrt(dx * dx + dy * dy + dz * dz) - r));
    }
  }
  return 0.0;
}

double sharp_wave_source(const double* prm, int dim, const double* x) {
  double alpha = prm[0], r = prm[1];
  double alpha_2 = alpha * alpha, alpha_3 = alpha_2 * alpha;
  double xc = prm[2], yc = prm[3], zc = prm[4];
  double x_minus_xc_2 = (x[0] - xc) * (x[0] - xc);
  double y_minus_yc_2 = (x[1] - yc) * (x[1] - yc);
  double term1, z_minus_zc_2 = 0.0;
  if (dim == 2) term1 = x_minus_xc_2 + y_minus_yc_2;
  else { z_minus_zc_2 = (x[2] - zc) * (x[2] - zc); term1 = x_minus_xc_2 + y_minus_yc_2 + z_minus_zc_2; }
  double sqrt_term1 = std::sqrt(term1);
  double term2 = sqrt_term1 - r;
  double term2_2 = term2 * term2;
  double denom1 = sqrt_term1 * (alpha_2 * term2_2 + 1.0);
  double denom2 = std::pow(term1, 1.5) * (alpha_2 * term2_2 + 1.0);
  double denom3 = term1 * (alpha_2 * term2_2 + 1.0) * (alpha_2 * term2_2 + 1.0);
  double dx2 = alpha / denom1 - (alpha * x_minus_xc_2) / denom2 - (2.0 * alpha_3 * x_minus_xc_2 * term2) / denom3;
  double dy2 = alpha / denom1 - (alpha * y_minus_yc_2) / denom2 - (2.0 * alpha_3 * y_minus_yc_2 * term2) / denom3;
  if (dim == 2) return -dx2 - dy2;
  double dz2 = alpha / denom1 - (alpha * z_minus_zc_2) / denom2 - (2.0 * alpha_3 * z_minus_zc_2 * term2) / denom3;
  return -dx2 - dy2 - dz2;
}

void fn_gradient(int fn, const double* prm, int dim, const double* x, double* g) {
  g[0] = g[1] = g[2] = 0.0;
  if (fn == ORC_FN_LINEAR) { g[0] = g[1] = 1.0; if (dim == 3) g[2] = 1.0; return; }
  if (fn == ORC_FN_SHARP_WAVE) {
    double alpha = prm[0], r = prm[1], alpha_2 = alpha * alpha;
    double xc = prm[2], yc = prm[3], zc = prm[4];
    double term1 = (x[0] - xc) * (x[0] - xc) + (x[1] - yc) * (x[1] - yc);
    if (dim == 3) term1 += (x[2] - zc) * (x[2] - zc);
    double sqrt_term1 = std::sqrt(term1);
    double term2 = sqrt_term1 - r, term2_2 = term2 * term2;
    g[0] = (alpha * (x[0] - xc)) / (sqrt_term1 * (alpha_2 * term2_2 + 1.0));
    g[1] = (alpha * (x[1] - yc)) / (sqrt_term1 * (alpha_2 * term2_2 + 1.0));
    if (dim == 3) g[2] = (alpha * (x[2] - zc)) / (sqrt_term1 * (alpha_2 * term2_2 + 1.0));
  }
}

}  // namespace

// ===========================================================================
struct orc_problem {
  orc_params p;
  int dim, order, ncomp;
  int n[3];
  int64_t ncells, nverts_lattice;
  RefFE fe, geo;
  int nd, nq, ngeo;
  std::vector<double> qx, qw;               // nq*3 reference qp coords, nq weights
  std::vector<double> shp, shg;             // fe: nnodes*nq values, nnodes*nq*3 reference gradients
  std::vector<double> gshp, gshg;           // geometry (Q1) at qps
  std::vector<double> gnod;                 // geometry Q1 shapes at fe nodes: 2^d * nnodes
  std::vector<double> coords;               // 3 * nverts_lattice
  std::vector<double> coef;                 // per cell
  std::vector<int32_t> gids;                // ncells*nd, reference convention
  int64_t nfree = 0, ndir = 0;
  std::vector<double> gvals;                // Dirichlet values, ndir
  // COO (upper, free only) and CSR
  int64_t coo_n = 0;
  std::vector<int64_t> irp;                 // nfree+1, 1-based
  std::vector<int32_t, NoInit<int32_t>> ja;  // 1-based
  std::vector<double, NoInit<double>> val;
  std::vector<double> rhs;
  double t_setup = 0, t_integrate = 0, t_compress = 0;
  std::vector<double> qp_source;            // copy of per-qp source if given
  // unstructured hexahedral mesh (GiD route): explicit cells, generated vefs
  bool unst = false;
  int64_t nverts_u = 0, nedges = 0, nfaces = 0, nvefs = 0;
  std::vector<int32_t> cellvert;            // ncells*8, 0-based vertex ids, lexicographic local order
  std::vector<int64_t> cellvef;             // ncells*26, 0-based vef gids (vertices, edges, faces)
  std::vector<int> vset;                    // nvefs boundary set ids

  int64_t vert_index(const int* v) const {
    return v[0] + (int64_t)(n[0] + 1) * (v[1] + (int64_t)(n[1] + 1) * (dim == 3 ? v[2] : 0));
  }
  void cell_ijk(int64_t c, int* ijk) const {
    ijk[0] = (int)(c % n[0]);
    int64_t r = c / n[0];
    ijk[1] = (int)(r % n[1]);
    ijk[2] = dim == 3 ? (int)(r / n[1]) : 0;
  }
  void cell_vertices(int64_t c, double* xv /*ngeo*3*/) const {
    if (unst) {
      for (int k = 0; k < 8; ++k)
        for (int l = 0; l < 3; ++l) xv[k * 3 + l] = coords[(size_t)cellvert[(size_t)c * 8 + k] * 3 + l];
      return;
    }
    int ijk[3];
    cell_ijk(c, ijk);
    for (int k = 0; k < ngeo; ++k) {
      int v[3] = {ijk[0] + (k & 1), ijk[1] + ((k >> 1) & 1), dim == 3 ? ijk[2] + ((k >> 2) & 1) : 0};
      int64_t vi = vert_index(v);
      for (int l = 0; l < 3; ++l) xv[k * 3 + l] = coords[vi * 3 + l];
    }
  }
};

namespace {

// Boundary set id of a global vef (uniform_hex_mesh_generator.f90:600-630).
int vef_set_id(const orc_problem& P, int type, const int* v, const std::vector<int>& codes) {
  int d = P.dim, anchor = 0, t = 0;
  for (int i = 0; i < d; ++i) {
    if (!((type >> i) & 1)) {
      if (v[i] == 0) {
      } else if (v[i] == P.n[i]) anchor |= 1 << i;
      else t |= 1 << i;
    } else t |= 1 << i;
  }
  int code = anchor | (t << d);
  for (size_t f = 0; f < codes.size(); ++f) if (codes[f] == code) return (int)f + 1;
  return 0;
}

// ---------------------------------------------------------------------------
// Unstructured hexahedral meshes (the mesh-data-files route of the serial triangulation,
// sbm_serial_triangulation.i90:120-188).
// Local vertices of n-face f of the hex: anchor | s for every subset s of its free directions.
std::vector<int> nface_vertices(int code) {
  int anchor = code & 7, t = code >> 3;
  std::vector<int> out;
  for (int s = 0; s < 8; ++s)
    if ((s & ~t) == 0) out.push_back(anchor | s);
  return out;
}
int nface_dim(int code) { return popcount(code >> 3); }

void generate_unstructured_topology(orc_problem& P, const orc_umesh* m) {
  const int64_t nc = P.ncells, nv = P.nverts_u;
  const std::vector<int>& codes = P.fe.codes;
  const int NV = 26;
  // cells around vertices, ascending (sbm_base_static_triangulation.i90:697-739)
  std::vector<std::vector<int64_t>> around(nv);
  for (int64_t c = 0; c < nc; ++c)
    for (int k = 0; k < 8; ++k) around[P.cellvert[c * 8 + k]].push_back(c);
  std::vector<std::vector<int>> fv(NV);
  for (int f = 0; f < NV; ++f) fv[f] = nface_vertices(codes[f]);
  auto sorted_gids = [&](int64_t c, int f) {
    std::vector<int64_t> g;
    for (int v : fv[f]) g.push_back(P.cellvert[c * 8 + v]);
    std::sort(g.begin(), g.end());
    return g;
  };
  // vefs: vertices keep their ids; edges, then faces, numbered on first appearance walking
  // the cells in order, later cells around the n-face's first vertex receive the same id
  // (sbm_fine_triangulation.i90:115-315)
  P.cellvef.assign((size_t)nc * NV, -1);
  for (int64_t c = 0; c < nc; ++c)
    for (int k = 0; k < 8; ++k) P.cellvef[c * NV + k] = P.cellvert[c * 8 + k];
  int64_t nvefs = nv;
  for (int dim = 1; dim <= 2; ++dim) {
    for (int64_t c = 0; c < nc; ++c)
      for (int f = 0; f < NV; ++f) {
        if (nface_dim(codes[f]) != dim || P.cellvef[c * NV + f] != -1) continue;
        const int64_t id = nvefs++;
        P.cellvef[c * NV + f] = id;
        std::vector<int64_t> gi = sorted_gids(c, f);
        const int64_t first = P.cellvert[c * 8 + fv[f][0]];
        for (int64_t c2 : around[first]) {
          if (c2 <= c) continue;
          for (int f2 = 0; f2 < NV; ++f2) {
            if (nface_dim(codes[f2]) != dim) continue;
            if (sorted_gids(c2, f2) == gi) { P.cellvef[c2 * NV + f2] = id; break; }
          }
        }
      }
    if (dim == 1) P.nedges = nvefs - nv;
    else P.nfaces = nvefs - nv - P.nedges;
  }
  P.nvefs = nvefs;
  // set ids of the given boundary vefs, in the given order (sbm_fine_triangulation.i90:317-444)
  P.vset.assign(nvefs, 0);
  for (int64_t ib = 0; ib < m->num_given_vefs; ++ib) {
    const int64_t b0 = m->given_vef_ptr[ib], nb = m->given_vef_ptr[ib + 1] - b0;
    const int sid = m->given_vef_set[ib];
    std::vector<int64_t> gv;
    for (int64_t k = 0; k < nb; ++k) gv.push_back((int64_t)m->given_vef_vertices[b0 + k] - 1);
    if (nb == 1) { P.vset[gv[0]] = sid; continue; }
    const int dim = nb == 2 ? 1 : 2;
    std::vector<int64_t> gs = gv;
    std::sort(gs.begin(), gs.end());
    bool done = false;
    for (int64_t c2 : around[gv[0]]) {
      for (int f2 = 0; f2 < NV && !done; ++f2) {
        if (nface_dim(codes[f2]) != dim || (int64_t)fv[f2].size() != nb) continue;
        if (sorted_gids(c2, f2) == gs) { P.vset[P.cellvef[c2 * NV + f2]] = sid; done = true; }
      }
      if (done) break;
    }
  }
  // boundary faces (one cell around) hand their set id to the edges and vertices of their
  // closure that have none, faces visited in gid order (sbm_fine_triangulation.i90:453-527)
  std::vector<int> ncell_around(nvefs, 0);
  std::vector<int64_t> first_cell(nvefs, -1);
  std::vector<int> first_pos(nvefs, -1);
  for (int64_t c = 0; c < nc; ++c)
    for (int f = 0; f < NV; ++f) {
      int64_t g = P.cellvef[c * NV + f];
      if (ncell_around[g]++ == 0) { first_cell[g] = c; first_pos[g] = f; }
    }
  for (int64_t g = nv + P.nedges; g < nvefs; ++g) {
    if (ncell_around[g] != 1) continue;
    const int sid = P.vset[g];
    const int64_t c = first_cell[g];
    const int fc = codes[first_pos[g]];
    for (int f = 0; f < NV; ++f) {
      const int code = codes[f];
      if (nface_dim(code) >= 2) continue;
      // sub-n-face of the facet: its vertices are a subset of the facet's
      bool sub = true;
      for (int v : fv[f]) {
        bool in = false;
        for (int w : nface_vertices(fc)) in = in || (w == v);
        sub = sub && in;
      }
      if (!sub) continue;
      int64_t s = P.cellvef[c * NV + f];
      if (P.vset[s] == 0) P.vset[s] = sid;
    }
  }
}

// Own dofs of a vef seen from cell c and from the cell that numbered them: node (i_k) of the
// vef in c and node (j_k) in the source are the same point once the corner vertices are matched
// (fetch_own_dofs_vef_from_source_fe, sbm_fe_cell_iterator.i90:736-856).
void fetch_unstructured(orc_problem& P, int64_t c, int f, int64_t sc, int sf) {
  const RefFE& fe = P.fe;
  const int p = P.order, code = fe.codes[f], scode = fe.codes[sf];
  int d[3], e[3], m = 0, m2 = 0;
  for (int i = 0; i < 3; ++i) if (((code >> 3) >> i) & 1) d[m++] = i;
  for (int i = 0; i < 3; ++i) if (((scode >> 3) >> i) & 1) e[m2++] = i;
  const int a = code & 7, a2 = scode & 7;
  auto corner = [&](int64_t cell, int anchor, const int* dirs, int bits) {
    int v = anchor;
    for (int k = 0; k < m; ++k) if ((bits >> k) & 1) v |= 1 << dirs[k];
    return P.cellvert[cell * 8 + v];
  };
  int M[4] = {0, 0, 0, 0};  // source corner bits -> corner bits in c
  for (int u = 0; u < (1 << m); ++u) {
    int32_t g = corner(sc, a2, e, u);
    for (int b = 0; b < (1 << m); ++b) if (corner(c, a, d, b) == g) M[u] = b;
  }
  int axis[2] = {0, 0}, flip[2] = {0, 0};
  for (int k = 0; k < m; ++k) {
    int diff = M[0] ^ M[1 << k];
    int r = 0;
    while (!((diff >> r) & 1)) ++r;
    axis[k] = r;
    flip[k] = (M[0] >> r) & 1;
  }
  int nn_f = 1;
  for (int k = 0; k < m; ++k) nn_f *= (p - 1);
  const std::vector<int>& t = fe.own[f];
  const std::vector<int>& s = fe.own[sf];
  if (nn_f == 0) return;
  for (int kn = 0; kn < nn_f; ++kn) {
    int i[2] = {0, 0}, r = kn;
    for (int k = 0; k < m; ++k) { i[k] = r % (p - 1) + 1; r /= (p - 1); }
    int kn2 = 0, mul = 1;
    for (int k = 0; k < m; ++k) {
      int j = flip[k] ? p - i[axis[k]] : i[axis[k]];
      kn2 += (j - 1) * mul;
      mul *= (p - 1);
    }
    for (int comp = 0; comp < fe.ncomp; ++comp)
      P.gids[(size_t)c * P.nd + t[comp * nn_f + kn]] = P.gids[(size_t)sc * P.nd + s[comp * nn_f + kn2]];
  }
}

void build_mesh_and_dofs(orc_problem& P) {
  const orc_params& p = P.p;
  P.dim = p.num_dims; P.order = p.order;
  P.ncomp = p.kind == ORC_ELASTICITY ? P.dim : 1;
  if (!P.unst) {
    P.n[0] = p.n[0]; P.n[1] = p.n[1]; P.n[2] = P.dim == 3 ? p.n[2] : 1;
    P.ncells = (int64_t)P.n[0] * P.n[1] * (P.dim == 3 ? P.n[2] : 1);
    P.nverts_lattice = (int64_t)(P.n[0] + 1) * (P.n[1] + 1) * (P.dim == 3 ? P.n[2] + 1 : 1);
  }
  P.fe.build(P.dim, P.order, P.ncomp);
  P.geo.build(P.dim, 1, 1);
  P.nd = P.fe.nshape;
  P.ngeo = P.geo.nnodes;
  int np1 = P.order + 1;
  P.nq = 1;
  for (int i = 0; i < P.dim; ++i) P.nq *= np1;
  // quadrature: degree 2p -> p+1 points per direction (sbm_lagrangian_reference_fe.i90:1414-1423,
  // sbm_hex_lagrangian_reference_fe.i90:320-327); x fastest (sbm_quadrature.i90:767-823)
  std::vector<double> x1(np1), w1(np1);
  gauss_legendre(np1, x1.data(), w1.data());
  P.qx.assign(P.nq * 3, 0.0);
  P.qw.assign(P.nq, 0.0);
  for (int q = 0; q < P.nq; ++q) {
    int i = q % np1, j = (q / np1) % np1, k = q / (np1 * np1);
    if (P.dim == 2) { P.qw[q] = w1[i] * w1[j]; P.qx[q * 3] = x1[i]; P.qx[q * 3 + 1] = x1[j]; }
    else { P.qw[q] = w1[i] * w1[j] * w1[k]; P.qx[q * 3] = x1[i]; P.qx[q * 3 + 1] = x1[j]; P.qx[q * 3 + 2] = x1[k]; }
  }
  tensor_shapes(P.dim, P.order, P.qx, P.nq, P.shp, P.shg);
  tensor_shapes(P.dim, 1, P.qx, P.nq, P.gshp, P.gshg);
  // geometry shapes at the FE nodes (nodal interpolation of Dirichlet data)
  {
    std::vector<double> npts(P.fe.nnodes * 3, 0.0), g;
    for (int nn = 0; nn < P.fe.nnodes; ++nn)
      for (int d = 0; d < P.dim; ++d)
        npts[nn * 3 + d] = P.order > 0 ? (2.0 / P.order) * P.fe.node_ijk[nn * 3 + d] - 1.0 : 0.0;
    tensor_shapes(P.dim, 1, npts, P.fe.nnodes, P.gnod, g);
  }
  // vertex coordinates: ijk/n mapped to the domain limits (uniform_hex_mesh_generator.f90:608-612,632-636)
  if (!P.unst) P.coords.assign(P.nverts_lattice * 3, 0.0);
  for (int64_t vi = 0; vi < (P.unst ? 0 : P.nverts_lattice); ++vi) {
    int64_t r = vi;
    int v[3];
    v[0] = (int)(r % (P.n[0] + 1)); r /= (P.n[0] + 1);
    v[1] = (int)(r % (P.n[1] + 1)); r /= (P.n[1] + 1);
    v[2] = (int)r;
    for (int d = 0; d < P.dim; ++d) {
      double c = (double)v[d] / (double)P.n[d];
      P.coords[vi * 3 + d] = (p.limits[2 * d + 1] - p.limits[2 * d]) * c + p.limits[2 * d];
    }
  }
  if (p.vertex_xyz && !P.unst)
    std::memcpy(P.coords.data(), p.vertex_xyz, sizeof(double) * 3 * P.nverts_lattice);
  P.coef.assign(P.ncells, 1.0);
  if (p.cell_coef) std::memcpy(P.coef.data(), p.cell_coef, sizeof(double) * P.ncells);

  // ---- dof numbering ----
  const RefFE& fe = P.fe;
  const int nvefs = fe.nfaces - 1;  // cell interior is the last n-face
  P.gids.assign((size_t)P.ncells * P.nd, 0);
  std::vector<char> is_dir_id(64, 0);
  for (int i = 0; i < p.n_dirichlet_ids; ++i)
    if (p.dirichlet_ids[i] >= 1 && p.dirichlet_ids[i] < 64) is_dir_id[p.dirichlet_ids[i]] = 1;
  const int ntypes = 1 << P.dim;
  const int64_t nkeys = P.unst ? P.nvefs : (int64_t)ntypes * P.nverts_lattice;
  auto vef_of = [&](int64_t c, int f, int* v, int& type) -> int64_t {
    if (P.unst) { type = fe.codes[f] >> 3; return P.cellvef[(size_t)c * 26 + f]; }
    int code = fe.codes[f];
    int anchor = code & (ntypes - 1);
    type = code >> P.dim;
    int ijk[3];
    P.cell_ijk(c, ijk);
    for (int d = 0; d < 3; ++d) v[d] = d < P.dim ? ijk[d] + ((anchor >> d) & 1) : 0;
    return (int64_t)type + ntypes * P.vert_index(v);
  };
  auto set_of = [&](int64_t key, int type, const int* v) {
    return P.unst ? P.vset[key] : vef_set_id(P, type, v, fe.codes);
  };
  auto fetch = [&](int64_t c, int f, int64_t src_c, int src_f) {
    if (P.unst) { fetch_unstructured(P, c, f, src_c, src_f); return; }
    // identity permutation: on a structured mesh all cells share one orientation,
    // so the k-th own dof of the n-face maps to the k-th own dof of the owner's n-face
    // (sbm_fe_cell_iterator.i90:736-856)
    const std::vector<int>& t = fe.own[f];
    const std::vector<int>& s = fe.own[src_f];
    for (size_t k = 0; k < t.size(); ++k)
      P.gids[(size_t)c * P.nd + t[k]] = P.gids[(size_t)src_c * P.nd + s[k]];
  };
  if (p.formulation == ORC_DG) {
    // dG space: every dof is a cell-interior own dof, numbered cell by cell in local order;
    // boundary data enter weakly (no strong Dirichlet dofs)
    for (int64_t c = 0; c < P.ncells; ++c)
      for (int s = 0; s < P.nd; ++s) P.gids[(size_t)c * P.nd + s] = (int32_t)(c * P.nd + s + 1);
    P.ndir = 0;
    P.nfree = P.ncells * P.nd;
    P.gvals.clear();
    return;
  }
  // (1) strong Dirichlet dofs, negative, first visit order (sbm_serial_fe_space.i90:525-716)
  {
    std::vector<int64_t> vis_cell(nkeys, -1);
    std::vector<int> vis_f(nkeys, -1);
    int64_t ndir = 0;
    for (int64_t c = 0; c < P.ncells; ++c) {
      for (int f = 0; f < nvefs; ++f) {
        int v[3], type;
        int64_t key = vef_of(c, f, v, type);
        int sid = set_of(key, type, v);
        if (sid == 0) continue;
        bool code = sid > 0 && sid < 64 && is_dir_id[sid] != 0;  // one condition per set id, all components
        int64_t prev = ndir;
        if (vis_cell[key] == -1) {
          for (int s : fe.own[f]) {
            int32_t& g = P.gids[(size_t)c * P.nd + s];
            if (g >= 0 && code) g = (int32_t)(-(++ndir));
          }
        }
        if (vis_cell[key] != -1) fetch(c, f, vis_cell[key], vis_f[key]);
        if (vis_cell[key] == -1 && prev < ndir) { vis_cell[key] = c; vis_f[key] = f; }
      }
    }
    P.ndir = ndir;
  }
  // (2) free dofs: cell interior first, then vefs in n-face order (sbm_serial_fe_space.i90:2623-2884)
  {
    std::vector<int64_t> own_cell(nkeys, -1);
    std::vector<int> own_f(nkeys, -1);
    int64_t cur = 0;
    for (int64_t c = 0; c < P.ncells; ++c) {
      for (int s : fe.own[nvefs]) P.gids[(size_t)c * P.nd + s] = (int32_t)(++cur);
      for (int f = 0; f < nvefs; ++f) {
        int v[3], type;
        int64_t key = vef_of(c, f, v, type);
        if (own_cell[key] == -1) {
          int64_t prev = cur;
          for (int s : fe.own[f]) {
            int32_t& g = P.gids[(size_t)c * P.nd + s];
            if (g >= 0) g = (int32_t)(++cur);
          }
          if (cur > prev) { own_cell[key] = c; own_f[key] = f; }
        } else {
          fetch(c, f, own_cell[key], own_f[key]);
        }
      }
    }
    P.nfree = cur;
  }
  // (3) nodal interpolation of the Dirichlet data (sbm_serial_fe_space.i90:997-1176); a vector
  // field takes the function's value for every component (the reference's elasticity test
  // functions give each component the same value: linear_elasticity_analytical_functions.f90
  // :128-142)
  P.gvals.assign(P.ndir, 0.0);
  if (P.ndir > 0) {
    std::vector<double> xv(P.ngeo * 3);
    for (int64_t c = 0; c < P.ncells; ++c) {
      bool any = false;
      for (int s = 0; s < P.nd; ++s) if (P.gids[(size_t)c * P.nd + s] < 0) { any = true; break; }
      if (!any) continue;
      P.cell_vertices(c, xv.data());
      for (int s = 0; s < P.nd; ++s) {
        int32_t g = P.gids[(size_t)c * P.nd + s];
        if (g >= 0) continue;
        int node = fe.node_of(s);
        double x[3] = {0, 0, 0};
        for (int k = 0; k < P.ngeo; ++k) {
          double a = P.gnod[(size_t)k * fe.nnodes + node];
          for (int l = 0; l < 3; ++l) x[l] = x[l] + a * xv[k * 3 + l];
        }
        P.gvals[-g - 1] = fn_value(p.boundary_fn, p.fn_param, P.dim, x);
      }
    }
  }
}

// Geometry at the quadrature points of one cell: inverse Jacobian (column-major
// 3x3 per qp), |det J| and physical qp coordinates.
// sbm_base_map.i90:91-106, field.f90:763-787, sbm_cell_map.i90:245-369
void cell_geometry(const orc_problem& P, int64_t c, std::vector<double>& invj, std::vector<double>& det,
                   std::vector<double>& xq) {
  std::vector<double> xv(P.ngeo * 3);
  P.cell_vertices(c, xv.data());
  invj.assign(P.nq * 9, 0.0);
  det.assign(P.nq, 0.0);
  xq.assign(P.nq * 3, 0.0);
  for (int q = 0; q < P.nq; ++q) {
    double J[9];
    for (int j = 0; j < 3; ++j) {
      for (int l = 0; l < 3; ++l) J[l + 3 * j] = 0.0;
      for (int k = 0; k < P.ngeo; ++k) {
        double alpha = P.gshg[((size_t)k * P.nq + q) * 3 + j];
        for (int l = 0; l < 3; ++l) J[l + 3 * j] = J[l + 3 * j] + alpha * xv[k * 3 + l];
      }
    }
    double* b = &invj[q * 9];
    for (int i = 0; i < 3; ++i) b[i + 3 * i] = 1.0;
    invmtx(P.dim, J, b, det[q]);
  }
  if (P.nq > 0 && det[0] < 0.0)
    for (int q = 0; q < P.nq; ++q) det[q] = std::fabs(det[q]);
  for (int q = 0; q < P.nq; ++q)
    for (int k = 0; k < P.ngeo; ++k) {
      double a = P.gshp[(size_t)k * P.nq + q];
      for (int l = 0; l < 3; ++l) xq[q * 3 + l] = xq[q * 3 + l] + a * xv[k * 3 + l];
    }
}

// Element matrix (column-major nd x nd) and vector of one cell, with the strong
// Dirichlet lifting applied to the vector.
void integrate_cell(const orc_problem& P, int64_t c, const std::vector<double>* invj0,
                    const std::vector<double>* det0, double* elmat, double* elvec) {
  const orc_params& p = P.p;
  const int nd = P.nd, nq = P.nq, nn = P.fe.nnodes;
  std::vector<double> invj, det, xq;
  cell_geometry(P, c, invj, det, xq);
  if (invj0) { invj = *invj0; det = *det0; }  // reference structured-mesh translation shortcut
  // physical gradients of the scalar shape functions (sbm_lagrangian_reference_fe.i90:1330-1342)
  std::vector<double> g((size_t)nn * nq * 3, 0.0);
  for (int q = 0; q < nq; ++q)
    for (int s = 0; s < nn; ++s)
      for (int i = 0; i < 3; ++i) {
        double acc = 0.0;
        for (int j = 0; j < 3; ++j) acc = acc + invj[q * 9 + j + 3 * i] * P.shg[((size_t)s * nq + q) * 3 + j];
        g[((size_t)s * nq + q) * 3 + i] = acc;
      }
  std::fill(elmat, elmat + (size_t)nd * nd, 0.0);
  std::fill(elvec, elvec + nd, 0.0);
  const double kc = P.coef[c];
  if (p.kind == ORC_POISSON) {
    for (int q = 0; q < nq; ++q) {
      // tutorial modules :114-128; a per-cell diffusion coefficient k scales the
      // bilinear form only: elmat += (factor*k) * grad(phi_j).grad(phi_i)
      double factor = det[q] * P.qw[q];
      double fk = factor * kc;
      for (int i = 0; i < nd; ++i)
        for (int j = 0; j < nd; ++j) {
          const double* gi = &g[((size_t)i * nq + q) * 3];
          const double* gj = &g[((size_t)j * nq + q) * 3];
          double dot = gj[0] * gi[0] + gj[1] * gi[1] + gj[2] * gi[2];
          elmat[i + (size_t)nd * j] = elmat[i + (size_t)nd * j] + fk * dot;
        }
      double f;
      if (p.source_fn == ORC_FN_SHARP_WAVE) f = sharp_wave_source(p.fn_param, P.dim, &xq[q * 3]);
      else if (p.source_fn == ORC_FN_QP_VALUES) f = P.qp_source[(size_t)c * nq + q];
      else if (p.source_fn == ORC_FN_CONST) f = p.fn_param[0];
      else f = 0.0;
      for (int i = 0; i < nd; ++i) elvec[i] = elvec[i] + factor * f * P.shp[(size_t)i * nq + q];
    }
  } else {
    // sbm_irreducible_discrete_integration.i90:100-121
    double E = kc, nu = p.nu;
    double lambda = (nu * E) / ((1.0 + nu) * (1.0 - 2.0 * nu));
    double mu = E / (2.0 * (1.0 + nu));
    const int dim = P.dim;
    for (int q = 0; q < nq; ++q) {
      double dV = det[q] * P.qw[q];
      double src[3] = {0, 0, 0};
      if (p.source_fn == ORC_FN_CONST) for (int d = 0; d < dim; ++d) src[d] = p.fn_param[d];
      else if (p.source_fn == ORC_FN_QP_VALUES) for (int d = 0; d < dim; ++d) src[d] = P.qp_source[((size_t)c * nq + q) * dim + d];
      for (int i = 0; i < nd; ++i) {
        int ci = P.fe.comp_of(i), ni = P.fe.node_of(i);
        const double* gi = &g[((size_t)ni * nq + q) * 3];
        double Gi[3][3] = {{0}};
        for (int a = 0; a < 3; ++a) Gi[a][ci] = gi[a];
        for (int j = 0; j < nd; ++j) {
          int cj = P.fe.comp_of(j), nj = P.fe.node_of(j);
          const double* gj = &g[((size_t)nj * nq + q) * 3];
          double Gj[3][3] = {{0}};
          for (int a = 0; a < 3; ++a) Gj[a][cj] = gj[a];
          double eps[3][3], tr = 0.0;
          for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) eps[a][b] = 0.5 * (Gj[a][b] + Gj[b][a]);
          for (int a = 0; a < 3; ++a) tr = tr + eps[a][a];
          double dc = 0.0;
          for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
              double sig = lambda * tr * (a == b ? 1.0 : 0.0) + 2.0 * mu * eps[a][b];
              dc = dc + Gi[a][b] * sig;
            }
          elmat[i + (size_t)nd * j] = elmat[i + (size_t)nd * j] + dV * dc;
        }
        elvec[i] = elvec[i] + dV * (src[ci] * P.shp[(size_t)ni * nq + q]);
      }
    }
  }
  // strong Dirichlet lifting (sbm_fe_cell_iterator.i90:1610-1637)
  for (int j = 0; j < nd; ++j) {
    int32_t gj = P.gids[(size_t)c * nd + j];
    if (gj < 0) {
      double gv = P.gvals[-gj - 1];
      for (int i = 0; i < nd; ++i) elvec[i] = elvec[i] - elmat[i + (size_t)nd * j] * gv;
    }
  }
}

// ---------------------------------------------------------------------------
// dG interior-penalty facet terms (tutorial_01 modules :146-322).  Facets are visited in
// order of first appearance (walking the cells, local faces in order); the left cell is the
// smaller cell id (cells around a vef are ascending).  Geometry per facet quadrature point:
//   facet map: x, dx/ds, dx/dt from the left cell's face vertices, normal = dx/ds x dx/dt,
//     |n| = area element, n/|n| times the orientation factor that makes it the left cell's
//     outward normal (sbm_facet_map.i90:74-128, sbm_reference_fe.i90:523-543);
//   each cell: its reference point (the right cell's through the face's shared corners),
//     Jacobian, inverse, shape values and physical gradients;
//   h = min over the cells of 2 (prod_i |grad xi_i|^-1)^(1/3) (sbm_cell_map.i90:429-461,
//     sbm_facet_integrator.i90:248-264).
struct FacetSide { int64_t c; int f; };

int64_t cell_vertex_id(const orc_problem& P, int64_t c, int k) {
  if (P.unst) return P.cellvert[(size_t)c * 8 + k];
  int ijk[3];
  P.cell_ijk(c, ijk);
  int v[3] = {ijk[0] + (k & 1), ijk[1] + ((k >> 1) & 1), ijk[2] + ((k >> 2) & 1)};
  return P.vert_index(v);
}

void face_dirs(int code, int& d1, int& d2, int& dn, int& anchor) {
  anchor = code & 7;
  int t = code >> 3, m = 0, dd[2] = {0, 0};
  for (int d = 0; d < 3; ++d) if ((t >> d) & 1) dd[m++] = d; else dn = d;
  d1 = dd[0]; d2 = dd[1];
}

// reference point in side S of the facet point with left-face coordinates (s, t)
void side_point(const orc_problem& P, FacetSide L, FacetSide S, double s, double t, double* xi) {
  int d1, d2, dn, a;
  face_dirs(P.fe.codes[S.f], d1, d2, dn, a);
  double u[2] = {s, t};
  if (S.c != L.c) {
    int ld1, ld2, ldn, la;
    face_dirs(P.fe.codes[L.f], ld1, ld2, ldn, la);
    auto corner = [&](FacetSide F, int fd1, int fd2, int fa, int b) {
      return cell_vertex_id(P, F.c, fa | ((b & 1) << fd1) | (((b >> 1) & 1) << fd2));
    };
    int M[4];
    for (int bs = 0; bs < 4; ++bs) {
      M[bs] = 0;
      for (int bl = 0; bl < 4; ++bl)
        if (corner(L, ld1, ld2, la, bl) == corner(S, d1, d2, a, bs)) M[bs] = bl;
    }
    for (int k = 0; k < 2; ++k) {
      int diff = M[0] ^ M[1 << k], r = (diff & 1) ? 0 : 1;
      u[k] = ((M[0] >> r) & 1) ? -(r == 0 ? s : t) : (r == 0 ? s : t);
    }
  }
  xi[d1] = u[0];
  xi[d2] = u[1];
  xi[dn] = ((a >> dn) & 1) ? 1.0 : -1.0;
}

struct SideEval {
  std::vector<double> val, grad;  // nn shape values, nn*3 physical gradients
  double h = 0.0, det = 0.0;
};

void eval_side(const orc_problem& P, int64_t c, const double* xi, SideEval& E) {
  std::vector<double> pt = {xi[0], xi[1], xi[2]}, gv, gg, sv, sg;
  tensor_shapes(3, 1, pt, 1, gv, gg);
  tensor_shapes(3, P.order, pt, 1, sv, sg);
  double xv[24];
  P.cell_vertices(c, xv);
  double J[9], b[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  for (int j = 0; j < 3; ++j) {
    for (int l = 0; l < 3; ++l) J[l + 3 * j] = 0.0;
    for (int k = 0; k < 8; ++k) {
      double alpha = gg[(size_t)k * 3 + j];
      for (int l = 0; l < 3; ++l) J[l + 3 * j] = J[l + 3 * j] + alpha * xv[k * 3 + l];
    }
  }
  invmtx(3, J, b, E.det);
  const int nn = P.fe.nnodes;
  E.val.assign(nn, 0.0);
  E.grad.assign((size_t)nn * 3, 0.0);
  for (int s = 0; s < nn; ++s) {
    E.val[s] = sv[s];
    for (int i = 0; i < 3; ++i) {
      double acc = 0.0;
      for (int j = 0; j < 3; ++j) acc = acc + b[j + 3 * i] * sg[(size_t)s * 3 + j];
      E.grad[(size_t)s * 3 + i] = acc;
    }
  }
  double ih[3] = {0.0, 0.0, 0.0};
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) ih[i] = ih[i] + b[i + 3 * j] * b[i + 3 * j];
    ih[i] = std::sqrt(ih[i]);
  }
  double vh = ih[0];
  for (int i = 1; i < 3; ++i) vh = vh * ih[i];
  vh = 1.0 / vh;
  vh = std::pow(vh, 1.0 / 3.0);
  E.h = 2.0 * vh;
}

double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

void dg_facets(orc_problem& P, std::vector<int32_t>& cia, std::vector<int32_t>& cja, std::vector<double>& cval) {
  const orc_params& p = P.p;
  const int nn = P.fe.nnodes, np1 = P.order + 1;
  const double C_IP = 10.0 * (double)(P.order * P.order);
  // facet key -> the (at most two) cells holding it, ascending
  const int ntypes = 8;
  auto key_of = [&](int64_t c, int f) -> int64_t {
    if (P.unst) return P.cellvef[(size_t)c * 26 + f];
    int ijk[3];
    P.cell_ijk(c, ijk);
    const int code = P.fe.codes[f], anchor = code & 7;
    int v[3] = {ijk[0] + (anchor & 1), ijk[1] + ((anchor >> 1) & 1), ijk[2] + ((anchor >> 2) & 1)};
    return (int64_t)(code >> 3) + ntypes * P.vert_index(v);
  };
  std::vector<std::pair<int64_t, int64_t>> occ;  // (key, c*32+f)
  for (int64_t c = 0; c < P.ncells; ++c)
    for (int f = 20; f < 26; ++f) occ.push_back({key_of(c, f), c * 32 + f});
  std::sort(occ.begin(), occ.end());
  std::vector<int64_t> other((size_t)P.ncells * 6, -1);
  for (size_t i = 0; i + 1 < occ.size(); ++i)
    if (occ[i].first == occ[i + 1].first) {
      int64_t a = occ[i].second, b = occ[i + 1].second;
      other[(a >> 5) * 6 + (a & 31) - 20] = b;
      other[(b >> 5) * 6 + (b & 31) - 20] = a;
    }
  std::vector<double> x1(np1), w1(np1);
  gauss_legendre(np1, x1.data(), w1.data());
  const int nq = np1 * np1;
  std::vector<double> fpts((size_t)nq * 3, 0.0), fv, fg;
  for (int q = 0; q < nq; ++q) { fpts[q * 3] = x1[q % np1]; fpts[q * 3 + 1] = x1[q / np1]; }
  tensor_shapes(2, 1, fpts, nq, fv, fg);  // facet geometry: 4 bilinear shapes on [-1,1]^2
  std::vector<double> facemat((size_t)4 * nn * nn), facevec((size_t)2 * nn);
  auto FM = [&](int i, int j, int I, int J) -> double& { return facemat[(((size_t)I * 2 + J) * nn + j) * nn + i]; };
  for (int64_t c = 0; c < P.ncells; ++c)
    for (int f = 20; f < 26; ++f) {
      const int64_t o = other[c * 6 + f - 20];
      if (o >= 0 && (o >> 5) < c) continue;  // visited from the smaller cell
      const bool boundary = o < 0;
      FacetSide side[2] = {{c, f}, {boundary ? -1 : (o >> 5), boundary ? -1 : (int)(o & 31)}};
      const int nsides = boundary ? 1 : 2;
      int d1, d2, dn, a;
      face_dirs(P.fe.codes[f], d1, d2, dn, a);
      double X[4][3];
      for (int k = 0; k < 4; ++k) {
        int64_t v = cell_vertex_id(P, c, a | ((k & 1) << d1) | (((k >> 1) & 1) << d2));
        for (int l = 0; l < 3; ++l) X[k][l] = P.coords[(size_t)v * 3 + l];
      }
      const double sigma = (d1 == 0 && d2 == 2) ? -1.0 : 1.0;
      const double outward = ((a >> dn) & 1) ? 1.0 : -1.0;
      std::fill(facemat.begin(), facemat.end(), 0.0);
      std::fill(facevec.begin(), facevec.end(), 0.0);
      double orient = 0.0;
      for (int q = 0; q < nq; ++q) {
        const double s = fpts[q * 3], t = fpts[q * 3 + 1];
        double xq[3] = {0, 0, 0}, js[3] = {0, 0, 0}, jt[3] = {0, 0, 0};
        for (int k = 0; k < 4; ++k) {
          const double ph = fv[(size_t)k * nq + q], ds = fg[((size_t)k * nq + q) * 3], dt = fg[((size_t)k * nq + q) * 3 + 1];
          for (int l = 0; l < 3; ++l) {
            xq[l] = xq[l] + ph * X[k][l];
            js[l] = js[l] + ds * X[k][l];
            jt[l] = jt[l] + dt * X[k][l];
          }
        }
        double n[3] = {js[1] * jt[2] - js[2] * jt[1], js[2] * jt[0] - js[0] * jt[2], js[0] * jt[1] - js[1] * jt[0]};
        const double det = std::sqrt(dot3(n, n));
        SideEval E[2];
        for (int I = 0; I < nsides; ++I) {
          double xi[3];
          side_point(P, side[0], side[I], s, t, xi);
          eval_side(P, side[I].c, xi, E[I]);
        }
        if (q == 0) orient = sigma * outward * (E[0].det > 0.0 ? 1.0 : -1.0);
        for (int l = 0; l < 3; ++l) n[l] = det != 0.0 ? n[l] / det * orient : 0.0;
        double nrm[2][3];
        for (int l = 0; l < 3; ++l) { nrm[0][l] = n[l]; nrm[1][l] = -n[l]; }
        const double h = nsides == 2 ? std::min(E[0].h, E[1].h) : E[0].h;
        const double factor = det * (w1[q % np1] * w1[q / np1]);
        if (!boundary) {
          for (int I = 0; I < 2; ++I)
            for (int J = 0; J < 2; ++J)
              for (int i = 0; i < nn; ++i)
                for (int j = 0; j < nn; ++j) {
                  const double t1 = 0.5 * dot3(&E[J].grad[(size_t)j * 3], nrm[I]) * E[I].val[i];
                  const double t2 = 0.5 * dot3(&E[I].grad[(size_t)i * 3], nrm[J]) * E[J].val[j];
                  const double sc = C_IP / h * E[J].val[j] * E[I].val[i];
                  const double t3 = (sc * nrm[I][0]) * nrm[J][0] + (sc * nrm[I][1]) * nrm[J][1] + (sc * nrm[I][2]) * nrm[J][2];
                  FM(i, j, I, J) = FM(i, j, I, J) + factor * (-t1 - t2 + t3);
                }
        } else {
          const double g = fn_value(p.boundary_fn, p.fn_param, 3, xq);
          for (int i = 0; i < nn; ++i) {
            for (int j = 0; j < nn; ++j) {
              const double t1 = dot3(&E[0].grad[(size_t)j * 3], n) * E[0].val[i];
              const double t2 = dot3(&E[0].grad[(size_t)i * 3], n) * E[0].val[j];
              const double t3 = C_IP / h * E[0].val[i] * E[0].val[j];
              FM(i, j, 0, 0) = FM(i, j, 0, 0) + factor * (-t1 - t2 + t3);
            }
            double gg[3] = {g * E[0].grad[(size_t)i * 3], g * E[0].grad[(size_t)i * 3 + 1], g * E[0].grad[(size_t)i * 3 + 2]};
            facevec[i] = facevec[i] + factor * (-dot3(gg, n) + C_IP / h * g * E[0].val[i]);
          }
        }
      }
      // COO append, upper entries (base_sparse_matrix.f90:3469-3513); facet rhs
      for (int I = 0; I < nsides; ++I)
        for (int J = 0; J < nsides; ++J)
          for (int j = 0; j < nn; ++j) {
            const int32_t jas = P.gids[(size_t)side[J].c * P.nd + j];
            for (int i = 0; i < nn; ++i) {
              const int32_t ias = P.gids[(size_t)side[I].c * P.nd + i];
              if (ias > jas) continue;
              cia.push_back(ias); cja.push_back(jas); cval.push_back(FM(i, j, I, J));
            }
          }
      if (boundary)
        for (int i = 0; i < nn; ++i) {
          const int32_t g = P.gids[(size_t)c * P.nd + i];
          P.rhs[g - 1] = P.rhs[g - 1] + facevec[i];
        }
    }
}

// Multi-threaded form of assemble() for the continuous Galerkin path, used when nthreads > 1.
// It produces the same CSR, bit for bit, as the serial COO append + sort_and_compress below:
// the cells are cut into nthreads consecutive chunks; pass A counts each chunk's upper free
// entries per row, so every (chunk, row) gets its slot range inside the row; pass B
// integrates the chunk's cells in order and writes each entry into its slot.  Every row then
// holds its entries in append (cell) order, exactly the order the stable counting sort by
// row gives; each row is stably sorted by column (insertion sort) and its duplicates summed
// in that order, as row_compress does.  The rhs is summed in cell order.
void assemble_parallel(orc_problem& P, int T) {
  const int nd = P.nd;
  const int64_t nr = P.nfree, nc = P.ncells;
  std::vector<double> invj0, det0, xq0;
  if (P.p.translated_jacobian) cell_geometry(P, 0, invj0, det0, xq0);
  std::vector<int64_t> cb(T + 1);
  for (int t = 0; t <= T; ++t) cb[t] = nc * t / T;
  // slot[t*nr + r]: entries of row r from chunk t (pass A), then the chunk's next slot in the row
  std::unique_ptr<uint32_t[]> slot(new uint32_t[(size_t)T * (size_t)nr]);
  std::unique_ptr<uint32_t[]> rowcnt(new uint32_t[(size_t)nr + 1]);
  std::vector<int64_t> rstart(nr + 1, 0), tsum(T + 1, 0);
  std::unique_ptr<double[]> evall(new double[(size_t)nc * nd]);
  std::unique_ptr<int32_t[]> cja;
  std::unique_ptr<double[]> cval;
#pragma omp parallel num_threads(T)
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    uint32_t* cnt = slot.get() + (size_t)t * nr;
    std::fill(cnt, cnt + nr, 0u);
    for (int64_t c = cb[t]; c < cb[t + 1]; ++c) {
      const int32_t* gid = &P.gids[(size_t)c * nd];
      for (int j = 0; j < nd; ++j) {
        const int32_t jas = gid[j];
        if (jas < 1) continue;
        for (int i = 0; i < nd; ++i) {
          const int32_t ias = gid[i];
          if (ias < 1 || ias > jas) continue;
          cnt[ias - 1]++;
        }
      }
    }
#pragma omp barrier
    const int64_t r0 = nr * t / T, r1 = nr * (t + 1) / T;
    int64_t mine = 0;
    for (int64_t r = r0; r < r1; ++r) {
      uint32_t acc = 0;
      for (int u = 0; u < T; ++u) {
        uint32_t k = slot[(size_t)u * nr + r];
        slot[(size_t)u * nr + r] = acc;
        acc += k;
      }
      rowcnt[r] = acc;
      mine += acc;
    }
    tsum[t + 1] = mine;
#pragma omp barrier
#pragma omp single
    {
      for (int u = 0; u < T; ++u) tsum[u + 1] += tsum[u];
      cja.reset(new int32_t[(size_t)tsum[T]]);
      cval.reset(new double[(size_t)tsum[T]]);
    }
    int64_t run = tsum[t];
    for (int64_t r = r0; r < r1; ++r) { rstart[r] = run; run += rowcnt[r]; }
    if (t == T - 1) rstart[nr] = run;
#pragma omp barrier
    std::vector<double> em((size_t)nd * nd);
    for (int64_t c = cb[t]; c < cb[t + 1]; ++c) {
      double* ev = &evall[(size_t)c * nd];
      integrate_cell(P, c, P.p.translated_jacobian && c > 0 ? &invj0 : nullptr,
                     P.p.translated_jacobian && c > 0 ? &det0 : nullptr, em.data(), ev);
      const int32_t* gid = &P.gids[(size_t)c * nd];
      for (int j = 0; j < nd; ++j) {
        const int32_t jas = gid[j];
        if (jas < 1) continue;
        for (int i = 0; i < nd; ++i) {
          const int32_t ias = gid[i];
          if (ias < 1 || ias > jas) continue;
          const int64_t pos = rstart[ias - 1] + cnt[ias - 1]++;
          cja[pos] = jas;
          cval[pos] = em[i + (size_t)nd * j];
        }
      }
    }
  }
  double t0 = now_s();
  P.coo_n = tsum[T];
  // rhs (serial_scalar_array_add_multiple_entries) in cell order
  P.rhs.assign(nr, 0.0);
  for (int64_t c = 0; c < nc; ++c) {
    const int32_t* gid = &P.gids[(size_t)c * nd];
    const double* ev = &evall[(size_t)c * nd];
    for (int i = 0; i < nd; ++i) if (gid[i] > 0) P.rhs[gid[i] - 1] = P.rhs[gid[i] - 1] + ev[i];
  }
  evall.reset();
  slot.reset();
#pragma omp parallel for schedule(dynamic, 1024) num_threads(T)
  for (int64_t r = 0; r < nr; ++r) {
    const int64_t s = rstart[r], e = rstart[r + 1];
    int32_t* cj = cja.get();
    double* cv = cval.get();
    for (int64_t k = s + 1; k < e; ++k) {  // stable insertion sort by column
      const int32_t kc = cj[k];
      const double kv = cv[k];
      int64_t m = k;
      while (m > s && cj[m - 1] > kc) { cj[m] = cj[m - 1]; cv[m] = cv[m - 1]; --m; }
      cj[m] = kc; cv[m] = kv;
    }
    int64_t w = s;
    for (int64_t k = s; k < e; ++k) {
      if (k > s && cj[w - 1] == cj[k]) cv[w - 1] = cv[w - 1] + cv[k];
      else { cj[w] = cj[k]; cv[w] = cv[k]; ++w; }
    }
    rowcnt[r] = (uint32_t)(w - s);
  }
  P.irp.assign(nr + 1, 1);
  for (int64_t r = 0; r < nr; ++r) P.irp[r + 1] = P.irp[r] + (int64_t)rowcnt[r];
  P.ja.resize((size_t)(P.irp[nr] - 1));
  P.val.resize((size_t)(P.irp[nr] - 1));
#pragma omp parallel for schedule(static) num_threads(T)
  for (int64_t r = 0; r < nr; ++r) {
    const int64_t d = P.irp[r] - 1;
    std::memcpy(&P.ja[d], &cja[rstart[r]], sizeof(int32_t) * rowcnt[r]);
    std::memcpy(&P.val[d], &cval[rstart[r]], sizeof(double) * rowcnt[r]);
  }
  P.t_compress = now_s() - t0;
}

void assemble(orc_problem& P) {
  if (P.p.nthreads > 1 && P.p.formulation != ORC_DG && P.nfree > 0) {
    assemble_parallel(P, P.p.nthreads);
    return;
  }
  const int nd = P.nd;
  std::vector<double> invj0, det0, xq0;
  if (P.p.translated_jacobian) cell_geometry(P, 0, invj0, det0, xq0);
  // COO append in cell order (base_sparse_matrix.f90:3469-3513); rhs add (serial_scalar_array.f90:247-262)
  std::vector<int32_t> cia, cja;
  std::vector<double> cval;
  P.rhs.assign(P.nfree, 0.0);
  const int64_t chunk = 4096;
  std::vector<double> em((size_t)chunk * nd * nd), ev((size_t)chunk * nd);
  int nth = P.p.nthreads > 0 ? P.p.nthreads : 1;
  (void)nth;
  for (int64_t c0 = 0; c0 < P.ncells; c0 += chunk) {
    int64_t c1 = std::min(P.ncells, c0 + chunk);
#pragma omp parallel for schedule(dynamic, 16) num_threads(nth) if (nth > 1)
    for (int64_t c = c0; c < c1; ++c)
      integrate_cell(P, c, P.p.translated_jacobian && c > 0 ? &invj0 : nullptr,
                     P.p.translated_jacobian && c > 0 ? &det0 : nullptr,
                     &em[(size_t)(c - c0) * nd * nd], &ev[(size_t)(c - c0) * nd]);
    for (int64_t c = c0; c < c1; ++c) {
      const int32_t* gid = &P.gids[(size_t)c * nd];
      const double* elmat = &em[(size_t)(c - c0) * nd * nd];
      for (int j = 0; j < nd; ++j) {
        int32_t jas = gid[j];
        if (jas < 1) continue;
        for (int i = 0; i < nd; ++i) {
          int32_t ias = gid[i];
          if (ias < 1 || ias > jas) continue;
          cia.push_back(ias); cja.push_back(jas); cval.push_back(elmat[i + (size_t)nd * j]);
        }
      }
      const double* elvec = &ev[(size_t)(c - c0) * nd];
      for (int i = 0; i < nd; ++i) if (gid[i] > 0) P.rhs[gid[i] - 1] = P.rhs[gid[i] - 1] + elvec[i];
    }
  }
  if (P.p.formulation == ORC_DG) dg_facets(P, cia, cja, cval);
  P.coo_n = (int64_t)cia.size();
  double t0 = now_s();
  // sort_and_compress (base_sparse_matrix.f90:4121-4829): stable bucket by row, stable
  // sort of the columns of each row, duplicates summed in sorted (= append) order.
  const int64_t nr = P.nfree;
  std::vector<int64_t> cnt(nr + 1, 0);
  for (int64_t e = 0; e < P.coo_n; ++e) cnt[cia[e]]++;
  std::vector<int64_t> start(nr + 1, 0);
  for (int64_t r = 1; r <= nr; ++r) start[r] = start[r - 1] + cnt[r];
  std::vector<int64_t> perm(P.coo_n);
  {
    std::vector<int64_t> pos(start.begin(), start.end());
    for (int64_t e = 0; e < P.coo_n; ++e) perm[pos[cia[e] - 1]++] = e;
  }
  std::vector<int64_t> rowlen(nr, 0);
  P.ja.clear(); P.val.clear();
  P.ja.reserve(P.coo_n / 2 + 16); P.val.reserve(P.coo_n / 2 + 16);
  std::vector<std::vector<int32_t>> rja(nth > 1 ? nr : 0);
  std::vector<std::vector<double>> rva(nth > 1 ? nr : 0);
  auto row_compress = [&](int64_t r, std::vector<int32_t>& oj, std::vector<double>& ov) {
    int64_t s = start[r], e = start[r + 1];
    std::stable_sort(perm.begin() + s, perm.begin() + e, [&](int64_t a, int64_t b) { return cja[a] < cja[b]; });
    for (int64_t k = s; k < e; ++k) {
      int64_t idx = perm[k];
      if (!oj.empty() && k > s && oj.back() == cja[idx]) ov.back() = ov.back() + cval[idx];
      else { oj.push_back(cja[idx]); ov.push_back(cval[idx]); }
    }
  };
  if (nth > 1) {
#pragma omp parallel for schedule(dynamic, 256) num_threads(nth)
    for (int64_t r = 0; r < nr; ++r) row_compress(r, rja[r], rva[r]);
    P.irp.assign(nr + 1, 1);
    for (int64_t r = 0; r < nr; ++r) {
      P.irp[r + 1] = P.irp[r] + (int64_t)rja[r].size();
      P.ja.insert(P.ja.end(), rja[r].begin(), rja[r].end());
      P.val.insert(P.val.end(), rva[r].begin(), rva[r].end());
    }
  } else {
    P.irp.assign(nr + 1, 1);
    for (int64_t r = 0; r < nr; ++r) {
      size_t before = P.ja.size();
      int64_t s = start[r], e = start[r + 1];
      std::stable_sort(perm.begin() + s, perm.begin() + e, [&](int64_t a, int64_t b) { return cja[a] < cja[b]; });
      for (int64_t k = s; k < e; ++k) {
        int64_t idx = perm[k];
        if (P.ja.size() > before && P.ja.back() == cja[idx]) P.val.back() = P.val.back() + cval[idx];
        else { P.ja.push_back(cja[idx]); P.val.push_back(cval[idx]); }
      }
      P.irp[r + 1] = P.irp[r] + (int64_t)(P.ja.size() - before);
    }
  }
  P.t_compress = now_s() - t0;
}

// ---- linear algebra of the CG path -------------------------------------------
// matvec_symmetric_storage (csr_sparse_matrix.f90:597-623), alpha=1, beta=0
void spmv_sym(const orc_problem& P, const double* x, double* y) {
  const int64_t n = P.nfree;
  for (int64_t i = 0; i < n; ++i) y[i] = 0.0;
  for (int64_t ir = 0; ir < n; ++ir) {
    int64_t s = P.irp[ir] - 1, e = P.irp[ir + 1] - 1;
    if (s >= e) continue;
    y[ir] = y[ir] + x[P.ja[s] - 1] * P.val[s];
    for (int64_t iz = s + 1; iz < e; ++iz) {
      int64_t ic = P.ja[iz] - 1;
      y[ir] = y[ir] + 1.0 * x[ic] * P.val[iz];
      y[ic] = y[ic] + 1.0 * x[ir] * P.val[iz];
    }
  }
}

// Multi-threaded symmetric-storage SpMV (the kernel above) for nthreads > 1.  Rows are cut
// into nthreads ranges of equal stored entries; thread t writes y of its own rows directly
// and the transposed contributions y(ic) += a x(ir) that land beyond its range into a private
// spill buffer, added to y afterwards in thread order.  Deterministic for a thread count; it
// sums in a different order than the serial kernel, so results agree to rounding.
//
// Gather form (full = true): the upper layout is first expanded to a full CSR (0-based, each
// row's columns ascending, expanded on nthreads threads) and every row is a plain dot
// product: twice the stored bytes, no scattered writes.
struct SymPar {
  int T = 1;
  bool full = false;
  std::vector<int64_t> rb;                  // row ranges
  std::vector<std::vector<double>> spill;   // per thread: y(rb[t+1] .. max column)
  std::vector<int64_t> frp;                 // full CSR
  std::vector<int32_t, NoInit<int32_t>> fci;
  std::vector<double, NoInit<double>> fv;
  void setup_full(const orc_problem& P, int nth) {
    T = nth;
    full = true;
    const int64_t n = P.nfree;
    std::unique_ptr<uint32_t[]> cnt(new uint32_t[(size_t)n]);
#pragma omp parallel for schedule(static) num_threads(T)
    for (int64_t r = 0; r < n; ++r) cnt[r] = (uint32_t)(P.irp[r + 1] - P.irp[r]);
#pragma omp parallel for schedule(static) num_threads(T)
    for (int64_t r = 0; r < n; ++r)
      for (int64_t k = P.irp[r]; k < P.irp[r + 1] - 1; ++k) {  // off-diagonal entries (diagonal first)
        const int64_t c = P.ja[k] - 1;
#pragma omp atomic
        cnt[c]++;
      }
    frp.assign(n + 1, 0);
    for (int64_t r = 0; r < n; ++r) frp[r + 1] = frp[r] + cnt[r];
    fci.resize((size_t)frp[n]);
    fv.resize((size_t)frp[n]);
    // lower part of row c: cursor from the row's start, filled in any order, sorted below
    std::unique_ptr<int64_t[]> cur(new int64_t[(size_t)n]);
#pragma omp parallel for schedule(static) num_threads(T)
    for (int64_t r = 0; r < n; ++r) cur[r] = frp[r];
#pragma omp parallel for schedule(static) num_threads(T)
    for (int64_t r = 0; r < n; ++r)
      for (int64_t k = P.irp[r]; k < P.irp[r + 1] - 1; ++k) {
        const int64_t c = P.ja[k] - 1;
        int64_t pos;
#pragma omp atomic capture
        pos = cur[c]++;
        fci[pos] = (int32_t)r;
        fv[pos] = P.val[k];
      }
#pragma omp parallel for schedule(dynamic, 1024) num_threads(T)
    for (int64_t r = 0; r < n; ++r) {
      const int64_t s = frp[r], m = cur[r];
      for (int64_t k = s + 1; k < m; ++k) {
        const int32_t kc = fci[k];
        const double kv = fv[k];
        int64_t q = k;
        while (q > s && fci[q - 1] > kc) { fci[q] = fci[q - 1]; fv[q] = fv[q - 1]; --q; }
        fci[q] = kc; fv[q] = kv;
      }
      int64_t w = m;
      for (int64_t k = P.irp[r] - 1; k < P.irp[r + 1] - 1; ++k) { fci[w] = P.ja[k] - 1; fv[w] = P.val[k]; ++w; }
    }
  }
  void apply_full(const double* x, double* y) const {
    const int64_t n = (int64_t)frp.size() - 1;
#pragma omp parallel for schedule(static, 4096) num_threads(T)
    for (int64_t r = 0; r < n; ++r) {
      double acc = 0.0;
      for (int64_t k = frp[r]; k < frp[r + 1]; ++k) acc = acc + fv[k] * x[fci[k]];
      y[r] = acc;
    }
  }
  void setup(const orc_problem& P, int nth) {
    T = nth;
    const int64_t n = P.nfree, nnz = P.irp[n] - 1;
    rb.assign(T + 1, n);
    rb[0] = 0;
    for (int t = 1; t < T; ++t)
      rb[t] = std::lower_bound(P.irp.begin(), P.irp.begin() + n, 1 + nnz * t / T) - P.irp.begin();
    for (int t = 1; t <= T; ++t) rb[t] = std::max(rb[t], rb[t - 1]);
    spill.assign(T, {});
#pragma omp parallel for schedule(static, 1) num_threads(T)
    for (int t = 0; t < T; ++t) {
      int64_t hi = rb[t + 1] - 1;
      for (int64_t r = rb[t]; r < rb[t + 1]; ++r)
        if (P.irp[r + 1] > P.irp[r]) hi = std::max<int64_t>(hi, P.ja[P.irp[r + 1] - 2] - 1);
      spill[t].assign((size_t)std::max<int64_t>(0, hi - rb[t + 1] + 1), 0.0);
    }
  }
  void apply(const orc_problem& P, const double* x, double* y) {
    if (full) { apply_full(x, y); return; }
#pragma omp parallel num_threads(T)
    {
      int t = 0;
#ifdef _OPENMP
      t = omp_get_thread_num();
#endif
      const int64_t a = rb[t], b = rb[t + 1];
      double* sp = spill[t].data();
      const int64_t ns = (int64_t)spill[t].size();
      for (int64_t i = a; i < b; ++i) y[i] = 0.0;
      for (int64_t k = 0; k < ns; ++k) sp[k] = 0.0;
      const int32_t* ja = P.ja.data();
      const double* va = P.val.data();
      for (int64_t ir = a; ir < b; ++ir) {
        const int64_t s = P.irp[ir] - 1, e = P.irp[ir + 1] - 1;
        if (s >= e) continue;
        // y(ir) in a register: the off-diagonal columns are > ir, so the sequence of sums
        // into y(ir) is the serial kernel's
        double acc = y[ir] + x[ja[s] - 1] * va[s];
        const double xr = x[ir];
        int64_t iz = s + 1;
        for (; iz < e && ja[iz] - 1 < b; ++iz) {
          const int64_t ic = ja[iz] - 1;
          acc = acc + x[ic] * va[iz];
          y[ic] = y[ic] + xr * va[iz];
        }
        for (; iz < e; ++iz) {
          const int64_t ic = ja[iz] - 1;
          acc = acc + x[ic] * va[iz];
          sp[ic - b] = sp[ic - b] + xr * va[iz];
        }
        y[ir] = acc;
      }
#pragma omp barrier
      for (int u = 0; u < T; ++u) {
        const int64_t bu = rb[u + 1];
        const double* su = spill[u].data();
#pragma omp for schedule(static)
        for (int64_t k = 0; k < (int64_t)spill[u].size(); ++k) y[bu + k] = y[bu + k] + su[k];
      }
    }
  }
};

}  // namespace

// ===========================================================================
extern "C" {

static bool dg_params_ok(const orc_params* p) {
  return p->formulation != ORC_DG || (p->num_dims == 3 && p->kind == ORC_POISSON && !p->cell_coef);
}

orc_problem* orc_create(const orc_params* p) {
  if (!p || (p->num_dims != 2 && p->num_dims != 3) || p->order < 1 || p->order > 8) return nullptr;
  if (!dg_params_ok(p)) return nullptr;
  orc_problem* P = new orc_problem();
  P->p = *p;
  double t0 = now_s();
  build_mesh_and_dofs(*P);
  if (p->source_fn == ORC_FN_QP_VALUES && p->qp_source)
    P->qp_source.assign(p->qp_source, p->qp_source + (size_t)P->ncells * P->nq * (p->kind == ORC_ELASTICITY ? P->dim : 1));
  double t1 = now_s();
  assemble(*P);
  double t2 = now_s();
  P->t_setup = t1 - t0;
  P->t_integrate = (t2 - t1) - P->t_compress;
  P->p.vertex_xyz = nullptr; P->p.cell_coef = nullptr; P->p.qp_source = nullptr;
  return P;
}

orc_problem* orc_create_unstructured(const orc_params* p, const orc_umesh* m) {
  if (!p || !m || p->num_dims != 3 || p->order < 1 || p->order > 8 || m->num_cells < 1) return nullptr;
  if (!dg_params_ok(p)) return nullptr;
  orc_problem* P = new orc_problem();
  P->p = *p;
  P->unst = true;
  P->dim = 3;
  P->ncells = m->num_cells;
  P->nverts_u = m->num_vertices;
  P->coords.assign(m->coords, m->coords + 3 * m->num_vertices);
  P->cellvert.resize((size_t)m->num_cells * 8);
  for (size_t k = 0; k < P->cellvert.size(); ++k) {
    int32_t v = m->cell_vertices[k] - 1;
    if (v < 0 || v >= m->num_vertices) { delete P; return nullptr; }
    P->cellvert[k] = v;
  }
  double t0 = now_s();
  P->fe.build(3, p->order, p->kind == ORC_ELASTICITY ? 3 : 1);
  generate_unstructured_topology(*P, m);
  build_mesh_and_dofs(*P);
  if (p->source_fn == ORC_FN_QP_VALUES && p->qp_source)
    P->qp_source.assign(p->qp_source, p->qp_source + (size_t)P->ncells * P->nq * (p->kind == ORC_ELASTICITY ? 3 : 1));
  double t1 = now_s();
  assemble(*P);
  double t2 = now_s();
  P->t_setup = t1 - t0;
  P->t_integrate = (t2 - t1) - P->t_compress;
  P->p.vertex_xyz = nullptr; P->p.cell_coef = nullptr; P->p.qp_source = nullptr;
  return P;
}

int64_t orc_num_vefs(const orc_problem* h, int64_t* num_edges, int64_t* num_faces) {
  if (num_edges) *num_edges = h->nedges;
  if (num_faces) *num_faces = h->nfaces;
  return h->nvefs;
}
void orc_get_cell_vefs(const orc_problem* h, int32_t* out) {
  for (size_t k = 0; k < h->cellvef.size(); ++k) out[k] = (int32_t)(h->cellvef[k] + 1);
}
void orc_get_vef_sets(const orc_problem* h, int32_t* out) {
  for (size_t k = 0; k < h->vset.size(); ++k) out[k] = h->vset[k];
}

void orc_destroy(orc_problem* h) { delete h; }
int64_t orc_num_cells(const orc_problem* h) { return h->ncells; }
int orc_dofs_per_cell(const orc_problem* h) { return h->nd; }
int orc_qp_per_cell(const orc_problem* h) { return h->nq; }
int64_t orc_num_free(const orc_problem* h) { return h->nfree; }
int64_t orc_num_dirichlet(const orc_problem* h) { return h->ndir; }
int64_t orc_nnz_upper(const orc_problem* h) { return (int64_t)h->ja.size(); }
int64_t orc_coo_entries(const orc_problem* h) { return h->coo_n; }

void orc_get_dof_map(const orc_problem* h, int32_t* out) { std::memcpy(out, h->gids.data(), sizeof(int32_t) * h->gids.size()); }
void orc_get_csr_upper(const orc_problem* h, int64_t* irp, int32_t* ja, double* val) {
  if (irp) std::memcpy(irp, h->irp.data(), sizeof(int64_t) * h->irp.size());
  if (ja) std::memcpy(ja, h->ja.data(), sizeof(int32_t) * h->ja.size());
  if (val) std::memcpy(val, h->val.data(), sizeof(double) * h->val.size());
}
void orc_get_rhs(const orc_problem* h, double* rhs) { std::memcpy(rhs, h->rhs.data(), sizeof(double) * h->rhs.size()); }
void orc_get_dirichlet_values(const orc_problem* h, double* g) { std::memcpy(g, h->gvals.data(), sizeof(double) * h->gvals.size()); }
void orc_get_elmat(const orc_problem* h, int64_t cell, double* elmat, double* elvec) {
  std::vector<double> invj0, det0, xq0;
  if (h->p.translated_jacobian && cell > 0) cell_geometry(*h, 0, invj0, det0, xq0);
  integrate_cell(*h, cell, h->p.translated_jacobian && cell > 0 ? &invj0 : nullptr,
                 h->p.translated_jacobian && cell > 0 ? &det0 : nullptr, elmat, elvec);
}
void orc_get_qp_coords(const orc_problem* h, double* out) {
  std::vector<double> invj, det, xq;
  for (int64_t c = 0; c < h->ncells; ++c) {
    cell_geometry(*h, c, invj, det, xq);
    std::memcpy(out + (size_t)c * h->nq * 3, xq.data(), sizeof(double) * h->nq * 3);
  }
}
void orc_get_timings(const orc_problem* h, double* t3) { t3[0] = h->t_setup; t3[1] = h->t_integrate; t3[2] = h->t_compress; }

void orc_spmv(const orc_problem* h, const double* x, double* y) { spmv_sym(*h, x, y); }

// cg_solve_body (cg.f90:101-238) with init_convergence_data / update_convergence_data...
// (cg.f90:279-407).  Vector kernels are the reference's BLAS calls restated as loops; with
// nthreads > 1 they run on that many threads (reductions summed in thread order) and the
// SpMV is SymPar's.  it_time (optional, length maxit) receives the seconds from the call's
// start (set-up included) to the end of each iteration.
int orc_cg_timed(const orc_problem* h, int precond, double rtol, double atol, int maxit, int criterion,
                 const double* b, const double* x0, double* x, int* iters, double* history, int nthreads,
                 double* it_time) {
  const double t_start = now_s();
  const int64_t n = h->nfree;
  const bool gather = nthreads < -1;
  const int nth = gather ? -nthreads : (nthreads > 0 ? nthreads : 1);
  std::vector<double, NoInit<double>> r(n), z(n), p(n), Ap(n), idiag(n);
  SymPar S;
  if (gather) S.setup_full(*h, nth);
  else if (nth > 1) S.setup(*h, nth);
  auto A = [&](const double* in, double* out) {
    if (nth > 1) S.apply(*h, in, out);
    else spmv_sym(*h, in, out);
  };
  std::vector<double> part(nth);
  auto dot = [&](const double* a, const double* c) {
    if (nth == 1) {
      double s = 0.0;
      for (int64_t i = 0; i < n; ++i) s = s + a[i] * c[i];
      return s;
    }
#pragma omp parallel num_threads(nth)
    {
      int t = 0;
#ifdef _OPENMP
      t = omp_get_thread_num();
#endif
      double s = 0.0;
      for (int64_t i = n * t / nth; i < n * (t + 1) / nth; ++i) s = s + a[i] * c[i];
      part[t] = s;
    }
    double s = 0.0;
    for (int t = 0; t < nth; ++t) s = s + part[t];
    return s;
  };
  auto nrm2 = [&](const double* a) { return std::sqrt(dot(a, a)); };
  // axpby: y = alpha*x + beta*y
  auto axpby = [&](double alpha, const double* xx, double beta, double* yy) {
#pragma omp parallel for schedule(static) num_threads(nth) if (nth > 1)
    for (int64_t i = 0; i < n; ++i) yy[i] = alpha * xx[i] + beta * yy[i];
  };
#pragma omp parallel for schedule(static) num_threads(nth) if (nth > 1)
  for (int64_t i = 0; i < n; ++i) {
    double d = 1.0;
    if (precond == 1) {
      // extract_diagonal (csr_sparse_matrix.f90:4231-4256) + entrywise_invert
      int64_t s = h->irp[i] - 1, e = h->irp[i + 1] - 1;
      const int32_t* lo = h->ja.data() + s;
      const int32_t* hi = h->ja.data() + e;
      const int32_t* it = std::lower_bound(lo, hi, (int32_t)(i + 1));
      d = (it != hi && *it == (int32_t)(i + 1)) ? h->val[s + (it - lo)] : 0.0;
      d = 1.0 / d;
    }
    idiag[i] = d;
    x[i] = x0 ? x0[i] : 0.0;
  }
  auto M = [&](const double* in, double* out) {
#pragma omp parallel for schedule(static) num_threads(nth) if (nth > 1)
    for (int64_t i = 0; i < n; ++i) out[i] = precond == 1 ? idiag[i] * in[i] : in[i];
  };
  double b_nrm_M = 0.0;
  if (criterion == ORC_RES_NRMGIVEN_RHS_NRMGIVEN) { M(b, r.data()); b_nrm_M = std::sqrt(dot(b, r.data())); }
  A(x, r.data());
  axpby(1.0, b, -1.0, r.data());
  M(r.data(), z.data());
  double r_z = dot(r.data(), z.data());
  double r_nrm_M = std::sqrt(r_z);
#pragma omp parallel for schedule(static) num_threads(nth) if (nth > 1)
  for (int64_t i = 0; i < n; ++i) p[i] = z[i];
  double rhs_test = 0.0;
  switch (criterion) {
    case ORC_RES_RHS: case ORC_DELTA_RHS: rhs_test = rtol * nrm2(b) + atol; break;
    case ORC_RES_RES: rhs_test = rtol * nrm2(r.data()) + atol; break;
    case ORC_RES_NRMGIVEN_RHS_NRMGIVEN: rhs_test = rtol * b_nrm_M + atol; break;
    case ORC_RES_NRMGIVEN_RES_NRMGIVEN: rhs_test = rtol * r_nrm_M + atol; break;
    default: break;
  }
  int it = 0;
  bool conv = false;
  double err = 0.0;
  while (true) {
    ++it;
    A(p.data(), Ap.data());
    double Ap_p = dot(Ap.data(), p.data());
    double alpha = Ap_p != 0.0 ? r_z / Ap_p : 0.0;
    axpby(alpha, p.data(), 1.0, x);
    axpby(-alpha, Ap.data(), 1.0, r.data());
    if (it == 1 && (criterion == ORC_DELTA_RHS || criterion == ORC_DELTA_DELTA)) {
      err = alpha * nrm2(p.data());
      if (criterion == ORC_DELTA_DELTA) rhs_test = rtol * err + atol;
    }
    switch (criterion) {
      case ORC_RES_RES: case ORC_RES_RHS: err = nrm2(r.data()); break;
      case ORC_DELTA_RHS: case ORC_DELTA_DELTA: if (it != 1) err = alpha * nrm2(p.data()); break;
      default: err = r_nrm_M; break;
    }
    if (history) history[it - 1] = err;
    conv = err <= rhs_test;
    if (!conv && it < maxit) {
      M(r.data(), z.data());
      double beta = 1.0 / r_z;
      r_z = dot(r.data(), z.data());
      beta = beta * r_z;
      r_nrm_M = std::sqrt(r_z);
      axpby(1.0, z.data(), beta, p.data());
    }
    if (it_time) it_time[it - 1] = now_s() - t_start;
    if (conv || it >= maxit) break;
  }
  if (iters) *iters = it;
  return conv ? 0 : 1;
}

int orc_cg(const orc_problem* h, int precond, double rtol, double atol, int maxit, int criterion,
           const double* b, const double* x0, double* x, int* iters, double* history, int nthreads) {
  return orc_cg_timed(h, precond, rtol, atol, maxit, criterion, b, x0, x, iters, history, nthreads, nullptr);
}

double orc_energy_error(const orc_problem* h, const double* x) {
  const orc_params& p = h->p;
  const int nd = h->nd, nq = h->nq;
  double total = 0.0;
  std::vector<double> invj, det, xq;
  for (int64_t c = 0; c < h->ncells; ++c) {
    cell_geometry(*h, c, invj, det, xq);
    double sq = 0.0;
    for (int q = 0; q < nq; ++q) {
      double gh[3] = {0, 0, 0};
      for (int s = 0; s < nd; ++s) {
        int32_t g = h->gids[(size_t)c * nd + s];
        double u = g > 0 ? x[g - 1] : h->gvals[-g - 1];
        double gp[3];
        for (int i = 0; i < 3; ++i) {
          double acc = 0.0;
          for (int j = 0; j < 3; ++j) acc = acc + invj[q * 9 + j + 3 * i] * h->shg[((size_t)s * nq + q) * 3 + j];
          gp[i] = acc;
        }
        for (int i = 0; i < 3; ++i) gh[i] = gh[i] + u * gp[i];
      }
      double ge[3];
      fn_gradient(p.boundary_fn, p.fn_param, h->dim, &xq[q * 3], ge);
      double factor = det[q] * h->qw[q];
      double e0 = ge[0] - gh[0], e1 = ge[1] - gh[1], e2 = ge[2] - gh[2];
      sq = sq + factor * (e0 * e0 + e1 * e1 + e2 * e2);
    }
    total += sq;
  }
  return std::sqrt(total);
}

// error_norms_scalar_compute_cell_contribution (sbm_error_norms_scalar.i90:115-241):
// e = exact - u_h at the Gauss points; cells summed in order (update_norm, error_norms.f90:160-172).
// out: mean, l1, l2^2, linfty, |grad e|^2, w1infty (before finalize_norm)
void orc_error_norms(const orc_problem* h, const double* x, int fn, const double* prm, double* out) {
  const int nd = h->nd, nq = h->nq;
  double mean = 0.0, l1 = 0.0, l2 = 0.0, linf = 0.0, h1 = 0.0, w1 = 0.0;
  std::vector<double> invj, det, xq;
  for (int64_t c = 0; c < h->ncells; ++c) {
    cell_geometry(*h, c, invj, det, xq);
    double cm = 0.0, cl1 = 0.0, cl2 = 0.0, cli = 0.0, ch1 = 0.0, cw1 = 0.0;
    for (int q = 0; q < nq; ++q) {
      double uh = 0.0, gh[3] = {0, 0, 0};
      for (int s = 0; s < nd; ++s) {
        int32_t g = h->gids[(size_t)c * nd + s];
        double u = g > 0 ? x[g - 1] : h->gvals[-g - 1];
        uh = uh + u * h->shp[(size_t)s * nq + q];
        for (int i = 0; i < 3; ++i) {
          double acc = 0.0;
          for (int j = 0; j < 3; ++j) acc = acc + invj[q * 9 + j + 3 * i] * h->shg[((size_t)s * nq + q) * 3 + j];
          gh[i] = gh[i] + u * acc;
        }
      }
      double e = fn_value(fn, prm, h->dim, &xq[q * 3]) - uh;
      double ge[3];
      fn_gradient(fn, prm, h->dim, &xq[q * 3], ge);
      double factor = det[q] * h->qw[q];
      double e0 = ge[0] - gh[0], e1 = ge[1] - gh[1], e2 = ge[2] - gh[2];
      cm = cm + e * factor;
      cl1 = cl1 + std::fabs(e) * factor;
      cl2 = cl2 + (e * e) * factor;
      cli = std::max(cli, std::fabs(e));
      ch1 = ch1 + (e0 * e0 + e1 * e1 + e2 * e2) * factor;
      cw1 = std::max(cw1, std::max(std::fabs(e0), std::max(std::fabs(e1), std::fabs(e2))));
    }
    mean += cm;
    l1 += cl1;
    l2 += cl2;
    linf = std::max(linf, cli);
    h1 += ch1;
    w1 = std::max(w1, cw1);
  }
  out[0] = mean;
  out[1] = l1;
  out[2] = l2;
  out[3] = linf;
  out[4] = h1;
  out[5] = w1;
}

void orc_gauss_legendre(int n, double* x, double* w) { gauss_legendre(n, x, w); }

int orc_own_dofs(int num_dims, int order, int ncomp, int iface, int32_t* out) {
  RefFE fe;
  fe.build(num_dims, order, ncomp);
  if (iface < 1 || iface > fe.nfaces) return -1;
  const std::vector<int>& l = fe.own[iface - 1];
  for (size_t k = 0; k < l.size(); ++k) out[k] = l[k];
  return (int)l.size();
}

int orc_polytope_codes(int num_dims, int32_t* codes) {
  std::vector<int> c = polytope_codes(num_dims);
  for (size_t i = 0; i < c.size(); ++i) codes[i] = c[i];
  return (int)c.size();
}

}  // extern "C"

// fg_refe.cpp -- host-side reference-element tables of the Lagrangian hex (and quad) FE.
//
// Node order, quadrature order and the polytope n-face order reproduce the reference
// element of FEMPAR (Sources/Lib/Integration/ReferenceFE):
//   * n-faces of the hex are bit codes (anchor vertex | free directions << 3) sorted by
//     (dimension, code)                               sbm_polytope.i90:175-269
//   * nodes are lexicographic, x fastest               sbm_polytope.i90:396-433
//   * Gauss-Legendre points, (p+1) per direction for the default degree 2p, x fastest
//                                                      sbm_quadrature.i90:767-823,
//                                                      sbm_lagrangian_reference_fe.i90:1414-1423
//   * equispaced 1D Lagrange basis on [-1,1], tensor-product values and gradients
//                                                      sbm_polynomial.i90:61-109,
//                                                      sbm_tensor_product_polynomial.i90:28-120
//   * geometry: trilinear (Q1) map                     sbm_fine_triangulation.i90:48
#include <algorithm>
#include <cmath>
#include <cstring>

#include "fg_internal.h"

namespace fg {

// Gauss-Legendre rule on [-1,1] (ascending) by Newton's method on the three-term
// recurrence of P_n; weights 2/((1-x^2) P_n'(x)^2).
void gl_rule(int n, double* x, double* w) {
  const double pi = 3.141592653589793238462643;
  for (int k = 0; k < (n + 1) / 2; ++k) {
    double t = std::cos(pi * (k + 0.75) / (n + 0.5));
    double d = 1.0;
    for (int it = 0; it < 64; ++it) {
      double pm = 1.0, pc = t;
      for (int m = 2; m <= n; ++m) {
        double pn = ((2 * m - 1) * t * pc - (m - 1) * pm) / m;
        pm = pc;
        pc = pn;
      }
      if (n == 1) { pc = t; pm = 1.0; }
      d = n * (t * pc - pm) / (t * t - 1.0);
      double step = pc / d;
      t -= step;
      if (std::fabs(step) <= 1e-16 * std::fabs(t) + 1e-300) break;
    }
    double pm = 1.0, pc = t;
    for (int m = 2; m <= n; ++m) {
      double pn = ((2 * m - 1) * t * pc - (m - 1) * pm) / m;
      pm = pc;
      pc = pn;
    }
    if (n == 1) { pc = t; pm = 1.0; }
    d = n * (t * pc - pm) / (t * t - 1.0);
    double wk = 2.0 / ((1.0 - t * t) * d * d);
    x[n - 1 - k] = std::fabs(t);
    x[k] = -std::fabs(t);
    w[k] = w[n - 1 - k] = wk;
  }
  if (n % 2 == 1) x[n / 2] = 0.0;
}

// 1D Lagrange basis l_j on nodes (2/p)i-1 and its derivative at x.
void lagrange_1d(int p, int j, double x, double& v, double& dv) {
  double xn[FG_MAX_ORDER + 1];
  for (int i = 0; i <= p; ++i) xn[i] = (2.0 / p) * i - 1.0;
  double den = 1.0;
  for (int i = 0; i <= p; ++i) if (i != j) den *= (xn[j] - xn[i]);
  double num = 1.0;
  for (int i = 0; i <= p; ++i) if (i != j) num *= (x - xn[i]);
  double dnum = 0.0;
  for (int k = 0; k <= p; ++k) {
    if (k == j) continue;
    double prod = 1.0;
    for (int i = 0; i <= p; ++i) if (i != j && i != k) prod *= (x - xn[i]);
    dnum += prod;
  }
  v = num / den;
  dv = dnum / den;
}

namespace {
int bitcount(int v) { return __builtin_popcount((unsigned)v); }
}  // namespace

void RefTables::build(int p, int nc) {
  dim = 3;
  order = p;
  ncomp = nc;
  const int np1 = p + 1;
  nn = np1 * np1 * np1;
  nd = nn * nc;
  nq = np1 * np1 * np1;
  // n-face codes: for every set of free directions t, the anchors with no bit in t.
  int cnt = 0;
  for (int t = 0; t < 8; ++t)
    for (int a = 0; a < 8; ++a)
      if ((a & t) == 0) codes[cnt++] = a | (t << 3);
  std::sort(codes, codes + 27, [](int u, int v) {
    int du = bitcount(u >> 3), dv = bitcount(v >> 3);
    return du != dv ? du < dv : u < v;
  });
  for (int i = 0; i < 64; ++i) code2idx[i] = -1;
  for (int i = 0; i < 27; ++i) code2idx[codes[i]] = i;

  double x1[FG_MAX_ORDER + 1], w1[FG_MAX_ORDER + 1];
  gl_rule(np1, x1, w1);
  qw.assign(nq, 0.0);
  for (int k = 0; k < np1; ++k)
    for (int j = 0; j < np1; ++j)
      for (int i = 0; i < np1; ++i) qw[i + np1 * (j + np1 * k)] = w1[i] * w1[j] * w1[k];

  // 1D tables at the 1D Gauss points
  double L[FG_MAX_ORDER + 1][FG_MAX_ORDER + 1], dL[FG_MAX_ORDER + 1][FG_MAX_ORDER + 1];
  for (int j = 0; j < np1; ++j)
    for (int q = 0; q < np1; ++q) lagrange_1d(p, j, x1[q], L[j][q], dL[j][q]);
  shp.assign((size_t)nn * nq, 0.0);
  shg.assign((size_t)nn * nq * 3, 0.0);
  for (int a = 0; a < nn; ++a) {
    int ai = a % np1, aj = (a / np1) % np1, ak = a / (np1 * np1);
    for (int q = 0; q < nq; ++q) {
      int qi = q % np1, qj = (q / np1) % np1, qk = q / (np1 * np1);
      shp[(size_t)a * nq + q] = L[ai][qi] * L[aj][qj] * L[ak][qk];
      shg[((size_t)a * nq + q) * 3 + 0] = dL[ai][qi] * L[aj][qj] * L[ak][qk];
      shg[((size_t)a * nq + q) * 3 + 1] = dL[aj][qj] * L[ai][qi] * L[ak][qk];
      shg[((size_t)a * nq + q) * 3 + 2] = dL[ak][qk] * L[ai][qi] * L[aj][qj];
    }
  }
  // Q1 geometry at the Gauss points and at the FE nodes
  gshp.assign(8 * nq, 0.0);
  gshg.assign(8 * nq * 3, 0.0);
  for (int k = 0; k < 8; ++k) {
    int bx = k & 1, by = (k >> 1) & 1, bz = (k >> 2) & 1;
    for (int q = 0; q < nq; ++q) {
      double xs = x1[q % np1], ys = x1[(q / np1) % np1], zs = x1[q / (np1 * np1)];
      double fx = bx ? 0.5 * (1 + xs) : 0.5 * (1 - xs), gx = bx ? 0.5 : -0.5;
      double fy = by ? 0.5 * (1 + ys) : 0.5 * (1 - ys), gy = by ? 0.5 : -0.5;
      double fz = bz ? 0.5 * (1 + zs) : 0.5 * (1 - zs), gz = bz ? 0.5 : -0.5;
      gshp[k * nq + q] = fx * fy * fz;
      gshg[(k * nq + q) * 3 + 0] = gx * fy * fz;
      gshg[(k * nq + q) * 3 + 1] = gy * fx * fz;
      gshg[(k * nq + q) * 3 + 2] = gz * fx * fy;
    }
  }
  gnod.assign(8 * nn, 0.0);
  for (int k = 0; k < 8; ++k) {
    int bx = k & 1, by = (k >> 1) & 1, bz = (k >> 2) & 1;
    for (int a = 0; a < nn; ++a) {
      double xs = (2.0 / p) * (a % np1) - 1.0, ys = (2.0 / p) * ((a / np1) % np1) - 1.0,
             zs = (2.0 / p) * (a / (np1 * np1)) - 1.0;
      double fx = bx ? 0.5 * (1 + xs) : 0.5 * (1 - xs);
      double fy = by ? 0.5 * (1 + ys) : 0.5 * (1 - ys);
      double fz = bz ? 0.5 * (1 + zs) : 0.5 * (1 - zs);
      gnod[k * nn + a] = fx * fy * fz;
    }
  }
}

void RefTables::build2d(int p, int nc) {
  dim = 2;
  order = p;
  ncomp = nc;
  const int np1 = p + 1;
  nn = np1 * np1;
  nd = nn * nc;
  nq = np1 * np1;
  // n-face codes of the quadrilateral: anchor | (free directions << 2), sorted by (dim, code)
  int cnt = 0;
  for (int t = 0; t < 4; ++t)
    for (int a = 0; a < 4; ++a)
      if ((a & t) == 0) codes[cnt++] = a | (t << 2);
  std::sort(codes, codes + 9, [](int u, int v) {
    int du = bitcount(u >> 2), dv = bitcount(v >> 2);
    return du != dv ? du < dv : u < v;
  });
  for (int i = 9; i < 27; ++i) codes[i] = -1;
  for (int i = 0; i < 64; ++i) code2idx[i] = -1;
  for (int i = 0; i < 9; ++i) code2idx[codes[i]] = i;

  double x1[FG_MAX_ORDER + 1], w1[FG_MAX_ORDER + 1];
  gl_rule(np1, x1, w1);
  qw.assign(nq, 0.0);
  for (int j = 0; j < np1; ++j)
    for (int i = 0; i < np1; ++i) qw[i + np1 * j] = w1[i] * w1[j];
  double L[FG_MAX_ORDER + 1][FG_MAX_ORDER + 1], dL[FG_MAX_ORDER + 1][FG_MAX_ORDER + 1];
  for (int j = 0; j < np1; ++j)
    for (int q = 0; q < np1; ++q) lagrange_1d(p, j, x1[q], L[j][q], dL[j][q]);
  shp.assign((size_t)nn * nq, 0.0);
  shg.assign((size_t)nn * nq * 3, 0.0);
  for (int a = 0; a < nn; ++a) {
    int ai = a % np1, aj = a / np1;
    for (int q = 0; q < nq; ++q) {
      int qi = q % np1, qj = q / np1;
      shp[(size_t)a * nq + q] = L[ai][qi] * L[aj][qj];
      shg[((size_t)a * nq + q) * 3 + 0] = dL[ai][qi] * L[aj][qj];
      shg[((size_t)a * nq + q) * 3 + 1] = dL[aj][qj] * L[ai][qi];
    }
  }
  gshp.assign(4 * nq, 0.0);
  gshg.assign(4 * nq * 3, 0.0);
  for (int k = 0; k < 4; ++k) {
    int bx = k & 1, by = (k >> 1) & 1;
    for (int q = 0; q < nq; ++q) {
      double xs = x1[q % np1], ys = x1[q / np1];
      double fx = bx ? 0.5 * (1 + xs) : 0.5 * (1 - xs), gx = bx ? 0.5 : -0.5;
      double fy = by ? 0.5 * (1 + ys) : 0.5 * (1 - ys), gy = by ? 0.5 : -0.5;
      gshp[k * nq + q] = fx * fy;
      gshg[(k * nq + q) * 3 + 0] = gx * fy;
      gshg[(k * nq + q) * 3 + 1] = gy * fx;
    }
  }
  gnod.assign(4 * nn, 0.0);
  for (int k = 0; k < 4; ++k) {
    int bx = k & 1, by = (k >> 1) & 1;
    for (int a = 0; a < nn; ++a) {
      double xs = (2.0 / p) * (a % np1) - 1.0, ys = (2.0 / p) * (a / np1) - 1.0;
      gnod[k * nn + a] = (bx ? 0.5 * (1 + xs) : 0.5 * (1 - xs)) * (by ? 0.5 * (1 + ys) : 0.5 * (1 - ys));
    }
  }
}

fg_status upload_tables(fg_ctx* ctx, const RefTables& t, DevTables& d) {
  size_t n = t.qw.size() + t.shp.size() + t.shg.size() + t.gshp.size() + t.gshg.size() + t.gnod.size();
  std::vector<double> h(n);
  size_t o = 0;
  auto put = [&](const std::vector<double>& v) {
    size_t at = o;
    std::memcpy(h.data() + o, v.data(), v.size() * sizeof(double));
    o += v.size();
    return at;
  };
  size_t oqw = put(t.qw), oshp = put(t.shp), oshg = put(t.shg), ogshp = put(t.gshp), ogshg = put(t.gshg),
         ognod = put(t.gnod);
  void* p = nullptr;
  FG_TRY(dev_alloc(ctx, &p, n * sizeof(double)));
  d.base = (double*)p;
  d.bytes = n * sizeof(double);
  FG_CUDA_TRY(cudaMemcpyAsync(d.base, h.data(), d.bytes, cudaMemcpyHostToDevice, ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  d.qw = d.base + oqw;
  d.shp = d.base + oshp;
  d.shg = d.base + oshg;
  d.gshp = d.base + ogshp;
  d.gshg = d.base + ogshg;
  d.gnod = d.base + ognod;
  // float-float copy of the reference gradients: hi = (float)v, lo = (float)(v - hi)
  const size_t ng = t.shg.size();
  std::vector<float> f(2 * ng);
  for (size_t i = 0; i < ng; ++i) {
    float hi = (float)t.shg[i];
    f[i] = hi;
    f[ng + i] = (float)(t.shg[i] - (double)hi);
  }
  void* pf = nullptr;
  FG_TRY(dev_alloc(ctx, &pf, f.size() * sizeof(float)));
  d.fbase = (float*)pf;
  FG_CUDA_TRY(cudaMemcpyAsync(d.fbase, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  d.shgh = d.fbase;
  d.shgl = d.fbase + ng;
  return FG_OK;
}

}  // namespace fg

// fg_errnorm.cu -- norms of the error of a discrete solution against an analytic function.
//
// Reference: error_norms_scalar_t%compute (Sources/Lib/Integration/ErrorNorms/
// sbm_error_norms_scalar.i90:67-241, error_norms.f90:160-221): per cell, e = u - u_h and
// grad(e) at the Gauss points; mean/l1/l2 (and the value part of h1) integrate e, |e|, e^2
// with |det J| w; linfty takes max |e|; h1_seminorm integrates |grad e|^2; w1infty takes the
// largest gradient component; cell contributions are summed (or maxed) over the cells and
// l2/h1 take square roots.  The tutorial's error estimator (tutorial_01 modules :542-679) is
// the squared energy norm per cell, here sum_q k |grad e|^2 |det J| w (k = 1 in the tutorial).
//
// One thread per cell writes its contributions; one block reduces them in a fixed order.
#include <cmath>

#include "fg_internal.h"

namespace fg {

namespace {

struct ErrGeom {
  int n[3], p, Ln[3];
  const int32_t* cellvert;  // unstructured meshes (null on the lattice)
  const int32_t* cellnode;
};

__device__ double exact_value(int fn, const double* prm, const double* x) {
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

// d/dx atan(a(r - r0)) = a / (1 + a^2 (r - r0)^2) * (x - c) / r
__device__ void exact_gradient(int fn, const double* prm, const double* x, double* g) {
  g[0] = g[1] = g[2] = 0.0;
  if (fn == FG_FN_LINEAR) {
    g[0] = g[1] = g[2] = 1.0;
  } else if (fn == FG_FN_SHARP_WAVE) {
    const double a = prm[0];
    double d[3] = {x[0] - prm[2], x[1] - prm[3], x[2] - prm[4]};
    const double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const double t = r - prm[1];
    const double s = a / (r * (a * a * t * t + 1.0));
    for (int i = 0; i < 3; ++i) g[i] = s * d[i];
  }
}

constexpr int kNC = 8;  // mean, l1, l2^2, linf, |grad|^2, w1inf, k|grad|^2, spare

template <int P>
__global__ void __launch_bounds__(128)
    k_cell_errors(ErrGeom g, int64_t ncells, const double* __restrict__ coords, DevTables tb,
                  const int32_t* __restrict__ latdof, const double* __restrict__ x, const double* __restrict__ gvals,
                  const double* __restrict__ coef, double coef_const, int fn, const double* __restrict__ prm_g,
                  double* __restrict__ C) {
  constexpr int NP1 = P + 1, NN = NP1 * NP1 * NP1, NQ = NN;
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  double prm[8];
  for (int i = 0; i < 8; ++i) prm[i] = prm_g[i];
  const int ci = (int)(c % g.n[0]), cj = (int)((c / g.n[0]) % g.n[1]), ck = (int)(c / ((int64_t)g.n[0] * g.n[1]));
  double xv[24];
  for (int k = 0; k < 8; ++k) {
    int64_t v = g.cellvert ? (int64_t)g.cellvert[c * 8 + k]
                           : (int64_t)(ci + (k & 1)) +
                                 (int64_t)(g.n[0] + 1) * ((cj + ((k >> 1) & 1)) + (int64_t)(g.n[1] + 1) * (ck + ((k >> 2) & 1)));
    for (int l = 0; l < 3; ++l) xv[k * 3 + l] = coords[v * 3 + l];
  }
  double u[NN];
  for (int s = 0; s < NN; ++s) {
    int ai = s % NP1, aj = (s / NP1) % NP1, ak = s / (NP1 * NP1);
    int64_t L = g.cellnode ? (int64_t)g.cellnode[c * NN + s]
                           : (int64_t)(P * ci + ai) + (int64_t)g.Ln[0] * ((P * cj + aj) + (int64_t)g.Ln[1] * (P * ck + ak));
    int32_t id = latdof[L];
    u[s] = id > 0 ? x[id - 1] : (id < 0 ? gvals[-id - 1] : 0.0);
  }
  const double kc = coef ? coef[c] : coef_const;
  double mean = 0.0, l1 = 0.0, l2 = 0.0, linf = 0.0, h1 = 0.0, w1inf = 0.0;
  bool neg = false;
  for (int q = 0; q < NQ; ++q) {
    double J[9];
    for (int j = 0; j < 3; ++j) {
      double a0 = 0.0, a1 = 0.0, a2 = 0.0;
      for (int k = 0; k < 8; ++k) {
        double alpha = tb.gshg[(k * NQ + q) * 3 + j];
        a0 = a0 + alpha * xv[k * 3 + 0];
        a1 = a1 + alpha * xv[k * 3 + 1];
        a2 = a2 + alpha * xv[k * 3 + 2];
      }
      J[0 + 3 * j] = a0;
      J[1 + 3 * j] = a1;
      J[2 + 3 * j] = a2;
    }
    double t1 = J[4] * J[8] - J[5] * J[7];
    double t2 = -J[1] * J[8] + J[2] * J[7];
    double t3 = J[1] * J[5] - J[2] * J[4];
    double det = J[0] * t1 + J[3] * t2 + J[6] * t3;
    double dn = 1.0 / det;
    double b[9];
    b[0] = t1 * dn;
    b[1] = t2 * dn;
    b[2] = t3 * dn;
    b[4] = (J[0] * J[8] - J[2] * J[6]) * dn;
    b[5] = (-J[0] * J[5] + J[3] * J[2]) * dn;
    b[8] = (J[0] * J[4] - J[1] * J[3]) * dn;
    b[3] = (-J[3] * J[8] + J[5] * J[6]) * dn;
    b[6] = (J[3] * J[7] - J[4] * J[6]) * dn;
    b[7] = (-J[0] * J[7] + J[1] * J[6]) * dn;
    if (q == 0) neg = det < 0.0;
    const double factor = (neg ? fabs(det) : det) * tb.qw[q];
    double xq[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 8; ++k) {
      double a = tb.gshp[k * NQ + q];
      xq[0] = xq[0] + a * xv[k * 3 + 0];
      xq[1] = xq[1] + a * xv[k * 3 + 1];
      xq[2] = xq[2] + a * xv[k * 3 + 2];
    }
    double uh = 0.0, gh[3] = {0.0, 0.0, 0.0};
    for (int s = 0; s < NN; ++s) {
      uh = uh + u[s] * tb.shp[s * NQ + q];
      for (int i = 0; i < 3; ++i) {
        double acc = 0.0;
        for (int j = 0; j < 3; ++j) acc = acc + b[j + 3 * i] * tb.shg[(s * NQ + q) * 3 + j];
        gh[i] = gh[i] + u[s] * acc;
      }
    }
    const double e = exact_value(fn, prm, xq) - uh;
    double ge[3];
    exact_gradient(fn, prm, xq, ge);
    const double e0 = ge[0] - gh[0], e1 = ge[1] - gh[1], e2 = ge[2] - gh[2];
    mean = mean + e * factor;
    l1 = l1 + fabs(e) * factor;
    l2 = l2 + (e * e) * factor;
    linf = fmax(linf, fabs(e));
    h1 = h1 + (e0 * e0 + e1 * e1 + e2 * e2) * factor;
    w1inf = fmax(w1inf, fmax(fabs(e0), fmax(fabs(e1), fabs(e2))));
  }
  double* o = C + c * kNC;
  o[0] = mean;
  o[1] = l1;
  o[2] = l2;
  o[3] = linf;
  o[4] = h1;
  o[5] = w1inf;
  o[6] = kc * h1;
  o[7] = 0.0;
}

// Quadrilaterals (2D): the same norms with the bilinear map (n = 2 branch of invmtx) and the
// 2D analytic functions.
__device__ double exact_value_2d(int fn, const double* prm, const double* x) {
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

__device__ void exact_gradient_2d(int fn, const double* prm, const double* x, double* g) {
  g[0] = g[1] = 0.0;
  if (fn == FG_FN_LINEAR) {
    g[0] = g[1] = 1.0;
  } else if (fn == FG_FN_SHARP_WAVE) {
    const double a = prm[0];
    const double d[2] = {x[0] - prm[2], x[1] - prm[3]};
    const double r = sqrt(d[0] * d[0] + d[1] * d[1]);
    const double t = r - prm[1];
    const double s = a / (r * (a * a * t * t + 1.0));
    g[0] = s * d[0];
    g[1] = s * d[1];
  }
}

template <int P>
__global__ void __launch_bounds__(128)
    k_cell_errors_2d(ErrGeom g, int64_t ncells, const double* __restrict__ coords, DevTables tb,
                     const int32_t* __restrict__ latdof, const double* __restrict__ x,
                     const double* __restrict__ gvals, const double* __restrict__ coef, double coef_const, int fn,
                     const double* __restrict__ prm_g, double* __restrict__ C) {
  constexpr int NP1 = P + 1, NN = NP1 * NP1, NQ = NN;
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  double prm[8];
  for (int i = 0; i < 8; ++i) prm[i] = prm_g[i];
  const int ci = (int)(c % g.n[0]), cj = (int)(c / g.n[0]);
  double xv[8];
  for (int k = 0; k < 4; ++k) {
    const int64_t v = (int64_t)(ci + (k & 1)) + (int64_t)(g.n[0] + 1) * (cj + (k >> 1));
    xv[k * 2 + 0] = coords[v * 3 + 0];
    xv[k * 2 + 1] = coords[v * 3 + 1];
  }
  double u[NN];
  for (int s = 0; s < NN; ++s) {
    const int64_t L = (int64_t)(P * ci + s % NP1) + (int64_t)g.Ln[0] * (P * cj + s / NP1);
    const int32_t id = latdof[L];
    u[s] = id > 0 ? x[id - 1] : (id < 0 ? gvals[-id - 1] : 0.0);
  }
  const double kc = coef ? coef[c] : coef_const;
  double mean = 0.0, l1 = 0.0, l2 = 0.0, linf = 0.0, h1 = 0.0, w1inf = 0.0;
  bool neg = false;
  for (int q = 0; q < NQ; ++q) {
    double J[2][2];  // J[l][j] = sum_k dN_k/dxi_j x_k(l)
    for (int j = 0; j < 2; ++j)
      for (int l = 0; l < 2; ++l) {
        double acc = 0.0;
        for (int k = 0; k < 4; ++k) acc = acc + tb.gshg[(k * NQ + q) * 3 + j] * xv[k * 2 + l];
        J[l][j] = acc;
      }
    const double det = J[0][0] * J[1][1] - J[1][0] * J[0][1];
    const double dn = 1.0 / det;
    const double b11 = J[1][1] * dn, b21 = -J[1][0] * dn, b12 = -J[0][1] * dn, b22 = J[0][0] * dn;
    if (q == 0) neg = det < 0.0;
    const double factor = (neg ? fabs(det) : det) * tb.qw[q];
    double xq[2] = {0.0, 0.0};
    for (int k = 0; k < 4; ++k) {
      const double a = tb.gshp[k * NQ + q];
      xq[0] = xq[0] + a * xv[k * 2 + 0];
      xq[1] = xq[1] + a * xv[k * 2 + 1];
    }
    double uh = 0.0, gh[2] = {0.0, 0.0};
    for (int s = 0; s < NN; ++s) {
      uh = uh + u[s] * tb.shp[s * NQ + q];
      const double r0 = tb.shg[(s * NQ + q) * 3 + 0], r1 = tb.shg[(s * NQ + q) * 3 + 1];
      gh[0] = gh[0] + u[s] * (b11 * r0 + b21 * r1);
      gh[1] = gh[1] + u[s] * (b12 * r0 + b22 * r1);
    }
    const double e = exact_value_2d(fn, prm, xq) - uh;
    double ge[2];
    exact_gradient_2d(fn, prm, xq, ge);
    const double e0 = ge[0] - gh[0], e1 = ge[1] - gh[1];
    mean = mean + e * factor;
    l1 = l1 + fabs(e) * factor;
    l2 = l2 + (e * e) * factor;
    linf = fmax(linf, fabs(e));
    h1 = h1 + (e0 * e0 + e1 * e1) * factor;
    w1inf = fmax(w1inf, fmax(fabs(e0), fabs(e1)));
  }
  double* o = C + c * kNC;
  o[0] = mean;
  o[1] = l1;
  o[2] = l2;
  o[3] = linf;
  o[4] = h1;
  o[5] = w1inf;
  o[6] = kc * h1;
  o[7] = 0.0;
}

// One block: column sums (max for linf / w1inf) over the cells, fixed order.
__global__ void __launch_bounds__(512) k_reduce_errors(int64_t ncells, const double* __restrict__ C, double* out) {
  __shared__ double sh[kNC][512];
  double acc[kNC] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int64_t c = threadIdx.x; c < ncells; c += blockDim.x)
    for (int k = 0; k < kNC; ++k) {
      double v = C[c * kNC + k];
      acc[k] = (k == 3 || k == 5) ? fmax(acc[k], v) : acc[k] + v;
    }
  for (int k = 0; k < kNC; ++k) sh[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int k = 0; k < kNC; ++k)
        sh[k][threadIdx.x] = (k == 3 || k == 5) ? fmax(sh[k][threadIdx.x], sh[k][threadIdx.x + s])
                                                : sh[k][threadIdx.x] + sh[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < kNC) out[threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void k_cell_energy(int64_t ncells, const double* __restrict__ C, double* __restrict__ e) {
  int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c < ncells) e[c] = C[c * kNC + 6];
}

}  // namespace

}  // namespace fg

using namespace fg;

extern "C" fg_status fg_system_error_norms(fg_system* sys, const double* x, int32_t on_device, int32_t fn,
                                           const double* fn_param, double* cell_sq_energy, fg_error_norms* out) {
  if (!sys || !x || !out) {
    set_error("bad argument: system/x/out");
    return FG_ERR_BADARG;
  }
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  if (sp->ncomp != 1) {
    set_error("error norms are built for scalar fields");
    return FG_ERR_UNSUPPORTED;
  }
  if (fn != FG_FN_ZERO && fn != FG_FN_CONST && fn != FG_FN_LINEAR && fn != FG_FN_SHARP_WAVE) {
    set_error("bad argument: exact-solution function");
    return FG_ERR_BADARG;
  }
  FG_CUDA_TRY(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  const int64_t nc = sp->mesh->ncells, n = sp->nfree;
  double *dx = nullptr, *dC = nullptr, *dout = nullptr, *dprm = nullptr, *de = nullptr;
  fg_status s = FG_OK;
  auto A = [&](double** p, size_t cnt) { if (s == FG_OK) s = dev_alloc(ctx, (void**)p, sizeof(double) * (cnt ? cnt : 1)); };
  if (!on_device) A(&dx, n);
  A(&dC, nc * kNC);
  A(&dout, kNC);
  A(&dprm, 8);
  if (cell_sq_energy) A(&de, nc);
  double prm[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (fn_param)
    for (int i = 0; i < 8; ++i) prm[i] = fn_param[i];
  cudaError_t e = cudaSuccess;
  if (s == FG_OK && !on_device && n > 0) e = cudaMemcpyAsync(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice, st);
  if (s == FG_OK && e == cudaSuccess) e = cudaMemcpyAsync(dprm, prm, sizeof(prm), cudaMemcpyHostToDevice, st);
  double h[kNC] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (s == FG_OK && e == cudaSuccess) {
    ErrGeom g;
    for (int d = 0; d < 3; ++d) {
      g.n[d] = sp->mesh->n[d];
      g.Ln[d] = sp->Ln[d];
    }
    g.p = sp->order;
    g.cellvert = sp->mesh->unst ? sp->mesh->d_cellvert : nullptr;
    g.cellnode = sp->d_cellnode;
    const double* xx = on_device ? x : dx;
    const unsigned blocks = (unsigned)((nc + 127) / 128);
    const double* coef = sys->d_coef;
    const double cc = sys->integ.coef_const;
    if (nc > 0 && sp->mesh->dim == 2) {
      if (sp->order == 1)
        k_cell_errors_2d<1><<<blocks, 128, 0, st>>>(g, nc, sp->mesh->d_coords, sp->dtab, sp->d_latdof, xx,
                                                    sys->d_gvals, coef, cc, fn, dprm, dC);
      else if (sp->order == 2)
        k_cell_errors_2d<2><<<blocks, 128, 0, st>>>(g, nc, sp->mesh->d_coords, sp->dtab, sp->d_latdof, xx,
                                                    sys->d_gvals, coef, cc, fn, dprm, dC);
      else
        k_cell_errors_2d<3><<<blocks, 128, 0, st>>>(g, nc, sp->mesh->d_coords, sp->dtab, sp->d_latdof, xx,
                                                    sys->d_gvals, coef, cc, fn, dprm, dC);
    } else if (nc > 0) {
      if (sp->order == 1)
        k_cell_errors<1><<<blocks, 128, 0, st>>>(g, nc, sp->mesh->d_coords, sp->dtab, sp->d_latdof, xx, sys->d_gvals,
                                                 coef, cc, fn, dprm, dC);
      else if (sp->order == 2)
        k_cell_errors<2><<<blocks, 128, 0, st>>>(g, nc, sp->mesh->d_coords, sp->dtab, sp->d_latdof, xx, sys->d_gvals,
                                                 coef, cc, fn, dprm, dC);
      else
        k_cell_errors<3><<<blocks, 128, 0, st>>>(g, nc, sp->mesh->d_coords, sp->dtab, sp->d_latdof, xx, sys->d_gvals,
                                                 coef, cc, fn, dprm, dC);
    }
    if (nc > 0) {
      k_reduce_errors<<<1, 512, 0, st>>>(nc, dC, dout);
      ctx->launches += 2;
      if (cell_sq_energy) {
        k_cell_energy<<<(unsigned)((nc + 255) / 256), 256, 0, st>>>(nc, dC, de);
        ctx->launches += 1;
      }
    }
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, dout, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && cell_sq_energy && nc > 0)
      e = cudaMemcpyAsync(cell_sq_energy, de, sizeof(double) * nc, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  dev_free(ctx, dx);
  dev_free(ctx, dC);
  dev_free(ctx, dout);
  dev_free(ctx, dprm);
  dev_free(ctx, de);
  if (s != FG_OK) return s;
  if (e != cudaSuccess) {
    set_error("error norms: %s", cudaGetErrorString(e));
    return FG_ERR_CUDA;
  }
  // finalize_norm (error_norms.f90:174-221)
  out->mean_norm = h[0];
  out->l1_norm = h[1];
  out->l2_norm = std::sqrt(h[2]);
  out->linfty_norm = h[3];
  out->h1_seminorm = std::sqrt(h[4]);
  out->h1_norm = std::sqrt(h[2] + h[4]);
  out->w1infty_seminorm = h[5];
  out->w1infty_norm = h[3] + h[5];
  out->energy_norm = std::sqrt(h[6]);
  return FG_OK;
}

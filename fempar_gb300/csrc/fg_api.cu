// fg_api.cu -- the extern "C" entry points of libfempar_gpu.so (include/fempar_gpu.h).
#include <cstdarg>
#include <cstdlib>
#include <cstring>

#include "fg_internal.h"

namespace fg {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

fg_status dev_alloc(fg_ctx* ctx, void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  if (ctx->budget && ctx->in_use + bytes > ctx->budget) {
    set_error("HBM budget exceeded: %llu + %llu > %llu bytes", (unsigned long long)ctx->in_use,
              (unsigned long long)bytes, (unsigned long long)ctx->budget);
    return FG_ERR_OOM;
  }
  // stream-ordered pool allocation on the context's stream: no device-wide
  // synchronisation on free, so contexts on other threads keep running
  cudaError_t e = cudaMallocAsync(p, bytes, ctx->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    set_error("cudaMallocAsync(%llu): %s", (unsigned long long)bytes, cudaGetErrorString(e));
    return FG_ERR_OOM;
  }
  ctx->allocs[*p] = bytes;
  ctx->in_use += bytes;
  return FG_OK;
}

void dev_free(fg_ctx* ctx, void* p) {
  if (!p) return;
  auto it = ctx->allocs.find(p);
  if (it != ctx->allocs.end()) {
    ctx->in_use -= it->second;
    ctx->allocs.erase(it);
  }
  cudaFreeAsync(p, ctx->stream);
}

}  // namespace fg

using namespace fg;

#define FG_CHECK_ARG(cond, msg)           \
  do {                                    \
    if (!(cond)) {                        \
      set_error("bad argument: %s", msg); \
      return FG_ERR_BADARG;               \
    }                                     \
  } while (0)

#define FG_DEVICE_GUARD(ctx) FG_CUDA_TRY(cudaSetDevice((ctx)->device))

extern "C" {

const char* fg_status_string(fg_status s) {
  switch (s) {
    case FG_OK: return "FG_OK";
    case FG_ERR_BADARG: return "FG_ERR_BADARG";
    case FG_ERR_OOM: return "FG_ERR_OOM";
    case FG_ERR_CUDA: return "FG_ERR_CUDA";
    case FG_ERR_NOT_CONVERGED: return "FG_ERR_NOT_CONVERGED";
    case FG_ERR_NUMERIC: return "FG_ERR_NUMERIC";
    case FG_ERR_TIMEOUT: return "FG_ERR_TIMEOUT";
    case FG_ERR_UNSUPPORTED: return "FG_ERR_UNSUPPORTED";
    case FG_ERR_NO_DEVICE: return "FG_ERR_NO_DEVICE";
    default: return "FG_ERR_UNKNOWN";
  }
}

const char* fg_last_error(void) { return g_err; }
const char* fg_version(void) { return "fempar-gb300 0.1 (sm_103a)"; }

void fg_solver_params_default(fg_solver_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->precond = FG_PREC_NONE;
  p->precision = FG_FP64;
  p->criterion = FG_RES_RES;
  p->rtol = 1e-6;
  p->atol = 0.0;
  p->max_iters = 1000;
}

void fg_integrand_default(fg_integrand* g) {
  if (!g) return;
  std::memset(g, 0, sizeof(*g));
  g->kind = FG_POISSON;
  g->coef_const = 1.0;
  g->nu = 0.3;
}

fg_status fg_ctx_create(int device, uint64_t hbm_budget_bytes, fg_ctx** out) {
  FG_CHECK_ARG(out, "out");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("no CUDA device: %s", cudaGetErrorString(e));
    return FG_ERR_NO_DEVICE;
  }
  FG_CHECK_ARG(device >= 0 && device < ndev, "device");
  FG_CUDA_TRY(cudaSetDevice(device));
  fg_ctx* c = new fg_ctx();
  c->device = device;
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    set_error("stream: %s", cudaGetErrorString(e));
    return FG_ERR_CUDA;
  }
  {
    // keep freed blocks in the device's pool (reused by later allocations of any context)
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      uint64_t thr = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    cudaGetLastError();
  }
  size_t freeb = 0, totalb = 0;
  cudaMemGetInfo(&freeb, &totalb);
  c->budget = hbm_budget_bytes ? hbm_budget_bytes : (uint64_t)freeb;
  *out = c;
  return FG_OK;
}

fg_status fg_ctx_destroy(fg_ctx* ctx) {
  if (!ctx) return FG_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto& kv : ctx->allocs) cudaFreeAsync(kv.first, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  ctx->allocs.clear();
  {
    // hand the pool's unused blocks back to the device when a context ends
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess) cudaMemPoolTrimTo(pool, 0);
    cudaGetLastError();
  }
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return FG_OK;
}

fg_status fg_ctx_memory(fg_ctx* ctx, uint64_t* in_use, uint64_t* budget) {
  FG_CHECK_ARG(ctx, "ctx");
  if (in_use) *in_use = ctx->in_use;
  if (budget) *budget = ctx->budget;
  return FG_OK;
}

fg_status fg_ctx_get_stream(fg_ctx* ctx, void** stream) {
  FG_CHECK_ARG(ctx && stream, "ctx/stream");
  *stream = (void*)ctx->stream;
  return FG_OK;
}

fg_status fg_ctx_kernel_launches(fg_ctx* ctx, int64_t* count) {
  FG_CHECK_ARG(ctx && count, "ctx/count");
  *count = ctx->launches;
  return FG_OK;
}

fg_status fg_mesh_create_structured(fg_ctx* ctx, int num_dims, const int32_t n[3], const double limits[6],
                                    const double* vertex_xyz, fg_mesh** out) {
  FG_CHECK_ARG(ctx && n && out, "ctx/n/out");
  *out = nullptr;
  if (num_dims != 2 && num_dims != 3) {
    set_error("num_dims must be 2 (quadrilaterals) or 3 (hexahedra)");
    return FG_ERR_UNSUPPORTED;
  }
  FG_CHECK_ARG(n[0] >= 1 && n[1] >= 1 && (num_dims == 2 || n[2] >= 1), "n");
  FG_DEVICE_GUARD(ctx);
  fg_mesh* m = new fg_mesh();
  m->ctx = ctx;
  m->dim = num_dims;
  // 2D: one layer of cells in the lattice bookkeeping (n[2] = 1), vertices at z = 0
  for (int d = 0; d < 3; ++d) m->n[d] = (num_dims == 2 && d == 2) ? 1 : n[d];
  for (int i = 0; i < 6; ++i) m->limits[i] = limits ? limits[i] : (i % 2 ? 1.0 : 0.0);
  m->ncells = (int64_t)m->n[0] * m->n[1] * (num_dims == 2 ? 1 : m->n[2]);
  m->nverts = (int64_t)(m->n[0] + 1) * (m->n[1] + 1) * (num_dims == 2 ? 1 : m->n[2] + 1);
  std::vector<double> h(3 * m->nverts);
  if (vertex_xyz) {
    std::memcpy(h.data(), vertex_xyz, sizeof(double) * h.size());
  } else {
    // ijk/n mapped to the domain limits (uniform_hex_mesh_generator.f90:608-612,632-636)
    for (int64_t v = 0; v < m->nverts; ++v) {
      int64_t r = v;
      int ijk[3];
      ijk[0] = (int)(r % (m->n[0] + 1)); r /= (m->n[0] + 1);
      ijk[1] = (int)(r % (m->n[1] + 1)); r /= (m->n[1] + 1);
      ijk[2] = (int)r;
      for (int d = 0; d < num_dims; ++d) {
        double c = (double)ijk[d] / (double)m->n[d];
        h[v * 3 + d] = (m->limits[2 * d + 1] - m->limits[2 * d]) * c + m->limits[2 * d];
      }
      if (num_dims == 2) h[v * 3 + 2] = 0.0;
    }
  }
  fg_status s = dev_alloc(ctx, (void**)&m->d_coords, sizeof(double) * h.size());
  if (s != FG_OK) { delete m; return s; }
  cudaError_t e = cudaMemcpyAsync(m->d_coords, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    dev_free(ctx, m->d_coords);
    delete m;
    set_error("mesh upload: %s", cudaGetErrorString(e));
    return FG_ERR_CUDA;
  }
  *out = m;
  return FG_OK;
}

static void mesh_free(fg_mesh* m) {
  fg_ctx* ctx = m->ctx;
  void* ptrs[] = {m->d_coords, m->d_cellvert, m->d_cellvef, m->d_vset, m->d_vowner, m->d_vnbr, m->d_vptr, m->d_vcells};
  for (void* p : ptrs) dev_free(ctx, p);
  delete m;
}

fg_status fg_mesh_destroy(fg_mesh* m) {
  if (!m) return FG_OK;
  cudaSetDevice(m->ctx->device);
  mesh_free(m);
  return FG_OK;
}

fg_status fg_mesh_create_unstructured(fg_ctx* ctx, int64_t num_vertices, const double* vertex_xyz,
                                      int64_t num_cells, const int32_t* cell_vertices, int64_t num_given_vefs,
                                      const int64_t* given_vef_ptr, const int32_t* given_vef_vertices,
                                      const int32_t* given_vef_set, fg_mesh** out) {
  FG_CHECK_ARG(ctx && out && vertex_xyz && cell_vertices, "ctx/out/vertex_xyz/cell_vertices");
  *out = nullptr;
  FG_CHECK_ARG(num_vertices >= 1 && num_vertices < (int64_t)0x7fffffff, "num_vertices");
  FG_CHECK_ARG(num_cells >= 1 && num_cells < (int64_t)0x7fffffff / 26, "num_cells");
  FG_CHECK_ARG(num_given_vefs >= 0 && (num_given_vefs == 0 || (given_vef_ptr && given_vef_vertices && given_vef_set)),
               "given vefs");
  // host-side validation: every index the device kernels follow stays inside its array
  std::vector<int32_t> cv((size_t)num_cells * 8);
  for (size_t k = 0; k < cv.size(); ++k) {
    const int32_t v = cell_vertices[k];
    if (v < 1 || v > num_vertices) {
      set_error("cell %lld: vertex id %d outside 1..%lld", (long long)(k / 8), v, (long long)num_vertices);
      return FG_ERR_BADARG;
    }
    cv[k] = v - 1;
  }
  for (int64_t c = 0; c < num_cells; ++c)
    for (int a = 0; a < 8; ++a)
      for (int b = a + 1; b < 8; ++b)
        if (cv[c * 8 + a] == cv[c * 8 + b]) {
          set_error("cell %lld repeats vertex %d", (long long)c, cv[c * 8 + a] + 1);
          return FG_ERR_BADARG;
        }
  if (num_given_vefs > 0) {
    if (given_vef_ptr[0] != 0) { set_error("given_vef_ptr[0] must be 0"); return FG_ERR_BADARG; }
    for (int64_t i = 0; i < num_given_vefs; ++i) {
      const int64_t n = given_vef_ptr[i + 1] - given_vef_ptr[i];
      if (n != 1 && n != 2 && n != 4) { set_error("given vef %lld has %lld vertices", (long long)i, (long long)n); return FG_ERR_BADARG; }
      for (int64_t k = given_vef_ptr[i]; k < given_vef_ptr[i + 1]; ++k)
        if (given_vef_vertices[k] < 1 || given_vef_vertices[k] > num_vertices) {
          set_error("given vef %lld: vertex id %d outside 1..%lld", (long long)i, given_vef_vertices[k], (long long)num_vertices);
          return FG_ERR_BADARG;
        }
    }
  }
  FG_DEVICE_GUARD(ctx);
  fg_mesh* m = new fg_mesh();
  m->ctx = ctx;
  m->dim = 3;
  m->unst = true;
  m->n[0] = (int)num_cells;
  m->n[1] = m->n[2] = 1;
  for (int i = 0; i < 6; ++i) m->limits[i] = 0.0;
  m->ncells = num_cells;
  m->nverts = num_vertices;
  fg_status s = dev_alloc(ctx, (void**)&m->d_coords, sizeof(double) * 3 * num_vertices);
  if (s == FG_OK) s = dev_alloc(ctx, (void**)&m->d_cellvert, sizeof(int32_t) * cv.size());
  if (s == FG_OK) {
    cudaError_t e = cudaMemcpyAsync(m->d_coords, vertex_xyz, sizeof(double) * 3 * num_vertices, cudaMemcpyHostToDevice,
                                    ctx->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(m->d_cellvert, cv.data(), sizeof(int32_t) * cv.size(), cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) { set_error("mesh upload: %s", cudaGetErrorString(e)); s = FG_ERR_CUDA; }
  }
  if (s == FG_OK) s = umesh_build_topology(m, num_given_vefs, given_vef_ptr, given_vef_vertices, given_vef_set);
  if (s == FG_OK) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { set_error("mesh: %s", cudaGetErrorString(e)); s = FG_ERR_CUDA; }
  }
  if (s != FG_OK) {
    cudaStreamSynchronize(ctx->stream);
    mesh_free(m);
    return s;
  }
  *out = m;
  return FG_OK;
}

fg_status fg_mesh_get_info(fg_mesh* m, fg_mesh_info* info) {
  FG_CHECK_ARG(m && info, "mesh/info");
  info->num_cells = m->ncells;
  info->num_vertices = m->nverts;
  if (m->unst) {
    info->num_edges = m->nedges;
    info->num_faces = m->nfaces;
  } else if (m->dim == 2) {
    const int64_t n0 = m->n[0], n1 = m->n[1];
    info->num_edges = n0 * (n1 + 1) + (n0 + 1) * n1;
    info->num_faces = 0;
  } else {
    const int64_t n0 = m->n[0], n1 = m->n[1], n2 = m->n[2];
    info->num_edges = n0 * (n1 + 1) * (n2 + 1) + (n0 + 1) * n1 * (n2 + 1) + (n0 + 1) * (n1 + 1) * n2;
    info->num_faces = n0 * n1 * (n2 + 1) + n0 * (n1 + 1) * n2 + (n0 + 1) * n1 * n2;
  }
  info->num_vefs = info->num_vertices + info->num_edges + info->num_faces;
  info->unstructured = m->unst ? 1 : 0;
  info->max_cells_around_vertex = m->unst ? m->max_vcells : (m->dim == 2 ? 4 : 8);
  return FG_OK;
}

fg_status fg_mesh_get_vefs(fg_mesh* m, int32_t* cell_vefs, int32_t* vef_set_ids) {
  FG_CHECK_ARG(m, "mesh");
  if (!m->unst) {
    set_error("vef tables are exported for unstructured meshes");
    return FG_ERR_UNSUPPORTED;
  }
  FG_DEVICE_GUARD(m->ctx);
  FG_TRY(umesh_export_vefs(m, cell_vefs, vef_set_ids));
  if (cell_vefs)
    for (int64_t k = 0; k < m->ncells * 26; ++k) cell_vefs[k] += 1;
  return FG_OK;
}

static void space_free(fg_space* sp) {
  fg_ctx* ctx = sp->mesh->ctx;
  dev_free(ctx, sp->dtab.base);
  dev_free(ctx, sp->dtab.fbase);
  dev_free(ctx, sp->d_latdof);
  dev_free(ctx, sp->d_free2lat);
  dev_free(ctx, sp->d_dir2lat);
  dev_free(ctx, sp->d_rowptr);
  dev_free(ctx, sp->d_col);
  dev_free(ctx, sp->d_perm);
  dev_free(ctx, sp->d_iperm);
  dev_free(ctx, sp->d_sptr);
  dev_free(ctx, sp->d_scol);
  if (sp->layout == FG_LAYOUT_STENCIL) dev_free(ctx, sp->d_row2vec);
  dev_free(ctx, sp->d_cellnode);
  dev_free(ctx, sp->d_nptr);
  dev_free(ctx, sp->d_ncl);
  dev_free(ctx, sp->d_dgnbr);
  dev_free(ctx, sp->d_dgnbrface);
  dev_free(ctx, sp->d_st_cls);
  dev_free(ctx, sp->d_st_off);
  dev_free(ctx, sp->d_st_scls);
  dev_free(ctx, sp->d_st_voff);
  dev_free(ctx, sp->d_st_row);
  dev_free(ctx, sp->d_row2st);
  dev_free(ctx, sp->d_st_slot2row);
  dev_free(ctx, sp->d_tcT);
  dev_free(ctx, sp->d_tcff);
  delete sp;
}

fg_status fg_space_create(fg_mesh* mesh, int order, int ncomp, const int32_t* dirichlet_ids, int n_ids,
                          fg_space** out) {
  FG_CHECK_ARG(mesh && out, "mesh/out");
  *out = nullptr;
  if (order < 1 || order > FG_MAX_ORDER) {
    set_error("order %d not built (1..%d)", order, FG_MAX_ORDER);
    return FG_ERR_UNSUPPORTED;
  }
  if (ncomp != 1 && ncomp != mesh->dim) {
    set_error("ncomp must be 1 or the number of dimensions (%d)", mesh->dim);
    return FG_ERR_UNSUPPORTED;
  }
  FG_CHECK_ARG(n_ids >= 0 && (n_ids == 0 || dirichlet_ids), "dirichlet ids");
  fg_ctx* ctx = mesh->ctx;
  FG_DEVICE_GUARD(ctx);
  fg_space* sp = new fg_space();
  sp->mesh = mesh;
  sp->order = order;
  sp->ncomp = ncomp;
  const int max_id = mesh->unst ? 31 : (mesh->dim == 2 ? 9 : 27);
  for (int i = 0; i < n_ids; ++i) {
    if (dirichlet_ids[i] < 1 || dirichlet_ids[i] > max_id) {
      delete sp;
      set_error("dirichlet id %d outside 1..%d", dirichlet_ids[i], max_id);
      return FG_ERR_BADARG;
    }
    sp->dirmask |= 1u << dirichlet_ids[i];
  }
  for (int d = 0; d < 3; ++d) sp->Ln[d] = (mesh->dim == 2 && d == 2) ? 1 : order * mesh->n[d] + 1;
  sp->nlat = (int64_t)sp->Ln[0] * sp->Ln[1] * sp->Ln[2];
  if (mesh->dim == 2) sp->tab.build2d(order, ncomp);
  else sp->tab.build(order, ncomp);
  fg_status s = upload_tables(ctx, sp->tab, sp->dtab);
  if (mesh->dim == 2) {
    // quadrilaterals: the solver runs on the explicit-column SELL layout
    if (s == FG_OK) s = q2_number_dofs(sp);
    if (s == FG_OK) s = q2_build_pattern(sp);
    sp->layout = FG_LAYOUT_SELL;
  } else if (mesh->unst) {
    // explicit nodes and cells around them; the solver runs on the explicit-column SELL layout
    sp->explicit_nodes = true;
    if (s == FG_OK) s = uspace_number_dofs(sp);
    if (s == FG_OK) s = uspace_build_pattern(sp);
    sp->layout = FG_LAYOUT_SELL;
  } else {
    if (s == FG_OK) s = space_number_dofs(sp);
    if (s == FG_OK) s = space_build_pattern(sp);
    // solver layout: lattice-implicit SELL unless FG_SOLVER_LAYOUT=sell asks for explicit columns
    const char* lay = getenv("FG_SOLVER_LAYOUT");
    sp->layout = (lay && std::strcmp(lay, "sell") == 0) ? FG_LAYOUT_SELL : FG_LAYOUT_STENCIL;
  }
  if (s == FG_OK) {
    if (sp->layout == FG_LAYOUT_SELL) {
      s = space_build_sell(sp);
      sp->nvec = sp->nfree;
      sp->d_row2vec = sp->d_iperm;
    } else {
      s = space_build_stencil(sp);
    }
  }
  if (s == FG_OK) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { set_error("space: %s", cudaGetErrorString(e)); s = FG_ERR_CUDA; }
  }
  if (s != FG_OK) {
    space_free(sp);
    return s;
  }
  *out = sp;
  return FG_OK;
}

fg_status fg_space_create_dg(fg_mesh* mesh, int order, fg_space** out) {
  FG_CHECK_ARG(mesh && out, "mesh/out");
  *out = nullptr;
  if (mesh->dim != 3) {
    set_error("the dG space is built on 3D meshes");
    return FG_ERR_UNSUPPORTED;
  }
  if (order < 1 || order > FG_MAX_ORDER) {
    set_error("order %d not built (1..%d)", order, FG_MAX_ORDER);
    return FG_ERR_UNSUPPORTED;
  }
  fg_ctx* ctx = mesh->ctx;
  FG_DEVICE_GUARD(ctx);
  fg_space* sp = new fg_space();
  sp->mesh = mesh;
  sp->order = order;
  sp->ncomp = 1;
  sp->dg = true;
  for (int d = 0; d < 3; ++d) sp->Ln[d] = order * mesh->n[d] + 1;
  sp->tab.build(order, 1);
  fg_status s = upload_tables(ctx, sp->tab, sp->dtab);
  if (s == FG_OK) s = dg_space_build(sp);
  sp->layout = FG_LAYOUT_SELL;
  if (s == FG_OK) {
    s = space_build_sell(sp);
    sp->nvec = sp->nfree;
    sp->d_row2vec = sp->d_iperm;
  }
  if (s == FG_OK) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { set_error("space: %s", cudaGetErrorString(e)); s = FG_ERR_CUDA; }
  }
  if (s != FG_OK) {
    space_free(sp);
    return s;
  }
  *out = sp;
  return FG_OK;
}

fg_status fg_space_destroy(fg_space* sp) {
  if (!sp) return FG_OK;
  cudaSetDevice(sp->mesh->ctx->device);
  space_free(sp);
  return FG_OK;
}

fg_status fg_space_release_pattern(fg_space* sp) {
  FG_CHECK_ARG(sp, "space");
  fg_ctx* ctx = sp->mesh->ctx;
  FG_DEVICE_GUARD(ctx);
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, sp->d_rowptr);
  dev_free(ctx, sp->d_col);
  sp->d_rowptr = nullptr;
  sp->d_col = nullptr;
  return FG_OK;
}

fg_status fg_space_get_info(fg_space* sp, fg_space_info* info) {
  FG_CHECK_ARG(sp && info, "space/info");
  info->num_dims = sp->mesh->dim;
  info->order = sp->order;
  info->ncomp = sp->ncomp;
  info->dofs_per_cell = sp->tab.nd;
  info->qp_per_cell = sp->tab.nq;
  info->num_cells = sp->mesh->ncells;
  info->num_free = sp->nfree;
  info->num_dirichlet = sp->ndir;
  info->nnz_full = sp->nnz;
  info->nnz_upper = sp->nnz_upper;
  info->solver_vec_len = sp->nvec;
  info->solver_entries = sp->layout == FG_LAYOUT_SELL ? sp->sell_nnz : sp->st_nvals;
  info->solver_layout = sp->layout;
  return FG_OK;
}

fg_status fg_space_get_dof_map(fg_space* sp, int32_t* lst) {
  FG_CHECK_ARG(sp && lst, "space/out");
  FG_DEVICE_GUARD(sp->mesh->ctx);
  return space_export_dof_map(sp, lst);
}

fg_status fg_space_get_dirichlet_coords(fg_space* sp, double* xyz) {
  FG_CHECK_ARG(sp && xyz, "space/out");
  fg_ctx* ctx = sp->mesh->ctx;
  FG_DEVICE_GUARD(ctx);
  if (sp->ndir == 0) return FG_OK;
  double* d = nullptr;
  FG_TRY(dev_alloc(ctx, (void**)&d, sizeof(double) * 3 * sp->ndir));
  fg_status s = space_dirichlet_coords(sp, d);
  if (s == FG_OK) {
    cudaError_t e = cudaMemcpyAsync(xyz, d, sizeof(double) * 3 * sp->ndir, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { set_error("%s", cudaGetErrorString(e)); s = FG_ERR_CUDA; }
  }
  dev_free(ctx, d);
  return s;
}

fg_status fg_space_get_qp_coords(fg_space* sp, double* xyz, int on_device) {
  FG_CHECK_ARG(sp && xyz, "space/out");
  fg_ctx* ctx = sp->mesh->ctx;
  FG_DEVICE_GUARD(ctx);
  const int64_t n = sp->mesh->ncells * sp->tab.nq * 3;
  if (n == 0) return FG_OK;
  if (on_device) {
    FG_TRY(space_qp_coords(sp, xyz));
    FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return FG_OK;
  }
  double* d = nullptr;
  FG_TRY(dev_alloc(ctx, (void**)&d, sizeof(double) * n));
  fg_status s = space_qp_coords(sp, d);
  if (s == FG_OK) {
    cudaError_t e = cudaMemcpyAsync(xyz, d, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { set_error("%s", cudaGetErrorString(e)); s = FG_ERR_CUDA; }
  }
  dev_free(ctx, d);
  return s;
}

static void system_free(fg_system* sys) {
  fg_ctx* ctx = sys->space->mesh->ctx;
  void* ptrs[] = {sys->d_val, sys->d_val32, sys->d_rhs, sys->d_gvals, sys->d_elmat, sys->d_elvec, sys->d_coef,
                  sys->d_qpsrc, sys->d_sval, sys->d_sval32, sys->d_tval, sys->d_tval32, sys->d_idiag, sys->d_idiag32, sys->d_work, sys->d_work32, sys->d_red, sys->d_ticket,
                  sys->d_val32s, sys->d_sdiag, sys->d_tcbuf};
  for (void* p : ptrs) dev_free(ctx, p);
  delete sys;
}

// copy (or alias-copy) an optional input array of n doubles to a device buffer
static fg_status stage_input(fg_ctx* ctx, const double* src, int64_t n, bool on_device, double** dst) {
  if (!src) return FG_OK;
  if (!*dst) FG_TRY(dev_alloc(ctx, (void**)dst, sizeof(double) * (n > 0 ? n : 1)));
  FG_CUDA_TRY(cudaMemcpyAsync(*dst, src, sizeof(double) * n, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                              ctx->stream));
  return FG_OK;
}

static fg_status numeric_phase(fg_system* sys, const fg_integrand* g) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  const bool dev = (g->flags & FG_INPUTS_ON_DEVICE) != 0;
  sys->integ = *g;
  if (g->kind == FG_ELASTICITY && sp->ncomp != sp->mesh->dim) {
    set_error("elasticity needs ncomp = %d", sp->mesh->dim);
    return FG_ERR_BADARG;
  }
  if (g->kind == FG_POISSON && sp->ncomp != 1) { set_error("Poisson needs ncomp=1"); return FG_ERR_BADARG; }
  if (g->cell_coef) FG_TRY(stage_input(ctx, g->cell_coef, sp->mesh->ncells, dev, &sys->d_coef));
  else if (sys->d_coef) { dev_free(ctx, sys->d_coef); sys->d_coef = nullptr; }
  if (g->source_fn == FG_FN_QP_VALUES) {
    FG_CHECK_ARG(g->qp_source, "qp_source");
    FG_TRY(stage_input(ctx, g->qp_source, sp->mesh->ncells * sp->tab.nq * sp->ncomp, dev, &sys->d_qpsrc));
  }
  if (g->dirichlet_values) {
    FG_TRY(stage_input(ctx, g->dirichlet_values, sp->ndir, dev, &sys->d_gvals));
  } else if (sp->ndir > 0) {
    FG_TRY(system_interpolate_dirichlet(sys, g->boundary_fn, g->fn_param));
  }
  FG_TRY(system_assemble(sys));
  sys->scaled_valid = false;
  if (sys->lean) {
    // element matrices are scratch of the scatter: release them before the solver layout
    dev_free(ctx, sys->d_elmat);
    dev_free(ctx, sys->d_elvec);
    dev_free(ctx, sys->d_tcbuf);
    sys->d_elmat = sys->d_elvec = nullptr;
    sys->d_tcbuf = nullptr;
    sys->tcbuf_bytes = 0;
    if (sp->layout == FG_LAYOUT_SELL) {
      FG_TRY(dev_alloc(ctx, (void**)&sys->d_sval, sizeof(double) * (sp->sell_nnz > 0 ? sp->sell_nnz : 1)));
      FG_TRY(dev_alloc(ctx, (void**)&sys->d_sval32, sizeof(float) * (sp->sell_nnz > 0 ? sp->sell_nnz : 1)));
    } else {
      FG_TRY(dev_alloc(ctx, (void**)&sys->d_tval, sizeof(double) * (sp->st_nvals > 0 ? sp->st_nvals : 1)));
      FG_TRY(dev_alloc(ctx, (void**)&sys->d_tval32, sizeof(float) * (sp->st_nvals > 0 ? sp->st_nvals : 1)));
    }
  }
  if (sp->layout == FG_LAYOUT_SELL) FG_TRY(system_fill_sell(sys));
  else if (!sys->direct) FG_TRY(system_fill_stencil(sys));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return FG_OK;
}

fg_status fg_assemble(fg_space* sp, const fg_integrand* g, fg_system** out) {
  FG_CHECK_ARG(sp && g && out, "space/integrand/out");
  *out = nullptr;
  fg_ctx* ctx = sp->mesh->ctx;
  FG_DEVICE_GUARD(ctx);
  if (!sp->d_rowptr || !sp->d_col) {
    set_error("the space's sparsity pattern was released");
    return FG_ERR_UNSUPPORTED;
  }
  fg_system* sys = new fg_system();
  sys->space = sp;
  sys->lean = (g->flags & FG_LEAN_SYSTEM) != 0;
  const int64_t ncells = sp->mesh->ncells, nd = sp->tab.nd;
  fg_status s = FG_OK;
  auto A = [&](void** p, size_t b) { if (s == FG_OK) s = dev_alloc(ctx, p, b); };
  // the row gather writes the lattice-implicit layout directly where it can (the CSR values
  // are then derived from it on export); otherwise it fills the CSR first
  if (sys->lean || !stencil_direct_ok(sp)) A((void**)&sys->d_val, sizeof(double) * (sp->nnz > 0 ? sp->nnz : 1));
  if (sys->lean) {
    // solver-layout arrays are allocated after the element matrices are released
  } else if (sp->layout == FG_LAYOUT_SELL) {
    A((void**)&sys->d_sval, sizeof(double) * (sp->sell_nnz > 0 ? sp->sell_nnz : 1));
    A((void**)&sys->d_sval32, sizeof(float) * (sp->sell_nnz > 0 ? sp->sell_nnz : 1));
  } else {
    A((void**)&sys->d_tval, sizeof(double) * (sp->st_nvals > 0 ? sp->st_nvals : 1));
    A((void**)&sys->d_tval32, sizeof(float) * (sp->st_nvals > 0 ? sp->st_nvals : 1));
  }
  A((void**)&sys->d_rhs, sizeof(double) * (sp->nfree > 0 ? sp->nfree : 1));
  A((void**)&sys->d_gvals, sizeof(double) * (sp->ndir > 0 ? sp->ndir : 1));
  A((void**)&sys->d_elmat, sizeof(double) * ncells * nd * nd);
  A((void**)&sys->d_elvec, sizeof(double) * ncells * nd);
  if (s == FG_OK) s = numeric_phase(sys, g);
  if (s == FG_OK) s = system_prepare_diag(sys);
  if (s == FG_OK) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { set_error("assemble: %s", cudaGetErrorString(e)); s = FG_ERR_CUDA; }
  }
  if (s == FG_OK && sys->lean) {
    dev_free(ctx, sys->d_val);
    sys->d_val = nullptr;
  }
  if (s != FG_OK) {
    system_free(sys);
    return s;
  }
  *out = sys;
  return FG_OK;
}

fg_status fg_system_reassemble(fg_system* sys, const fg_integrand* g) {
  FG_CHECK_ARG(sys && g, "system/integrand");
  if (sys->lean) {
    set_error("the system was assembled lean (FG_LEAN_SYSTEM): reassembly needs a full system");
    return FG_ERR_UNSUPPORTED;
  }
  FG_DEVICE_GUARD(sys->space->mesh->ctx);
  FG_TRY(numeric_phase(sys, g));
  FG_TRY(system_prepare_diag(sys));
  FG_CUDA_TRY(cudaStreamSynchronize(sys->space->mesh->ctx->stream));
  return FG_OK;
}

fg_status fg_system_destroy(fg_system* sys) {
  if (!sys) return FG_OK;
  cudaSetDevice(sys->space->mesh->ctx->device);
  cudaStreamSynchronize(sys->space->mesh->ctx->stream);
  system_free(sys);
  return FG_OK;
}

fg_status fg_system_export_csr(fg_system* sys, int symmetric_storage, int one_based, int64_t* irp, int32_t* ja,
                               double* val) {
  FG_CHECK_ARG(sys, "system");
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  FG_DEVICE_GUARD(ctx);
  if (sys->direct) FG_TRY(system_ensure_csr(sys));
  if (!sys->d_val || !sp->d_rowptr || !sp->d_col) {
    set_error("the CSR of this system was released (FG_LEAN_SYSTEM / fg_space_release_pattern)");
    return FG_ERR_UNSUPPORTED;
  }
  one_based = one_based ? 1 : 0;
  if (symmetric_storage) return space_export_upper(sp, sys->d_val, one_based, irp, ja, val);
  const int64_t n = sp->nfree;
  if (irp) {
    FG_CUDA_TRY(cudaMemcpyAsync(irp, sp->d_rowptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, ctx->stream));
  }
  if (ja && sp->nnz) FG_CUDA_TRY(cudaMemcpyAsync(ja, sp->d_col, sizeof(int32_t) * sp->nnz, cudaMemcpyDeviceToHost, ctx->stream));
  if (val && sp->nnz) FG_CUDA_TRY(cudaMemcpyAsync(val, sys->d_val, sizeof(double) * sp->nnz, cudaMemcpyDeviceToHost, ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (one_based) {
    if (irp) for (int64_t i = 0; i <= n; ++i) irp[i] += 1;
    if (ja) for (int64_t i = 0; i < sp->nnz; ++i) ja[i] += 1;
  }
  return FG_OK;
}

fg_status fg_system_export_rhs(fg_system* sys, double* rhs) {
  FG_CHECK_ARG(sys && rhs, "system/rhs");
  fg_ctx* ctx = sys->space->mesh->ctx;
  FG_DEVICE_GUARD(ctx);
  if (sys->space->nfree == 0) return FG_OK;
  FG_CUDA_TRY(cudaMemcpyAsync(rhs, sys->d_rhs, sizeof(double) * sys->space->nfree, cudaMemcpyDeviceToHost, ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return FG_OK;
}

fg_status fg_system_export_dirichlet_values(fg_system* sys, double* g) {
  FG_CHECK_ARG(sys && g, "system/g");
  fg_ctx* ctx = sys->space->mesh->ctx;
  FG_DEVICE_GUARD(ctx);
  if (sys->space->ndir == 0) return FG_OK;
  FG_CUDA_TRY(cudaMemcpyAsync(g, sys->d_gvals, sizeof(double) * sys->space->ndir, cudaMemcpyDeviceToHost, ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return FG_OK;
}

fg_status fg_system_spmv_device(fg_system* sys, int precision, const void* x, void* y) {
  FG_CHECK_ARG(sys && x && y, "system/x/y");
  fg_ctx* ctx = sys->space->mesh->ctx;
  FG_DEVICE_GUARD(ctx);
  FG_TRY(system_spmv(sys, precision, x, y, ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return FG_OK;
}

fg_status fg_system_spmv_solver_layout_device(fg_system* sys, int precision, const void* x_slot, void* y_slot,
                                              int reps) {
  FG_CHECK_ARG(sys && x_slot && y_slot && reps >= 0, "system/x/y/reps");
  FG_DEVICE_GUARD(sys->space->mesh->ctx);
  return system_spmv_slot(sys, precision, x_slot, y_slot, reps, sys->space->mesh->ctx->stream);
}

static fg_status check_params(const fg_solver_params* p) {
  if (!p) { set_error("params"); return FG_ERR_BADARG; }
  if (p->precision != FG_FP64 && p->precision != FG_MIXED) { set_error("precision"); return FG_ERR_BADARG; }
  if (p->precond != FG_PREC_NONE && p->precond != FG_PREC_JACOBI) { set_error("precond"); return FG_ERR_BADARG; }
  if (p->criterion < FG_RES_RES || p->criterion > FG_RES_NRMGIVEN_RES_NRMGIVEN) { set_error("criterion"); return FG_ERR_BADARG; }
  if (p->precision == FG_MIXED && p->criterion != FG_RES_RES && p->criterion != FG_RES_RHS) {
    set_error("mixed precision supports the res_res and res_rhs criteria");
    return FG_ERR_UNSUPPORTED;
  }
  if (!(p->rtol >= 0.0) || !(p->atol >= 0.0) || p->max_iters < 1) { set_error("rtol/atol/max_iters"); return FG_ERR_BADARG; }
  return FG_OK;
}

fg_status fg_solve_device(fg_system* sys, const fg_solver_params* params, const double* b_dev, const double* x0_dev,
                          double* x_dev, fg_solve_info* info) {
  FG_CHECK_ARG(sys && x_dev, "system/x");
  FG_TRY(check_params(params));
  FG_DEVICE_GUARD(sys->space->mesh->ctx);
  return system_solve(sys, params, b_dev, x0_dev, x_dev, info);
}

fg_status fg_solve(fg_system* sys, const fg_solver_params* params, const double* b, const double* x0, double* x,
                   fg_solve_info* info) {
  FG_CHECK_ARG(sys && x, "system/x");
  FG_TRY(check_params(params));
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  FG_DEVICE_GUARD(ctx);
  const int64_t n = sp->nfree;
  double *db = nullptr, *dx0 = nullptr, *dx = nullptr;
  fg_status s = FG_OK;
  auto cleanup = [&]() { dev_free(ctx, db); dev_free(ctx, dx0); dev_free(ctx, dx); };
  if (b) { s = stage_input(ctx, b, n, false, &db); }
  if (s == FG_OK && x0) s = stage_input(ctx, x0, n, false, &dx0);
  if (s == FG_OK) s = dev_alloc(ctx, (void**)&dx, sizeof(double) * (n > 0 ? n : 1));
  if (s != FG_OK) { cleanup(); return s; }
  fg_status ss = system_solve(sys, params, db, dx0, dx, info);
  if (ss == FG_OK || ss == FG_ERR_NOT_CONVERGED) {
    cudaError_t e = cudaMemcpyAsync(x, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { set_error("%s", cudaGetErrorString(e)); ss = FG_ERR_CUDA; }
  }
  cleanup();
  return ss;
}

}  // extern "C"

// fg_unstructured.cu -- unstructured hexahedral meshes on the device: the mesh-data-files
// route of the serial triangulation (sbm_serial_triangulation.i90:120-188).
//
// Topology (fg_mesh_create_unstructured).
//   - cells around every vertex, ascending (sbm_base_static_triangulation.i90:697-739);
//   - edges, then faces, numbered in order of first appearance when the cells are walked
//     in order and each cell's n-faces in the reference FE's local order
//     (sbm_fine_triangulation.i90:115-315).  On the device every (cell, local n-face)
//     looks for an earlier cell around its smallest vertex that holds the same vertex set;
//     the first holders are flagged, an exclusive scan over the flags in (cell, n-face)
//     order gives each new vef its id, and the other holders copy it.  Same ids as the
//     reference's sequential walk;
//   - set ids of the given boundary vefs, later entries overwrite earlier ones
//     (sbm_fine_triangulation.i90:317-444);
//   - boundary faces (one cell around) hand their set id to the edges and vertices of their
//     closure that have none; the face with the smallest id wins, as in the reference's walk
//     over the vefs in id order (sbm_fine_triangulation.i90:453-527).
//
// Space (fg_space_create on such a mesh).  Nodes: vertices, then p-1 per edge, (p-1)^2
// per face, (p-1)^3 per cell.  A vef's own nodes are numbered in the local order of its
// first cell (the cell that numbers its dofs); another cell reaches them through the
// corner correspondence of the shared vef (the reference's own-dof permutations,
// fetch_own_dofs_vef_from_source_fe in sbm_fe_cell_iterator.i90:736-856).  Dof numbering
// is the structured path's rule with explicit owners: the Dirichlet pass numbers the own
// dofs of Dirichlet vefs -1,-2,... and the free pass cell interiors then vefs 1,2,...,
// each in the first cell that visits them (sbm_serial_fe_space.i90:525-716, :2623-2884).
//
// Sparsity: one warp per row gathers the dofs of the cells around the row's node, sorts
// them (bitonic, shared memory) and keeps the distinct free ones -- the set and order of
// the reference's COO -> sort_and_compress.  Assembly: one warp per row walks the cells
// around the row's node in increasing cell order and adds their element-matrix rows, so
// every entry is summed in the reference's order; no atomics.
#include "fg_internal.h"

namespace fg {

static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// Local n-faces of the hexahedron in the reference FE's order (dimension, then code).
struct HexNF {
  int8_t code[26];
  int8_t dim[26];
  int8_t nvert[26];
  int8_t vert[26][4];
  int8_t sub[6][8];  // edges and vertices on each face
};

static HexNF make_hexnf(const int* codes) {
  HexNF h;
  for (int f = 0; f < 26; ++f) {
    const int code = codes[f], anchor = code & 7, t = code >> 3;
    h.code[f] = (int8_t)code;
    h.dim[f] = (int8_t)__builtin_popcount(t);
    int n = 0;
    for (int s = 0; s < 8; ++s)
      if ((s & ~t) == 0) h.vert[f][n++] = (int8_t)(anchor | s);
    h.nvert[f] = (int8_t)n;
    for (int k = n; k < 4; ++k) h.vert[f][k] = -1;
  }
  for (int fi = 0; fi < 6; ++fi) {
    const int f = 20 + fi;
    int n = 0;
    for (int f2 = 0; f2 < 20; ++f2) {
      bool in = true;
      for (int k = 0; k < h.nvert[f2]; ++k) {
        bool hit = false;
        for (int m = 0; m < 4; ++m) hit = hit || (h.vert[f][m] == h.vert[f2][k]);
        in = in && hit;
      }
      if (in) h.sub[fi][n++] = (int8_t)f2;
    }
  }
  return h;
}

__device__ __forceinline__ void sort_small(int32_t* g, int n) {
  for (int i = 1; i < n; ++i) {
    int32_t v = g[i];
    int j = i - 1;
    while (j >= 0 && g[j] > v) { g[j + 1] = g[j]; --j; }
    g[j + 1] = v;
  }
}

__device__ __forceinline__ void nface_sorted(const HexNF& h, const int32_t* cellvert, int64_t c, int f, int32_t* g) {
  const int n = h.nvert[f];
  for (int k = 0; k < n; ++k) g[k] = cellvert[c * 8 + h.vert[f][k]];
  sort_small(g, n);
}

// ---- cells around vertices -------------------------------------------------------------
__global__ void k_vcount(int64_t n, const int32_t* cellvert, unsigned long long* cnt) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(&cnt[cellvert[i]], 1ull);
}
__global__ void k_vfill(int64_t n, const int32_t* cellvert, unsigned long long* cursor, int32_t* vcells) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) vcells[atomicAdd(&cursor[cellvert[i]], 1ull)] = (int32_t)(i / 8);
}
__global__ void k_sort_segments_i32(int64_t nseg, const int64_t* ptr, int32_t* v, int* maxlen) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const int64_t a = ptr[s], b = ptr[s + 1];
  for (int64_t i = a + 1; i < b; ++i) {
    int32_t x = v[i];
    int64_t j = i - 1;
    while (j >= a && v[j] > x) { v[j + 1] = v[j]; --j; }
    v[j + 1] = x;
  }
  atomicMax(maxlen, (int)(b - a));
}
__global__ void k_sort_segments_i64(int64_t nseg, const int64_t* ptr, int64_t* v, int* maxlen) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const int64_t a = ptr[s], b = ptr[s + 1];
  for (int64_t i = a + 1; i < b; ++i) {
    int64_t x = v[i];
    int64_t j = i - 1;
    while (j >= a && v[j] > x) { v[j + 1] = v[j]; --j; }
    v[j + 1] = x;
  }
  atomicMax(maxlen, (int)(b - a));
}

// ---- edges and faces by first appearance -------------------------------------------------
// (cell, local n-face) of dimension DIM: is it the first holder of its vertex set, who is,
// and how many cells hold it.
template <int DIM>
__global__ void k_nface_match(int64_t nc, const int32_t* __restrict__ cellvert, const int64_t* __restrict__ vptr,
                              const int32_t* __restrict__ vcells, HexNF h, int64_t* flag, int64_t* src,
                              int32_t* nbr) {
  constexpr int NF = DIM == 1 ? 12 : 6, F0 = DIM == 1 ? 8 : 20, NV = DIM == 1 ? 2 : 4;
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= nc * NF) return;
  const int64_t c = idx / NF;
  const int f = F0 + (int)(idx % NF);
  int32_t g[4], g2[4];
  nface_sorted(h, cellvert, c, f, g);
  int64_t found = -1;
  int count = 0;
  for (int64_t k = vptr[g[0]]; k < vptr[g[0] + 1]; ++k) {
    const int64_t c2 = vcells[k];
    if (c2 == c) { ++count; continue; }
    for (int f2 = F0; f2 < F0 + NF; ++f2) {
      nface_sorted(h, cellvert, c2, f2, g2);
      bool eq = true;
#pragma unroll
      for (int m = 0; m < NV; ++m) eq = eq && (g[m] == g2[m]);
      if (eq) {
        ++count;
        if (c2 < c && found < 0) found = c2 * 32 + f2;
        break;
      }
    }
  }
  flag[idx] = found < 0 ? 1 : 0;
  src[idx] = found < 0 ? c * 32 + f : found;
  nbr[idx] = count;
}

template <int DIM>
__global__ void k_nface_ids(int64_t nc, const int64_t* __restrict__ rank, const int64_t* __restrict__ src,
                            const int32_t* __restrict__ nbr, int64_t base, int64_t nv, int32_t* cellvef,
                            int64_t* vowner, int32_t* vnbr) {
  constexpr int NF = DIM == 1 ? 12 : 6, F0 = DIM == 1 ? 8 : 20;
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= nc * NF) return;
  const int64_t c = idx / NF;
  const int f = F0 + (int)(idx % NF);
  const int64_t s = src[idx];
  const int64_t c0 = s >> 5;
  const int f0 = (int)(s & 31);
  const int64_t id = base + rank[c0 * NF + (f0 - F0)];
  cellvef[c * 26 + f] = (int32_t)id;
  if (c0 == c && f0 == f) {
    vowner[id - nv] = s;
    vnbr[id - nv] = nbr[idx];
  }
}

__global__ void k_cell_vertices_as_vefs(int64_t nc, const int32_t* cellvert, int32_t* cellvef) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < nc * 8) cellvef[(i / 8) * 26 + (i % 8)] = cellvert[i];
}

// ---- set ids ---------------------------------------------------------------------------
__global__ void k_given_find(int64_t nb, const int64_t* __restrict__ bptr, const int32_t* __restrict__ bverts,
                             const int32_t* __restrict__ cellvert, const int32_t* __restrict__ cellvef,
                             const int64_t* __restrict__ vptr, const int32_t* __restrict__ vcells, HexNF h,
                             int32_t* gid, unsigned long long* win) {
  const int64_t ib = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (ib >= nb) return;
  const int64_t b0 = bptr[ib];
  const int n = (int)(bptr[ib + 1] - b0);
  int32_t g = -1;
  if (n == 1) {
    g = bverts[b0] - 1;
  } else if (n == 2 || n == 4) {
    const int dim = n == 2 ? 1 : 2, F0 = n == 2 ? 8 : 20, NF = n == 2 ? 12 : 6;
    int32_t gv[4], g2[4];
    for (int k = 0; k < n; ++k) gv[k] = bverts[b0 + k] - 1;
    const int32_t v0 = gv[0];
    sort_small(gv, n);
    for (int64_t k = vptr[v0]; k < vptr[v0 + 1] && g < 0; ++k) {
      const int64_t c2 = vcells[k];
      for (int f2 = F0; f2 < F0 + NF; ++f2) {
        if (h.dim[f2] != dim) continue;
        nface_sorted(h, cellvert, c2, f2, g2);
        bool eq = true;
        for (int m = 0; m < n; ++m) eq = eq && (gv[m] == g2[m]);
        if (eq) { g = cellvef[c2 * 26 + f2]; break; }
      }
    }
  }
  gid[ib] = g;
  if (g >= 0) atomicMax(&win[g], (unsigned long long)(ib + 1));
}

__global__ void k_given_apply(int64_t nb, const int32_t* gid, const unsigned long long* win, const int32_t* bset,
                              int32_t* vset) {
  const int64_t ib = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (ib >= nb) return;
  const int32_t g = gid[ib];
  if (g >= 0 && win[g] == (unsigned long long)(ib + 1)) vset[g] = bset[ib];
}

__global__ void k_face_propagate(int64_t nfaces, int64_t nv, int64_t ne, const int64_t* __restrict__ vowner,
                                 const int32_t* __restrict__ vnbr, const int32_t* __restrict__ cellvef,
                                 const int32_t* __restrict__ vset, HexNF h, int32_t* win) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nfaces) return;
  const int64_t gid = nv + ne + i;
  if (vnbr[ne + i] != 1) return;
  const int32_t sid = vset[gid];
  if (sid == 0) return;
  const int64_t s = vowner[ne + i];
  const int64_t c = s >> 5;
  const int f = (int)(s & 31);
  for (int k = 0; k < 8; ++k) {
    const int32_t sv = cellvef[c * 26 + h.sub[f - 20][k]];
    if (vset[sv] == 0) atomicMin(&win[sv], (int32_t)gid);
  }
}

__global__ void k_face_apply(int64_t n, const int32_t* win, int32_t* vset) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int32_t w = win[s];
  if (w != 0x7f7f7f7f) vset[s] = vset[w];
}

// exclusive scan of n int64 in place (cub, as fg_space.cu), total returned
fg_status scan_i64(fg_ctx* ctx, int64_t* a, int64_t n, int64_t* total);

static fg_status upload(fg_ctx* ctx, void** d, const void* h, size_t bytes) {
  FG_TRY(dev_alloc(ctx, d, bytes > 0 ? bytes : 8));
  if (bytes) FG_CUDA_TRY(cudaMemcpyAsync(*d, h, bytes, cudaMemcpyHostToDevice, ctx->stream));
  return FG_OK;
}

// Cells around each of the n vertices referenced by the ne = 8*ncells entries of the cell
// vertex table (ascending).
static fg_status build_adjacency_i32(fg_ctx* ctx, const int32_t* keys, int64_t ne, int64_t n, int64_t** ptr,
                                     int32_t** list, int* maxlen) {
  unsigned long long* cnt = nullptr;
  FG_TRY(dev_alloc(ctx, (void**)ptr, sizeof(int64_t) * (n + 1)));
  FG_CUDA_TRY(cudaMemsetAsync(*ptr, 0, sizeof(int64_t) * (n + 1), ctx->stream));
  k_vcount<<<nblk(ne, 256), 256, 0, ctx->stream>>>(ne, keys, (unsigned long long*)*ptr);
  int64_t tot = 0;
  FG_TRY(scan_i64(ctx, *ptr, n + 1, &tot));
  FG_TRY(dev_alloc(ctx, (void**)list, sizeof(int32_t) * (ne > 0 ? ne : 1)));
  FG_TRY(dev_alloc(ctx, (void**)&cnt, sizeof(int64_t) * (n + 1)));
  FG_CUDA_TRY(cudaMemcpyAsync(cnt, *ptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToDevice, ctx->stream));
  k_vfill<<<nblk(ne, 256), 256, 0, ctx->stream>>>(ne, keys, cnt, *list);
  int* dmax = (int*)cnt;
  FG_CUDA_TRY(cudaMemsetAsync(dmax, 0, sizeof(int), ctx->stream));
  k_sort_segments_i32<<<nblk(n, 128), 128, 0, ctx->stream>>>(n, *ptr, *list, dmax);
  FG_CUDA_TRY(cudaMemcpyAsync(maxlen, dmax, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, cnt);
  return FG_OK;
}

fg_status umesh_build_topology(fg_mesh* m, int64_t nb, const int64_t* bptr, const int32_t* bverts,
                               const int32_t* bset) {
  fg_ctx* ctx = m->ctx;
  int codes[27];
  {
    RefTables t;
    t.build(1, 1);
    for (int i = 0; i < 27; ++i) codes[i] = t.codes[i];
  }
  const HexNF h = make_hexnf(codes);
  const int64_t nc = m->ncells, nv = m->nverts;
  FG_TRY(build_adjacency_i32(ctx, m->d_cellvert, nc * 8, nv, &m->d_vptr, &m->d_vcells, &m->max_vcells));
  FG_TRY(dev_alloc(ctx, (void**)&m->d_cellvef, sizeof(int32_t) * nc * 26));
  k_cell_vertices_as_vefs<<<nblk(nc * 8, 256), 256, 0, ctx->stream>>>(nc, m->d_cellvert, m->d_cellvef);
  // edges then faces; the match/flag arrays of both are kept until the ids are written
  int64_t *eflag = nullptr, *esrc = nullptr, *fflag = nullptr, *fsrc = nullptr;
  int32_t *enbr = nullptr, *fnbr = nullptr;
  const int64_t ne_loc = nc * 12, nf_loc = nc * 6;
  FG_TRY(dev_alloc(ctx, (void**)&eflag, sizeof(int64_t) * ne_loc));
  FG_TRY(dev_alloc(ctx, (void**)&esrc, sizeof(int64_t) * ne_loc));
  FG_TRY(dev_alloc(ctx, (void**)&enbr, sizeof(int32_t) * ne_loc));
  FG_TRY(dev_alloc(ctx, (void**)&fflag, sizeof(int64_t) * nf_loc));
  FG_TRY(dev_alloc(ctx, (void**)&fsrc, sizeof(int64_t) * nf_loc));
  FG_TRY(dev_alloc(ctx, (void**)&fnbr, sizeof(int32_t) * nf_loc));
  k_nface_match<1><<<nblk(ne_loc, 128), 128, 0, ctx->stream>>>(nc, m->d_cellvert, m->d_vptr, m->d_vcells, h, eflag,
                                                                esrc, enbr);
  k_nface_match<2><<<nblk(nf_loc, 128), 128, 0, ctx->stream>>>(nc, m->d_cellvert, m->d_vptr, m->d_vcells, h, fflag,
                                                               fsrc, fnbr);
  FG_CUDA_TRY(cudaGetLastError());
  FG_TRY(scan_i64(ctx, eflag, ne_loc, &m->nedges));
  FG_TRY(scan_i64(ctx, fflag, nf_loc, &m->nfaces));
  m->nvefs = nv + m->nedges + m->nfaces;
  if (m->nvefs >= (int64_t)0x7f7f7f7f) {
    set_error("vef count exceeds int32 ids");
    return FG_ERR_UNSUPPORTED;
  }
  const int64_t nef = m->nedges + m->nfaces;
  FG_TRY(dev_alloc(ctx, (void**)&m->d_vowner, sizeof(int64_t) * (nef > 0 ? nef : 1)));
  FG_TRY(dev_alloc(ctx, (void**)&m->d_vnbr, sizeof(int32_t) * (nef > 0 ? nef : 1)));
  k_nface_ids<1><<<nblk(ne_loc, 256), 256, 0, ctx->stream>>>(nc, eflag, esrc, enbr, nv, nv, m->d_cellvef, m->d_vowner,
                                                             m->d_vnbr);
  k_nface_ids<2><<<nblk(nf_loc, 256), 256, 0, ctx->stream>>>(nc, fflag, fsrc, fnbr, nv + m->nedges, nv, m->d_cellvef,
                                                             m->d_vowner, m->d_vnbr);
  FG_CUDA_TRY(cudaGetLastError());
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, eflag);
  dev_free(ctx, esrc);
  dev_free(ctx, enbr);
  dev_free(ctx, fflag);
  dev_free(ctx, fsrc);
  dev_free(ctx, fnbr);
  // set ids
  FG_TRY(dev_alloc(ctx, (void**)&m->d_vset, sizeof(int32_t) * m->nvefs));
  FG_CUDA_TRY(cudaMemsetAsync(m->d_vset, 0, sizeof(int32_t) * m->nvefs, ctx->stream));
  if (nb > 0) {
    int64_t* d_bptr = nullptr;
    int32_t *d_bverts = nullptr, *d_bset = nullptr, *d_gid = nullptr;
    unsigned long long* win = nullptr;
    FG_TRY(upload(ctx, (void**)&d_bptr, bptr, sizeof(int64_t) * (nb + 1)));
    FG_TRY(upload(ctx, (void**)&d_bverts, bverts, sizeof(int32_t) * bptr[nb]));
    FG_TRY(upload(ctx, (void**)&d_bset, bset, sizeof(int32_t) * nb));
    FG_TRY(dev_alloc(ctx, (void**)&d_gid, sizeof(int32_t) * nb));
    FG_TRY(dev_alloc(ctx, (void**)&win, sizeof(unsigned long long) * m->nvefs));
    FG_CUDA_TRY(cudaMemsetAsync(win, 0, sizeof(unsigned long long) * m->nvefs, ctx->stream));
    k_given_find<<<nblk(nb, 128), 128, 0, ctx->stream>>>(nb, d_bptr, d_bverts, m->d_cellvert, m->d_cellvef, m->d_vptr,
                                                         m->d_vcells, h, d_gid, win);
    k_given_apply<<<nblk(nb, 256), 256, 0, ctx->stream>>>(nb, d_gid, win, d_bset, m->d_vset);
    FG_CUDA_TRY(cudaGetLastError());
    FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    dev_free(ctx, d_bptr);
    dev_free(ctx, d_bverts);
    dev_free(ctx, d_bset);
    dev_free(ctx, d_gid);
    dev_free(ctx, win);
  }
  if (m->nfaces > 0) {
    const int64_t nlow = nv + m->nedges;
    int32_t* win = nullptr;
    FG_TRY(dev_alloc(ctx, (void**)&win, sizeof(int32_t) * nlow));
    // 0x7f7f7f7f (every byte 0x7f) marks "no face"; vef ids stay below it (checked above)
    FG_CUDA_TRY(cudaMemsetAsync(win, 0x7f, sizeof(int32_t) * nlow, ctx->stream));
    k_face_propagate<<<nblk(m->nfaces, 256), 256, 0, ctx->stream>>>(m->nfaces, nv, m->nedges, m->d_vowner, m->d_vnbr,
                                                                    m->d_cellvef, m->d_vset, h, win);
    k_face_apply<<<nblk(nlow, 256), 256, 0, ctx->stream>>>(nlow, win, m->d_vset);
    FG_CUDA_TRY(cudaGetLastError());
    FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    dev_free(ctx, win);
  }
  ctx->launches += 12;
  return FG_OK;
}

// ================================ space ===================================================
struct UGeom {
  int p, ncomp, nn;
  int64_t nc, nv, ne, nf;
  int64_t ebase, fbase, ibase;  // first node of edges, faces, cell interiors
  uint32_t dirmask;
  int code2idx[64];
  HexNF h;
};

static UGeom make_ugeom(const fg_space* sp) {
  UGeom g;
  const fg_mesh* m = sp->mesh;
  g.p = sp->order;
  g.ncomp = sp->ncomp;
  g.nn = sp->tab.nn;
  g.nc = m->ncells;
  g.nv = m->nverts;
  g.ne = m->nedges;
  g.nf = m->nfaces;
  const int64_t pm1 = g.p - 1;
  g.ebase = g.nv;
  g.fbase = g.ebase + g.ne * pm1;
  g.ibase = g.fbase + g.nf * pm1 * pm1;
  g.dirmask = sp->dirmask;
  for (int i = 0; i < 64; ++i) g.code2idx[i] = sp->tab.code2idx[i];
  g.h = make_hexnf(sp->tab.codes);
  return g;
}

// First node of the own nodes of vef `gid` (dimension m).
__device__ __forceinline__ int64_t vef_node_base(const UGeom& g, int m, int64_t gid) {
  const int64_t pm1 = g.p - 1;
  return m == 1 ? g.ebase + (gid - g.nv) * pm1 : g.fbase + (gid - g.nv - g.ne) * pm1 * pm1;
}

// node id of local node a of every cell
__global__ void k_ucellnode(UGeom g, int64_t nnodes, const int32_t* __restrict__ cellvert,
                            const int32_t* __restrict__ cellvef, const int64_t* __restrict__ vowner, int32_t* cellnode,
                            int* err) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= g.nc * g.nn) return;
  const int64_t c = idx / g.nn;
  const int a = (int)(idx % g.nn);
  const int p = g.p, np1 = p + 1, pm1 = p - 1;
  const int ijk[3] = {a % np1, (a / np1) % np1, a / (np1 * np1)};
  int anchor = 0, t = 0;
  for (int d = 0; d < 3; ++d) {
    if (ijk[d] == p) anchor |= 1 << d;
    else if (ijk[d] > 0) t |= 1 << d;
  }
  int64_t node;
  if (t == 0) {
    node = cellvert[c * 8 + anchor];
  } else if (t == 7) {
    node = g.ibase + c * pm1 * pm1 * pm1 + (ijk[0] - 1) + pm1 * ((ijk[1] - 1) + pm1 * (ijk[2] - 1));
  } else {
    const int f = g.code2idx[anchor | (t << 3)];
    const int64_t gid = cellvef[c * 26 + f];
    const int m = __popc(t);
    const int64_t s = vowner[gid - g.nv];
    const int64_t c0 = s >> 5;
    const int code0 = g.h.code[s & 31];
    const int a0 = code0 & 7, t0 = code0 >> 3;
    int d[2], e[2], md = 0, me = 0;
    for (int k = 0; k < 3; ++k) {
      if ((t >> k) & 1) d[md++] = k;
      if ((t0 >> k) & 1) e[me++] = k;
    }
    // corner bits of the owner -> corner bits of this cell, through the vertex ids
    int M[4] = {0, 0, 0, 0};
    for (int u = 0; u < (1 << m); ++u) {
      int v0 = a0;
      for (int k = 0; k < m; ++k) if ((u >> k) & 1) v0 |= 1 << e[k];
      const int32_t gv = cellvert[c0 * 8 + v0];
      for (int b = 0; b < (1 << m); ++b) {
        int v = anchor;
        for (int k = 0; k < m; ++k) if ((b >> k) & 1) v |= 1 << d[k];
        if (cellvert[c * 8 + v] == gv) M[u] = b;
      }
    }
    int kn = 0, mul = 1;
    for (int k = 0; k < m; ++k) {
      const int diff = M[0] ^ M[1 << k];
      if (__popc(diff) != 1) { atomicExch(err, 1); cellnode[idx] = -1; return; }  // corners do not match
      const int r = __ffs(diff) - 1;     // axis of this cell's n-face along the owner's axis k
      const int flip = (M[0] >> r) & 1;  // owner's axis runs the other way
      const int i = ijk[d[r]];
      const int j = flip ? p - i : i;
      kn += (j - 1) * mul;
      mul *= pm1;
    }
    node = vef_node_base(g, m, gid) + kn;
  }
  if (node < 0 || node >= nnodes) { atomicExch(err, 1); node = -1; }
  cellnode[idx] = (int32_t)node;
}

__device__ __forceinline__ bool is_owner(const UGeom& g, int64_t c, int f, int64_t gid, const int64_t* vptr,
                                         const int32_t* vcells, const int64_t* vowner) {
  if (f < 8) return vcells[vptr[gid]] == c;
  return (vowner[gid - g.nv] >> 5) == c;
}

__device__ __forceinline__ bool vef_dirichlet(const UGeom& g, int32_t sid) {
  return sid > 0 && sid < 32 && ((g.dirmask >> sid) & 1u);
}

__global__ void k_ucount(UGeom g, const int32_t* __restrict__ cellvef, const int64_t* __restrict__ vptr,
                         const int32_t* __restrict__ vcells, const int64_t* __restrict__ vowner,
                         const int32_t* __restrict__ vset, int64_t* cnt_free, int64_t* cnt_dir) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= g.nc) return;
  const int pm1 = g.p - 1;
  int64_t nf = (int64_t)pm1 * pm1 * pm1 * g.ncomp, nd = 0;
  for (int f = 0; f < 26; ++f) {
    const int m = g.h.dim[f];
    int cnt = 1;
    for (int k = 0; k < m; ++k) cnt *= pm1;
    if (cnt == 0) continue;
    const int64_t gid = cellvef[c * 26 + f];
    if (!is_owner(g, c, f, gid, vptr, vcells, vowner)) continue;
    if (vef_dirichlet(g, vset[gid])) nd += (int64_t)cnt * g.ncomp;
    else nf += (int64_t)cnt * g.ncomp;
  }
  cnt_free[c] = nf;
  cnt_dir[c] = nd;
}

__global__ void k_uassign(UGeom g, const int32_t* __restrict__ cellvef, const int64_t* __restrict__ vptr,
                          const int32_t* __restrict__ vcells, const int64_t* __restrict__ vowner,
                          const int32_t* __restrict__ vset, const int64_t* __restrict__ base_free,
                          const int64_t* __restrict__ base_dir, int32_t* latdof, int32_t* free2node,
                          int32_t* dir2node) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= g.nc) return;
  const int pm1 = g.p - 1;
  int64_t id = base_free[c], did = base_dir[c];
  const int64_t ib = g.ibase + c * pm1 * pm1 * pm1;
  // cell interior: component-major, nodes lexicographic
  for (int comp = 0; comp < g.ncomp; ++comp)
    for (int k = 0; k < pm1 * pm1 * pm1; ++k) {
      const int32_t slot = (int32_t)((ib + k) * g.ncomp + comp);
      latdof[slot] = (int32_t)(++id);
      free2node[id - 1] = slot;
    }
  for (int f = 0; f < 26; ++f) {
    const int m = g.h.dim[f];
    int cnt = 1;
    for (int k = 0; k < m; ++k) cnt *= pm1;
    if (cnt == 0) continue;
    const int64_t gid = cellvef[c * 26 + f];
    if (!is_owner(g, c, f, gid, vptr, vcells, vowner)) continue;
    const bool dir = vef_dirichlet(g, vset[gid]);
    const int64_t nb = m == 0 ? gid : vef_node_base(g, m, gid);
    for (int comp = 0; comp < g.ncomp; ++comp)
      for (int k = 0; k < cnt; ++k) {
        const int32_t slot = (int32_t)((nb + k) * g.ncomp + comp);
        if (dir) {
          latdof[slot] = (int32_t)(-(++did));
          dir2node[did - 1] = slot;
        } else {
          latdof[slot] = (int32_t)(++id);
          free2node[id - 1] = slot;
        }
      }
  }
}

// (cell << 6 | local node) of every cell around each node
__global__ void k_ncount(int64_t n, const int32_t* cellnode, unsigned long long* cnt) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(&cnt[cellnode[i]], 1ull);
}
__global__ void k_nfill(int64_t n, int nn, const int32_t* cellnode, unsigned long long* cursor, int64_t* ncl) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) ncl[atomicAdd(&cursor[cellnode[i]], 1ull)] = ((i / nn) << 6) | (i % nn);
}

fg_status uspace_number_dofs(fg_space* sp) {
  fg_mesh* m = sp->mesh;
  fg_ctx* ctx = m->ctx;
  const UGeom g = make_ugeom(sp);
  const int64_t nc = m->ncells, nn = sp->tab.nn;
  sp->nlat = g.ibase + nc * (int64_t)(g.p - 1) * (g.p - 1) * (g.p - 1);
  if (sp->nlat * sp->ncomp >= (int64_t)0x7fffffff || nc * nn >= ((int64_t)1 << 40)) {
    set_error("node count exceeds int32 ids");
    return FG_ERR_UNSUPPORTED;
  }
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_cellnode, sizeof(int32_t) * nc * nn));
  {
    int* derr = nullptr;
    int herr = 0;
    FG_TRY(dev_alloc(ctx, (void**)&derr, sizeof(int)));
    FG_CUDA_TRY(cudaMemsetAsync(derr, 0, sizeof(int), ctx->stream));
    k_ucellnode<<<nblk(nc * nn, 256), 256, 0, ctx->stream>>>(g, sp->nlat, m->d_cellvert, m->d_cellvef, m->d_vowner,
                                                             sp->d_cellnode, derr);
    FG_CUDA_TRY(cudaGetLastError());
    FG_CUDA_TRY(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    dev_free(ctx, derr);
    if (herr) {
      set_error("cells sharing an edge or face do not agree on its corners (invalid mesh)");
      return FG_ERR_BADARG;
    }
  }
  int64_t *cf = nullptr, *cd = nullptr;
  FG_TRY(dev_alloc(ctx, (void**)&cf, sizeof(int64_t) * nc));
  FG_TRY(dev_alloc(ctx, (void**)&cd, sizeof(int64_t) * nc));
  k_ucount<<<nblk(nc, 256), 256, 0, ctx->stream>>>(g, m->d_cellvef, m->d_vptr, m->d_vcells, m->d_vowner, m->d_vset,
                                                   cf, cd);
  FG_CUDA_TRY(cudaGetLastError());
  int64_t nfree = 0, ndir = 0;
  FG_TRY(scan_i64(ctx, cf, nc, &nfree));
  FG_TRY(scan_i64(ctx, cd, nc, &ndir));
  if (nfree >= (int64_t)0x7fffffff) {
    set_error("dof count exceeds int32 ids");
    return FG_ERR_UNSUPPORTED;
  }
  sp->nfree = nfree;
  sp->ndir = ndir;
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_latdof, sizeof(int32_t) * sp->nlat * sp->ncomp));
  FG_CUDA_TRY(cudaMemsetAsync(sp->d_latdof, 0, sizeof(int32_t) * sp->nlat * sp->ncomp, ctx->stream));
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_free2lat, sizeof(int32_t) * (nfree > 0 ? nfree : 1)));
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_dir2lat, sizeof(int32_t) * (ndir > 0 ? ndir : 1)));
  k_uassign<<<nblk(nc, 128), 128, 0, ctx->stream>>>(g, m->d_cellvef, m->d_vptr, m->d_vcells, m->d_vowner, m->d_vset,
                                                    cf, cd, sp->d_latdof, sp->d_free2lat, sp->d_dir2lat);
  FG_CUDA_TRY(cudaGetLastError());
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, cf);
  dev_free(ctx, cd);
  FG_TRY(uspace_build_adjacency(sp));
  ctx->launches += 4;
  return FG_OK;
}

// cells around every node (nlat nodes, the cell node table d_cellnode), ascending
fg_status uspace_build_adjacency(fg_space* sp) {
  fg_ctx* ctx = sp->mesh->ctx;
  const int64_t nc = sp->mesh->ncells, nn = sp->tab.nn;
  {
    const int64_t ne = nc * nn, n = sp->nlat;
    FG_TRY(dev_alloc(ctx, (void**)&sp->d_nptr, sizeof(int64_t) * (n + 1)));
    FG_CUDA_TRY(cudaMemsetAsync(sp->d_nptr, 0, sizeof(int64_t) * (n + 1), ctx->stream));
    k_ncount<<<nblk(ne, 256), 256, 0, ctx->stream>>>(ne, sp->d_cellnode, (unsigned long long*)sp->d_nptr);
    int64_t tot = 0;
    FG_TRY(scan_i64(ctx, sp->d_nptr, n + 1, &tot));
    FG_TRY(dev_alloc(ctx, (void**)&sp->d_ncl, sizeof(int64_t) * ne));
    unsigned long long* cur = nullptr;
    FG_TRY(dev_alloc(ctx, (void**)&cur, sizeof(int64_t) * (n + 1)));
    FG_CUDA_TRY(cudaMemcpyAsync(cur, sp->d_nptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToDevice, ctx->stream));
    k_nfill<<<nblk(ne, 256), 256, 0, ctx->stream>>>(ne, (int)nn, sp->d_cellnode, cur, sp->d_ncl);
    int* dmax = (int*)cur;
    FG_CUDA_TRY(cudaMemsetAsync(dmax, 0, sizeof(int), ctx->stream));
    k_sort_segments_i64<<<nblk(n, 128), 128, 0, ctx->stream>>>(n, sp->d_nptr, sp->d_ncl, dmax);
    FG_CUDA_TRY(cudaMemcpyAsync(&sp->max_ncells, dmax, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    dev_free(ctx, cur);
  }
  ctx->launches += 3;
  return FG_OK;
}

// ---- sparsity -------------------------------------------------------------------------
// One warp per row: the dofs of the cells around the row's node, sorted, distinct, free.
template <bool FILL>
__global__ void k_urow(int64_t nfree, int nn, int ncomp, int cap_max, const int32_t* __restrict__ free2node,
                       const int32_t* __restrict__ latdof, const int32_t* __restrict__ cellnode,
                       const int64_t* __restrict__ nptr, const int64_t* __restrict__ ncl, const int64_t* rowptr,
                       int64_t* rowlen, int32_t* col) {
  extern __shared__ int32_t s_keys[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  int32_t* keys = s_keys + (size_t)wib * cap_max;
  const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (r >= nfree) return;
  const int64_t node = free2node[r] / ncomp;
  const int64_t e0 = nptr[node];
  const int per = nn * ncomp;
  const int total = (int)(nptr[node + 1] - e0) * per;
  int cap = 32;
  while (cap < total) cap <<= 1;
  for (int t = lane; t < cap; t += 32) {
    int32_t key = 0x7fffffff;
    if (t < total) {
      const int e = t / per, rem = t - e * per;
      const int b = rem % nn, comp = rem / nn;
      const int64_t c = ncl[e0 + e] >> 6;
      const int32_t id = latdof[(int64_t)cellnode[c * nn + b] * ncomp + comp];
      if (id > 0) key = id - 1;
    }
    keys[t] = key;
  }
  __syncwarp();
  for (int k = 2; k <= cap; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = lane; t < cap; t += 32) {
        const int u = t ^ j;
        if (u > t) {
          const int32_t a = keys[t], b = keys[u];
          const bool up = (t & k) == 0;
          if ((a > b) == up) { keys[t] = b; keys[u] = a; }
        }
      }
      __syncwarp();
    }
  int64_t pos = 0;
  const int64_t base = FILL ? rowptr[r] : 0;
  for (int t0 = 0; t0 < cap; t0 += 32) {
    const int t = t0 + lane;
    const int32_t k = keys[t];
    const bool u = k != 0x7fffffff && (t == 0 || keys[t - 1] != k);
    const unsigned bal = __ballot_sync(0xffffffffu, u);
    if (FILL && u) col[base + pos + __popc(bal & ((1u << lane) - 1u))] = k;
    pos += __popc(bal);
  }
  if (!FILL && lane == 0) rowlen[r] = pos;
}

__global__ void k_row_max(int64_t n, const int64_t* rowptr, int* mx) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r < n) atomicMax(mx, (int)(rowptr[r + 1] - rowptr[r]));
}

fg_status uspace_build_pattern(fg_space* sp) {
  fg_ctx* ctx = sp->mesh->ctx;
  const int64_t n = sp->nfree;
  const int nn = sp->tab.nn, ncomp = sp->ncomp;
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_rowptr, sizeof(int64_t) * (n + 1)));
  if (n == 0) {  // no free dofs: an empty pattern (row pointer 0, a one-slot column array)
    FG_CUDA_TRY(cudaMemsetAsync(sp->d_rowptr, 0, sizeof(int64_t), ctx->stream));
    FG_TRY(dev_alloc(ctx, (void**)&sp->d_col, sizeof(int32_t)));
    sp->nnz = 0;
    return FG_OK;
  }
  const int64_t cand = (int64_t)sp->max_ncells * nn * ncomp;
  int cap = 32;
  while (cap < cand) cap <<= 1;
  if (cap > 16384) {
    set_error("a node lies in %d cells: row gather of %lld dofs exceeds 16384", sp->max_ncells, (long long)cand);
    return FG_ERR_UNSUPPORTED;
  }
  sp->box_cap = cap;
  const int warps = cap >= 8192 ? 1 : (cap >= 2048 ? 2 : 4);
  const size_t smem = (size_t)warps * cap * sizeof(int32_t);
  const unsigned grid = nblk(n, warps);
  FG_CUDA_TRY(cudaFuncSetAttribute((const void*)k_urow<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  FG_CUDA_TRY(cudaFuncSetAttribute((const void*)k_urow<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_urow<false><<<grid, warps * 32, smem, ctx->stream>>>(n, nn, ncomp, cap, sp->d_free2lat, sp->d_latdof,
                                                         sp->d_cellnode, sp->d_nptr, sp->d_ncl, nullptr, sp->d_rowptr,
                                                         nullptr);
  FG_CUDA_TRY(cudaGetLastError());
  int64_t nnz = 0;
  FG_TRY(scan_i64(ctx, sp->d_rowptr, n, &nnz));
  FG_CUDA_TRY(cudaMemcpyAsync(sp->d_rowptr + n, &nnz, sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
  sp->nnz = nnz;
  FG_TRY(dev_alloc(ctx, (void**)&sp->d_col, sizeof(int32_t) * (nnz > 0 ? nnz : 1)));
  k_urow<true><<<grid, warps * 32, smem, ctx->stream>>>(n, nn, ncomp, cap, sp->d_free2lat, sp->d_latdof,
                                                        sp->d_cellnode, sp->d_nptr, sp->d_ncl, sp->d_rowptr, nullptr,
                                                        sp->d_col);
  FG_CUDA_TRY(cudaGetLastError());
  int* dmax = nullptr;
  FG_TRY(dev_alloc(ctx, (void**)&dmax, sizeof(int)));
  FG_CUDA_TRY(cudaMemsetAsync(dmax, 0, sizeof(int), ctx->stream));
  k_row_max<<<nblk(n, 256), 256, 0, ctx->stream>>>(n, sp->d_rowptr, dmax);
  int mx = 0;
  FG_CUDA_TRY(cudaMemcpyAsync(&mx, dmax, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, dmax);
  int rc = 32;
  while (rc < mx) rc <<= 1;
  sp->row_cap = rc;
  FG_TRY(space_count_upper(sp));
  ctx->launches += 4;
  return FG_OK;
}

// ---- numeric assembly -----------------------------------------------------------------
// One warp per free row: the rows of the element matrices of the cells around the row's
// node, added in increasing cell order (the reference's COO append + sort_and_compress).
__global__ void __launch_bounds__(128)
    k_uscatter_rows(int64_t nfree, int nn, int ncomp, int row_cap, const int32_t* __restrict__ free2node,
                    const int32_t* __restrict__ latdof, const int32_t* __restrict__ cellnode,
                    const int64_t* __restrict__ nptr, const int64_t* __restrict__ ncl,
                    const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                    const double* __restrict__ E, const double* __restrict__ EV, double* __restrict__ val,
                    float* __restrict__ val32, double* __restrict__ rhs) {
  extern __shared__ double s_acc[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  double* acc = s_acc + (size_t)wib * row_cap;
  int32_t* cols = reinterpret_cast<int32_t*>(s_acc + (size_t)(blockDim.x >> 5) * row_cap) + (size_t)wib * row_cap;
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
  if (r >= nfree) return;
  const int32_t slot = free2node[r];
  const int64_t node = slot / ncomp;
  const int comp = slot % ncomp;
  const int ND = nn * ncomp;
  const int64_t s = rowptr[r];
  const int len = (int)(rowptr[r + 1] - s);
  for (int t = lane; t < len; t += 32) {
    cols[t] = col[s + t];
    acc[t] = 0.0;
  }
  __syncwarp();
  double rsum = 0.0;
  for (int64_t e = nptr[node]; e < nptr[node + 1]; ++e) {
    const int64_t packed = ncl[e];
    const int64_t c = packed >> 6;
    const int a = (int)(packed & 63) + comp * nn;
    const double* Erow = E + ((size_t)c * ND + a) * ND;
    for (int b = lane; b < ND; b += 32) {
      const int32_t id = latdof[(int64_t)cellnode[c * nn + (b % nn)] * ncomp + b / nn];
      if (id > 0) {
        const int32_t key = id - 1;
        int lo = 0, hi = len;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (cols[mid] < key) lo = mid + 1;
          else hi = mid;
        }
        if (lo < len && cols[lo] == key) acc[lo] = acc[lo] + Erow[b];
      }
    }
    if (lane == 0) rsum = rsum + EV[c * ND + a];
    __syncwarp();
  }
  for (int t = lane; t < len; t += 32) {
    const double v = acc[t];
    val[s + t] = v;
    if (val32) val32[s + t] = (float)v;
  }
  if (lane == 0) rhs[r] = rsum;
}

fg_status usystem_scatter(fg_system* sys) {
  fg_space* sp = sys->space;
  fg_ctx* ctx = sp->mesh->ctx;
  const int64_t n = sp->nfree;
  if (n == 0) return FG_OK;
  int warps = 4;
  while (warps > 1 && (size_t)warps * sp->row_cap * (sizeof(double) + sizeof(int32_t)) > 200 * 1024) warps >>= 1;
  const size_t smem = (size_t)warps * sp->row_cap * (sizeof(double) + sizeof(int32_t));
  if (smem > 227 * 1024) {
    set_error("row of %d entries too long for the row gather", sp->row_cap);
    return FG_ERR_UNSUPPORTED;
  }
  FG_CUDA_TRY(cudaFuncSetAttribute((const void*)k_uscatter_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_uscatter_rows<<<nblk(n, warps), warps * 32, smem, ctx->stream>>>(
      n, sp->tab.nn, sp->ncomp, sp->row_cap, sp->d_free2lat, sp->d_latdof, sp->d_cellnode, sp->d_nptr, sp->d_ncl,
      sp->d_rowptr, sp->d_col, sys->d_elmat, sys->d_elvec, sys->d_val, sys->d_val32, sys->d_rhs);
  ctx->launches += 1;
  FG_CUDA_TRY(cudaGetLastError());
  return FG_OK;
}

// ---- exports and Dirichlet coordinates --------------------------------------------------
__global__ void k_ucell_dof_map(int64_t nc, int nn, int nd, int ncomp, const int32_t* cellnode, const int32_t* latdof,
                                int32_t* out) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= nc * nd) return;
  const int64_t c = idx / nd;
  const int s = (int)(idx % nd);
  out[idx] = latdof[(int64_t)cellnode[c * nn + s % nn] * ncomp + s / nn];
}

fg_status uspace_export_dof_map(fg_space* sp, int32_t* out_host) {
  fg_ctx* ctx = sp->mesh->ctx;
  const int64_t total = sp->mesh->ncells * sp->tab.nd;
  int32_t* d = nullptr;
  FG_TRY(dev_alloc(ctx, (void**)&d, sizeof(int32_t) * total));
  k_ucell_dof_map<<<nblk(total, 256), 256, 0, ctx->stream>>>(sp->mesh->ncells, sp->tab.nn, sp->tab.nd, sp->ncomp,
                                                              sp->d_cellnode, sp->d_latdof, d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out_host, d, sizeof(int32_t) * total, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  dev_free(ctx, d);
  if (e != cudaSuccess) { set_error("dof map export: %s", cudaGetErrorString(e)); return FG_ERR_CUDA; }
  return FG_OK;
}

// Coordinates of a node through the trilinear map of the last cell (in cell order) around it:
// the reference's interpolate_dirichlet_values walks the cells in order, the last write wins
// (sbm_serial_fe_space.i90:1140-1152).
__global__ void k_udirichlet_coords(int64_t ndir, int p, int ncomp, const int32_t* dir2node, const int64_t* nptr,
                                    const int64_t* ncl, const int32_t* cellvert, const double* coords, double* xyz) {
  const int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (d >= ndir) return;
  const int64_t node = dir2node[d] / ncomp;
  const int64_t packed = ncl[nptr[node + 1] - 1];
  const int64_t c = packed >> 6;
  const int a = (int)(packed & 63), np1 = p + 1;
  const int ijk[3] = {a % np1, (a / np1) % np1, a / (np1 * np1)};
  double xi[3];
  for (int k = 0; k < 3; ++k) xi[k] = (2.0 / p) * ijk[k] - 1.0;
  double x[3] = {0.0, 0.0, 0.0};
  for (int k = 0; k < 8; ++k) {
    const int bx = k & 1, by = (k >> 1) & 1, bz = (k >> 2) & 1;
    const double fx = bx ? 0.5 * (1 + xi[0]) : 0.5 * (1 - xi[0]);
    const double fy = by ? 0.5 * (1 + xi[1]) : 0.5 * (1 - xi[1]);
    const double fz = bz ? 0.5 * (1 + xi[2]) : 0.5 * (1 - xi[2]);
    const double w = fx * fy * fz;
    const int64_t v = cellvert[c * 8 + k];
    for (int l = 0; l < 3; ++l) x[l] = x[l] + w * coords[v * 3 + l];
  }
  for (int l = 0; l < 3; ++l) xyz[d * 3 + l] = x[l];
}

fg_status uspace_dirichlet_coords(fg_space* sp, double* d_xyz) {
  if (sp->ndir == 0) return FG_OK;
  fg_mesh* m = sp->mesh;
  k_udirichlet_coords<<<nblk(sp->ndir, 256), 256, 0, m->ctx->stream>>>(sp->ndir, sp->order, sp->ncomp, sp->d_dir2lat,
                                                                       sp->d_nptr, sp->d_ncl, m->d_cellvert,
                                                                       m->d_coords, d_xyz);
  FG_CUDA_TRY(cudaGetLastError());
  return FG_OK;
}

fg_status umesh_export_vefs(fg_mesh* m, int32_t* cell_vefs, int32_t* vef_sets) {
  fg_ctx* ctx = m->ctx;
  if (cell_vefs)
    FG_CUDA_TRY(cudaMemcpyAsync(cell_vefs, m->d_cellvef, sizeof(int32_t) * m->ncells * 26, cudaMemcpyDeviceToHost,
                                ctx->stream));
  if (vef_sets)
    FG_CUDA_TRY(cudaMemcpyAsync(vef_sets, m->d_vset, sizeof(int32_t) * m->nvefs, cudaMemcpyDeviceToHost, ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return FG_OK;
}

}  // namespace fg

// fg_partition.cu -- partitioned assembly on one device: FEMPAR's element-based parallel FE
// space (par_fe_space_t, Sources/Lib/Integration/FESpace/sbm_par_fe_space.i90), its
// nearest-neighbour communication plan (dof_import_t, Sources/Lib/LinearAlgebra/Vector/
// dof_import.f90) and the subassembled -> assembled vector exchange (par_scalar_array_t%comm,
// par_scalar_array.f90:498-533), for a structured mesh split into np0 x np1 x np2 box parts.
//
// Host (setup, closed forms on the lattice):
//   - local cells of a part in the generator's order: cells away from neighbour parts first,
//     cells next to a neighbour part last in reverse visiting order
//     (uniform_hex_mesh_generator.f90:255-360);
//   - local free dofs: the serial first-visitor numbering run over the local cells
//     (sbm_serial_fe_space.i90:2623-2884);
//   - interface couplings, one column per (local interface dof, other part sharing it) with
//     (neighbour part, number of sharing parts, non-consecutive dof ggid) -- the ggid made of
//     the largest global cell around the dof and the dof's position in it
//     (sbm_par_fe_space.i90:1103-1118, :1877-2034) -- sorted lexicographically, owners decided
//     as :2737-2853 (two sharers: first half of each neighbour's run to the larger part id,
//     the rest to the smaller; more sharers: the largest part id);
//   - dof_import_create (dof_import.f90:102-213) and the interior-then-interface renumbering
//     (:365-421, sbm_par_fe_space.i90:449-470).
// Device: all parts' local dofs form one concatenated space (part p's dofs at an offset); its
// node table makes every part's box lattice a separate set of nodes, so the explicit-node row
// gather assembles every part's subassembled matrix (block diagonal) and rhs in one pass.
// comm: stage 1 adds each owner copy's senders in the reference's receive order, stage 2
// copies the owner value back to the other copies.  The partitioned Jacobi-PCG runs on the
// concatenated space with comm after every SpMV and dots weighted by the dof_import weights
// (par_scalar_array.f90:303-345) -- the same iterates as the global PCG up to rounding.
// A multi-device run would keep each part on its device and replace the gathers of comm by
// sends/receives of the pack/unpack lists; this build has one device and no such collective.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "fg_internal.h"

struct fg_partition;

namespace fg {

static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

struct PartMeta {
  std::vector<int64_t> cells;   // global cell ids, local order
  std::vector<int32_t> l2g;     // final local dof -> global free id (1-based)
  int32_t num_dofs = 0, num_interior = 0, num_interface = 0;
  std::vector<double> weight;
  std::vector<int32_t> list_rcv, rcv_ptrs, unpack_idx, list_snd, snd_ptrs, pack_idx;  // 1-based
  int64_t node_off = 0, dof_off = 0;
  int Lb[3] = {0, 0, 0}, c0[3] = {0, 0, 0};
};

}  // namespace fg

struct fg_partition {
  fg_space* gsp = nullptr;
  fg_space* psp = nullptr;  // concatenated local dofs of all parts
  int np[3] = {1, 1, 1};
  int nparts = 1;
  std::vector<fg::PartMeta> parts;
  int64_t nl = 0, ncouplings = 0;
  int32_t* d_l2g = nullptr;     // nl: global free id (0-based)
  double* d_weight = nullptr;   // nl
  int64_t nown = 0, nnon = 0;
  int32_t* d_own_idx = nullptr;  // owner copies receiving
  int64_t* d_own_ptr = nullptr;  // nown+1
  int32_t* d_own_src = nullptr;  // their senders, in receive order
  int32_t* d_non_idx = nullptr;  // non-owner copies
  int32_t* d_non_src = nullptr;  // their owner copies
};

namespace fg {

// own dofs of every n-face (codes order, volume last): local dof ids, first free direction
// fastest, components component-major
static std::vector<std::vector<int>> own_lists(const RefTables& t, int p, int ncomp) {
  const int np1 = p + 1, nn = np1 * np1 * np1;
  std::vector<std::vector<int>> own(27);
  for (int f = 0; f < 27; ++f) {
    const int code = t.codes[f], anchor = code & 7, ty = code >> 3;
    std::vector<int> freed;
    for (int d = 0; d < 3; ++d) if ((ty >> d) & 1) freed.push_back(d);
    std::vector<int> nodes;
    if (p >= 2 || freed.empty()) {
      std::vector<int> disp(freed.size(), 1);
      while (true) {
        int ijk[3];
        for (int d = 0; d < 3; ++d) ijk[d] = ((anchor >> d) & 1) ? p : 0;
        for (size_t k = 0; k < freed.size(); ++k) ijk[freed[k]] = disp[k];
        nodes.push_back(ijk[0] + np1 * (ijk[1] + np1 * ijk[2]));
        size_t k = 0;
        for (; k < freed.size(); ++k) {
          if (++disp[k] <= p - 1) break;
          disp[k] = 1;
        }
        if (k == freed.size()) break;
      }
    }
    for (int c = 0; c < ncomp; ++c)
      for (int a : nodes) own[f].push_back(a + c * nn);
  }
  return own;
}

static fg_status build_meta(fg_partition* P) {
  fg_space* g = P->gsp;
  fg_ctx* ctx = g->mesh->ctx;
  const int p = g->order, ncomp = g->ncomp, np1 = p + 1, nn = np1 * np1 * np1;
  const int n[3] = {g->mesh->n[0], g->mesh->n[1], g->mesh->n[2]};
  const int64_t Ln0 = g->Ln[0], Ln1 = g->Ln[1];
  int nloc[3];
  for (int d = 0; d < 3; ++d) {
    if (P->np[d] < 1 || n[d] % P->np[d] != 0) {
      set_error("partition: %d parts do not divide %d cells in direction %d", P->np[d], n[d], d);
      return FG_ERR_BADARG;
    }
    nloc[d] = n[d] / P->np[d];
  }
  std::vector<int32_t> latdof((size_t)g->nlat * ncomp), free2lat(g->nfree > 0 ? g->nfree : 1);
  FG_CUDA_TRY(cudaMemcpyAsync(latdof.data(), g->d_latdof, sizeof(int32_t) * latdof.size(), cudaMemcpyDeviceToHost,
                              ctx->stream));
  if (g->nfree > 0)
    FG_CUDA_TRY(cudaMemcpyAsync(free2lat.data(), g->d_free2lat, sizeof(int32_t) * g->nfree, cudaMemcpyDeviceToHost,
                                ctx->stream));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  const auto own = own_lists(g->tab, p, ncomp);
  auto gdof = [&](int64_t c, int s) {
    const int64_t ci = c % n[0], cj = (c / n[0]) % n[1], ck = c / ((int64_t)n[0] * n[1]);
    const int a = s % nn, comp = s / nn;
    const int ai = a % np1, aj = (a / np1) % np1, ak = a / (np1 * np1);
    const int64_t L = (p * ci + ai) + Ln0 * ((p * cj + aj) + Ln1 * (p * ck + ak));
    return latdof[L * ncomp + comp];
  };
  // sharing parts, largest part, and the non-consecutive ggid of a global free dof
  auto dof_info = [&](int32_t gid, int* pmin, int* pmax, int64_t& key) {
    const int32_t slot = free2lat[gid - 1];
    const int64_t L = slot / ncomp;
    const int comp = slot % ncomp;
    const int64_t I[3] = {L % Ln0, (L / Ln0) % Ln1, L / (Ln0 * Ln1)};
    int64_t cm[3];
    int loc[3];
    for (int d = 0; d < 3; ++d) {
      const int64_t cmin = I[d] == 0 ? 0 : (I[d] - 1) / p;
      const int64_t cmax = std::min<int64_t>(n[d] - 1, I[d] / p);
      pmin[d] = (int)(cmin / nloc[d]);
      pmax[d] = (int)(cmax / nloc[d]);
      cm[d] = cmax;
      loc[d] = (int)(I[d] - p * cmax);
    }
    const int64_t cell = cm[0] + (int64_t)n[0] * (cm[1] + (int64_t)n[1] * cm[2]);
    const int s = loc[0] + np1 * (loc[1] + np1 * loc[2]) + comp * nn;
    key = cell + ((int64_t)s << 40);
  };
  auto part_id = [&](int px, int py, int pz) { return 1 + px + P->np[0] * (py + P->np[1] * pz); };
  const int nparts = P->nparts;
  P->parts.assign(nparts, PartMeta());
  std::vector<int32_t> stamp(g->nfree > 0 ? g->nfree : 1, 0), lidx(g->nfree > 0 ? g->nfree : 1, 0);
  const int walk[27] = {26, 0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 21, 22, 23, 24, 25};
  int64_t dof_off = 0, node_off = 0;
  for (int pid = 1; pid <= nparts; ++pid) {
    PartMeta& M = P->parts[pid - 1];
    const int pi = (pid - 1) % P->np[0], pj = ((pid - 1) / P->np[0]) % P->np[1], pk = (pid - 1) / (P->np[0] * P->np[1]);
    const int pijk[3] = {pi, pj, pk};
    int left[3], right[3], tot[3], first[3];
    for (int d = 0; d < 3; ++d) {
      left[d] = pijk[d] > 0;
      right[d] = pijk[d] < P->np[d] - 1;
      tot[d] = nloc[d] + left[d] + right[d];
      first[d] = pijk[d] * nloc[d] - left[d];
      M.c0[d] = pijk[d] * nloc[d];
      M.Lb[d] = nloc[d] * p + 1;
    }
    std::vector<int64_t> interior, itfc;
    for (int k = 0; k < tot[2]; ++k)
      for (int j = 0; j < tot[1]; ++j)
        for (int i = 0; i < tot[0]; ++i) {
          const int ijk[3] = {i, j, k};
          bool ghost = false, inter = false;
          for (int d = 0; d < 3; ++d) {
            ghost = ghost || (left[d] && ijk[d] == 0) || (right[d] && ijk[d] == tot[d] - 1);
            inter = inter || (left[d] && ijk[d] == 1) || (right[d] && ijk[d] == tot[d] - 2);
          }
          if (ghost) continue;
          const int64_t cid = (first[0] + i) + (int64_t)n[0] * ((first[1] + j) + (int64_t)n[1] * (first[2] + k));
          (inter ? itfc : interior).push_back(cid);
        }
    M.cells = interior;
    M.cells.insert(M.cells.end(), itfc.rbegin(), itfc.rend());
    // serial numbering over the local cells
    std::vector<int32_t> l2g0;
    for (int64_t c : M.cells)
      for (int f : walk)
        for (int s : own[f]) {
          const int32_t gd = gdof(c, s);
          if (gd > 0 && stamp[gd - 1] != pid) {
            stamp[gd - 1] = pid;
            lidx[gd - 1] = (int32_t)l2g0.size();
            l2g0.push_back(gd);
          }
        }
    const int32_t nloc_d = (int32_t)l2g0.size();
    // interface columns: (neighbour, sharers, key, local dof, largest part)
    struct Col { int32_t q, nsh; int64_t key; int32_t l; int32_t mx; };
    std::vector<Col> cols;
    for (int32_t l = 0; l < nloc_d; ++l) {
      int pmin[3], pmax[3];
      int64_t key;
      dof_info(l2g0[l], pmin, pmax, key);
      const int nsh = (pmax[0] - pmin[0] + 1) * (pmax[1] - pmin[1] + 1) * (pmax[2] - pmin[2] + 1);
      if (nsh < 2) continue;
      const int mx = part_id(pmax[0], pmax[1], pmax[2]);
      for (int z = pmin[2]; z <= pmax[2]; ++z)
        for (int y = pmin[1]; y <= pmax[1]; ++y)
          for (int x = pmin[0]; x <= pmax[0]; ++x) {
            const int q = part_id(x, y, z);
            if (q != pid) cols.push_back({q, nsh, key, l, mx});
          }
    }
    std::sort(cols.begin(), cols.end(), [](const Col& a, const Col& b) {
      if (a.q != b.q) return a.q < b.q;
      if (a.nsh != b.nsh) return a.nsh < b.nsh;
      return a.key < b.key;
    });
    enum { OWN = 1, NON = 2, UNC = 3 };
    std::vector<int> flag(cols.size(), 0);
    for (size_t i = 0; i < cols.size();) {
      if (cols[i].nsh == 2) {
        const size_t s0 = i;
        while (i < cols.size() && cols[i].nsh == 2 && cols[i].q == cols[s0].q) ++i;
        const size_t size = i - s0;
        const bool first_owner = pid == std::max(pid, (int)cols[s0].q);
        for (size_t j = s0; j < i; ++j) {
          const bool in_first = j < s0 + size / 2;
          flag[j] = (in_first == first_owner) ? OWN : NON;
        }
      } else {
        flag[i] = pid == cols[i].mx ? OWN : (cols[i].q == cols[i].mx ? NON : UNC);
        ++i;
      }
    }
    // dof_import_create
    std::vector<double> weight(nloc_d, 1.0);
    std::vector<int32_t> rcv_of(nparts + 1, -1), snd_of(nparts + 1, -1);
    std::vector<std::vector<int32_t>> rcv, snd;
    std::vector<char> itf(nloc_d, 0);
    for (size_t i = 0; i < cols.size(); ++i) {
      const int q = cols[i].q;
      const int32_t loc1 = cols[i].l + 1;
      if (flag[i] == OWN) {
        if (rcv_of[q] < 0) { rcv_of[q] = (int32_t)rcv.size(); rcv.push_back({}); M.list_rcv.push_back(q); }
        rcv[rcv_of[q]].push_back(loc1);
      } else if (flag[i] == NON) {
        if (snd_of[q] < 0) { snd_of[q] = (int32_t)snd.size(); snd.push_back({}); M.list_snd.push_back(q); }
        snd[snd_of[q]].push_back(loc1);
        weight[loc1 - 1] = 0.0;
      }
      itf[loc1 - 1] = 1;
    }
    M.rcv_ptrs.assign(1, 1);
    for (auto& v : rcv) { M.unpack_idx.insert(M.unpack_idx.end(), v.begin(), v.end()); M.rcv_ptrs.push_back(M.rcv_ptrs.back() + (int32_t)v.size()); }
    M.snd_ptrs.assign(1, 1);
    for (auto& v : snd) { M.pack_idx.insert(M.pack_idx.end(), v.begin(), v.end()); M.snd_ptrs.push_back(M.snd_ptrs.back() + (int32_t)v.size()); }
    int32_t nitf = 0;
    for (char c : itf) nitf += c;
    M.num_dofs = nloc_d;
    M.num_interface = nitf;
    M.num_interior = nloc_d - nitf;
    // interior first, then interface in pack order, then unpack order
    std::vector<int32_t> perm(nloc_d + 1, -1);
    int32_t cur = M.num_interior + 1;
    for (int32_t v : M.pack_idx) if (perm[v] == -1) perm[v] = cur++;
    for (int32_t v : M.unpack_idx) if (perm[v] == -1) perm[v] = cur++;
    cur = 1;
    for (int32_t v = 1; v <= nloc_d; ++v) if (perm[v] == -1) perm[v] = cur++;
    for (auto& v : M.pack_idx) v = perm[v];
    for (auto& v : M.unpack_idx) v = perm[v];
    M.weight.assign(nloc_d, 0.0);
    M.l2g.assign(nloc_d, 0);
    for (int32_t v = 1; v <= nloc_d; ++v) {
      M.weight[perm[v] - 1] = weight[v - 1];
      M.l2g[perm[v] - 1] = l2g0[v - 1];
    }
    M.dof_off = dof_off;
    M.node_off = node_off;
    dof_off += nloc_d;
    node_off += (int64_t)M.Lb[0] * M.Lb[1] * M.Lb[2];
    P->ncouplings += (int64_t)cols.size();
  }
  P->nl = dof_off;
  if (dof_off >= (int64_t)0x7fffffff || node_off * ncomp >= (int64_t)0x7fffffff) {
    set_error("partitioned dof count exceeds int32 ids");
    return FG_ERR_UNSUPPORTED;
  }
  // part space: node tables, dof tables
  fg_space* s = P->psp;
  s->nlat = node_off;
  s->nfree = dof_off;
  s->ndir = g->ndir;
  std::vector<int32_t> platdof((size_t)node_off * ncomp, 0), pfree2lat(dof_off > 0 ? dof_off : 1),
      cellnode((size_t)g->mesh->ncells * nn);
  for (int pid = 1; pid <= nparts; ++pid) {
    const PartMeta& M = P->parts[pid - 1];
    for (int32_t l = 0; l < M.num_dofs; ++l) lidx[M.l2g[l] - 1] = l;
    for (int64_t k = 0; k < M.Lb[2]; ++k)
      for (int64_t j = 0; j < M.Lb[1]; ++j)
        for (int64_t i = 0; i < M.Lb[0]; ++i) {
          const int64_t L = (M.c0[0] * p + i) + Ln0 * ((M.c0[1] * p + j) + Ln1 * (M.c0[2] * p + k));
          const int64_t node = M.node_off + i + M.Lb[0] * (j + (int64_t)M.Lb[1] * k);
          for (int c = 0; c < ncomp; ++c) {
            const int32_t gd = latdof[L * ncomp + c];
            int32_t v = gd;
            if (gd > 0) {
              const int64_t r = M.dof_off + lidx[gd - 1];
              v = (int32_t)(r + 1);
              pfree2lat[r] = (int32_t)(node * ncomp + c);
            }
            platdof[node * ncomp + c] = v;
          }
        }
    for (int64_t c : M.cells) {
      const int64_t ci = c % n[0], cj = (c / n[0]) % n[1], ck = c / ((int64_t)n[0] * n[1]);
      for (int a = 0; a < nn; ++a) {
        const int ai = a % np1, aj = (a / np1) % np1, ak = a / (np1 * np1);
        const int64_t i = p * (ci - M.c0[0]) + ai, j = p * (cj - M.c0[1]) + aj, k = p * (ck - M.c0[2]) + ak;
        cellnode[(size_t)c * nn + a] = (int32_t)(M.node_off + i + M.Lb[0] * (j + (int64_t)M.Lb[1] * k));
      }
    }
  }
  FG_TRY(dev_alloc(ctx, (void**)&s->d_latdof, sizeof(int32_t) * platdof.size()));
  FG_TRY(dev_alloc(ctx, (void**)&s->d_free2lat, sizeof(int32_t) * pfree2lat.size()));
  FG_TRY(dev_alloc(ctx, (void**)&s->d_cellnode, sizeof(int32_t) * cellnode.size()));
  FG_TRY(dev_alloc(ctx, (void**)&s->d_dir2lat, sizeof(int32_t) * (g->ndir > 0 ? g->ndir : 1)));
  FG_CUDA_TRY(cudaMemcpyAsync(s->d_latdof, platdof.data(), sizeof(int32_t) * platdof.size(), cudaMemcpyHostToDevice, ctx->stream));
  FG_CUDA_TRY(cudaMemcpyAsync(s->d_free2lat, pfree2lat.data(), sizeof(int32_t) * pfree2lat.size(), cudaMemcpyHostToDevice, ctx->stream));
  FG_CUDA_TRY(cudaMemcpyAsync(s->d_cellnode, cellnode.data(), sizeof(int32_t) * cellnode.size(), cudaMemcpyHostToDevice, ctx->stream));
  if (g->ndir > 0)
    FG_CUDA_TRY(cudaMemcpyAsync(s->d_dir2lat, g->d_dir2lat, sizeof(int32_t) * g->ndir, cudaMemcpyDeviceToDevice, ctx->stream));
  // comm plan
  std::vector<int32_t> l2g_all(dof_off > 0 ? dof_off : 1);
  std::vector<double> w_all(dof_off > 0 ? dof_off : 1);
  std::vector<std::vector<int32_t>> srcs(dof_off > 0 ? dof_off : 1);
  std::vector<int32_t> non_idx, non_src;
  for (int pid = 1; pid <= nparts; ++pid) {
    const PartMeta& M = P->parts[pid - 1];
    for (int32_t l = 0; l < M.num_dofs; ++l) {
      l2g_all[M.dof_off + l] = M.l2g[l] - 1;
      w_all[M.dof_off + l] = M.weight[l];
    }
    for (size_t k = 0; k < M.list_rcv.size(); ++k) {
      const PartMeta& Q = P->parts[M.list_rcv[k] - 1];
      auto it = std::find(Q.list_snd.begin(), Q.list_snd.end(), pid);
      const size_t kk = it - Q.list_snd.begin();
      const int32_t nm = M.rcv_ptrs[k + 1] - M.rcv_ptrs[k];
      if (it == Q.list_snd.end() || Q.snd_ptrs[kk + 1] - Q.snd_ptrs[kk] != nm) {
        set_error("partition: message sizes between parts %d and %d disagree", pid, M.list_rcv[k]);
        return FG_ERR_NUMERIC;
      }
      for (int32_t e = 0; e < nm; ++e) {
        const int64_t dst = M.dof_off + M.unpack_idx[M.rcv_ptrs[k] - 1 + e] - 1;
        const int64_t src = Q.dof_off + Q.pack_idx[Q.snd_ptrs[kk] - 1 + e] - 1;
        srcs[dst].push_back((int32_t)src);
        non_idx.push_back((int32_t)src);
        non_src.push_back((int32_t)dst);
      }
    }
  }
  std::vector<int32_t> own_idx, own_src;
  std::vector<int64_t> own_ptr(1, 0);
  for (int64_t r = 0; r < dof_off; ++r)
    if (!srcs[r].empty()) {
      own_idx.push_back((int32_t)r);
      own_src.insert(own_src.end(), srcs[r].begin(), srcs[r].end());
      own_ptr.push_back((int64_t)own_src.size());
    }
  P->nown = (int64_t)own_idx.size();
  P->nnon = (int64_t)non_idx.size();
  auto up = [&](void** d, const void* h, size_t bytes) -> fg_status {
    FG_TRY(dev_alloc(ctx, d, bytes > 0 ? bytes : 8));
    if (bytes) FG_CUDA_TRY(cudaMemcpyAsync(*d, h, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return FG_OK;
  };
  FG_TRY(up((void**)&P->d_l2g, l2g_all.data(), sizeof(int32_t) * dof_off));
  FG_TRY(up((void**)&P->d_weight, w_all.data(), sizeof(double) * dof_off));
  FG_TRY(up((void**)&P->d_own_idx, own_idx.data(), sizeof(int32_t) * own_idx.size()));
  FG_TRY(up((void**)&P->d_own_ptr, own_ptr.data(), sizeof(int64_t) * own_ptr.size()));
  FG_TRY(up((void**)&P->d_own_src, own_src.data(), sizeof(int32_t) * own_src.size()));
  FG_TRY(up((void**)&P->d_non_idx, non_idx.data(), sizeof(int32_t) * non_idx.size()));
  FG_TRY(up((void**)&P->d_non_src, non_src.data(), sizeof(int32_t) * non_src.size()));
  FG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return FG_OK;
}

// ---- comm and the partitioned PCG --------------------------------------------------------
__global__ void k_comm_gather(int64_t nown, const int32_t* idx, const int64_t* ptr, const int32_t* src, double* x) {
  const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= nown) return;
  double v = x[idx[o]];
  for (int64_t k = ptr[o]; k < ptr[o + 1]; ++k) v = v + x[src[k]];
  x[idx[o]] = v;
}
__global__ void k_comm_scatter(int64_t nnon, const int32_t* idx, const int32_t* src, double* x) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < nnon) x[idx[i]] = x[src[i]];
}

fg_status partition_comm(fg_partition* P, double* x) {
  fg_ctx* ctx = P->gsp->mesh->ctx;
  if (P->nown > 0)
    k_comm_gather<<<nblk(P->nown, 256), 256, 0, ctx->stream>>>(P->nown, P->d_own_idx, P->d_own_ptr, P->d_own_src, x);
  if (P->nnon > 0)
    k_comm_scatter<<<nblk(P->nnon, 256), 256, 0, ctx->stream>>>(P->nnon, P->d_non_idx, P->d_non_src, x);
  ctx->launches += 2;
  FG_CUDA_TRY(cudaGetLastError());
  return FG_OK;
}

// weighted dot: fixed grid, per-block partials in a fixed order, summed by one block
constexpr int kDotBlocks = 304;
__global__ void k_wdot_partial(int64_t n, const double* w, const double* a, const double* b, double* part) {
  __shared__ double s[256];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc += w[i] * a[i] * b[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if ((int)threadIdx.x < k) s[threadIdx.x] += s[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}
__global__ void k_sum_partials(int n, const double* part, double* out) {
  __shared__ double s[512];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += part[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int k = 256; k > 0; k >>= 1) {
    if ((int)threadIdx.x < k) s[threadIdx.x] += s[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}
// x += alpha p; r -= alpha q; z = dinv r
__global__ void k_pcg_update(int64_t n, double alpha, const double* p, const double* q, const double* dinv, double* x,
                             double* r, double* z) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  x[i] = x[i] + alpha * p[i];
  const double ri = r[i] - alpha * q[i];
  r[i] = ri;
  z[i] = dinv[i] * ri;
}
__global__ void k_pcg_pupdate(int64_t n, double beta, const double* z, double* p) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) p[i] = z[i] + beta * p[i];
}
__global__ void k_pcg_init(int64_t n, const double* b, const double* d, double* x, double* r, double* z, double* p,
                           double* dinv) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double di = d[i] != 0.0 ? 1.0 / d[i] : 0.0;
  dinv[i] = di;
  x[i] = 0.0;
  r[i] = b[i];
  z[i] = di * b[i];
  p[i] = z[i];
}
__global__ void k_extract_diag(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val, double* d) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  double v = 0.0;
  for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
    if (col[k] == r) v = val[k];
  d[r] = v;
}
__global__ void k_gather_owned(int64_t n, const int32_t* l2g, const double* w, const double* x, double* xg) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n && w[i] != 0.0) xg[l2g[i]] = x[i];
}

}  // namespace fg

using namespace fg;

extern "C" {

fg_status fg_partition_create(fg_space* space, const int32_t num_parts_x_dir[3], fg_partition** out) {
  if (!space || !num_parts_x_dir || !out) { set_error("bad argument: space/num_parts_x_dir/out"); return FG_ERR_BADARG; }
  *out = nullptr;
  if (space->mesh->unst || space->dg || space->explicit_nodes || space->mesh->dim != 3) {
    set_error("partitioned spaces are built from continuous spaces on structured 3D meshes");
    return FG_ERR_UNSUPPORTED;
  }
  fg_ctx* ctx = space->mesh->ctx;
  FG_CUDA_TRY(cudaSetDevice(ctx->device));
  fg_partition* P = new fg_partition();
  P->gsp = space;
  for (int d = 0; d < 3; ++d) P->np[d] = num_parts_x_dir[d];
  P->nparts = P->np[0] * P->np[1] * P->np[2];
  fg_space* s = new fg_space();
  s->mesh = space->mesh;
  s->order = space->order;
  s->ncomp = space->ncomp;
  s->dirmask = space->dirmask;
  for (int d = 0; d < 3; ++d) s->Ln[d] = space->Ln[d];
  s->explicit_nodes = true;
  s->layout = FG_LAYOUT_SELL;
  s->tab.build(space->order, space->ncomp);
  P->psp = s;
  fg_status st = upload_tables(ctx, s->tab, s->dtab);
  if (st == FG_OK) st = build_meta(P);
  if (st == FG_OK) st = uspace_build_adjacency(s);
  if (st == FG_OK) st = uspace_build_pattern(s);
  if (st == FG_OK) {
    st = space_build_sell(s);
    s->nvec = s->nfree;
    s->d_row2vec = s->d_iperm;
  }
  if (st == FG_OK) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { set_error("partition: %s", cudaGetErrorString(e)); st = FG_ERR_CUDA; }
  }
  if (st != FG_OK) {
    fg_partition_destroy(P);
    return st;
  }
  *out = P;
  return FG_OK;
}

fg_status fg_partition_destroy(fg_partition* P) {
  if (!P) return FG_OK;
  fg_ctx* ctx = P->gsp->mesh->ctx;
  cudaSetDevice(ctx->device);
  void* ptrs[] = {P->d_l2g, P->d_weight, P->d_own_idx, P->d_own_ptr, P->d_own_src, P->d_non_idx, P->d_non_src};
  for (void* q : ptrs) dev_free(ctx, q);
  if (P->psp) fg_space_destroy(P->psp);
  delete P;
  return FG_OK;
}

fg_status fg_partition_get_info(fg_partition* P, fg_partition_info* info) {
  if (!P || !info) { set_error("bad argument: partition/info"); return FG_ERR_BADARG; }
  info->num_parts = P->nparts;
  info->num_local_dofs = P->nl;
  int64_t mx = 0;
  for (auto& M : P->parts) mx = std::max<int64_t>(mx, M.num_dofs);
  info->max_part_dofs = mx;
  info->num_couplings = P->ncouplings;
  info->nnz_full = P->psp->nnz;
  info->nnz_upper = P->psp->nnz_upper;
  info->num_dirichlet = P->psp->ndir;
  return FG_OK;
}

fg_status fg_partition_get_dof_import_sizes(fg_partition* P, int32_t part_id, fg_dof_import_sizes* sz) {
  if (!P || !sz || part_id < 1 || part_id > P->nparts) { set_error("bad argument: partition/part_id/sizes"); return FG_ERR_BADARG; }
  const PartMeta& M = P->parts[part_id - 1];
  sz->num_dofs = M.num_dofs;
  sz->num_interior_dofs = M.num_interior;
  sz->num_interface_dofs = M.num_interface;
  sz->num_rcv = (int32_t)M.list_rcv.size();
  sz->num_snd = (int32_t)M.list_snd.size();
  sz->num_unpack = (int32_t)M.unpack_idx.size();
  sz->num_pack = (int32_t)M.pack_idx.size();
  sz->num_cells = (int64_t)M.cells.size();
  sz->first_local_dof = M.dof_off;
  return FG_OK;
}

fg_status fg_partition_get_dof_import(fg_partition* P, int32_t part_id, int32_t* l2g, double* weight, int32_t* list_rcv,
                                      int32_t* rcv_ptrs, int32_t* unpack_idx, int32_t* list_snd, int32_t* snd_ptrs,
                                      int32_t* pack_idx, int64_t* cells) {
  if (!P || part_id < 1 || part_id > P->nparts) { set_error("bad argument: partition/part_id"); return FG_ERR_BADARG; }
  const PartMeta& M = P->parts[part_id - 1];
  auto cp = [](void* dst, const void* src, size_t bytes) { if (dst && bytes) std::memcpy(dst, src, bytes); };
  cp(l2g, M.l2g.data(), sizeof(int32_t) * M.l2g.size());
  cp(weight, M.weight.data(), sizeof(double) * M.weight.size());
  cp(list_rcv, M.list_rcv.data(), sizeof(int32_t) * M.list_rcv.size());
  cp(rcv_ptrs, M.rcv_ptrs.data(), sizeof(int32_t) * M.rcv_ptrs.size());
  cp(unpack_idx, M.unpack_idx.data(), sizeof(int32_t) * M.unpack_idx.size());
  cp(list_snd, M.list_snd.data(), sizeof(int32_t) * M.list_snd.size());
  cp(snd_ptrs, M.snd_ptrs.data(), sizeof(int32_t) * M.snd_ptrs.size());
  cp(pack_idx, M.pack_idx.data(), sizeof(int32_t) * M.pack_idx.size());
  cp(cells, M.cells.data(), sizeof(int64_t) * M.cells.size());
  return FG_OK;
}

fg_status fg_partition_assemble(fg_partition* P, const fg_integrand* integrand, fg_system** out) {
  if (!P || !integrand || !out) { set_error("bad argument: partition/integrand/out"); return FG_ERR_BADARG; }
  return fg_assemble(P->psp, integrand, out);
}

fg_status fg_partition_comm_device(fg_partition* P, double* x) {
  if (!P || !x) { set_error("bad argument: partition/x"); return FG_ERR_BADARG; }
  FG_CUDA_TRY(cudaSetDevice(P->gsp->mesh->ctx->device));
  FG_TRY(partition_comm(P, x));
  FG_CUDA_TRY(cudaStreamSynchronize(P->gsp->mesh->ctx->stream));
  return FG_OK;
}

fg_status fg_partition_solve(fg_partition* P, fg_system* sub, const fg_solver_params* prm, double* x_global,
                             fg_solve_info* info) {
  if (!P || !sub || !prm || !x_global) { set_error("bad argument: partition/system/params/x"); return FG_ERR_BADARG; }
  if (sub->space != P->psp) { set_error("the system was not assembled on this partition"); return FG_ERR_BADARG; }
  if (prm->precond != FG_PREC_JACOBI && prm->precond != FG_PREC_NONE) {
    set_error("the partitioned PCG takes Jacobi or no preconditioner");
    return FG_ERR_UNSUPPORTED;
  }
  if (!sub->d_val) { set_error("the partitioned system was assembled lean"); return FG_ERR_UNSUPPORTED; }
  fg_ctx* ctx = P->gsp->mesh->ctx;
  FG_CUDA_TRY(cudaSetDevice(ctx->device));
  const int64_t n = P->nl;
  double* w = nullptr;  // b d x r z p q dinv | partials | scalar
  FG_TRY(dev_alloc(ctx, (void**)&w, sizeof(double) * (8 * (size_t)n + kDotBlocks + 8)));
  double *b = w, *d = w + n, *x = w + 2 * n, *r = w + 3 * n, *z = w + 4 * n, *p = w + 5 * n, *q = w + 6 * n,
         *dinv = w + 7 * n, *part = w + 8 * n, *scal = part + kDotBlocks;
  double* xg = nullptr;
  FG_TRY(dev_alloc(ctx, (void**)&xg, sizeof(double) * (P->gsp->nfree > 0 ? P->gsp->nfree : 1)));
  cudaStream_t st = ctx->stream;
  auto wdot = [&](const double* a, const double* c, double* res) -> fg_status {
    k_wdot_partial<<<kDotBlocks, 256, 0, st>>>(n, P->d_weight, a, c, part);
    k_sum_partials<<<1, 512, 0, st>>>(kDotBlocks, part, scal);
    FG_CUDA_TRY(cudaMemcpyAsync(res, scal, sizeof(double), cudaMemcpyDeviceToHost, st));
    FG_CUDA_TRY(cudaStreamSynchronize(st));
    ctx->launches += 2;
    return FG_OK;
  };
  fg_status s = FG_OK;
  FG_CUDA_TRY(cudaMemcpyAsync(b, sub->d_rhs, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  FG_TRY(partition_comm(P, b));
  fg_space* ps = P->psp;
  k_extract_diag<<<nblk(n, 256), 256, 0, st>>>(n, ps->d_rowptr, ps->d_col, sub->d_val, d);
  FG_TRY(partition_comm(P, d));
  if (prm->precond == FG_PREC_NONE) {
    // identity preconditioner: d = 1
    std::vector<double> ones(n, 1.0);
    FG_CUDA_TRY(cudaMemcpyAsync(d, ones.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
  }
  k_pcg_init<<<nblk(n, 256), 256, 0, st>>>(n, b, d, x, r, z, p, dinv);
  ctx->launches += 2;
  double rz = 0.0, rr = 0.0, bb = 0.0;
  FG_TRY(wdot(b, b, &bb));
  FG_TRY(wdot(r, z, &rz));
  const double tol = prm->rtol * std::sqrt(bb) + prm->atol;
  int it = 0;
  bool conv = std::sqrt(bb) <= tol;
  const auto t0 = std::chrono::steady_clock::now();
  while (!conv && it < prm->max_iters) {
    FG_TRY(system_spmv(sub, FG_FP64, p, q, st));
    FG_TRY(partition_comm(P, q));
    double pq = 0.0;
    FG_TRY(wdot(p, q, &pq));
    if (!(pq != 0.0) || !std::isfinite(pq)) { s = FG_ERR_NUMERIC; break; }
    const double alpha = rz / pq;
    k_pcg_update<<<nblk(n, 256), 256, 0, st>>>(n, alpha, p, q, dinv, x, r, z);
    ctx->launches += 1;
    ++it;
    FG_TRY(wdot(r, r, &rr));
    if (std::sqrt(rr) <= tol) { conv = true; break; }
    double rzn = 0.0;
    FG_TRY(wdot(r, z, &rzn));
    const double beta = rzn / rz;
    rz = rzn;
    k_pcg_pupdate<<<nblk(n, 256), 256, 0, st>>>(n, beta, z, p);
    ctx->launches += 1;
  }
  const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  k_gather_owned<<<nblk(n, 256), 256, 0, st>>>(n, P->d_l2g, P->d_weight, x, xg);
  ctx->launches += 1;
  FG_CUDA_TRY(cudaMemcpyAsync(x_global, xg, sizeof(double) * P->gsp->nfree, cudaMemcpyDeviceToHost, st));
  FG_CUDA_TRY(cudaStreamSynchronize(st));
  dev_free(ctx, w);
  dev_free(ctx, xg);
  if (info) {
    info->iterations = it;
    info->outer_iterations = 0;
    info->converged = conv ? 1 : 0;
    info->error_estimate = std::sqrt(rr);
    info->tolerance = tol;
    info->solve_ms = ms;
    info->kernel_launches = ctx->launches;
  }
  if (s != FG_OK) { set_error("partitioned PCG breakdown"); return s; }
  if (!conv) { set_error("partitioned PCG: not converged in %d iterations", it); return FG_ERR_NOT_CONVERGED; }
  return FG_OK;
}

}  // extern "C"

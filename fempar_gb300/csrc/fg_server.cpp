// fg_server.cpp -- device-resident request loop (serving form of the hot path).
//
// Worker threads each own an fg_ctx (its own CUDA stream) on one device.  A request is
// admitted when its estimated device footprint fits the remaining HBM budget; requests
// wait in per-size-class FIFO queues (class = log2 of the free dofs) and a free worker
// takes the oldest request among the class heads that fits.  While the globally oldest
// request does not fit, newer requests may still be admitted (backfill) only during its
// first 2 s of waiting, so a large request is not starved by a stream of small ones.
// Admitted requests run concurrently: their kernels overlap on the GPU.  Each request
// builds mesh, space and system on the device, solves (mixed precision by default) and
// copies its solution to a host buffer, then frees its device memory.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "fg_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t id = 0;
  fg_request r;
  std::vector<double> coef;
  std::vector<int32_t> ids;
  uint64_t bytes = 0;
  int64_t nfree = 0;
  int cls = 0;
  Clock::time_point t_submit, t_start, t_end;
  fg_result res;
  std::vector<double> x;
  bool done = false;
};

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

// Boundary set id of the vef that owns lattice node (I,J,K) (uniform_hex_mesh_generator
// numbering of the 27 regions of the box), host version.
int node_set_id(const int* IJK, const int* n, int p, const int* code2idx) {
  int anchor = 0, t = 0;
  for (int d = 0; d < 3; ++d) {
    if (IJK[d] % p != 0) { t |= 1 << d; continue; }  // inside a cell in this direction
    const int v = IJK[d] / p;
    if (v == 0) {
    } else if (v == n[d]) anchor |= 1 << d;
    else t |= 1 << d;
  }
  return code2idx[anchor | (t << 3)] + 1;
}

}  // namespace

struct fg_server {
  int device = 0;
  uint64_t budget = 0, reserved = 0, peak = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::map<int, std::deque<Request*>> queues;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
  std::vector<std::thread> workers;
  bool stop = false;
  uint64_t next_id = 1;
  int64_t completed = 0;
};

namespace fg {

// free dofs and footprint of a request (exact dof count; matrix sizes bounded from above)
static fg_status footprint(const fg_request* q, uint64_t* bytes, int64_t* nfree_out) {
  if (!q || q->n[0] < 1 || q->n[1] < 1 || q->n[2] < 1 || q->order < 1 || q->order > FG_MAX_ORDER) {
    set_error("bad request");
    return FG_ERR_BADARG;
  }
  const int p = q->order, ncomp = q->kind == FG_ELASTICITY ? 3 : 1;
  RefTables t;
  t.build(p, ncomp);
  uint32_t mask = 0;
  for (int i = 0; i < q->n_ids; ++i) {
    if (q->dirichlet_ids[i] < 1 || q->dirichlet_ids[i] > 27) { set_error("dirichlet id"); return FG_ERR_BADARG; }
    mask |= 1u << q->dirichlet_ids[i];
  }
  const int Ln[3] = {p * q->n[0] + 1, p * q->n[1] + 1, p * q->n[2] + 1};
  // lattice nodes by region: per direction the low plane (1 node), the high plane (1) or
  // the Ln-2 nodes in between; a region's nodes are free unless its set id is Dirichlet
  int64_t nfree_nodes = 0;
  for (int rz = 0; rz < 3; ++rz)
    for (int ry = 0; ry < 3; ++ry)
      for (int rx = 0; rx < 3; ++rx) {
        const int rr[3] = {rx, ry, rz};
        int IJK[3];
        int64_t cnt = 1;
        for (int d = 0; d < 3; ++d) {
          IJK[d] = rr[d] == 0 ? 0 : (rr[d] == 2 ? Ln[d] - 1 : 1);
          cnt *= rr[d] == 1 ? (int64_t)(Ln[d] - 2) : 1;
        }
        if (cnt <= 0) continue;
        // a node strictly inside (1 <= I <= Ln-2) has the set id of any interior node of its
        // region; I = 1 is inside a cell (p > 1) or on an interior plane (p = 1): both give
        // a free direction in node_set_id
        if (!((mask >> node_set_id(IJK, q->n, p, t.code2idx)) & 1u)) nfree_nodes += cnt;
      }
  const int64_t nfree = nfree_nodes * ncomp;
  const double ncells = (double)q->n[0] * q->n[1] * q->n[2];
  const double nlat = (double)Ln[0] * Ln[1] * Ln[2];
  const double box_d = ((2.0 * p + 1.0) + (p - 1.0) * (p + 1.0)) / p;  // mean box width per direction
  const double nnz = (double)nfree * box_d * box_d * box_d * ncomp;
  const double nd = (double)t.nd;
  const double nvec = std::pow((double)p * std::max({q->n[0], q->n[1], q->n[2]}) + 1.0 + 3.0 * p, 3.0) * ncomp;
  // requests are assembled lean (FG_LEAN_SYSTEM): the element matrices are released before
  // the solver layout is allocated, the CSR after it is filled, so the peak is the larger of
  // (element matrices + CSR) and (CSR + solver layout), plus what lives throughout
  double elm = ncells * nd * nd * 8 + ncells * nd * 8;  // element matrices and vectors
  if (ncomp == 1) {
    // Poisson element matrices on the tensor cores: geometric factors (K = 6 NQ per cell),
    // packed upper triangles and the digit workspace (7 bf16 digits, K padded to 16)
    const double K = 6.0 * t.nq, npair = nd * (nd + 1) / 2;
    elm += ncells * (K * 8 + npair * 8 + std::ceil(K / 16.0) * 16 * 7 * 2) + npair * K * 8;
  }
  const double csr = nnz * (4 + 8) + nfree * 8.0;             // CSR pattern + FP64 values + row pointers
  const double lay = nnz * 1.15 * (8 + 4);                    // solver layout FP64 + FP32 (padding)
  double b = std::max(elm, lay) + csr;
  b += nvec * (6 * 8 + 4 * 4 + 12);                 // solver vectors + Jacobi
  b += nlat * ncomp * (4 + 14) + nfree * 12.0;      // dof maps + symbolic-phase temporaries
  b += (double)(q->n[0] + 1) * (q->n[1] + 1) * (q->n[2] + 1) * 24 + ncells * 8;
  b = b * 1.10 + (64u << 20);
  *bytes = (uint64_t)b;
  *nfree_out = nfree;
  return FG_OK;
}

static void run_request(fg_ctx* ctx, Request* R) {
  fg_status s = FG_OK;
  fg_mesh* mesh = nullptr;
  fg_space* sp = nullptr;
  fg_system* sys = nullptr;
  const double lim[6] = {0, 1, 0, 1, 0, 1};
  const int ncomp = R->r.kind == FG_ELASTICITY ? 3 : 1;
  s = fg_mesh_create_structured(ctx, 3, R->r.n, lim, nullptr, &mesh);
  if (s == FG_OK) s = fg_space_create(mesh, R->r.order, ncomp, R->ids.data(), (int)R->ids.size(), &sp);
  if (s == FG_OK) {
    fg_integrand g;
    fg_integrand_default(&g);
    g.kind = R->r.kind;
    g.cell_coef = R->coef.empty() ? nullptr : R->coef.data();
    g.coef_const = R->r.coef_const;
    g.nu = R->r.nu;
    g.source_fn = R->r.source_fn;
    for (int i = 0; i < 8; ++i) g.fn_param[i] = R->r.fn_param[i];
    g.flags = FG_LEAN_SYSTEM;
    s = fg_assemble(sp, &g, &sys);
    if (s == FG_OK) s = fg_space_release_pattern(sp);
  }
  fg_solve_info info;
  std::memset(&info, 0, sizeof(info));
  if (s == FG_OK) {
    fg_space_info si;
    fg_space_get_info(sp, &si);
    R->x.assign(si.num_free, 0.0);
    R->res.num_free = si.num_free;
    s = fg_solve(sys, &R->r.solver, nullptr, nullptr, R->x.data(), &info);
  }
  R->res.status = s;
  R->res.iterations = info.iterations;
  R->res.outer_iterations = info.outer_iterations;
  R->res.solve_ms = info.solve_ms;
  fg_system_destroy(sys);
  fg_space_destroy(sp);
  fg_mesh_destroy(mesh);
}

static Request* pick(fg_server* S) {
  Request* oldest = nullptr;
  for (auto& kv : S->queues)
    if (!kv.second.empty() && (!oldest || kv.second.front()->id < oldest->id)) oldest = kv.second.front();
  if (!oldest) return nullptr;
  const uint64_t room = S->budget - S->reserved;
  if (oldest->bytes <= room) return oldest;
  // backfill with newer requests only during the oldest one's first 2 s of waiting
  if (ms_between(oldest->t_submit, Clock::now()) > 2000.0) return nullptr;
  Request* best = nullptr;
  for (auto& kv : S->queues)
    if (!kv.second.empty() && kv.second.front()->bytes <= room && (!best || kv.second.front()->id < best->id))
      best = kv.second.front();
  return best;
}

static void worker_main(fg_server* S) {
  fg_ctx* ctx = nullptr;
  if (fg_ctx_create(S->device, 0, &ctx) != FG_OK) return;
  for (;;) {
    Request* R = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_work.wait_for(lk, std::chrono::milliseconds(100), [&] { return S->stop || pick(S) != nullptr; });
      if (S->stop) break;
      R = pick(S);
      if (!R) continue;
      S->queues[R->cls].pop_front();
      S->reserved += R->bytes;
      S->peak = std::max(S->peak, S->reserved);
      R->t_start = Clock::now();
    }
    run_request(ctx, R);
    {
      std::lock_guard<std::mutex> lk(S->mu);
      R->t_end = Clock::now();
      S->reserved -= R->bytes;
      R->res.t_queue_ms = ms_between(R->t_submit, R->t_start);
      R->res.t_run_ms = ms_between(R->t_start, R->t_end);
      R->res.t_total_ms = ms_between(R->t_submit, R->t_end);
      R->res.footprint_bytes = R->bytes;
      R->done = true;
      ++S->completed;
    }
    S->cv_done.notify_all();
    S->cv_work.notify_all();
  }
  fg_ctx_destroy(ctx);
}

}  // namespace fg

using namespace fg;

extern "C" {

fg_status fg_request_footprint(const fg_request* req, uint64_t* bytes, int64_t* num_free) {
  if (!bytes || !num_free) { set_error("bad argument"); return FG_ERR_BADARG; }
  return footprint(req, bytes, num_free);
}

fg_status fg_server_create(int device, uint64_t hbm_budget_bytes, int nworkers, fg_server** out) {
  if (!out || nworkers < 1 || nworkers > 64) { set_error("bad argument"); return FG_ERR_BADARG; }
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    set_error("no such CUDA device");
    return FG_ERR_NO_DEVICE;
  }
  fg_server* S = new fg_server();
  S->device = device;
  if (!hbm_budget_bytes) {
    size_t fr = 0, tot = 0;
    cudaSetDevice(device);
    cudaMemGetInfo(&fr, &tot);
    hbm_budget_bytes = (uint64_t)(fr * 0.9);
  }
  S->budget = hbm_budget_bytes;
  for (int i = 0; i < nworkers; ++i) S->workers.emplace_back(worker_main, S);
  *out = S;
  return FG_OK;
}

fg_status fg_server_submit(fg_server* S, const fg_request* req, uint64_t* ticket) {
  if (!S || !req || !ticket) { set_error("bad argument"); return FG_ERR_BADARG; }
  std::unique_ptr<Request> R(new Request());
  R->r = *req;
  FG_TRY(footprint(req, &R->bytes, &R->nfree));
  if (R->bytes > S->budget) {
    set_error("request needs %llu bytes, above the server's HBM budget of %llu", (unsigned long long)R->bytes,
              (unsigned long long)S->budget);
    return FG_ERR_OOM;
  }
  const int64_t ncells = (int64_t)req->n[0] * req->n[1] * req->n[2];
  if (req->cell_coef) R->coef.assign(req->cell_coef, req->cell_coef + ncells);
  if (req->n_ids > 0) R->ids.assign(req->dirichlet_ids, req->dirichlet_ids + req->n_ids);
  R->r.cell_coef = nullptr;
  R->r.dirichlet_ids = nullptr;
  R->cls = R->nfree > 0 ? (int)std::floor(std::log2((double)R->nfree)) : 0;
  std::memset(&R->res, 0, sizeof(R->res));
  {
    std::lock_guard<std::mutex> lk(S->mu);
    R->id = S->next_id++;
    R->t_submit = Clock::now();
    *ticket = R->id;
    S->queues[R->cls].push_back(R.get());
    S->reqs[R->id] = std::move(R);
  }
  S->cv_work.notify_all();
  return FG_OK;
}

fg_status fg_server_wait(fg_server* S, uint64_t ticket, int timeout_ms, fg_result* res) {
  if (!S) { set_error("bad argument"); return FG_ERR_BADARG; }
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) { set_error("unknown ticket %llu", (unsigned long long)ticket); return FG_ERR_BADARG; }
  Request* R = it->second.get();
  if (timeout_ms < 0) S->cv_done.wait(lk, [&] { return R->done; });
  else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return R->done; }))
    return FG_ERR_TIMEOUT;
  if (res) *res = R->res;
  return FG_OK;
}

fg_status fg_server_take_solution(fg_server* S, uint64_t ticket, double* x) {
  if (!S) { set_error("bad argument"); return FG_ERR_BADARG; }
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end() || !it->second->done) { set_error("ticket not finished or unknown"); return FG_ERR_BADARG; }
  if (x && !it->second->x.empty()) std::memcpy(x, it->second->x.data(), sizeof(double) * it->second->x.size());
  S->reqs.erase(it);
  return FG_OK;
}

fg_status fg_server_stats(fg_server* S, uint64_t* peak_reserved, int64_t* completed) {
  if (!S) { set_error("bad argument"); return FG_ERR_BADARG; }
  std::lock_guard<std::mutex> lk(S->mu);
  if (peak_reserved) *peak_reserved = S->peak;
  if (completed) *completed = S->completed;
  return FG_OK;
}

fg_status fg_server_destroy(fg_server* S) {
  if (!S) return FG_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  for (auto& t : S->workers) t.join();
  delete S;
  return FG_OK;
}

}  // extern "C"

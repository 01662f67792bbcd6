"""Serving form of the GB300 path: a device-resident request loop (fg_server_* C-ABI).

    srv = Server(device=0, hbm_budget_bytes=150 << 30, nworkers=4)
    t = srv.submit(kind=POISSON, n=(32, 32, 32), order=2, cell_coef=k)   # returns at once
    res = srv.wait(t); x = srv.take(t)                                   # per-request latency

Open-loop benchmark (``python -m fempar_gb300.serving``): requests arrive with exponential
inter-arrival times at a given rate; each is Poisson or linear elasticity (50/50) on an n^3
hex mesh with n log-uniform in [nmin, nmax], order Q1 or Q2, lognormal(sigma=1) cellwise
coefficients, homogeneous Dirichlet (Poisson: whole boundary; elasticity: clamped at x=0),
source 1 / body force (0,0,-1); admitted by HBM budget, solved by mixed-precision PCG
(Jacobi) to 1e-8.  Reports p50/p99 latency, throughput and, for a sample, the error
against the FP64 solve of the same request.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import threading
import time

import numpy as np

from . import _lib as L

POISSON, ELASTICITY = L.FG_POISSON, L.FG_ELASTICITY
ALL_BOUNDARY_IDS = list(range(1, 27))
CLAMP_X0_IDS = [1, 3, 5, 7, 13, 15, 17, 19, 25]


def make_request(kind, n, order, cell_coef=None, coef_const=1.0, nu=0.3, source_fn=L.FG_FN_CONST,
                 fn_param=None, dirichlet_ids=None, precision=L.FG_MIXED, rtol=1e-8, max_iters=200000,
                 precond=L.FG_PREC_JACOBI):
    r = L.Request()
    keep = []
    r.kind = kind
    for i in range(3):
        r.n[i] = int(n[i])
    r.order = order
    if cell_coef is not None:
        a = np.ascontiguousarray(cell_coef, dtype=np.float64)
        keep.append(a)
        r.cell_coef = a.ctypes.data
    r.coef_const = coef_const
    r.nu = nu
    r.source_fn = source_fn
    if fn_param is None:
        fn_param = [0.0, 0.0, -1.0] if kind == ELASTICITY else [1.0]
    for i, v in enumerate(fn_param):
        r.fn_param[i] = float(v)
    ids = dirichlet_ids if dirichlet_ids is not None else (CLAMP_X0_IDS if kind == ELASTICITY else ALL_BOUNDARY_IDS)
    ia = np.ascontiguousarray(ids, dtype=np.int32)
    keep.append(ia)
    r.dirichlet_ids = ia.ctypes.data
    r.n_ids = len(ids)
    L.lib().fg_solver_params_default(C.byref(r.solver))
    r.solver.precision = precision
    r.solver.precond = precond
    r.solver.rtol = rtol
    r.solver.max_iters = max_iters
    return r, keep


def footprint(**kw):
    r, keep = make_request(**kw)
    b, n = C.c_uint64(), C.c_int64()
    L.check(L.lib().fg_request_footprint(C.byref(r), C.byref(b), C.byref(n)), "fg_request_footprint")
    return b.value, n.value


class Server:
    def __init__(self, device=0, hbm_budget_bytes=0, nworkers=4):
        h = C.c_void_p()
        L.check(L.lib().fg_server_create(device, hbm_budget_bytes, nworkers, C.byref(h)), "fg_server_create")
        self.h = h

    def submit(self, **kw) -> int:
        r, keep = make_request(**kw)
        t = C.c_uint64()
        L.check(L.lib().fg_server_submit(self.h, C.byref(r), C.byref(t)), "fg_server_submit")
        del keep  # copied by the server at submit
        return t.value

    def wait(self, ticket, timeout_ms=-1):
        res = L.Result()
        st = L.lib().fg_server_wait(self.h, ticket, timeout_ms, C.byref(res))
        if st == -6:
            return None
        L.check(st, "fg_server_wait")
        return {k: getattr(res, k) for k, _ in L.Result._fields_}

    def take(self, ticket, num_free):
        x = np.zeros(num_free)
        L.check(L.lib().fg_server_take_solution(self.h, ticket, x.ctypes.data), "fg_server_take_solution")
        return x

    def stats(self):
        p, c = C.c_uint64(), C.c_int64()
        L.check(L.lib().fg_server_stats(self.h, C.byref(p), C.byref(c)), "fg_server_stats")
        return {"peak_reserved_bytes": p.value, "completed": c.value}

    def close(self):
        if getattr(self, "h", None):
            L.lib().fg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def request_stream(count, nmin, nmax, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(count):
        kind = ELASTICITY if rng.random() < 0.5 else POISSON
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        order = int(rng.integers(1, 3))
        coef = np.exp(rng.normal(0.0, 1.0, size=n ** 3))
        out.append({"kind": kind, "n": (n, n, n), "order": order, "cell_coef": coef})
    return out


def run_open_loop(rate, count=200, nmin=16, nmax=48, budget_gb=150, nworkers=4, seed=20261203, check_every=25,
                  device=0):
    reqs = request_stream(count, nmin, nmax, seed)
    rng = np.random.Generator(np.random.PCG64(seed + 7))
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=count))
    srv = Server(device=device, hbm_budget_bytes=int(budget_gb * (1 << 30)), nworkers=nworkers)
    tickets = [None] * count
    t0 = time.perf_counter()

    def submitter():
        for i, rq in enumerate(reqs):
            dt = arrivals[i] - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            tickets[i] = srv.submit(**rq)

    th = threading.Thread(target=submitter)
    th.start()
    th.join()
    results, sols = [], {}
    dofs = 0
    for i, t in enumerate(tickets):
        res = srv.wait(t)
        results.append(res)
        dofs += res["num_free"]
        x = srv.take(t, res["num_free"])
        if i % check_every == 0:
            sols[i] = x
    wall = time.perf_counter() - t0
    # error of sampled mixed-precision solutions vs the FP64 solve of the same request
    errs = []
    for i, x in sols.items():
        rq = dict(reqs[i])
        t = srv.submit(**rq, precision=L.FG_FP64)
        res = srv.wait(t)
        x64 = srv.take(t, res["num_free"])
        errs.append(float(np.linalg.norm(x - x64) / max(np.linalg.norm(x64), 1e-300)))
    stats = srv.stats()
    srv.close()
    lat = np.array([r["t_total_ms"] for r in results])
    ok = sum(1 for r in results if r["status"] == 0)
    return {"rate_req_s": rate, "requests": count, "completed_ok": ok, "wall_s": wall,
            "throughput_req_s": count / wall, "throughput_dof_s": dofs / wall,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_queue_ms": float(np.mean([r["t_queue_ms"] for r in results])),
            "max_err_vs_fp64": max(errs) if errs else None, "n_err_samples": len(errs),
            "peak_reserved_gb": stats["peak_reserved_bytes"] / 1e9, "nworkers": nworkers,
            "n_range": [nmin, nmax], "budget_gb": budget_gb}


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--rates", type=float, nargs="+", default=[50.0, 200.0])
    ap.add_argument("--count", type=int, default=120)
    ap.add_argument("--nmin", type=int, default=16)
    ap.add_argument("--nmax", type=int, default=40)
    ap.add_argument("--workers", type=int, default=4)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    args = ap.parse_args()
    from . import build
    build.build()
    for rate in args.rates:
        out = run_open_loop(rate, count=args.count, nmin=args.nmin, nmax=args.nmax, budget_gb=args.budget_gb,
                            nworkers=args.workers)
        print(json.dumps({"metric": "serving p50/p99 solve latency", **out}), flush=True)


if __name__ == "__main__":
    main()

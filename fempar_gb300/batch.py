"""Batched independent Poisson solves in one persistent launch (fg_batch_* C-ABI).

    b = BatchSolver(ctx, problems, rtol=1e-8)      # plan: buffers, team schedule, block size, graph
    results = b.run()                               # assemble + Jacobi-PCG for every problem

``problems`` is a list of dicts ``{"n", "order", "coef", "qp_source", "x"}``: numpy arrays
(host mode, copied in/out by every run) or torch CUDA float64 tensors (device mode).

Benchmark (``python -m fempar_gb300.batch``): 4096 problems, n = round(exp(U(ln 8, ln 48))),
order uniform in {1,2,3}, k ~ U[0.1, 10], f ~ N(0,1) i.i.d. at every Gauss point, seeded;
FP32 CG with float-float refinement to 1e-8.  Reports DOF/s (total free dofs / device time
of one run) beside the estimated stencil work, and checks a sample against FP64 solves of
the same problems through the general (assembled) path.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import time

import numpy as np

from . import _lib as L

SEED = 20261203


def _ptr(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return C.c_void_p(a.ctypes.data)


class BatchSolver:
    def __init__(self, ctx, problems, rtol=1e-8, atol=0.0, max_iters=100000, threads=0, on_device=None):
        self.ctx = ctx
        self.problems = problems
        if on_device is None:
            on_device = hasattr(problems[0]["qp_source"], "data_ptr")
        arr = (L.BatchProblem * len(problems))()
        for i, q in enumerate(problems):
            n, p = int(q["n"]), int(q["order"])
            nf = n ** 3 * (p + 1) ** 3
            nx = max(p * n - 1, 0) ** 3
            src, x = q["qp_source"], q["x"]
            for t, m in ((src, nf), (x, nx)):
                if (t.numel() if hasattr(t, "numel") else t.size) != m:
                    raise ValueError(f"problem {i}: expected {nf} source values and {nx} outputs")
            arr[i].n, arr[i].order, arr[i].coef = n, p, float(q["coef"])
            arr[i].qp_source = _ptr(src).value
            arr[i].x = _ptr(x).value
        self._arr = arr
        prm = L.SolverParams()
        L.lib().fg_solver_params_default(C.byref(prm))
        prm.rtol, prm.atol, prm.max_iters = rtol, atol, max_iters
        h = C.c_void_p()
        L.check(L.lib().fg_batch_create(ctx.h, len(problems), arr, L.FG_INPUTS_ON_DEVICE if on_device else 0,
                                        C.byref(prm), int(threads), C.byref(h)), "fg_batch_create")
        self.h = h

    def run(self, raise_on_error=True):
        res = (L.BatchResult * len(self.problems))()
        st = L.lib().fg_batch_run(self.h, res)
        if st != L.FG_OK and raise_on_error:
            raise L.FGError(st, "fg_batch_run")
        return [{k: getattr(r, k) for k, _ in L.BatchResult._fields_} for r in res]

    def info(self):
        i = L.BatchInfo()
        L.check(L.lib().fg_batch_get_info(self.h, C.byref(i)), "fg_batch_get_info")
        return {k: getattr(i, k) for k, _ in L.BatchInfo._fields_}

    def close(self):
        if getattr(self, "h", None):
            L.lib().fg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def problem_set(count, seed=SEED, nmin=8, nmax=48, orders=(1, 2, 3)):
    """Sizes, orders and coefficients of the cfg-style batch (sources drawn separately)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = np.round(np.exp(rng.uniform(np.log(nmin), np.log(nmax), size=count))).astype(int)
    p = rng.choice(np.array(orders), size=count)
    k = rng.uniform(0.1, 10.0, size=count)
    return [{"n": int(n[i]), "order": int(p[i]), "coef": float(k[i])} for i in range(count)]


def lattice_index_map(dof_map, n, p):
    """Index map: interior-lattice position (x fastest) -> 0-based free dof id of the
    reference numbering, from a (ncells, (p+1)^3) scalar dof map."""
    F = p * n - 1
    nn = (p + 1) ** 3
    c = np.arange(n ** 3)
    a = np.arange(nn)
    ci, cj, ck = c % n, (c // n) % n, c // (n * n)
    ai, aj, ak = a % (p + 1), (a // (p + 1)) % (p + 1), a // ((p + 1) ** 2)
    I = p * ci[:, None] + ai[None, :]
    J = p * cj[:, None] + aj[None, :]
    K = p * ck[:, None] + ak[None, :]
    dm = np.asarray(dof_map).reshape(n ** 3, nn)
    free = dm > 0
    out = np.full(max(F, 0) ** 3, -1, dtype=np.int64)
    out[((I - 1) + F * ((J - 1) + F * (K - 1)))[free]] = dm[free] - 1
    return out


def benchmark(ctx, count=4096, nmin=8, nmax=48, threads=0, runs=3, rtols=(1e-8,), check=16, seed=SEED):
    """The batched benchmark on `ctx`: `count` problems of the cfg-style distribution, solved
    `runs` times in one persistent launch each, for every residual tolerance in `rtols`.  A
    sample of `check` problems is also solved by the plain FP64 drop-in (assembled CSR,
    Jacobi-CG) at each tolerance (timed) and at 1e-13, and the batch solutions are compared
    with both.  Returns a JSON-ready dict: the first tolerance's figures at the top level,
    every tolerance's under "by_rtol"."""
    import torch

    from .fe import FEAffineOperator, IterativeLinearSolver, PoissonIntegration, SerialFESpace, SerialTriangulation
    dev = f"cuda:{ctx.device}"
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    probs = problem_set(count, seed=seed, nmin=nmin, nmax=nmax)
    for q in probs:
        n, p = q["n"], q["order"]
        q["qp_source"] = torch.randn(n ** 3 * (p + 1) ** 3, dtype=torch.float64, device=dev, generator=g)
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    small = [i for i, q in enumerate(probs) if (q["order"] * q["n"] - 1) ** 3 <= 2000000]
    sample = [int(i) for i in rng.choice(small, size=min(check, len(small)), replace=False)]
    # FP64 reference solutions of the sample (drop-in at 1e-13), kept on the host
    ref = {}
    for i in sample:
        q = probs[i]
        n, p = q["n"], q["order"]
        tri = SerialTriangulation(ctx, (n, n, n))
        sp = SerialFESpace(tri, order=p, dirichlet_ids=list(range(1, 27)))
        op = FEAffineOperator(sp, PoissonIntegration(coef_const=q["coef"], source_fn=L.FG_FN_QP_VALUES,
                                                     qp_source=q["qp_source"].cpu().numpy())).compute()
        s = IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
        s.set_parameters_from_pl({"ILS_RTOL": 1e-13, "ILS_MAX_NUM_ITERATIONS": 200000})
        ref[i] = (s.solve(), lattice_index_map(sp.get_dof_map(), n, p), tri, sp, op)
    by = {}
    for rtol in rtols:
        for q in probs:
            q["x"] = torch.zeros(max(q["order"] * q["n"] - 1, 0) ** 3, dtype=torch.float64, device=dev)
        t0 = time.perf_counter()
        B = BatchSolver(ctx, probs, rtol=rtol, threads=threads)
        plan_s = time.perf_counter() - t0
        times = []
        for _ in range(runs):
            res = B.run()
            times.append(B.info()["run_ms"])
        info = B.info()
        dofs = info["total_dofs"]
        its = np.array([r["iterations"] for r in res])
        # algorithmic stencil work: iterations x interior nodes x mean stencil width x 2 flops
        width = {1: 27.0, 2: 64.0, 3: 125.0}
        flops = sum(2.0 * r["iterations"] * max(q["order"] * q["n"] - 1, 0) ** 3 * width[q["order"]]
                    for q, r in zip(probs, res))
        rec = {"rtol": rtol, "problems": count, "total_dofs": dofs, "run_ms": min(times), "runs_ms": times,
               "dof_per_s": dofs / (min(times) * 1e-3), "plan_s": plan_s, "info": info,
               "iterations": {"mean": float(its.mean()), "max": int(its.max())},
               "stencil_tflop": flops / 1e12, "stencil_tflops_per_s": flops / (min(times) * 1e-3) / 1e12,
               "refinements_mean": float(np.mean([r["refinements"] for r in res])),
               "all_converged": all(r["status"] == 0 for r in res)}
        errs, errs_same, errs_fp64, t64, d64 = [], [], [], 0.0, 0
        for i in sample:
            q = probs[i]
            x13, idx, tri, sp, op = ref[i]
            # the plain FP64 drop-in at the same rtol: assembly + solve, timed
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            op.compute()
            s8 = IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
            s8.set_parameters_from_pl({"ILS_RTOL": rtol, "ILS_MAX_NUM_ITERATIONS": 200000})
            x8 = s8.solve()
            t64 += time.perf_counter() - t1
            d64 += sp.num_free_dofs
            xb = q["x"].cpu().numpy()
            errs.append(float(np.linalg.norm(xb - x13[idx]) / np.linalg.norm(x13)))
            errs_same.append(float(np.linalg.norm(xb - x8[idx]) / np.linalg.norm(x8)))
            errs_fp64.append(float(np.linalg.norm(x8 - x13) / np.linalg.norm(x13)))
        rec["max_err_vs_fp64_rtol1e-13"] = max(errs) if errs else None
        rec["max_err_vs_fp64_same_rtol"] = max(errs_same) if errs_same else None
        # what the stopping rule itself allows: the FP64 drop-in at rtol vs the same at 1e-13
        rec["max_err_fp64_dropin_vs_rtol1e-13"] = max(errs_fp64) if errs_fp64 else None
        if d64:
            rec["fp64_dropin_sample"] = {"problems": len(errs), "dofs": d64, "seconds": t64, "dof_per_s": d64 / t64}
            rec["batch_over_fp64_dropin"] = rec["dof_per_s"] / (d64 / t64)
        by[str(rtol)] = rec
        B.close()
    for i in sample:
        ref[i][4].close()
    return {"metric": "batched Poisson: DOF/s to rtol (assembly + Jacobi-PCG), one persistent launch",
            **by[str(rtols[0])], "by_rtol": by}


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--count", type=int, default=4096)
    ap.add_argument("--nmin", type=int, default=8)
    ap.add_argument("--nmax", type=int, default=48)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--runs", type=int, default=3)
    ap.add_argument("--rtol", type=float, nargs="+", default=[1e-8])
    ap.add_argument("--check", type=int, default=16, help="problems checked against FP64 assembled solves")
    args = ap.parse_args()
    from . import build
    from .fe import Context
    build.build()
    ctx = Context(0)
    out = benchmark(ctx, count=args.count, nmin=args.nmin, nmax=args.nmax, threads=args.threads, runs=args.runs,
                    rtols=tuple(args.rtol), check=args.check)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()

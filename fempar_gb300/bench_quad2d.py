"""2D benchmark: tutorial_01's continuous Poisson problem on quadrilaterals
(``python -m fempar_gb300.bench_quad2d``).

Workload (seeded, synthetic): unit square, n^2 quadrilaterals with interior vertices perturbed
by U(-0.15h, 0.15h), k = exp(N(0,1)) per cell, the tutorial's sharp circular wave in 2D
(alpha 200, r 0.7, centre (-0.05, -0.05)) as source and Dirichlet data on every boundary set,
Q_p elements, Jacobi-PCG to 1e-8.  Times: space (numbering, pattern, SELL layout), numeric
assembly, solve in FP64 and mixed precision; L2 / H1 errors against the exact solution.

Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import _lib as L
from .fe import Context, FEAffineOperator, IterativeLinearSolver, PoissonIntegration, SerialFESpace, SerialTriangulation

SEED = 20261203
SHARP = [200.0, 0.7, -0.05, -0.05, 0.0]


def perturbed_vertices(n, rng):
    h = 1.0 / n
    j, i = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    ii, jj = i.ravel(), j.ravel()
    xyz = np.stack([ii * h, jj * h, np.zeros(ii.size)], axis=-1)
    interior = (ii > 0) & (ii < n) & (jj > 0) & (jj < n)
    xyz[interior, :2] += rng.uniform(-0.15 * h, 0.15 * h, size=(int(interior.sum()), 2))
    return xyz.ravel()


def run(n=2048, order=2, rtol=1e-8, device=0):
    rng = np.random.Generator(np.random.PCG64(SEED))
    xyz = perturbed_vertices(n, rng)
    k = np.exp(rng.normal(0.0, 1.0, size=n * n))
    ctx = Context(device)
    tri = SerialTriangulation(ctx, (n, n), vertex_xyz=xyz)
    out = {"metric": "2D Poisson (quadrilaterals): DOF/s to 1e-8 (assembly + Jacobi-PCG)", "n": [n, n],
           "order": order}
    t0 = time.perf_counter()
    sp = SerialFESpace(tri, order=order, dirichlet_ids=list(range(1, 9)))
    out["space_ms"] = (time.perf_counter() - t0) * 1e3
    out["dofs"] = sp.num_free_dofs
    out["nnz_full"] = sp.info.nnz_full
    integ = PoissonIntegration(cell_coef=k, source_fn=L.FG_FN_SHARP_WAVE, boundary_fn=L.FG_FN_SHARP_WAVE,
                               fn_param=SHARP)
    op = FEAffineOperator(sp, integ)
    op.compute()
    t0 = time.perf_counter()
    op.compute()
    out["assembly_ms"] = (time.perf_counter() - t0) * 1e3
    for prec in ("fp64", "mixed"):
        s = IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
        s.set_parameters_from_pl({"ILS_RTOL": rtol, "ILS_MAX_NUM_ITERATIONS": 400000, "PRECISION": prec})
        x = s.solve()
        inf = s.info()
        step = out["assembly_ms"] + inf["solve_ms"]
        err = op.error_norms(x, L.FG_FN_SHARP_WAVE, SHARP)
        out[prec] = {"iterations": inf["iterations"], "outer_iterations": inf["outer_iterations"],
                     "converged": inf["converged"], "solve_ms": inf["solve_ms"], "step_ms": step,
                     "dof_per_s": sp.num_free_dofs / (step * 1e-3),
                     "ms_per_iteration": inf["solve_ms"] / max(inf["iterations"], 1),
                     "l2_error": err["l2_norm"], "h1_error": err["h1_norm"]}
    out["mixed_vs_fp64"] = out["mixed"]["dof_per_s"] / out["fp64"]["dof_per_s"]
    out["note"] = "host wall time around the synchronous assembly; solve_ms from CUDA events"
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--order", type=int, default=2)
    args = ap.parse_args()
    from . import build
    build.build()
    print(json.dumps(run(args.n, args.order)), flush=True)


if __name__ == "__main__":
    main()

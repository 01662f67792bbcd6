"""dG benchmark: tutorial_01's interior-penalty formulation on the device
(``python -m fempar_gb300.bench_dg``).

Workload (seeded, synthetic): unit cube, n^3 hexahedra with interior vertices perturbed by
U(-0.15h, 0.15h), the tutorial's sharp circular wave (alpha 200, r 0.7, centre -0.05) as source
and weak boundary data, dG of order p (C_IP = 10 p^2), Jacobi-PCG to 1e-8.  Times: space
(neighbours, pattern, SELL), numeric assembly (volume kernel + facet-row kernel), solve in
FP64 and mixed precision; L2 / H1 errors against the exact solution; the continuous Q_p
discretisation of the same problem beside it.

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
SHARP = [200.0, 0.7, -0.05, -0.05, -0.05]


def perturbed_vertices(n, rng):
    h = 1.0 / n
    k, j, i = np.meshgrid(np.arange(n + 1), np.arange(n + 1), np.arange(n + 1), indexing="ij")
    xyz = np.stack([i * h, j * h, k * h], axis=-1).reshape(-1, 3)
    ii, jj, kk = i.ravel(), j.ravel(), k.ravel()
    interior = (ii > 0) & (ii < n) & (jj > 0) & (jj < n) & (kk > 0) & (kk < n)
    xyz[interior] += rng.uniform(-0.15 * h, 0.15 * h, size=xyz.shape)[interior]
    return xyz.ravel()


def solve(op, prec, rtol):
    s = IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": rtol, "ILS_MAX_NUM_ITERATIONS": 400000, "PRECISION": prec})
    x = s.solve()
    return x, s.info()


def run(n=48, order=2, rtol=1e-8, device=0, cg=True):
    rng = np.random.Generator(np.random.PCG64(SEED))
    xyz = perturbed_vertices(n, rng)
    ctx = Context(device)
    tri = SerialTriangulation(ctx, (n, n, n), vertex_xyz=xyz)
    out = {"metric": "dG (interior penalty) Poisson: DOF/s to 1e-8 (assembly + Jacobi-PCG)", "n": n, "order": order}
    t0 = time.perf_counter()
    sp = SerialFESpace(tri, order=order, dg=True)
    out["space_ms"] = (time.perf_counter() - t0) * 1e3
    out["dofs"] = sp.num_free_dofs
    out["nnz_full"] = sp.info.nnz_full
    integ = PoissonIntegration(source_fn=L.FG_FN_SHARP_WAVE, boundary_fn=L.FG_FN_SHARP_WAVE, fn_param=SHARP)
    op = FEAffineOperator(sp, integ)
    op.compute()
    t0 = time.perf_counter()
    op.compute()
    t_asm = (time.perf_counter() - t0) * 1e3
    out["assembly_ms"] = t_asm
    for prec in ("fp64", "mixed"):
        x, inf = solve(op, prec, rtol)
        step = t_asm + inf["solve_ms"]
        e = op.error_norms(x, L.FG_FN_SHARP_WAVE, SHARP)
        out[prec] = {"iterations": inf["iterations"], "solve_ms": inf["solve_ms"],
                     "ms_per_iteration": inf["solve_ms"] / max(inf["iterations"], 1), "step_ms": step,
                     "dof_per_s": sp.num_free_dofs / (step * 1e-3), "converged": inf["converged"],
                     "l2_error": e["l2_norm"], "h1_semi_error": e["h1_seminorm"]}
    op.close()
    sp.close()
    if cg:
        spc = SerialFESpace(tri, order=order, dirichlet_ids=list(range(1, 27)))
        opc = FEAffineOperator(spc, integ).compute()
        x, inf = solve(opc, "fp64", rtol)
        e = opc.error_norms(x, L.FG_FN_SHARP_WAVE, SHARP)
        out["cg_fp64"] = {"dofs": spc.num_free_dofs, "iterations": inf["iterations"], "solve_ms": inf["solve_ms"],
                          "l2_error": e["l2_norm"], "h1_semi_error": e["h1_seminorm"]}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=48)
    ap.add_argument("--order", type=int, default=2)
    ap.add_argument("--no-cg", action="store_true")
    a = ap.parse_args()
    print(json.dumps(run(a.n, a.order, cg=not a.no_cg)))


if __name__ == "__main__":
    main()

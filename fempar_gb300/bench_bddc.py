"""BDDC benchmark: linear elasticity, Q2, box subdomains (``python -m fempar_gb300.bench_bddc``).

Workload (seeded, synthetic): unit cube, n^3 hexahedra with interior vertices perturbed by
U(-0.15h, 0.15h) per component, Q2 elements, Young's modulus lognormal(sigma=1.5) per cell,
nu = 0.3, clamped at x = 0, body force (0,0,-1); nsub^3 box subdomains (corner + edge coarse
space; diagonal-stiffness weights unless --multiplicity; --faces adds face averages).  One step = numerical assembly + BDDC numerical setup + PCG
to ||r|| <= 1e-8 ||b||, once with the FP64 preconditioner and once with its FP32 copy
(FP64 Krylov vectors either way).  Beside it, Jacobi-PCG (FP64 and mixed) on the same system.

Prints one JSON line: dofs, partition sizes, per-stage times, iterations, DOF/s, the error
of each solution against the FP64 BDDC one, and the batched Cholesky's FP64 rate.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import _lib as L
from .fe import (MLBDDC, Context, ElasticityIntegration, FEAffineOperator, IterativeLinearSolver, SerialFESpace,
                 SerialTriangulation, bddc_cuts)

SEED = 20261203
CLAMP_X0_IDS = [1, 3, 5, 7, 13, 15, 17, 19, 25]


def perturbed_vertices(n, frac, rng):
    h = 1.0 / n
    K, J, I = np.meshgrid(np.arange(n + 1), np.arange(n + 1), np.arange(n + 1), indexing="ij")
    I, J, K = I.ravel(), J.ravel(), K.ravel()
    xyz = np.stack([I * h, J * h, K * h], axis=1)
    interior = (I > 0) & (I < n) & (J > 0) & (J < n) & (K > 0) & (K < n)
    xyz[interior] += rng.uniform(-frac * h, frac * h, size=xyz.shape)[interior]
    return xyz.ravel()


def run_jacobi_only(n, rtol=1e-8, device=0, precisions=("mixed",)):
    """The same elasticity problem with Jacobi-PCG only, assembled lean (fits 96^3 Q2, the
    size at which dense subdomain factors do not fit)."""
    rng = np.random.Generator(np.random.PCG64(SEED))
    xyz = perturbed_vertices(n, 0.15, rng)
    E = np.exp(rng.normal(0.0, 1.5, size=n ** 3))
    ctx = Context(device)
    t0 = time.perf_counter()
    tri = SerialTriangulation(ctx, (n, n, n), vertex_xyz=xyz)
    sp = SerialFESpace(tri, order=2, ncomp=3, dirichlet_ids=CLAMP_X0_IDS)
    t_sym = (time.perf_counter() - t0) * 1e3
    integ = ElasticityIntegration(cell_coef=E, nu=0.3, source_fn=L.FG_FN_CONST, fn_param=[0.0, 0.0, -1.0])
    t0 = time.perf_counter()
    op = FEAffineOperator(sp, integ, lean=True).compute()
    t_asm = (time.perf_counter() - t0) * 1e3
    out = {"metric": "elasticity Q2: DOF/s to 1e-8 (assembly + Jacobi-PCG)", "n": n, "dofs": sp.num_free_dofs,
           "nnz_full": sp.info.nnz_full, "symbolic_ms": t_sym, "assembly_ms": t_asm,
           "device_gb_after_assembly": ctx.memory()[0] / 1e9}
    for prec in precisions:
        s = IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
        s.set_parameters_from_pl({"ILS_RTOL": rtol, "ILS_MAX_NUM_ITERATIONS": 400000, "PRECISION": prec})
        s.solve()
        inf = s.info()
        total = t_asm + inf["solve_ms"]
        out["jacobi_" + prec] = {"iterations": inf["iterations"], "outer_iterations": inf["outer_iterations"],
                                 "converged": inf["converged"], "solve_ms": inf["solve_ms"], "step_ms": total,
                                 "dof_per_s": sp.num_free_dofs / (total * 1e-3),
                                 "ms_per_iteration": inf["solve_ms"] / max(inf["iterations"], 1)}
    return out


def run(n=32, nsub=8, jitter=0.0, rtol=1e-8, device=0, faces=False, weighting=L.FG_BDDC_WEIGHT_MULTIPLICITY,
        jacobi=True, handler=L.FG_BDDC_HANDLER_STANDARD):
    rng = np.random.Generator(np.random.PCG64(SEED))
    xyz = perturbed_vertices(n, 0.15, rng)
    E = np.exp(rng.normal(0.0, 1.5, size=n ** 3))
    ctx = Context(device)
    tri = SerialTriangulation(ctx, (n, n, n), vertex_xyz=xyz)
    sp = SerialFESpace(tri, order=2, ncomp=3, dirichlet_ids=CLAMP_X0_IDS)
    integ = ElasticityIntegration(cell_coef=E, nu=0.3, source_fn=L.FG_FN_CONST, fn_param=[0.0, 0.0, -1.0])
    op = FEAffineOperator(sp, integ).compute()
    t0 = time.perf_counter()
    op.compute()  # numerical re-assembly, timed
    t_asm = (time.perf_counter() - t0) * 1e3
    cuts = bddc_cuts((n, n, n), (nsub, nsub, nsub), jitter=jitter, seed=SEED)
    t0 = time.perf_counter()
    rigid = handler == L.FG_BDDC_HANDLER_ELASTICITY
    M = MLBDDC(op, nsub=(nsub,) * 3, cuts=cuts, use_edges=not rigid, use_faces=faces, weighting=weighting,
               coarse_handler=handler)
    t_create = (time.perf_counter() - t0) * 1e3
    info = M.info()
    t0 = time.perf_counter()
    M.numerical_setup()
    t_num = (time.perf_counter() - t0) * 1e3
    out = {"metric": "BDDC elasticity Q2: DOF/s to 1e-8 (assembly + BDDC numerical setup + PCG)",
           "n": n, "nsub": [nsub] * 3, "jitter": jitter, "faces": faces,
           "coarse_handler": "elasticity (vertices + rigid-body face functionals)" if rigid
           else "standard (vertices + edge/face averages)",
           "weighting": "stiffness" if weighting == L.FG_BDDC_WEIGHT_STIFFNESS else "multiplicity",
           "dofs": sp.num_free_dofs,
           "max_local_dofs": info["max_local_dofs"], "coarse_dofs": info["num_coarse_dofs"],
           "interface_dofs": info["num_interface_dofs"], "bddc_device_gb": info["device_bytes"] / 1e9,
           "assembly_ms": t_asm, "bddc_create_ms": t_create, "bddc_symbolic_ms": info["symbolic_ms"],
           "bddc_numeric_ms": t_num}
    info = M.info()
    out["subdomain_cholesky"] = {"fp64_gflop": info["factor_flops"] / 1e9, "ms": info["factor_ms"],
                                 "fp64_tflops": info["factor_flops"] / (info["factor_ms"] * 1e-3) / 1e12}
    out["coarse_setup_ms"] = info["coarse_ms"]
    sols = {}
    runs = [("bddc_fp64", "fp64", M), ("bddc_mixed", "mixed", M)]
    if jacobi:
        runs += [("jacobi_mixed", "mixed", "jacobi"), ("jacobi_fp64", "fp64", "jacobi")]
    for name, prec, M_ in runs:
        s = IterativeLinearSolver().set_type_from_string("CG").set_operators(op, M_)
        s.set_parameters_from_pl({"ILS_RTOL": rtol, "PRECISION": prec,
                                  "ILS_MAX_NUM_ITERATIONS": 5000 if name.startswith("bddc") else 200000})
        t0 = time.perf_counter()
        x = s.solve()
        wall = (time.perf_counter() - t0) * 1e3
        inf = s.info()
        sols[name] = x
        total = t_asm + (t_num if name.startswith("bddc") else 0.0) + inf["solve_ms"]
        out[name] = {"iterations": inf["iterations"], "outer_iterations": inf["outer_iterations"],
                     "converged": inf["converged"], "solve_ms": inf["solve_ms"], "solve_wall_ms": wall,
                     "step_ms": total, "dof_per_s": sp.num_free_dofs / (total * 1e-3)}
    ref = sols["bddc_fp64"]
    for name, x in sols.items():
        out[name]["rel_err_vs_bddc_fp64"] = float(np.linalg.norm(x - ref) / np.linalg.norm(ref))
    out["clocks_note"] = "host wall times around synchronous library calls; solve_ms from CUDA events"
    M.close()
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--n", type=int, default=32)
    ap.add_argument("--nsub", type=int, default=8)
    ap.add_argument("--jitter", type=float, default=0.0)
    ap.add_argument("--faces", action="store_true")
    ap.add_argument("--multiplicity", action="store_true",
                    help="1/(subdomains around) weights (the reference's standard handler); "
                         "default: diag(A_i)/sum diag(A_j)")
    ap.add_argument("--elasticity-handler", action="store_true",
                    help="the reference's elasticity coarse handler: vertices and six rigid-body "
                         "functionals per face, no edge constraints (implies --faces)")
    ap.add_argument("--no-jacobi", action="store_true")
    ap.add_argument("--jacobi-only", action="store_true",
                    help="no BDDC: lean assembly + mixed Jacobi-PCG (e.g. --n 96, the cfg size)")
    args = ap.parse_args()
    from . import build
    build.build()
    if args.jacobi_only:
        print(json.dumps(run_jacobi_only(args.n)), flush=True)
        return
    wt = L.FG_BDDC_WEIGHT_MULTIPLICITY if args.multiplicity else L.FG_BDDC_WEIGHT_STIFFNESS
    handler = L.FG_BDDC_HANDLER_ELASTICITY if args.elasticity_handler else L.FG_BDDC_HANDLER_STANDARD
    print(json.dumps(run(args.n, args.nsub, args.jitter, faces=args.faces or args.elasticity_handler, weighting=wt,
                         jacobi=not args.no_jacobi, handler=handler)), flush=True)


if __name__ == "__main__":
    main()

"""Numeric assembly time of Poisson Q2 on an n^3 mesh for each way of forming the element
matrices (``python -m fempar_gb300.bench_assembly --n 128``).

Modes (FG_TC_INTEGRATION with the integrand's precision request):
  fp64_pipe        FP64 integration kernel (k_integrate_poisson<P, false>)
  float_float      float-float integration kernel (k_integrate_poisson<P, true>)
  tensor_core_fp64 one emulated-FP64 tcgen05 product of the cells' geometric factors with the
                   shared reference-gradient table (k_poisson_geom, k_oz_gemm, k_poisson_unpack):
                   the FP64 request's default
  tensor_core      the same with the geometric factors in float-float (k_poisson_geom_ff): the
                   fast request's default (the mixed solver's)
Each assembly includes the row gather into the solver layout.  The mesh is the unit cube with
interior vertices moved by U(+-0.15 h) and k = exp(N(0,1)) per cell, f = 1, u = 0 on the
boundary (seeded).  Times are CUDA events on the library's stream, the minimum of --reps
after one warm-up assembly.  Up to 64^3 the matrices are also compared with the FP64-pipe
kernel's (largest difference over each row's largest entry).  Prints one JSON line.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os

import numpy as np

SEED = 20261203


def workload(n: int, seed: int = SEED):
    rng = np.random.Generator(np.random.PCG64(seed))
    h = 1.0 / n
    k, j, i = np.meshgrid(np.arange(n + 1), np.arange(n + 1), np.arange(n + 1), indexing="ij")
    xyz = np.stack([i * h, j * h, k * h], axis=-1).reshape(-1, 3)
    ii, jj, kk = i.ravel(), j.ravel(), k.ravel()
    inner = (ii > 0) & (ii < n) & (jj > 0) & (jj < n) & (kk > 0) & (kk < n)
    d = rng.uniform(-0.15 * h, 0.15 * h, size=xyz.shape)
    xyz[inner] += d[inner]
    return np.ascontiguousarray(xyz.ravel()), np.exp(rng.normal(0.0, 1.0, size=n ** 3))


MODES = {"fp64_pipe": ("0", False), "float_float": ("0", True), "tensor_core_fp64": ("2", False),
         "tensor_core": ("2", True)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--modes", default="fp64_pipe,float_float,tensor_core_fp64,tensor_core")
    args = ap.parse_args()
    import torch
    import fempar_gb300 as fg
    from fempar_gb300 import _lib as L

    xyz, coef = workload(args.n)
    ctx = fg.Context(0)
    sp_ptr = C.c_void_p()
    L.lib().fg_ctx_get_stream(ctx.h, C.byref(sp_ptr))
    stream = torch.cuda.ExternalStream(sp_ptr.value, device="cuda:0")
    tri = fg.SerialTriangulation(ctx, [args.n] * 3, vertex_xyz=xyz)
    space = fg.SerialFESpace(tri, order=2, dirichlet_ids=fg.ALL_BOUNDARY_IDS)
    coef_dev = torch.from_numpy(coef).to("cuda:0")
    out = {"n": args.n, "num_cells": args.n ** 3, "num_free_dofs": space.num_free_dofs}
    op, ref = None, None
    for name in args.modes.split(","):
        env, fast = MODES[name]
        os.environ["FG_TC_INTEGRATION"] = env
        integ = fg.PoissonIntegration(cell_coef=coef_dev, source_fn=fg.FG_FN_CONST, fn_param=[1.0],
                                      fast_integration=fast)
        if op is None:
            op = fg.FEAffineOperator(space, integ)
        op.integration = integ
        op.compute()
        ts = []
        for _ in range(args.reps):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            op.compute()
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        out[name + "_ms"] = min(ts)
        if args.n <= 64:
            irp, ja, val = op.get_matrix(symmetric_storage=True, one_based=False)
            if name == "fp64_pipe":
                ref = (irp, val)
            elif ref is not None:
                rows = np.repeat(np.arange(len(irp) - 1), np.diff(irp))
                scale = np.zeros(len(irp) - 1)
                np.maximum.at(scale, rows, np.abs(ref[1]))
                out[name + "_max_diff_rowscaled"] = float((np.abs(val - ref[1]) / scale[rows]).max())
    os.environ.pop("FG_TC_INTEGRATION", None)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()

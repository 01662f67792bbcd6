"""Dense FP64 products on the bf16 tensor cores (``fg_dense_gemm_nt``) and their benchmark.

``gemm_nt(ctx, A, B, C, alpha, beta, lower)`` computes C = alpha A B^T + beta C on float64
CUDA tensors of any strides (B None: B = A).  FP64 is emulated by seven signed 8-bit digits
per value and row on tcgen05 (Ozaki scheme), the building block of the BDDC set-up's dense
factorisations.

``python -m fempar_gb300.dense`` times it against the FP64 pipe (torch.matmul on float64,
i.e. cuBLAS DGEMM) on a square product and on rank-128 updates (the shape of a blocked
Cholesky factorisation's trailing updates), and reports the largest difference from DGEMM
per element, relative to k max_l |A_il| max_l |B_jl|.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json

from . import _lib as L


def gemm_nt(ctx, A, B=None, Cm=None, alpha=1.0, beta=0.0, lower=False):
    """C = alpha A B^T + beta C (float64 CUDA tensors); returns C (allocated if None)."""
    import torch
    m, k = A.shape
    n = m if B is None else B.shape[0]
    if B is not None and B.shape[1] != k:
        raise ValueError("A and B need the same number of columns")
    if Cm is None:
        Cm = torch.zeros((m, n), dtype=torch.float64, device=A.device)
        beta = 0.0
    for t in (A, B, Cm):
        if t is not None and (t.dtype != torch.float64 or not t.is_cuda):
            raise TypeError("float64 CUDA tensors expected")
    torch.cuda.synchronize(A.device)
    bp = C.c_void_p(B.data_ptr()) if B is not None else None
    bs = B.stride() if B is not None else (0, 0)
    L.check(L.lib().fg_dense_gemm_nt(ctx.h, m, n, k, float(alpha), C.c_void_p(A.data_ptr()), A.stride(0),
                                     A.stride(1), bp, bs[0], bs[1], float(beta), C.c_void_p(Cm.data_ptr()),
                                     Cm.stride(0), Cm.stride(1), L.FG_DENSE_LOWER if lower else 0),
            "fg_dense_gemm_nt")
    return Cm


def _time(fn, reps):
    import torch
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def benchmark(ctx, sizes=((4096, 4096, 4096), (8192, 8192, 128), (16384, 16384, 128)), reps=5, seed=7):
    import torch
    dev = f"cuda:{ctx.device}"
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    out = []
    for m, n, k in sizes:
        A = torch.randn((m, k), dtype=torch.float64, device=dev, generator=g)
        B = torch.randn((n, k), dtype=torch.float64, device=dev, generator=g)
        Cm = torch.empty((m, n), dtype=torch.float64, device=dev)
        flops = 2.0 * m * n * k
        t_oz = _time(lambda: gemm_nt(ctx, A, B, Cm), reps)
        t_64 = _time(lambda: torch.matmul(A, B.T, out=Cm), reps)
        ref = torch.matmul(A, B.T)
        X = gemm_nt(ctx, A, B)
        # error against cuBLAS DGEMM, per element relative to |A_i||B_j| (the dot-product scale)
        scale = torch.outer(A.abs().max(dim=1).values, B.abs().max(dim=1).values) * k
        err = float(((X - ref).abs() / scale).max())
        out.append({"m": m, "n": n, "k": k, "emulated_ms": t_oz, "emulated_tflops": flops / t_oz / 1e9,
                    "dgemm_ms": t_64, "dgemm_tflops": flops / t_64 / 1e9, "speedup": t_64 / t_oz,
                    "max_err_vs_dgemm_rel_to_k_max_max": err})
        del A, B, Cm, ref, X
        torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--reps", type=int, default=5)
    args = ap.parse_args()
    from . import Context
    ctx = Context(0)
    for r in benchmark(ctx, reps=args.reps):
        print(json.dumps(r), flush=True)


if __name__ == "__main__":
    main()

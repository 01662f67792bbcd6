"""Dense FP64 products on the bf16 tensor cores (fg_dense_gemm_nt, digit slicing on tcgen05)
against cuBLAS DGEMM (torch.matmul on float64).

* integer inputs whose rows need one digit: the product is exact, so it equals DGEMM bit for
  bit (ragged tiles, several K chunks);
* normal inputs: every element within 1e-13 k max|A_i.| max|B_j.| of DGEMM (the FP64
  dot-product scale), for row-major and column-major operands, alpha, beta;
* rows scaled by powers of two from 2^-60 to 2^60 (per-row exponents);
* the lower-triangle flag writes nothing above the diagonal; B = NULL is A A^T, e.g. the
  trailing update of a column-major Cholesky panel;
* k = 0 gives beta C;
* a bounded wait that runs out (test switch) returns FG_ERR_TIMEOUT and leaves the context
  usable.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fempar_gb300 as fg
    from fempar_gb300 import build
    build.build()
    return fg, fg.Context(0), torch


def scaled_err(X, ref, A, B, k):
    scale = np.outer(np.abs(A).max(axis=1), np.abs(B).max(axis=1)) * max(k, 1)
    scale[scale == 0] = 1.0
    return float((np.abs(X - ref) / scale).max())


def test_integer_inputs_exact(env):
    fg, ctx, torch = env
    from fempar_gb300.dense import gemm_nt
    rng = np.random.default_rng(1)
    m, n, k = 200, 130, 300
    A = rng.integers(-100, 101, size=(m, k)).astype(np.float64)
    B = rng.integers(-100, 101, size=(n, k)).astype(np.float64)
    dA, dB = torch.tensor(A, device="cuda"), torch.tensor(B, device="cuda")
    X = gemm_nt(ctx, dA, dB).cpu().numpy()
    assert np.array_equal(X, A @ B.T)


@pytest.mark.parametrize("m,n,k,colmajor", [(128, 64, 128, False), (300, 257, 1000, False), (517, 190, 129, True),
                                            (64, 1000, 40, True)])
def test_normal_inputs_against_dgemm(env, m, n, k, colmajor):
    fg, ctx, torch = env
    from fempar_gb300.dense import gemm_nt
    g = torch.Generator(device="cuda")
    g.manual_seed(m * 7 + n)
    if colmajor:
        dA = torch.randn((k, m), dtype=torch.float64, device="cuda", generator=g).T
        dB = torch.randn((k, n), dtype=torch.float64, device="cuda", generator=g).T
    else:
        dA = torch.randn((m, k), dtype=torch.float64, device="cuda", generator=g)
        dB = torch.randn((n, k), dtype=torch.float64, device="cuda", generator=g)
    C0 = torch.randn((m, n), dtype=torch.float64, device="cuda", generator=g)
    Cm = C0.clone()
    gemm_nt(ctx, dA, dB, Cm, alpha=-0.75, beta=1.5)
    ref = -0.75 * (dA @ dB.T) + 1.5 * C0
    A, B = dA.cpu().numpy(), dB.cpu().numpy()
    err = scaled_err(Cm.cpu().numpy(), ref.cpu().numpy(), A, B, k)
    assert err <= TOL, err


def test_row_scales_over_120_binades(env):
    fg, ctx, torch = env
    from fempar_gb300.dense import gemm_nt
    rng = np.random.default_rng(3)
    m, n, k = 256, 192, 256
    A = rng.normal(size=(m, k)) * np.ldexp(1.0, rng.integers(-60, 61, size=m))[:, None]
    B = rng.normal(size=(n, k)) * np.ldexp(1.0, rng.integers(-60, 61, size=n))[:, None]
    dA, dB = torch.tensor(A, device="cuda"), torch.tensor(B, device="cuda")
    X = gemm_nt(ctx, dA, dB).cpu().numpy()
    ref = (dA @ dB.T).cpu().numpy()
    assert scaled_err(X, ref, A, B, k) <= TOL


def test_lower_syrk_of_a_cholesky_panel(env):
    """C[j1:, j1:] -= P P^T (lower) with P = M[j1:, j0:j1] of a column-major matrix."""
    fg, ctx, torch = env
    from fempar_gb300.dense import gemm_nt
    N, j0, j1 = 700, 100, 228
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    Mt = torch.randn((N, N), dtype=torch.float64, device="cuda", generator=g)  # Mt[c, r] = M[r, c]
    M = Mt.T                                                                     # column-major view
    before = M.clone()
    P = M[j1:, j0:j1]
    Cv = M[j1:, j1:]
    ref = (before[j1:, j1:] - P @ P.T).cpu().numpy()
    gemm_nt(ctx, P, None, Cv, alpha=-1.0, beta=1.0, lower=True)
    X = M[j1:, j1:].cpu().numpy()
    Pn = P.cpu().numpy()
    low = np.tril(np.ones_like(X, dtype=bool))
    err = scaled_err(np.where(low, X, 0), np.where(low, ref, 0), Pn, Pn, j1 - j0)
    assert err <= TOL, err
    assert np.array_equal(X[~low], before[j1:, j1:].cpu().numpy()[~low]), "wrote above the diagonal"
    assert torch.equal(M[:, :j1], before[:, :j1]) and torch.equal(M[:j1, :], before[:j1, :])


def test_k_zero_scales_c(env):
    fg, ctx, torch = env
    from fempar_gb300.dense import gemm_nt
    A = torch.zeros((70, 0), dtype=torch.float64, device="cuda")
    B = torch.zeros((50, 0), dtype=torch.float64, device="cuda")
    C0 = torch.randn((70, 50), dtype=torch.float64, device="cuda")
    Cm = C0.clone()
    gemm_nt(ctx, A, B, Cm, alpha=1.0, beta=2.0)
    assert torch.equal(Cm, 2.0 * C0)


def test_bounded_wait_runs_out_and_context_survives(env, monkeypatch):
    """Failure detection without a GPU fault: CTA 0 never issues the copies of its third stage
    (test switch), its bounded wait runs out after ~1 s, the call returns FG_ERR_TIMEOUT after
    draining what is in flight, and the same context then computes the product correctly."""
    fg, ctx, torch = env
    from fempar_gb300 import FGError
    from fempar_gb300.dense import gemm_nt
    A = torch.randn((256, 256), dtype=torch.float64, device="cuda")
    B = torch.randn((192, 256), dtype=torch.float64, device="cuda")
    monkeypatch.setenv("FG_OZ_TEST_DROP_STAGE", "2")
    with pytest.raises(FGError) as ei:
        gemm_nt(ctx, A, B)
    assert "FG_ERR_TIMEOUT" in str(ei.value)
    monkeypatch.delenv("FG_OZ_TEST_DROP_STAGE")
    X = gemm_nt(ctx, A, B).cpu().numpy()
    ref = (A @ B.T).cpu().numpy()
    assert scaled_err(X, ref, A.cpu().numpy(), B.cpu().numpy(), 256) <= TOL

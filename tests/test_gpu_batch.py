"""Batched persistent Poisson solves (fg_batch_* through the C-ABI) against the oracle.

Bar: every problem's solution within 1e-8 (relative 2-norm) of the oracle's FP64 Jacobi-CG
solution at rtol 1e-13, with the batch solved to rtol 1e-10; a multi-CTA team problem within
1e-8 of the general FP64 device path; bitwise equal results run to run and between host and
device input modes of the same plan.
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fg():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fempar_gb300 as fg
    from fempar_gb300 import build
    build.build()
    return fg


@pytest.fixture(scope="module")
def ctx(fg):
    return fg.Context(0)


def small_set(seed=5):
    rng = np.random.default_rng(seed)
    out = []
    for n, p in [(2, 1), (3, 1), (5, 1), (2, 2), (3, 2), (4, 2), (2, 3), (3, 3), (1, 3), (4, 1), (1, 1)]:
        out.append({"n": n, "order": p, "coef": float(rng.uniform(0.1, 10.0)),
                    "qp_source": rng.normal(size=n ** 3 * (p + 1) ** 3),
                    "x": np.zeros(max(p * n - 1, 0) ** 3)})
    return out


def oracle_solution(q):
    n, p = q["n"], q["order"]
    P = O.Problem((n, n, n), order=p, cell_coef=np.full(n ** 3, q["coef"]), source_fn=O.FN_QP_VALUES,
                  qp_source=q["qp_source"])
    if P.nfree == 0:
        return np.zeros(0)
    ref = P.cg(precond=1, rtol=1e-13, maxit=100000)
    from fempar_gb300.batch import lattice_index_map
    idx = lattice_index_map(P.dof_map(), n, p)
    return ref["x"][idx]


def test_batch_matches_oracle(fg, ctx):
    from fempar_gb300.batch import BatchSolver
    probs = small_set()
    B = BatchSolver(ctx, probs, rtol=1e-10, threads=256)
    res = B.run()
    assert all(r["status"] == 0 for r in res)
    for q, r in zip(probs, res):
        xo = oracle_solution(q)
        if xo.size == 0:
            continue
        err = np.linalg.norm(q["x"] - xo) / np.linalg.norm(xo)
        assert err <= 1e-8, (q["n"], q["order"], err)
        assert r["rel_residual"] <= 1e-10
    x1 = [q["x"].copy() for q in probs]
    B.run()
    for a, q in zip(x1, probs):
        assert np.array_equal(a, q["x"])
    B.close()


def test_batch_device_inputs_and_teams(fg, ctx):
    """One large problem among small ones gets a multi-CTA team; device inputs give the same
    bits as host inputs under the same plan."""
    import torch
    from fempar_gb300.batch import BatchSolver
    rng = np.random.default_rng(9)
    probs = small_set(seed=7)
    big = {"n": 20, "order": 3, "coef": 2.5, "qp_source": rng.normal(size=20 ** 3 * 64), "x": np.zeros(59 ** 3)}
    probs.append(big)
    B = BatchSolver(ctx, probs, rtol=1e-10, threads=256)
    res = B.run()
    info = B.info()
    assert res[-1]["team"] > 1 and info["teams_gt1"] >= 1
    assert all(r["status"] == 0 for r in res)
    # the team problem against the general FP64 device path (assembled CSR, Jacobi-CG)
    tri = fg.SerialTriangulation(ctx, (20, 20, 20))
    sp = fg.SerialFESpace(tri, order=3, dirichlet_ids=list(range(1, 27)))
    op = fg.FEAffineOperator(sp, fg.PoissonIntegration(coef_const=2.5, source_fn=fg.FG_FN_QP_VALUES,
                                                       qp_source=big["qp_source"])).compute()
    s = fg.IterativeLinearSolver().set_type_from_string("CG").set_operators(op, "jacobi")
    s.set_parameters_from_pl({"ILS_RTOL": 1e-12, "ILS_MAX_NUM_ITERATIONS": 100000})
    x64 = s.solve()
    dm = sp.get_dof_map()
    n, p, F = 20, 3, 59
    idx = np.full(F ** 3, -1, dtype=np.int64)
    for c in range(n ** 3):
        ci, cj, ck = c % n, (c // n) % n, c // (n * n)
        for a in range(64):
            g = dm[c, a]
            if g > 0:
                ai, aj, ak = a % 4, (a // 4) % 4, a // 16
                idx[(p * ci + ai - 1) + F * ((p * cj + aj - 1) + F * (p * ck + ak - 1))] = g - 1
    err = np.linalg.norm(big["x"] - x64[idx]) / np.linalg.norm(x64)
    assert err <= 1e-8, err
    # device mode, same plan parameters
    dprobs = [{"n": q["n"], "order": q["order"], "coef": q["coef"],
               "qp_source": torch.tensor(q["qp_source"], device="cuda:0"),
               "x": torch.zeros(q["x"].size, dtype=torch.float64, device="cuda:0")} for q in probs]
    D = BatchSolver(ctx, dprobs, rtol=1e-10, threads=256)
    D.run()
    for q, d in zip(probs, dprobs):
        assert np.array_equal(q["x"], d["x"].cpu().numpy())
    B.close()
    D.close()


def test_batch_reports_non_convergence_and_bad_input(fg, ctx):
    from fempar_gb300 import FGError
    from fempar_gb300.batch import BatchSolver
    probs = small_set()[:3]
    B = BatchSolver(ctx, probs, rtol=1e-12, max_iters=2, threads=128)
    res = B.run(raise_on_error=False)
    assert any(r["status"] == -4 for r in res)
    with pytest.raises(FGError):
        B.run()
    bad = [{"n": 2, "order": 4, "coef": 1.0, "qp_source": np.zeros(8 * 125), "x": np.zeros(343)}]
    with pytest.raises(FGError):
        BatchSolver(ctx, bad)


def test_batch_autotune_picks_a_block_size(fg, ctx, monkeypatch):
    from fempar_gb300.batch import BatchSolver
    probs = small_set(seed=11)
    B = BatchSolver(ctx, probs, rtol=1e-8, threads=0)
    info = B.info()
    assert info["threads"] in (128, 256, 512) and info["autotune_ms"] > 0 and info["team_share"] == 0.5
    res = B.run()
    assert all(r["status"] == 0 for r in res)
    # team sizing from the environment: more and larger teams at 0.25, same convergence
    monkeypatch.setenv("FG_BATCH_TEAM_SHARE", "0.25")
    B2 = BatchSolver(ctx, probs, rtol=1e-8, threads=256)
    assert B2.info()["team_share"] == 0.25
    assert all(r["status"] == 0 for r in B2.run())


def test_batch_bounded_team_wait_runs_out_and_context_survives(fg, ctx, monkeypatch):
    """Failure detection without a GPU fault: one member of every multi-CTA team skips its
    first barrier arrival (test switch), the team waits run out after 200 ms, the run reports
    FG_ERR_TIMEOUT, and the same context then solves normally."""
    import time
    from fempar_gb300 import FGError
    from fempar_gb300.batch import BatchSolver
    rng = np.random.default_rng(9)

    def problems():
        ps = small_set(seed=7)
        ps.append({"n": 20, "order": 3, "coef": 2.5, "qp_source": rng.normal(size=20 ** 3 * 64),
                   "x": np.zeros(59 ** 3)})
        return ps

    monkeypatch.setenv("FG_BATCH_BARRIER_TIMEOUT_MS", "200")
    monkeypatch.setenv("FG_BATCH_TEST_DROP_ARRIVAL", "1")
    B = BatchSolver(ctx, problems(), rtol=1e-10, threads=256)
    t0 = time.perf_counter()
    res = B.run(raise_on_error=False)
    assert time.perf_counter() - t0 < 30.0
    assert res[-1]["team"] > 1 and res[-1]["status"] == -6  # FG_ERR_TIMEOUT
    with pytest.raises(FGError):
        B.run()
    B.close()
    monkeypatch.delenv("FG_BATCH_TEST_DROP_ARRIVAL")
    monkeypatch.delenv("FG_BATCH_BARRIER_TIMEOUT_MS")
    ps = problems()
    C = BatchSolver(ctx, ps, rtol=1e-10, threads=256)
    res = C.run()
    assert all(r["status"] == 0 for r in res)
    xo = oracle_solution(ps[2])
    assert np.linalg.norm(ps[2]["x"] - xo) <= 1e-8 * np.linalg.norm(xo)
    C.close()

"""Serving loop on the GPU: concurrent requests give the same solutions as the same requests
run alone, and a served solution matches the CPU oracle."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fempar_gb300 import build, serving
    build.build()
    return serving


def _mix():
    rng = np.random.default_rng(5)
    reqs = []
    for i in range(8):
        kind = [0, 1][i % 2]
        n = [4, 6, 5, 7, 3, 6, 8, 5][i]
        order = [1, 2][(i // 2) % 2]
        reqs.append({"kind": kind, "n": (n, n, n), "order": order,
                     "cell_coef": np.exp(rng.normal(0.0, 1.0, size=n ** 3)), "rtol": 1e-10})
    return reqs


def test_results_same_alone_and_in_the_mix(S):
    reqs = _mix()
    alone = []
    srv1 = S.Server(nworkers=1)
    for rq in reqs:
        t = srv1.submit(**rq)
        r = srv1.wait(t)
        assert r["status"] == 0
        alone.append(srv1.take(t, r["num_free"]))
    srv1.close()
    srv = S.Server(nworkers=4)
    tickets = [srv.submit(**rq) for rq in reqs]
    mixed = []
    for t in tickets:
        r = srv.wait(t)
        assert r["status"] == 0 and r["t_total_ms"] >= r["t_run_ms"] > 0
        mixed.append(srv.take(t, r["num_free"]))
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs)
    for a, m in zip(alone, mixed):
        # same kernels, fixed grids and reduction orders: identical bits
        assert np.array_equal(a, m)


def test_served_solution_matches_oracle(S):
    n = (5, 4, 6)
    coef = np.exp(np.random.default_rng(2).normal(0.0, 1.0, size=n[0] * n[1] * n[2]))
    srv = S.Server(nworkers=2)
    t = srv.submit(kind=S.POISSON, n=n, order=2, cell_coef=coef, rtol=1e-12)
    r = srv.wait(t)
    x = srv.take(t, r["num_free"])
    srv.close()
    P = O.Problem(n, order=2, cell_coef=coef, source_fn=O.FN_CONST, fn_param=[1.0])
    ref = P.cg(precond=1, rtol=1e-13, maxit=20000)
    assert np.linalg.norm(x - ref["x"]) / np.linalg.norm(ref["x"]) <= 1e-9


def test_every_request_of_the_mix_matches_oracle(S):
    """Per-request error against the oracle: the Poisson and elasticity requests of the mix
    (Q1/Q2, lognormal coefficients, mixed precision to 1e-10), served concurrently, each within
    1e-8 of the oracle's FP64 solution of the same request (rtol 1e-13)."""
    reqs = _mix()
    srv = S.Server(nworkers=4)
    tickets = [srv.submit(**rq) for rq in reqs]
    sols = []
    for t in tickets:
        r = srv.wait(t)
        assert r["status"] == 0
        sols.append(srv.take(t, r["num_free"]))
    srv.close()
    for rq, x in zip(reqs, sols):
        if rq["kind"] == S.ELASTICITY:
            P = O.Problem(rq["n"], order=rq["order"], kind=O.ELASTICITY, dirichlet_ids=S.CLAMP_X0_IDS,
                          cell_coef=rq["cell_coef"], nu=0.3, source_fn=O.FN_CONST, fn_param=[0.0, 0.0, -1.0])
        else:
            P = O.Problem(rq["n"], order=rq["order"], cell_coef=rq["cell_coef"], source_fn=O.FN_CONST, fn_param=[1.0])
        ref = P.cg(precond=1, rtol=1e-13, maxit=100000)
        err = np.linalg.norm(x - ref["x"]) / np.linalg.norm(ref["x"])
        assert err <= 1e-8, (rq["kind"], rq["n"], rq["order"], err)


def test_budget_refuses_oversized_request(S):
    from fempar_gb300 import FGError
    srv = S.Server(hbm_budget_bytes=64 << 20, nworkers=1)
    with pytest.raises(FGError):
        srv.submit(kind=S.POISSON, n=(40, 40, 40), order=2)
    srv.close()


def test_lean_system_solves_identically_and_refuses_exports(S):
    """FG_LEAN_SYSTEM (what served requests use): same solution bits as a full system,
    smaller resident memory, export and reassembly refused."""
    import numpy as np
    import fempar_gb300 as fg
    from fempar_gb300 import FGError
    ctx = fg.Context(0)
    n = (10, 9, 8)
    k = np.exp(np.random.default_rng(4).normal(size=n[0] * n[1] * n[2]))
    xs, mem = [], []
    for lean in (False, True):
        tri = fg.SerialTriangulation(ctx, n)
        sp = fg.SerialFESpace(tri, order=2, dirichlet_ids=list(range(1, 27)))
        op = fg.FEAffineOperator(sp, fg.PoissonIntegration(cell_coef=k, source_fn=fg.FG_FN_CONST, fn_param=[1.0]),
                                 lean=lean).compute()
        if lean:
            sp.release_pattern()
            with pytest.raises(FGError):
                op.get_matrix()
            with pytest.raises(FGError):
                op.compute()
        mem.append(ctx.memory()[0])
        s = fg.IterativeLinearSolver().set_type_from_string("GPU_MPCG").set_operators(op, "jacobi")
        s.set_parameters_from_pl({"ILS_RTOL": 1e-8, "ILS_MAX_NUM_ITERATIONS": 10000})
        xs.append(s.solve())
        op.close()
        sp.close()
        tri.close()
    assert np.array_equal(xs[0], xs[1])
    assert mem[1] < 0.7 * mem[0]

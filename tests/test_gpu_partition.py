"""Partitioned assembly on the device (fg_partition_*) against the oracle's restatement of
par_fe_space_t / dof_import_t.

Bar: every part's cells (local order), local-to-global map, weights and exchange lists
bit-exact; the subassembled matrices summed over the parts (through the local-to-global maps)
equal the global matrix to 1e-13 of the row max; comm of the subassembled rhs equals the global
rhs to 1e-13; the partitioned Jacobi-PCG solution equals the oracle's to 1e-10 (rtol 1e-13).
"""
import numpy as np
import pytest

import oracle as O
import partition as PT

pytestmark = pytest.mark.gpu
SHARP = [20.0, 0.3, -0.05, -0.05, -0.05]
CLAMP = [1, 3, 5, 7, 13, 15, 17, 19, 25]


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


def build_pair(fg, ctx, n, order, kind):
    rng = np.random.default_rng(sum(n) + order)
    coef = np.exp(rng.normal(size=int(np.prod(n))))
    tri = fg.SerialTriangulation(ctx, n)
    if kind == O.ELASTICITY:
        P = O.Problem(n, order=order, kind=O.ELASTICITY, dirichlet_ids=CLAMP, cell_coef=coef, source_fn=O.FN_CONST,
                      fn_param=[0.0, 0.0, -1.0])
        sp = fg.SerialFESpace(tri, order=order, ncomp=3, dirichlet_ids=CLAMP)
        integ = fg.ElasticityIntegration(cell_coef=coef, nu=0.3, source_fn=O.FN_CONST, fn_param=[0.0, 0.0, -1.0])
    else:
        P = O.Problem(n, order=order, cell_coef=coef, source_fn=O.FN_SHARP_WAVE, boundary_fn=O.FN_SHARP_WAVE,
                      fn_param=SHARP)
        sp = fg.SerialFESpace(tri, order=order, dirichlet_ids=list(range(1, 27)))
        integ = fg.PoissonIntegration(cell_coef=coef, source_fn=O.FN_SHARP_WAVE, boundary_fn=O.FN_SHARP_WAVE,
                                      fn_param=SHARP)
    return P, tri, sp, integ


@pytest.mark.parametrize("n,nparts,order,kind", [((4, 4, 2), (2, 2, 1), 1, O.POISSON),
                                                 ((4, 6, 4), (2, 3, 2), 2, O.POISSON),
                                                 ((6, 4, 4), (3, 2, 2), 3, O.POISSON),
                                                 ((4, 4, 4), (2, 2, 2), 1, O.ELASTICITY),
                                                 ((4, 2, 4), (2, 1, 2), 2, O.ELASTICITY),
                                                 ((3, 2, 2), (3, 2, 2), 1, O.POISSON),
                                                 ((3, 2, 1), (3, 2, 1), 2, O.POISSON)])
def test_partition_parity(fg, ctx, n, nparts, order, kind):
    import torch
    from fempar_gb300.partition import PartitionedFESpace
    P, tri, sp, integ = build_pair(fg, ctx, n, order, kind)
    parts = PT.build(P, nparts)
    ps = PartitionedFESpace(sp, nparts)
    assert ps.num_parts == len(parts)
    assert ps.num_local_dofs == sum(p["num_dofs"] for p in parts)
    offs = []
    for pid, o in enumerate(parts, start=1):
        d = ps.dof_import(pid)
        offs.append(d["first_local_dof"])
        assert (d["num_dofs"], d["num_interior"], d["num_interface"]) == (o["num_dofs"], o["num_interior"], o["num_interface"])
        assert np.array_equal(d["cells"], o["cells"])
        assert np.array_equal(d["l2g"], o["l2g"])
        assert np.array_equal(d["weight"], o["weight"])
        for k in ("list_rcv", "rcv_ptrs", "unpack_idx", "list_snd", "snd_ptrs", "pack_idx"):
            assert np.array_equal(d[k], np.asarray(o[k], dtype=np.int32)), k
    op = ps.assemble(integ)
    # subassembled matrices summed through the local-to-global maps = the global matrix
    rp, ci, v = op.get_matrix(symmetric_storage=False, one_based=False)
    l2g = np.concatenate([np.asarray(o["l2g"]) - 1 for o in parts])
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    G = {}
    for r, c, x in zip(l2g[rows], l2g[ci], v):
        G[(r, c)] = G.get((r, c), 0.0) + x
    orp, oci, ov = P.csr_full()
    orow = np.repeat(np.arange(P.nfree), np.diff(orp))
    scale = np.zeros(P.nfree)
    np.maximum.at(scale, orow, np.abs(ov))
    assert len(G) == len(ov)
    err = max(abs(G[(r, c)] - x) / scale[r] for r, c, x in zip(orow, oci, ov))
    assert err <= 1e-13, err
    # comm of the subassembled rhs
    b = torch.tensor(op.get_translation(), device="cuda:0")
    ps.comm_device(b)
    ob = P.rhs()
    assert np.max(np.abs(b.cpu().numpy() - ob[l2g])) <= 1e-13 * np.max(np.abs(ob))
    # partitioned PCG
    ref = P.cg(precond=1, rtol=1e-13, maxit=50000)
    x = op.solve(rtol=1e-13, max_iters=50000)
    assert op.last_info["converged"]
    assert np.linalg.norm(x - ref["x"]) <= 1e-10 * np.linalg.norm(ref["x"])
    assert abs(op.last_info["iterations"] - ref["iters"]) <= 2
    op.close()
    ps.close()


def test_partition_rejects_bad_splits(fg, ctx):
    from fempar_gb300 import FGError
    from fempar_gb300.partition import PartitionedFESpace
    tri = fg.SerialTriangulation(ctx, (4, 4, 3))
    sp = fg.SerialFESpace(tri, order=1, dirichlet_ids=list(range(1, 27)))
    with pytest.raises(FGError):
        PartitionedFESpace(sp, (2, 2, 2))   # 3 cells do not split in 2
    dsp = fg.SerialFESpace(tri, order=1, dg=True)
    with pytest.raises(FGError):
        PartitionedFESpace(dsp, (2, 1, 1))

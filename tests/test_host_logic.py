"""Host-side logic that needs no GPU: the serving footprint / dof-count model and the
no-device error path."""
import pytest

import oracle as O


@pytest.mark.parametrize("kind", ["poisson", "elasticity"])
@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("ids", ["all", "clamp", "faces", "none"])
def test_request_footprint_counts_free_dofs_like_the_oracle(kind, order, ids):
    from fempar_gb300 import build, serving as S
    build.build()
    dirichlet = {"all": S.ALL_BOUNDARY_IDS, "clamp": S.CLAMP_X0_IDS, "faces": [21, 24, 26], "none": []}[ids]
    k = S.ELASTICITY if kind == "elasticity" else S.POISSON
    for n in ((3, 4, 5), (2, 2, 2), (1, 3, 2)):
        b, nf = S.footprint(kind=k, n=n, order=order, dirichlet_ids=dirichlet)
        P = O.Problem(n, order=order, kind=O.ELASTICITY if k == S.ELASTICITY else O.POISSON, dirichlet_ids=dirichlet)
        assert nf == P.nfree
        assert b > 0


def test_footprint_grows_with_problem_size():
    from fempar_gb300 import build, serving as S
    build.build()
    small = S.footprint(kind=S.POISSON, n=(16, 16, 16), order=2)[0]
    big = S.footprint(kind=S.POISSON, n=(32, 32, 32), order=2)[0]
    assert 4 * small < big < 10 * small  # ~8x the data plus a fixed per-request reserve


@pytest.mark.parametrize("order", [1, 2, 3])
def test_footprint_covers_the_tensor_core_assembly_scratch(order):
    """A Poisson request is assembled with its element matrices on the tensor cores: the
    admission footprint must cover, besides the element matrices and vectors, the product's
    scratch per cell -- the 6 NQ geometric factors, the packed upper triangle and the 7 bf16
    digits of the factors (K padded to 16) -- and the shared table T."""
    import math
    from fempar_gb300 import build, serving as S
    build.build()
    n = (24, 20, 16)
    b, nf = S.footprint(kind=S.POISSON, n=n, order=order)
    ncells = n[0] * n[1] * n[2]
    nd = nq = (order + 1) ** 3
    K, npair = 6 * nq, nd * (nd + 1) // 2
    elm = ncells * (nd * nd + nd) * 8
    tc = ncells * (K * 8 + npair * 8 + math.ceil(K / 16) * 16 * 7 * 2) + npair * K * 8
    assert b >= elm + tc


def test_server_and_context_without_device_report_status():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    from fempar_gb300 import FGError, build, serving as S
    import fempar_gb300 as fg
    build.build()
    with pytest.raises(FGError):
        fg.Context(0)
    with pytest.raises(FGError):
        S.Server(device=0)

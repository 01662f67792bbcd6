"""Solver parameters on the host (no GPU): the C-ABI defaults are the reference's CG
defaults (iterative_solver_parameters.f90:168-178: rtol 1e-6, atol 0, 1000 iterations,
res_res), and the host mirror maps the reference's ILS_* keys onto them."""
import pytest


@pytest.fixture(scope="module")
def fe():
    from fempar_gb300 import _lib as L
    try:
        L.lib()
    except (ImportError, OSError) as e:
        pytest.skip(f"library not built: {e}")
    from fempar_gb300 import fe
    return fe


def test_defaults_are_the_reference_cg_defaults(fe):
    from fempar_gb300 import _lib as L
    s = fe.IterativeLinearSolver()
    p = s.params
    assert p.rtol == 1e-6 and p.atol == 0.0 and p.max_iters == 1000
    assert p.criterion == L.FG_RES_RES and p.precision == L.FG_FP64 and p.precond == L.FG_PREC_NONE


def test_parameter_keys_map_onto_the_c_struct(fe):
    from fempar_gb300 import _lib as L
    s = fe.IterativeLinearSolver().set_type_from_string("GPU_MPCG")
    assert s.params.precision == L.FG_MIXED
    s.set_parameters_from_pl({"ILS_RTOL": 1e-9, "ILS_ATOL": 1e-14, "ILS_MAX_NUM_ITERATIONS": 77,
                              "ILS_STOPPING_CRITERIUM": "DELTA_RHS", "PRECISION": "fp64"})
    p = s.params
    assert p.rtol == 1e-9 and p.atol == 1e-14 and p.max_iters == 77
    assert p.criterion == L.FG_DELTA_RHS and p.precision == L.FG_FP64
    with pytest.raises(KeyError):
        s.set_parameters_from_pl({"ILS_NOT_A_KEY": 1})
    with pytest.raises(ValueError):
        fe.IterativeLinearSolver().set_type_from_string("RGMRES")

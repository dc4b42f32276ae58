"""Host-side solver settings (no GPU): the reference's solver.* keys onto the
C ABI's agb_solver_opts, and the defaults Linear::PrepareMLMG gives MLMG."""
import pytest


def test_default_cycle_is_the_reference_f_cycle(agb):
    """Linear::PrepareMLMG calls setMaxFmgIter(100000000) and Parse leaves
    it unless solver.max_fmg_iter is given (Linear.H:261-266)."""
    assert agb.default_opts().max_fmg_iter == 100000000


def test_parse_maps_reference_keys(agb):
    from alamo_gb300 import _lib
    from alamo_gb300.elastic import parse_solver_opts
    o, extra = parse_solver_opts({
        "max_iter": "500", "bottom_max_iter": 50, "max_fmg_iter": "0", "fixed_iter": 4, "verbose": 3,
        "pre_smooth": 1, "post_smooth": "3", "final_smooth": 6, "bottom_smooth": 2, "bottom_solver": "smoother",
        "bottom_tol_rel": "1e-6", "bottom_tol_abs": 1e-12, "omega": 0.5, "tol_rel": "1e-9", "tol_abs": 0,
        "average_down_coeffs": "true", "normalize_ddw": 1, "abort_on_fail": "false"})
    assert (o.max_iter, o.bottom_max_iter, o.max_fmg_iter, o.fixed_iter, o.verbose) == (500, 50, 0, 4, 3)
    assert (o.pre_smooth, o.post_smooth, o.final_smooth, o.bottom_smooth) == (1, 3, 6, 2)
    assert o.bottom_solver == _lib.BOTTOM_SMOOTHER
    assert (o.bottom_tol_rel, o.bottom_tol_abs, o.omega) == (1e-6, 1e-12, 0.5)
    assert extra == {"tol_rel": 1e-9, "tol_abs": 0.0, "abort_on_fail": False}
    # untouched fields keep the defaults they started from
    d = agb.default_opts()
    assert (o.precision, o.solver, o.krylov_dim) == (d.precision, d.solver, d.krylov_dim)


@pytest.mark.parametrize("kv,err", [({"max_fixed_iter": 3}, ValueError), ({"cg_tol_rel": 1e-3}, ValueError),
                                    ({"cg_tol_abs": 1e-3}, ValueError), ({"bottom_solver": "cg"}, ValueError),
                                    ({"bottom_solver": "jacobi"}, KeyError), ({"max_iters": 3}, KeyError)])
def test_parse_rejects(agb, kv, err):
    from alamo_gb300.elastic import parse_solver_opts
    with pytest.raises(err):
        parse_solver_opts(kv)


@pytest.mark.parametrize("field,value", [
    ("pre_smooth", -1), ("post_smooth", -1), ("final_smooth", -1), ("bottom_smooth", -1),
    ("bottom_max_iter", -1), ("max_iter", -1), ("omega", 0.0), ("omega", 2.5), ("precision", 5),
    ("solver", 3), ("bottom_solver", 7), ("fine_kernel", 2), ("tma_min_nodes", -1)])
def test_create_rejects_bad_options(agb, field, value):
    """agb_elastic_create checks the options before it touches the GPU and
    answers AGB_BAD_ARG with a message naming the problem."""
    import ctypes
    from alamo_gb300 import _lib
    o = agb.default_opts()
    setattr(o, field, value)
    h = ctypes.c_void_p()
    dx = (ctypes.c_double * 3)(1, 1, 1)
    assert agb.lib().agb_elastic_create(ctypes.byref(h), 5, 5, 5, dx, 0, ctypes.byref(o)) == _lib.AGB_BAD_ARG
    assert not h.value
    assert _lib.last_error()


@pytest.mark.parametrize("field,value", [("krylov_dim", 0), ("krylov_dim", 40), ("inner_tol", 0.0),
                                         ("inner_tol", 1.0)])
def test_create_rejects_bad_fgmres_options(agb, field, value):
    import ctypes
    from alamo_gb300 import _lib
    o = agb.default_opts(solver="fgmres")
    setattr(o, field, value)
    h = ctypes.c_void_p()
    dx = (ctypes.c_double * 3)(1, 1, 1)
    assert agb.lib().agb_elastic_create(ctypes.byref(h), 5, 5, 5, dx, 0, ctypes.byref(o)) == _lib.AGB_BAD_ARG


def test_parse_newton_keys(agb):
    """Newton::Parse adds nriters and nrtolerance to the linear keys
    (src/Solver/Nonlocal/Newton.H:643-652; defaults 1 and 0, :630-631); the
    linear solver refuses them."""
    from alamo_gb300.elastic import parse_solver_opts
    o, extra = parse_solver_opts({"nriters": "10", "nrtolerance": "1e-6", "max_iter": 30}, newton=True)
    assert (extra["nriters"], extra["nrtolerance"], o.max_iter) == (10, 1e-6, 30)
    with pytest.raises(KeyError):
        parse_solver_opts({"nriters": 10})

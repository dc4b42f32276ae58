"""ctypes binding of the oracle (TEST INFRASTRUCTURE ONLY).

The oracle is a plain C++ restatement of the reference's CPU path (see the
header of ``elastic_oracle.cpp`` for the file:line map).  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import this
module, and only as the checker; the product package never does.

Arrays: node grids are nx*ny*nz with x fastest.  Vector fields are float64
arrays of shape (3, nz, ny, nx) (component slowest).  Stiffness is float64
(nz, ny, nx, nc) with nc = 2 (lambda, mu) or 21 (major-minor data[]).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

ISO, MM, MAJ = 0, 1, 2


class Opts(ctypes.Structure):
    _fields_ = [
        ("max_iter", ctypes.c_int),
        ("pre_smooth", ctypes.c_int),
        ("post_smooth", ctypes.c_int),
        ("final_smooth", ctypes.c_int),
        ("bottom_smooth", ctypes.c_int),
        ("bottom_max_iter", ctypes.c_int),
        ("bottom_tol_rel", ctypes.c_double),
        ("bottom_tol_abs", ctypes.c_double),
        ("omega", ctypes.c_double),
        ("max_coarsening_level", ctypes.c_int),
        ("fixed_iter", ctypes.c_int),
        ("verbose", ctypes.c_int),
        ("bottom_solver", ctypes.c_int),
        ("max_fmg_iter", ctypes.c_int),
        ("smoother", ctypes.c_int),
    ]


class Report(ctypes.Structure):
    _fields_ = [
        ("iters", ctypes.c_int),
        ("status", ctypes.c_int),
        ("nlevels", ctypes.c_int),
        ("bottom_iters_total", ctypes.c_int),
        ("resnorm0", ctypes.c_double),
        ("rhsnorm0", ctypes.c_double),
        ("final_resnorm", ctypes.c_double),
        ("seconds", ctypes.c_double),
        ("setup_seconds", ctypes.c_double),
    ]


def build(force=False):
    """Compile liboracle.so with the Makefile beside this file."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB_PATH)
        d = ctypes.c_double
        i = ctypes.c_int
        p = ctypes.c_void_p
        _lib.orc_residual.restype = d
        _lib.orc_num_levels.restype = i
        _lib.orc_num_threads.restype = i
        _lib.orc_solve.restype = i
        for name in ["orc_fapply", "orc_diagonal", "orc_fsmooth", "orc_restrict", "orc_restrict_C",
                     "orc_prolong_add", "orc_bc_init", "orc_build_rhs", "orc_stress_strain", "orc_cubic",
                     "orc_default_opts", "orc_jacobi_sweep", "orc_set_threads"]:
            getattr(_lib, name).restype = None
        del p
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays must be C-contiguous"
    return a.ctypes.data_as(ctypes.c_void_p)


def _dx(dx):
    return np.ascontiguousarray(np.broadcast_to(np.asarray(dx, dtype=np.float64), (3,)))


def _bct(bc_type):
    return np.ascontiguousarray(np.asarray(bc_type, dtype=np.int32).reshape(26, 3))


def _dims(u_or_C, vector=True):
    if vector:
        return u_or_C.shape[3], u_or_C.shape[2], u_or_C.shape[1]
    return u_or_C.shape[2], u_or_C.shape[1], u_or_C.shape[0]


def sym_of(C):
    return {2: ISO, 21: MM, 45: MAJ}[C.shape[-1]]


def set_threads(n):
    lib().orc_set_threads(ctypes.c_int(int(n)))


def num_threads():
    return lib().orc_num_threads()


def fapply(C, bc_type, u, dx):
    nx, ny, nz = _dims(C, vector=False)
    f = np.empty_like(u)
    d, b = _dx(dx), _bct(bc_type)
    lib().orc_fapply(sym_of(C), nx, ny, nz, _p(d), _p(C), _p(b), _p(u), _p(f))
    return f


def diagonal(C, bc_type, dx):
    nx, ny, nz = _dims(C, vector=False)
    dg = np.empty((3, nz, ny, nx))
    d, b = _dx(dx), _bct(bc_type)
    lib().orc_diagonal(sym_of(C), nx, ny, nz, _p(d), _p(C), _p(b), _p(dg))
    return dg


def fsmooth(C, bc_type, diag, x, b, dx, omega=2.0 / 3.0, ncalls=1):
    nx, ny, nz = _dims(C, vector=False)
    x = x.copy()
    d, bt = _dx(dx), _bct(bc_type)
    lib().orc_fsmooth(sym_of(C), nx, ny, nz, _p(d), _p(C), _p(bt), _p(diag), _p(x), _p(b),
                      ctypes.c_double(omega), ncalls)
    return x


def gs_smooth(C, bc_type, diag, x, b, dx, omega=2.0 / 3.0, ncalls=1):
    """ncalls multicolour Gauss-Seidel smoother calls (two sweeps each;
    weight 1 on interior rows, omega on boundary rows)."""
    nx, ny, nz = _dims(C, vector=False)
    x = x.copy()
    d, bt = _dx(dx), _bct(bc_type)
    lib().orc_gs_smooth(sym_of(C), nx, ny, nz, _p(d), _p(C), _p(bt), _p(diag), _p(x), _p(b), ctypes.c_double(omega),
                        ncalls)
    return x


def jacobi_sweep(C, bc_type, diag, x, b, dx, omega=2.0 / 3.0):
    nx, ny, nz = _dims(C, vector=False)
    out = np.empty_like(x)
    d, bt = _dx(dx), _bct(bc_type)
    lib().orc_jacobi_sweep(sym_of(C), nx, ny, nz, _p(d), _p(C), _p(bt), _p(diag), _p(x), _p(b),
                           ctypes.c_double(omega), _p(out))
    return out


def residual(C, bc_type, x, b, dx):
    nx, ny, nz = _dims(C, vector=False)
    r = np.empty_like(x)
    d, bt = _dx(dx), _bct(bc_type)
    nrm = lib().orc_residual(sym_of(C), nx, ny, nz, _p(d), _p(C), _p(bt), _p(x), _p(b), _p(r))
    return r, nrm


def restrict(fine):
    nzf, nyf, nxf = fine.shape[1:]
    c = np.empty((3, (nzf - 1) // 2 + 1, (nyf - 1) // 2 + 1, (nxf - 1) // 2 + 1))
    lib().orc_restrict(nxf, nyf, nzf, _p(fine), _p(c))
    return c


def restrict_C(Cf):
    nzf, nyf, nxf, nc = Cf.shape
    Cc = np.empty(((nzf - 1) // 2 + 1, (nyf - 1) // 2 + 1, (nxf - 1) // 2 + 1, nc))
    lib().orc_restrict_C({2: ISO, 21: MM, 45: MAJ}[nc], nxf, nyf, nzf, _p(Cf), _p(Cc))
    return Cc


def prolong_add(crse, fine):
    fine = fine.copy()
    nzf, nyf, nxf = fine.shape[1:]
    lib().orc_prolong_add(nxf, nyf, nzf, _p(crse), _p(fine))
    return fine


def bc_init(b, bc_type, bc_val, homogeneous=False):
    b = b.copy()
    nz, ny, nx = b.shape[1:]
    bt = _bct(bc_type)
    bv = np.ascontiguousarray(np.asarray(bc_val, dtype=np.float64).reshape(26, 3))
    lib().orc_bc_init(nx, ny, nz, _p(bt), _p(bv), int(bool(homogeneous)), _p(b))
    return b


def build_rhs(C, F0, bc_type, u, b, dx):
    nx, ny, nz = _dims(C, vector=False)
    rhs = np.empty_like(u)
    if F0 is None:
        f0n, F0p = 0, None
    else:
        F0 = np.ascontiguousarray(F0, dtype=np.float64)
        f0n = 1 if F0.ndim == 3 else 9
        F0p = F0
    d, bt = _dx(dx), _bct(bc_type)
    lib().orc_build_rhs(sym_of(C), nx, ny, nz, _p(d), _p(C), _p(F0p), f0n, _p(bt), _p(u), _p(b), _p(rhs))
    return rhs


def stress_strain(C, F0, u, dx):
    nx, ny, nz = _dims(C, vector=False)
    stress = np.empty((nz, ny, nx, 9))
    strain = np.empty((nz, ny, nx, 9))
    energy = np.empty((nz, ny, nx))
    if F0 is None:
        f0n, F0p = 0, None
    else:
        F0 = np.ascontiguousarray(F0, dtype=np.float64)
        f0n = 1 if F0.ndim == 3 else 9
        F0p = F0
    d = _dx(dx)
    lib().orc_stress_strain(sym_of(C), nx, ny, nz, _p(d), _p(C), _p(F0p), f0n, _p(u), _p(stress), _p(strain),
                            _p(energy))
    return stress, strain, energy


def cubic(C11, C12, C44, R):
    R = np.ascontiguousarray(R, dtype=np.float64).reshape(3, 3)
    out = np.empty(21)
    lib().orc_cubic(ctypes.c_double(C11), ctypes.c_double(C12), ctypes.c_double(C44), _p(R), _p(out))
    return out


def default_opts(**kw):
    o = Opts()
    lib().orc_default_opts(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def num_levels(nx, ny, nz, max_coarsening_level=-1):
    return lib().orc_num_levels(nx, ny, nz, max_coarsening_level)


def solve(C, bc_type, rhs, dx, tol_rel=1e-10, tol_abs=0.0, x0=None, opts=None, **kw):
    """Multigrid solve of A x = rhs; returns (x, report, residual history)."""
    nx, ny, nz = _dims(C, vector=False)
    x = np.zeros_like(rhs) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    o = opts if opts is not None else default_opts(**kw)
    rep = Report()
    hist = np.zeros(max(o.max_iter, o.fixed_iter) + 2)
    d, bt = _dx(dx), _bct(bc_type)
    lib().orc_solve(sym_of(C), nx, ny, nz, _p(d), _p(C), _p(bt), ctypes.byref(o), ctypes.c_double(tol_rel),
                    ctypes.c_double(tol_abs), _p(x), _p(rhs), ctypes.byref(rep), _p(hist))
    return x, rep, hist[: rep.iters + 1]


def derivative(which, f, dx):
    """Central FD derivative of a scalar node field (nz, ny, nx) at interior
    nodes; ``which`` is the reference's order code, e.g. 110 for d2/dxdy."""
    nz, ny, nx = f.shape
    out = np.empty_like(f)
    d = _dx(dx)
    lib().orc_derivative.restype = None
    lib().orc_derivative(int(which), nx, ny, nz, _p(d), _p(np.ascontiguousarray(f)), _p(out))
    return out


def vcycle(C, bc_type, res, dx, opts=None, **kw):
    """One V-cycle on A cor = res from cor = 0."""
    nx, ny, nz = _dims(C, vector=False)
    o = opts if opts is not None else default_opts(**kw)
    cor = np.empty_like(res)
    d, bt = _dx(dx), _bct(bc_type)
    lib().orc_vcycle.restype = None
    lib().orc_vcycle(sym_of(C), nx, ny, nz, _p(d), _p(C), _p(bt), ctypes.byref(o), _p(res), _p(cor))
    return cor


def set_uniform(uniform):
    """Operator::Elastic::SetUniform: True drops the grad-C term."""
    lib().orc_set_uniform.restype = None
    lib().orc_set_uniform(int(bool(uniform)))


_psi_keep = None


def psi_ghosted(psi_cells):
    """(nz-1, ny-1, nx-1) cell values -> (nz+1, ny+1, nx+1) with one ghost
    layer of 1.0 on every side (the reference's define-time fill)."""
    pc = np.asarray(psi_cells, dtype=np.float64)
    g = np.ones(tuple(s + 2 for s in pc.shape))
    g[1:-1, 1:-1, 1:-1] = pc
    return g


def set_psi(psi_cells, small=1e-8):
    """Operator::Elastic::SetPsi for the calls that follow (None clears):
    psi_cells is the (nz-1, ny-1, nx-1) cell field of a node grid."""
    global _psi_keep
    lib().orc_set_psi.restype = None
    if psi_cells is None:
        _psi_keep = None
        lib().orc_set_psi(None, ctypes.c_double(0.0))
        return
    _psi_keep = np.ascontiguousarray(psi_ghosted(psi_cells))
    lib().orc_set_psi(_p(_psi_keep), ctypes.c_double(small))


def coarsen_psi(psi_cells):
    """One multigrid coarsening of a cell psi field (Elastic.cpp:839-905):
    (nz-1, ny-1, nx-1) fine cells -> coarse cells."""
    g = np.ascontiguousarray(psi_ghosted(psi_cells))
    nz, ny, nx = (s - 1 for s in g.shape)
    out = np.empty(((nz - 1) // 2 + 2, (ny - 1) // 2 + 2, (nx - 1) // 2 + 2))
    lib().orc_coarsen_psi.restype = None
    lib().orc_coarsen_psi(nx, ny, nz, _p(g), _p(out))
    return out[1:-1, 1:-1, 1:-1].copy()


def neohookean(mu, kappa, F):
    """Model::Solid::Finite::NeoHookean at one F: (W, DW (3, 3), DDW (45,))."""
    F = np.ascontiguousarray(F, dtype=np.float64).reshape(9)
    W = ctypes.c_double()
    dw = np.empty(9)
    ddw = np.empty(45)
    lib().orc_neohookean.restype = None
    lib().orc_neohookean(ctypes.c_double(mu), ctypes.c_double(kappa), _p(F), ctypes.byref(W), _p(dw), _p(ddw))
    return W.value, dw.reshape(3, 3), ddw


def neohookean_field(model, u, dx):
    """dw (nz, ny, nx, 9) and ddw (nz, ny, nx, 45) at F = I + grad u for a
    per-node (mu, kappa) model (nz, ny, nx, 2)."""
    nz, ny, nx = model.shape[:3]
    dw = np.empty((nz, ny, nx, 9))
    ddw = np.empty((nz, ny, nx, 45))
    d = _dx(dx)
    lib().orc_neohookean_field.restype = None
    lib().orc_neohookean_field(nx, ny, nz, _p(d), _p(np.ascontiguousarray(model)), _p(np.ascontiguousarray(u)),
                               _p(dw), _p(ddw))
    return dw, ddw


def rhs_dw(dw, bc_type, u, b, dx):
    """b - div(dw) / b - BC(u, grad u, dw) for a nodal stress field dw."""
    nz, ny, nx = dw.shape[:3]
    rhs = np.empty_like(u)
    d, bt = _dx(dx), _bct(bc_type)
    lib().orc_rhs_dw.restype = None
    lib().orc_rhs_dw(nx, ny, nz, _p(d), _p(np.ascontiguousarray(dw)), _p(bt), _p(np.ascontiguousarray(u)),
                     _p(np.ascontiguousarray(b)), _p(rhs))
    return rhs

"""Host-side mirror of the reference's operator and solver classes.

    Elastic  ->  Operator::Elastic<SYM>          (src/Operator/Elastic.H:21-190)
    Linear   ->  Solver::Nonlocal::Linear        (src/Solver/Nonlocal/Linear.H:18-389)
    Newton   ->  Solver::Nonlocal::Newton        (src/Solver/Nonlocal/Newton.H:14-654)

Method names follow the reference (SetModel, SetBC, Fapply, Fsmooth,
Diagonal, solve, ...).  Every call goes through the C ABI of
``include/agb.h`` into the CUDA library; nothing is computed on the CPU.

Host arrays are numpy float64: vector fields (3, nz, ny, nx), stiffness
(nz, ny, nx, 2 | 21), eigenstrain (nz, ny, nx) for F0 = s I or
(nz, ny, nx, 3, 3).  Device arrays are passed as ``DevicePtr(address)``.
"""
import ctypes

import numpy as np

from . import _lib as L
from .bc import Constant


class DevicePtr:
    """A raw CUDA device address (e.g. ``torch.Tensor.data_ptr()``)."""

    def __init__(self, addr):
        self.addr = int(addr)


def _arg(a, dtype=np.float64):
    """(pointer, where) for a host numpy array or a DevicePtr."""
    if a is None:
        return None, L.MEM_HOST
    if isinstance(a, DevicePtr):
        return ctypes.c_void_p(a.addr), L.MEM_DEVICE
    if not (isinstance(a, np.ndarray) and a.dtype == dtype and a.flags["C_CONTIGUOUS"]):
        raise TypeError("expected a C-contiguous %s numpy array or DevicePtr" % np.dtype(dtype).name)
    return a.ctypes.data_as(ctypes.c_void_p), L.MEM_HOST


def _same_where(*ws):
    ws = [w for w in ws if w is not None]
    if len(set(ws)) > 1:
        raise TypeError("mixing host arrays and device pointers in one call")
    return ws[0] if ws else L.MEM_HOST


def default_opts(**kw):
    o = L.SolverOpts()
    L.check(L.lib().agb_default_opts(ctypes.byref(o)))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise TypeError("unknown solver option %r" % k)
        if k == "precision" and isinstance(v, str):
            v = {"fp64": L.PRECISION_FP64, "mixed": L.PRECISION_MIXED}[v]
        if k == "solver" and isinstance(v, str):
            v = {"vcycle": L.SOLVER_VCYCLE, "fgmres": L.SOLVER_FGMRES}[v]
        if k == "outer_residual" and isinstance(v, str):
            v = {"fp64": L.OUTER_FP64, "dfloat": L.OUTER_DFLOAT}[v]
        if k == "precond_cycle" and isinstance(v, str):
            v = {"v": L.PRECOND_V, "f": L.PRECOND_F}[v]
        if k == "smoother" and isinstance(v, str):
            v = {"jacobi": L.SMOOTHER_JACOBI, "gs": L.SMOOTHER_GS}[v]
        if k == "bottom_solver" and isinstance(v, str):
            v = {"bicgstab": L.BOTTOM_BICGSTAB, "direct": L.BOTTOM_DIRECT, "smoother": L.BOTTOM_SMOOTHER}[v]
        setattr(o, k, v)
    return o


class Elastic:
    """Operator::Elastic<SYM> on one uniform node grid (one AMR level)."""

    def __init__(self, n, dx, sym="isotropic", opts=None):
        if isinstance(n, int):
            n = (n, n, n)
        self.n = tuple(int(v) for v in n)
        dxa = np.ascontiguousarray(np.broadcast_to(np.asarray(dx, dtype=np.float64), (3,)))
        self.dx = dxa
        self.sym = {"isotropic": L.SYM_ISOTROPIC, "majorminor": L.SYM_MAJORMINOR, "major": L.SYM_MAJOR}.get(sym, sym)
        self.nc = {L.SYM_ISOTROPIC: 2, L.SYM_MAJORMINOR: 21, L.SYM_MAJOR: 45}[self.sym]
        self.opts = opts if opts is not None else default_opts()
        h = ctypes.c_void_p()
        L.check(L.lib().agb_elastic_create(ctypes.byref(h), self.n[0], self.n[1], self.n[2],
                                           dxa.ctypes.data_as(ctypes.c_void_p), self.sym, ctypes.byref(self.opts)))
        self.h = h
        self.bc = Constant()

    def close(self):
        if getattr(self, "h", None):
            L.lib().agb_elastic_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def N(self):
        return self.n[0] * self.n[1] * self.n[2]

    def num_levels(self):
        v = ctypes.c_int()
        L.check(L.lib().agb_elastic_num_levels(self.h, ctypes.byref(v)))
        return v.value

    def level_dims(self, level):
        d = (ctypes.c_int * 3)()
        L.check(L.lib().agb_elastic_level_dims(self.h, int(level), d))
        return tuple(d)

    def _vec_shape(self, level=0):
        nx, ny, nz = self.level_dims(level)
        return (3, nz, ny, nx)

    # --- Operator::Elastic user API -------------------------------------
    def SetModel(self, C):
        p, w = _arg(C)
        L.check(L.lib().agb_elastic_set_model(self.h, p, w))

    def GetModel(self, level=0):
        nx, ny, nz = self.level_dims(level)
        out = np.empty((nz, ny, nx, self.nc))
        p, w = _arg(out)
        L.check(L.lib().agb_elastic_get_model(self.h, int(level), p, w))
        return out

    def SetBC(self, bc):
        """Elastic::SetBC (src/Operator/Elastic.H:61-65).  The tables are
        copied with the values at the BC's current time (``bc.set_time``);
        after moving the time, call SetBC again."""
        self.bc = bc
        t, v = bc.tables()
        L.check(L.lib().agb_elastic_set_bc(self.h, t.ctypes.data_as(ctypes.c_void_p),
                                           v.ctypes.data_as(ctypes.c_void_p)))

    def SetPsi(self, psi, small=1e-8):
        """Elastic::SetPsi (src/Operator/Elastic.cpp:118-137): psi is the
        (nz-1, ny-1, nx-1) cell field of the void indicator; None clears it.
        small is m_psi_small."""
        if psi is None:
            L.check(L.lib().agb_elastic_set_psi(self.h, None, ctypes.c_double(0.0), L.MEM_HOST))
            self.psi = None
            return
        nx, ny, nz = self.n
        shape = (nz - 1, ny - 1, nx - 1)
        if isinstance(psi, np.ndarray) and tuple(psi.shape) != shape:
            raise ValueError(f"psi must have the cell shape {shape}, got {tuple(psi.shape)}")
        self.psi = psi
        p, w = _arg(psi)
        L.check(L.lib().agb_elastic_set_psi(self.h, p, ctypes.c_double(small), w))

    def SetOpts(self, opts):
        self.opts = opts
        L.check(L.lib().agb_elastic_set_opts(self.h, ctypes.byref(opts)))

    def prepareForSolve(self):
        L.check(L.lib().agb_elastic_prepare(self.h))

    # --- MLNodeLinOp hooks ----------------------------------------------
    def Fapply(self, u, f=None, level=0):
        if f is None:
            f = np.empty(self._vec_shape(level))
        pu, wu = _arg(u)
        pf, wf = _arg(f)
        L.check(L.lib().agb_elastic_fapply(self.h, int(level), pu, pf, _same_where(wu, wf)))
        return f

    def Fapply_f32(self, u, f=None, level=0):
        if f is None:
            f = np.empty(self._vec_shape(level), dtype=np.float32)
        pu, wu = _arg(u, np.float32)
        pf, wf = _arg(f, np.float32)
        L.check(L.lib().agb_elastic_fapply_f32(self.h, int(level), pu, pf, _same_where(wu, wf)))
        return f

    def Diagonal(self, level=0, diag=None):
        if diag is None:
            diag = np.empty(self._vec_shape(level))
        p, w = _arg(diag)
        L.check(L.lib().agb_elastic_diagonal(self.h, int(level), p, w))
        return diag

    def Fsmooth(self, x, b, ncalls=1, level=0):
        """Two damped-Jacobi sweeps per call, in place on x."""
        px, wx = _arg(x)
        pb, wb = _arg(b)
        L.check(L.lib().agb_elastic_fsmooth(self.h, int(level), px, pb, int(ncalls), _same_where(wx, wb)))
        return x

    def residual_dfloat(self, x, b, r=None):
        """The fine-level residual in double-float arithmetic (FP64 arrays in
        and out); returns (r, (inf-norm, 2-norm))."""
        if r is None:
            r = np.empty(self._vec_shape(0))
        norms = (ctypes.c_double * 2)()
        px, wx = _arg(x)
        pb, wb = _arg(b)
        pr, wr = _arg(r)
        L.check(L.lib().agb_elastic_residual_dfloat(self.h, px, pb, pr, norms, _same_where(wx, wb, wr)))
        return r, (norms[0], norms[1])

    def Fsmooth_f32(self, x, b, ncalls=1, level=0):
        """The mixed-precision cycle's FP32 Fsmooth, in place on x (float32)."""
        px, wx = _arg(x, np.float32)
        pb, wb = _arg(b, np.float32)
        L.check(L.lib().agb_elastic_fsmooth_f32(self.h, int(level), px, pb, int(ncalls), _same_where(wx, wb)))
        return x

    def residual_f32(self, x, b, r=None, level=0):
        """The mixed-precision cycle's FP32 residual r = b - A x (float32)."""
        if r is None:
            r = np.empty(self._vec_shape(level), dtype=np.float32)
        px, wx = _arg(x, np.float32)
        pb, wb = _arg(b, np.float32)
        pr, wr = _arg(r, np.float32)
        L.check(L.lib().agb_elastic_residual_f32(self.h, int(level), px, pb, pr, _same_where(wx, wb, wr)))
        return r

    def residual(self, x, b, r=None, level=0):
        """r = b - A x; returns (r, (inf-norm, 2-norm))."""
        if r is None:
            r = np.empty(self._vec_shape(level))
        norms = (ctypes.c_double * 2)()
        px, wx = _arg(x)
        pb, wb = _arg(b)
        pr, wr = _arg(r)
        L.check(L.lib().agb_elastic_residual(self.h, int(level), px, pb, pr, norms, _same_where(wx, wb, wr)))
        return r, (norms[0], norms[1])

    def restriction(self, crse_level, fine, crse=None):
        if crse is None:
            crse = np.empty(self._vec_shape(crse_level))
        pf, wf = _arg(fine)
        pc, wc = _arg(crse)
        L.check(L.lib().agb_elastic_restrict(self.h, int(crse_level), pf, pc, _same_where(wf, wc)))
        return crse

    def interpolation(self, fine_level, fine, crse):
        """fine += P crse (in place)."""
        pc, wc = _arg(crse)
        pf, wf = _arg(fine)
        L.check(L.lib().agb_elastic_prolong_add(self.h, int(fine_level), pc, pf, _same_where(wc, wf)))
        return fine

    def vcycle(self, res, cor=None, precision="fp64"):
        """One multigrid V-cycle on A cor = res from cor = 0 (MLMG::mgVcycle)."""
        if cor is None:
            cor = np.empty(self._vec_shape(0))
        pr, wr = _arg(res)
        pc, wc = _arg(cor)
        prec = {"fp64": L.PRECISION_FP64, "mixed": L.PRECISION_MIXED, "fp32": L.PRECISION_MIXED}.get(precision,
                                                                                                      precision)
        L.check(L.lib().agb_elastic_vcycle(self.h, pr, pc, int(prec), _same_where(wr, wc)))
        return cor

    # --- BC / RHS / post-processing -------------------------------------
    def bc_init(self, b=None, homogeneous=False):
        if b is None:
            b = np.zeros(self._vec_shape(0))
        p, w = _arg(b)
        L.check(L.lib().agb_elastic_bc_init(self.h, p, int(bool(homogeneous)), w))
        return b

    @staticmethod
    def _f0(F0):
        if F0 is None:
            return None, 0, None
        if isinstance(F0, tuple):  # (DevicePtr, ncomp)
            return ctypes.c_void_p(F0[0].addr), int(F0[1]), L.MEM_DEVICE
        F0 = np.ascontiguousarray(F0, dtype=np.float64)
        return F0.ctypes.data_as(ctypes.c_void_p), (1 if F0.ndim == 3 else 9), L.MEM_HOST

    def build_rhs(self, u, b, F0=None, rhs=None):
        if rhs is None:
            rhs = np.empty(self._vec_shape(0))
        pF, nF, wF = self._f0(F0)
        pu, wu = _arg(u)
        pb, wb = _arg(b)
        pr, wr = _arg(rhs)
        L.check(L.lib().agb_elastic_build_rhs(self.h, pu, pb, pF, nF, pr, _same_where(wu, wb, wr, wF)))
        return rhs

    def stress_strain(self, u, F0=None):
        """(stress, strain, energy): (nz,ny,nx,3,3), (nz,ny,nx,3,3), (nz,ny,nx)."""
        nz, ny, nx = self._vec_shape(0)[1:]
        s = np.empty((nz, ny, nx, 3, 3))
        e = np.empty((nz, ny, nx, 3, 3))
        en = np.empty((nz, ny, nx))
        pF, nF, wF = self._f0(F0)
        pu, wu = _arg(u)
        L.check(L.lib().agb_elastic_stress_strain(self.h, pu, pF, nF, s.ctypes.data_as(ctypes.c_void_p),
                                                  e.ctypes.data_as(ctypes.c_void_p),
                                                  en.ctypes.data_as(ctypes.c_void_p), _same_where(wu, wF)))
        return s, e, en

    def Stress(self, u, F0=None):
        return self.stress_strain(u, F0)[0]

    def OpStress(self, u, voigt=False):
        """Elastic::Stress (src/Operator/Elastic.cpp:483-549): (C grad u)
        psi_avg, SoA (6 Voigt or 9 components, nz, ny, nx)."""
        return self._tensor(u, 0, voigt)

    def OpStrain(self, u, voigt=False):
        """Elastic::Strain (src/Operator/Elastic.cpp:426-480): sym grad u,
        SoA (6 Voigt or 9 components, nz, ny, nx)."""
        return self._tensor(u, 1, voigt)

    def _tensor(self, u, which, voigt):
        nx, ny, nz = self.n
        out = np.empty((6 if voigt else 9, nz, ny, nx))
        pu, wu = _arg(u)
        po, wo = _arg(out)
        L.check(L.lib().agb_elastic_tensor(self.h, pu, int(which), int(bool(voigt)), po, _same_where(wu, wo)))
        return out

    def Strain(self, u):
        return self.stress_strain(u)[1]

    def Energy(self, u, F0=None):
        return self.stress_strain(u, F0)[2]

    # --- profiling --------------------------------------------------------
    def profile(self, on=True):
        L.check(L.lib().agb_profile_enable(self.h, int(bool(on))))
        L.check(L.lib().agb_profile_reset(self.h))

    def profile_get(self, family):
        n = ctypes.c_int64()
        ms = ctypes.c_double()
        L.check(L.lib().agb_profile_get(self.h, int(family), ctypes.byref(n), ctypes.byref(ms)))
        return n.value, ms.value

    def profile_bytes(self, family):
        """Algorithmic bytes of the family's timed launches since the reset."""
        b = ctypes.c_double()
        L.check(L.lib().agb_profile_bytes(self.h, int(family), ctypes.byref(b)))
        return b.value

    def launch_count(self):
        n = ctypes.c_int64()
        L.check(L.lib().agb_launch_count(self.h, ctypes.byref(n)))
        return n.value


# solver.* keys of Solver::Nonlocal::Linear::Parse (src/Solver/Nonlocal/Linear.H:296-382)
# that map one to one onto agb_solver_opts fields
_INT_KEYS = ["max_iter", "bottom_max_iter", "max_fmg_iter", "fixed_iter", "verbose", "pre_smooth", "post_smooth",
             "final_smooth", "bottom_smooth"]
_FLOAT_KEYS = ["bottom_tol_rel", "bottom_tol_abs", "omega"]
# keys with no effect on a single-level solve: average_down_coeffs averages
# stiffness between AMR levels only (Elastic.cpp:611-613); normalize_ddw is
# stored but read by no operator code; dump_on_fail writes diagnostics files
_NO_EFFECT_KEYS = ["average_down_coeffs", "normalize_ddw", "dump_on_fail"]


def _flag(v):
    if isinstance(v, str):
        return v.strip().lower() in ("1", "true")
    return bool(v)


def parse_solver_opts(kv, opts=None, newton=False):
    """``Linear::Parse`` (src/Solver/Nonlocal/Linear.H:296-382) and
    ``PrepareMLMG`` (:255-290): the reference's ``solver.*`` keys (given
    without the prefix) onto an agb_solver_opts, starting from ``opts`` or
    the defaults.  Returns (opts, extra) with extra = {"tol_rel", "tol_abs",
    "abort_on_fail"} for the keys that are arguments of the solve.  The
    deprecated keys abort in the reference and raise ValueError here, as do
    unknown keys and the CG bottom solver (not provided: BiCGStab, the direct
    bottom and the smoother are).  newton=True also takes Newton::Parse's
    nriters and nrtolerance (src/Solver/Nonlocal/Newton.H:643-652) into
    extra."""
    o = default_opts() if opts is None else opts
    extra = {"tol_rel": None, "tol_abs": None, "abort_on_fail": True}
    if newton:
        extra.update(nriters=None, nrtolerance=None)
    for k, v in kv.items():
        if k in ("max_fixed_iter", "cg_tol_rel", "cg_tol_abs"):
            raise ValueError(k + " is deprecated in the reference (Linear.H:308-335)")
        if k in _INT_KEYS:
            setattr(o, k, int(v))
        elif k in _FLOAT_KEYS:
            setattr(o, k, float(v))
        elif k == "bottom_solver":
            name = str(v).strip()
            if name == "cg":
                raise ValueError("the CG bottom solver is not provided (bicgstab, direct, smoother are)")
            o.bottom_solver = {"bicgstab": L.BOTTOM_BICGSTAB, "direct": L.BOTTOM_DIRECT,
                               "smoother": L.BOTTOM_SMOOTHER}[name]
        elif k in ("tol_rel", "tol_abs"):
            extra[k] = float(v)
        elif k == "abort_on_fail":
            extra["abort_on_fail"] = _flag(v)
        elif k in _NO_EFFECT_KEYS:
            pass
        elif newton and k == "nriters":
            extra["nriters"] = int(v)
        elif newton and k == "nrtolerance":
            extra["nrtolerance"] = float(v)
        else:
            raise KeyError("unknown solver key " + k)
    return o, extra


class Linear:
    """Solver::Nonlocal::Linear: multigrid solve of A sol = rhs."""

    def __init__(self, op=None):
        self.op = None
        if op is not None:
            self.Define(op)

    def Define(self, op):
        if self.op is not None:
            raise RuntimeError("Solver cannot be re-defined")
        self.op = op

    def Clear(self):
        self.op = None

    def _set(self, **kw):
        o = self.op.opts
        for k, v in kw.items():
            setattr(o, k, v)
        self.op.SetOpts(o)

    def Parse(self, kv):
        """Apply the reference's ``solver.*`` keys (parse_solver_opts) to the
        operator's options; tol_rel / tol_abs / abort_on_fail are kept on
        the solver for the caller."""
        o, extra = parse_solver_opts(kv, self.op.opts)
        self.op.SetOpts(o)
        self.parsed = extra
        return extra

    def apply(self, rhs, sol):
        """Linear::apply (src/Solver/Nonlocal/Linear.H:169-174): rhs = A sol
        on the fine level, boundary rows included."""
        return self.op.Fapply(sol, rhs)

    def setMaxIter(self, v): self._set(max_iter=int(v))
    def setMaxFmgIter(self, v): self._set(max_fmg_iter=int(v))
    def setBottomMaxIter(self, v): self._set(bottom_max_iter=int(v))
    def setFixedIter(self, v): self._set(fixed_iter=int(v))
    def setVerbose(self, v): self._set(verbose=int(v))
    def setPreSmooth(self, v): self._set(pre_smooth=int(v))
    def setPostSmooth(self, v): self._set(post_smooth=int(v))
    def setPrecision(self, p): self._set(precision={"fp64": 0, "mixed": 1}.get(p, p))

    def solve(self, sol, rhs, tol_rel, tol_abs, allow_not_converged=False):
        """Returns the agb_solve_report as a dict; sol is updated in place."""
        rep = L.SolveReport()
        ps, ws = _arg(sol)
        pr, wr = _arg(rhs)
        st = L.lib().agb_linear_solve(self.op.h, ps, pr, ctypes.c_double(tol_rel), ctypes.c_double(tol_abs),
                                      ctypes.byref(rep), _same_where(ws, wr))
        L.check(st, (L.AGB_OK, L.AGB_NOT_CONVERGED) if allow_not_converged else (L.AGB_OK,))
        return rep.as_dict()


class Newton(Linear):
    """Solver::Nonlocal::Newton for linear models (setNRIters /
    nrtolerance of the reference; nriters = 1 by default)."""

    def __init__(self, op, nriters=1, nrtolerance=0.0):
        super().__init__(op)
        self.nriters = int(nriters)
        self.nrtolerance = float(nrtolerance)

    def setNRIters(self, n):
        """Newton::setNRIters (src/Solver/Nonlocal/Newton.H:44)."""
        self.nriters = int(n)

    def Parse(self, kv):
        """Newton::Parse (src/Solver/Nonlocal/Newton.H:643-652): the linear
        solver keys plus nriters and nrtolerance."""
        o, extra = parse_solver_opts(kv, self.op.opts, newton=True)
        self.op.SetOpts(o)
        if extra["nriters"] is not None:
            self.nriters = extra["nriters"]
        if extra["nrtolerance"] is not None:
            self.nrtolerance = extra["nrtolerance"]
        self.parsed = extra
        return extra

    def setPsi(self, psi, small=1e-8):
        """Newton::setPsi (src/Solver/Nonlocal/Newton.H:46-49): the operator's
        psi for the solves that follow (Elastic.SetPsi)."""
        self.op.SetPsi(psi, small)

    def solve(self, u, b, F0=None, tol_rel=1e-8, tol_abs=0.0, allow_not_converged=False):
        """Returns the last linear solve's report as a dict, plus "relnorm"
        (max |increment| of the last iteration) when nriters > 1."""
        rep = L.SolveReport()
        pF, nF, wF = Elastic._f0(F0)
        pu, wu = _arg(u)
        pb, wb = _arg(b)
        where = _same_where(wu, wb, wF)
        if self.nriters == 1:
            st = L.lib().agb_newton_solve(self.op.h, pu, pb, pF, nF, ctypes.c_double(tol_rel),
                                          ctypes.c_double(tol_abs), ctypes.byref(rep), where)
            rn = None
        else:
            r = ctypes.c_double()
            st = L.lib().agb_newton_solve_n(self.op.h, pu, pb, pF, nF, ctypes.c_double(tol_rel),
                                            ctypes.c_double(tol_abs), self.nriters, ctypes.c_double(self.nrtolerance),
                                            ctypes.byref(rep), ctypes.byref(r), where)
            rn = r.value
        L.check(st, (L.AGB_OK, L.AGB_NOT_CONVERGED) if allow_not_converged else (L.AGB_OK,))
        d = rep.as_dict()
        if rn is not None:
            d["relnorm"] = rn
        return d

    def solve_neohookean(self, model, u, b, tol_rel=1e-8, tol_abs=0.0, allow_not_converged=False):
        """Newton iterations for a NeoHookean medium (agb_newton_solve_neohookean):
        model (nz, ny, nx, 2) = (mu, kappa) per node; u in/out.  The handle
        must be of symmetry "major".  Returns the last linear solve's report
        plus "relnorm" (max |increment| of the last iteration)."""
        rep = L.SolveReport()
        pm, wm = _arg(model)
        pu, wu = _arg(u)
        pb, wb = _arg(b)
        r = ctypes.c_double()
        st = L.lib().agb_newton_solve_neohookean(self.op.h, pm, pu, pb, ctypes.c_double(tol_rel),
                                                 ctypes.c_double(tol_abs), self.nriters,
                                                 ctypes.c_double(self.nrtolerance), ctypes.byref(rep), ctypes.byref(r),
                                                 _same_where(wm, wu, wb))
        L.check(st, (L.AGB_OK, L.AGB_NOT_CONVERGED) if allow_not_converged else (L.AGB_OK,))
        d = rep.as_dict()
        d["relnorm"] = r.value
        return d

    def solve_guess(self, net, u, b, F0=None, tol_rel=1e-8, tol_abs=0.0, allow_not_converged=False):
        """One Newton step from u = 0 whose linear solve starts from the
        learned guess of `net` (agb_newton_solve_guess): u is output only.
        Returns the solve report as a dict plus "guess_used"."""
        rep = L.SolveReport()
        pF, nF, wF = Elastic._f0(F0)
        pu, wu = _arg(u)
        pb, wb = _arg(b)
        used = ctypes.c_int()
        st = L.lib().agb_newton_solve_guess(self.op.h, net.h, pu, pb, pF, nF, ctypes.c_double(tol_rel),
                                            ctypes.c_double(tol_abs), ctypes.byref(rep), ctypes.byref(used),
                                            _same_where(wu, wb, wF))
        L.check(st, (L.AGB_OK, L.AGB_NOT_CONVERGED) if allow_not_converged else (L.AGB_OK,))
        d = rep.as_dict()
        d["guess_used"] = bool(used.value)
        return d

"""AMR composite solve (agb_composite_*): Solver::Nonlocal::Linear on a
hierarchy of nested boxes, one per level, refinement ratio 2.

Level 0 is the domain; level l >= 1 is a box of `nv` valid nodes per axis
starting at level index `lo`, and its arrays (stiffness, eigenstrain,
solution) cover the box plus one ring of ghost nodes (nv + 2 per axis).
"""
import ctypes

import numpy as np

from . import _lib as L
from .elastic import _arg, default_opts


class Composite:
    def __init__(self, n0, dx0, boxes, sym="isotropic", opts=None):
        """boxes: [(lo, nv), ...] of levels 1.. (each an int or a 3-tuple)."""
        n0 = (n0,) * 3 if isinstance(n0, int) else tuple(n0)
        dx0 = np.ascontiguousarray(np.broadcast_to(np.asarray(dx0, dtype=np.float64), (3,)))
        self.nlev = 1 + len(boxes)
        lo = np.zeros((self.nlev, 3), dtype=np.int32)
        nv = np.zeros((self.nlev, 3), dtype=np.int32)
        for l, (b_lo, b_nv) in enumerate(boxes, start=1):
            lo[l] = np.broadcast_to(b_lo, (3,))
            nv[l] = np.broadcast_to(b_nv, (3,))
        self.sym = {"isotropic": L.SYM_ISOTROPIC, "majorminor": L.SYM_MAJORMINOR}[sym]
        self.nc = 2 if self.sym == L.SYM_ISOTROPIC else 21
        self.opts = opts if opts is not None else default_opts()
        h = ctypes.c_void_p()
        n0a = (ctypes.c_int * 3)(*n0)
        L.check(L.lib().agb_composite_create(ctypes.byref(h), self.nlev, n0a, dx0.ctypes.data_as(ctypes.c_void_p),
                                             self.sym, lo.ctypes.data_as(ctypes.c_void_p),
                                             nv.ctypes.data_as(ctypes.c_void_p), ctypes.byref(self.opts)))
        self.h = h
        self.dims = []
        for l in range(self.nlev):
            d = (ctypes.c_int * 3)()
            L.check(L.lib().agb_composite_level_dims(self.h, l, d))
            self.dims.append((d[0], d[1], d[2]))

    def close(self):
        if self.h:
            L.lib().agb_composite_destroy(self.h)
            self.h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def SetBC(self, bc):
        t, v = bc.tables()
        t = np.ascontiguousarray(t, dtype=np.int32)
        v = np.ascontiguousarray(v, dtype=np.float64)
        L.check(L.lib().agb_composite_set_bc(self.h, t.ctypes.data_as(ctypes.c_void_p),
                                             v.ctypes.data_as(ctypes.c_void_p)))

    def SetModel(self, level, C):
        p, w = _arg(np.ascontiguousarray(C) if isinstance(C, np.ndarray) else C)
        L.check(L.lib().agb_composite_set_model(self.h, int(level), p, w))

    def solve(self, F0=None, tol_rel=1e-10, tol_abs=0.0, allow_not_converged=False):
        """Host arrays: F0 None or a list of per-level eigenstrain arrays
        (scalar (nz, ny, nx) or None entries).  Returns (u per level, iters,
        final relative composite residual)."""
        us = [np.zeros((3,) + tuple(d[::-1])) for d in self.dims]
        uptr = (ctypes.c_void_p * self.nlev)(*[u.ctypes.data for u in us])
        fptr, f0n = None, 0
        keep = []
        if F0 is not None:
            arrs = [None if f is None else np.ascontiguousarray(f, dtype=np.float64) for f in F0]
            keep = arrs
            f0n = 1
            for f in arrs:
                if f is not None and f.ndim == 4:
                    f0n = 9
            fptr = (ctypes.c_void_p * self.nlev)(*[None if f is None else f.ctypes.data for f in arrs])
        it = ctypes.c_int()
        rn = ctypes.c_double()
        st = L.lib().agb_composite_solve(self.h, uptr, fptr, f0n, ctypes.c_double(tol_rel), ctypes.c_double(tol_abs),
                                         ctypes.byref(it), ctypes.byref(rn), L.MEM_HOST)
        del keep
        L.check(st, (L.AGB_OK, L.AGB_NOT_CONVERGED) if allow_not_converged else (L.AGB_OK,))
        return us, it.value, rn.value

"""Synthetic inputs of the benchmark workloads (wrappers of agb_synth_*).

The shapes, sizes and value distributions are the ones the benchmark
configurations name; no dataset is involved.  All generators are
deterministic for a given seed (std::mt19937_64).
"""
import ctypes

import numpy as np

from . import _lib as L

SEED_FAPPLY = 20261203


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _dx(dx):
    return np.ascontiguousarray(np.broadcast_to(np.asarray(dx, dtype=np.float64), (3,)))


def uniform(seed, shape, lo=-1.0, hi=1.0):
    out = np.empty(shape)
    L.check(L.lib().agb_synth_uniform(ctypes.c_uint64(seed), ctypes.c_int64(out.size), ctypes.c_double(lo),
                                      ctypes.c_double(hi), _p(out)))
    return out


def cubic_stiffness(C11, C12, C44, R=None):
    R = np.eye(3) if R is None else np.ascontiguousarray(R, dtype=np.float64)
    out = np.empty(21)
    L.check(L.lib().agb_cubic_stiffness(ctypes.c_double(C11), ctypes.c_double(C12), ctypes.c_double(C44), _p(R),
                                        _p(out)))
    return out


def inclusion_iso(n, center=(0.5, 0.5, 0.5), radius=0.25, lam_in=10.0, mu_in=10.0, lam_out=1.0, mu_out=1.0,
                  eps_in=0.01, L_box=1.0):
    """One spherical inclusion on the unit cube (node coordinates i*dx)."""
    dx = L_box / (n - 1)
    C = np.empty((n, n, n, 2))
    F0 = np.empty((n, n, n))
    c = np.asarray(center, dtype=np.float64)
    L.check(L.lib().agb_synth_inclusion_iso(n, n, n, _p(_dx(dx)), _p(c), ctypes.c_double(radius),
                                            ctypes.c_double(lam_in), ctypes.c_double(mu_in), ctypes.c_double(lam_out),
                                            ctypes.c_double(mu_out), ctypes.c_double(eps_in), _p(C), _p(F0)))
    return C, F0, dx


def voronoi_cubic(n, nseeds=64, seed=1, C11=1.68, C12=1.21, C44=0.75, L_box=1.0, with_grain=False):
    """Cubic polycrystal, one grain per Voronoi seed, Haar-random rotations."""
    dx = L_box / (n - 1)
    C = np.empty((n, n, n, 21))
    grain = np.empty((n, n, n), dtype=np.int32) if with_grain else None
    L.check(L.lib().agb_synth_voronoi_cubic(n, n, n, _p(_dx(dx)), int(nseeds), ctypes.c_uint64(seed),
                                            ctypes.c_double(C11), ctypes.c_double(C12), ctypes.c_double(C44), _p(C),
                                            _p(grain) if grain is not None else None))
    return (C, dx, grain) if with_grain else (C, dx)


def spheres_iso(n, nspheres=200, seed=1, rmin=0.02, rmax=0.06, contrast=10.0, smin=0.0, smax=0.02, L_box=1.0):
    """Two-phase isotropic medium of non-overlapping spheres with eigenstrain."""
    dx = L_box / (n - 1)
    C = np.empty((n, n, n, 2))
    F0 = np.empty((n, n, n))
    placed = ctypes.c_int()
    L.check(L.lib().agb_synth_spheres_iso(n, n, n, _p(_dx(dx)), int(nspheres), ctypes.c_uint64(seed),
                                          ctypes.c_double(rmin), ctypes.c_double(rmax), ctypes.c_double(contrast),
                                          ctypes.c_double(contrast), ctypes.c_double(1.0), ctypes.c_double(1.0),
                                          ctypes.c_double(smin), ctypes.c_double(smax), _p(C), _p(F0),
                                          ctypes.byref(placed)))
    return C, F0, dx, placed.value


def spheres_diffuse(n, nspheres=200, seed=1, rmin=0.02, rmax=0.06, eps=None, contrast=10.0, smin=0.0, smax=0.02,
                    L_box=1.0):
    """The spheres of spheres_iso with a diffuse interface (the reference's
    ellipse initial condition); eps defaults to 4 node spacings."""
    dx = L_box / (n - 1)
    if eps is None:
        eps = 4.0 * dx
    C = np.empty((n, n, n, 2))
    F0 = np.empty((n, n, n))
    placed = ctypes.c_int()
    L.check(L.lib().agb_synth_spheres_diffuse(n, n, n, _p(_dx(dx)), int(nspheres), ctypes.c_uint64(seed),
                                              ctypes.c_double(rmin), ctypes.c_double(rmax), ctypes.c_double(eps),
                                              ctypes.c_double(contrast), ctypes.c_double(contrast),
                                              ctypes.c_double(1.0), ctypes.c_double(1.0), ctypes.c_double(smin),
                                              ctypes.c_double(smax), _p(C), _p(F0), ctypes.byref(placed)))
    return C, F0, dx, placed.value

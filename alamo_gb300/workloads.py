"""Synthetic inputs of the benchmark workloads, in numpy only.

The benchmark's two arms (the CUDA library and the reference's CPU path)
must see the same bytes without the CPU arm loading the CUDA library, so the
generators live here as plain numpy.  They reproduce the library's own
generators (``agb_synth_*``, ``csrc/synth.cpp``) value for value: the same
std::mt19937_64 stream (restated below from the recurrence the C++ standard
fixes), the same floating-point expressions in the same order.  The one
exception is the diffuse-sphere profile, whose erf comes from scipy here and
from the C library there (equal to about one unit in the last place).

Workloads (unit cube, node coordinates i*dx):
  inclusion_iso    one isotropic spherical inclusion with eigenstrain
                   (Model::Solid::Affine::Isotropic per node)
  voronoi_cubic    cubic polycrystal, one grain per Voronoi seed, Haar-random
                   rotations (Model::Solid::Linear::Cubic with
                   Set::Matrix4<3,MajorMinor>::Cubic,
                   src/Set/Matrix4_MajorMinor.H:518-547)
  spheres_diffuse  non-overlapping spheres with the diffuse profile of the
                   reference's ellipse initial condition (src/IC/Ellipse.H:56-75)
"""
import math

import numpy as np

_MASK = (1 << 64) - 1


class MT19937_64:
    """std::mt19937_64: word size 64, degree 312, middle 156, twist matrix
    0xB5026F5AA96619E9, tempering (29, 0x5555555555555555), (17,
    0x71D67FFFEDA60000), (37, 0xFFF7EEE000000000), 43; initialisation
    multiplier 6364136223846793005 (the parameters the C++ standard names)."""
    N, M = 312, 156

    def __init__(self, seed):
        mt = [0] * self.N
        mt[0] = seed & _MASK
        for i in range(1, self.N):
            mt[i] = (6364136223846793005 * (mt[i - 1] ^ (mt[i - 1] >> 62)) + i) & _MASK
        self.mt = mt
        self.i = self.N

    def _twist(self):
        mt = self.mt
        upper, lower = 0xFFFFFFFF80000000, 0x7FFFFFFF
        for k in range(self.N):
            y = (mt[k] & upper) | (mt[(k + 1) % self.N] & lower)
            v = mt[(k + self.M) % self.N] ^ (y >> 1)
            if y & 1:
                v ^= 0xB5026F5AA96619E9
            mt[k] = v
        self.i = 0

    def next(self):
        if self.i >= self.N:
            self._twist()
        y = self.mt[self.i]
        self.i += 1
        y ^= (y >> 29) & 0x5555555555555555
        y ^= (y << 17) & 0x71D67FFFEDA60000
        y ^= (y << 37) & 0xFFF7EEE000000000
        y ^= y >> 43
        return y & _MASK


class Rng:
    """The library's random numbers: doubles (x >> 11) * 2^-53, normals by
    Box-Muller on two of them."""

    def __init__(self, seed):
        self.g = MT19937_64(seed)

    def uniform(self, lo=None, hi=None):
        u = float(self.g.next() >> 11) * (1.0 / 9007199254740992.0)
        return u if lo is None else lo + (hi - lo) * u

    def normal(self):
        u1 = self.uniform()
        while u1 <= 0.0:
            u1 = self.uniform()
        u2 = self.uniform()
        return math.sqrt(-2.0 * math.log(u1)) * math.cos(6.283185307179586 * u2)


def random_rotation(r):
    """Haar-uniform rotation: a normalised quaternion of four normals."""
    while True:
        q = [r.normal() for _ in range(4)]
        n2 = 0.0
        for v in q:
            n2 += v * v
        if not n2 < 1e-12:
            break
    inv = 1.0 / math.sqrt(n2)
    w, x, y, z = q[0] * inv, q[1] * inv, q[2] * inv, q[3] * inv
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


_PAIR = ((0, 1, 2), (1, 3, 4), (2, 4, 5))


def _ut(a, b):
    if a > b:
        a, b = b, a
    return (a * 11 - a * a) // 2 + b


def cubic_stiffness(C11, C12, C44, Rs):
    """Major-minor entries (21 per rotation) of the rotated cubic table for
    a stack of rotations Rs (m, 3, 3): C11 on iiii, C44 on ijij (i != j), C12
    on iijj (i != j), rotated entrywise, each major-minor class keeping the
    value of its last (p, q, s, t) in lexicographic order."""
    Rs = np.asarray(Rs, dtype=np.float64).reshape(-1, 3, 3)
    Ct = np.zeros((3, 3, 3, 3))
    for i in range(3):
        for j in range(3):
            for k in range(3):
                for l in range(3):
                    if i == j == k == l:
                        Ct[i, j, k, l] = C11
                    elif i == k and j == l:
                        Ct[i, j, k, l] = C44
                    elif i == j and k == l:
                        Ct[i, j, k, l] = C12
    out = np.zeros((Rs.shape[0], 21))
    for p in range(3):
        for q in range(3):
            for s in range(3):
                for t in range(3):
                    acc = np.zeros(Rs.shape[0])
                    for i in range(3):
                        for j in range(3):
                            for k in range(3):
                                for l in range(3):
                                    acc = acc + Rs[:, p, i] * Rs[:, s, k] * Ct[i, j, k, l] * Rs[:, q, j] * Rs[:, t, l]
                    out[:, _ut(_PAIR[p][q], _PAIR[s][t])] = acc
    return out


def inclusion_iso(n, center=(0.5, 0.5, 0.5), radius=0.25, lam_in=10.0, mu_in=10.0, lam_out=1.0, mu_out=1.0,
                  eps_in=0.01):
    """One spherical inclusion on the unit cube: C (n, n, n, 2) as
    (lambda, mu) per node, F0 (n, n, n) the dilatational eigenstrain, dx."""
    dx = 1.0 / (n - 1)
    i = np.arange(n, dtype=np.float64)
    x = i * dx - center[0]
    y = i * dx - center[1]
    z = i * dx - center[2]
    d = np.sqrt(x[None, None, :] * x[None, None, :] + y[None, :, None] * y[None, :, None]
                + z[:, None, None] * z[:, None, None])
    inside = d < radius
    C = np.empty((n, n, n, 2))
    C[..., 0] = np.where(inside, lam_in, lam_out)
    C[..., 1] = np.where(inside, mu_in, mu_out)
    F0 = np.where(inside, eps_in, 0.0)
    return C, F0, dx


def voronoi_grains(n, nseeds=64, seed=1, C11=1.68, C12=1.21, C44=0.75):
    """Grain id per node (n, n, n) int32 and each grain's 21 stiffness
    entries (nseeds, 21); dx."""
    dx = 1.0 / (n - 1)
    r = Rng(seed)
    Lb = (n - 1) * dx
    sx, sy, sz = np.empty(nseeds), np.empty(nseeds), np.empty(nseeds)
    for s in range(nseeds):
        sx[s] = r.uniform() * Lb
        sy[s] = r.uniform() * Lb
        sz[s] = r.uniform() * Lb
    Rs = np.stack([random_rotation(r) for _ in range(nseeds)])
    Cg = cubic_stiffness(C11, C12, C44, Rs)
    coord = np.arange(n, dtype=np.float64) * dx
    grain = np.empty((n, n, n), dtype=np.int32)
    for k in range(n):
        z = coord[k]
        best = np.zeros((n, n), dtype=np.int32)
        bd = np.full((n, n), 1e300)
        for s in range(nseeds):
            ddx = coord[None, :] - sx[s]
            ddy = coord[:, None] - sy[s]
            ddz = z - sz[s]
            d2 = (ddx * ddx + ddy * ddy) + ddz * ddz
            closer = d2 < bd
            bd = np.where(closer, d2, bd)
            best = np.where(closer, s, best)
        grain[k] = best
    return grain, Cg, dx


def voronoi_cubic(n, nseeds=64, seed=1, C11=1.68, C12=1.21, C44=0.75, with_grain=False):
    """Cubic polycrystal: C (n, n, n, 21) in the reference's major-minor
    storage order, dx (and the grain ids)."""
    grain, Cg, dx = voronoi_grains(n, nseeds, seed, C11, C12, C44)
    C = np.take(Cg, grain, axis=0)
    return (C, dx, grain) if with_grain else (C, dx)


def _place_spheres(r, nspheres, Lb, rmin, rmax, smin, smax):
    sp = []
    max_tries = 1000 * (nspheres + 1)
    t = 0
    while t < max_tries and len(sp) < nspheres:
        t += 1
        c = (r.uniform() * Lb, r.uniform() * Lb, r.uniform() * Lb, r.uniform(rmin, rmax), r.uniform(smin, smax))
        ok = True
        for o in sp:
            ddx, ddy, ddz = c[0] - o[0], c[1] - o[1], c[2] - o[2]
            if ddx * ddx + ddy * ddy + ddz * ddz < (c[3] + o[3]) * (c[3] + o[3]):
                ok = False
                break
        if ok:
            sp.append(c)
    return sp


def spheres_diffuse(n, nspheres=200, seed=3, rmin=0.02, rmax=0.06, eps=None, contrast=10.0, smin=0.0, smax=0.02):
    """Isotropic two-phase medium: non-overlapping spheres (rejection
    sampling) with the diffuse profile 0.5 - 0.5 erf((d^2 - r^2) / (eps d)),
    C = (1 - eta) C_matrix + eta C_sphere (lambda = mu = 1 and contrast),
    F0 = sum of eta times the sphere's eigenstrain; eps defaults to four node
    spacings.  Returns C, F0, dx and the number of spheres placed."""
    from scipy.special import erf
    dx = 1.0 / (n - 1)
    if eps is None:
        eps = 4.0 * dx
    r = Rng(seed)
    sp = _place_spheres(r, nspheres, (n - 1) * dx, rmin, rmax, smin, smax)
    eta = np.zeros((n, n, n))
    f0 = np.zeros((n, n, n))
    coord = np.arange(n, dtype=np.float64) * dx
    for (cx, cy, cz, rad, s) in sp:
        ext = rad + 3.0 * eps
        i0, i1 = max(0, math.floor((cx - ext) / dx)), min(n - 1, math.ceil((cx + ext) / dx))
        j0, j1 = max(0, math.floor((cy - ext) / dx)), min(n - 1, math.ceil((cy + ext) / dx))
        k0, k1 = max(0, math.floor((cz - ext) / dx)), min(n - 1, math.ceil((cz + ext) / dx))
        ddx = coord[i0:i1 + 1] - cx
        ddy = coord[j0:j1 + 1] - cy
        ddz = coord[k0:k1 + 1] - cz
        d2 = (ddx[None, None, :] * ddx[None, None, :] + ddy[None, :, None] * ddy[None, :, None]) \
            + ddz[:, None, None] * ddz[:, None, None]
        d = np.sqrt(d2)
        with np.errstate(divide="ignore", invalid="ignore"):
            e = np.where(d > 0, 0.5 - 0.5 * erf((d * d - rad * rad) / (eps * d)), 1.0)
        eta[k0:k1 + 1, j0:j1 + 1, i0:i1 + 1] += e
        f0[k0:k1 + 1, j0:j1 + 1, i0:i1 + 1] += e * s
    e = np.clip(eta, 0.0, 1.0)
    C = np.empty((n, n, n, 2))
    C[..., 0] = (1.0 - e) * 1.0 + e * contrast
    C[..., 1] = (1.0 - e) * 1.0 + e * contrast
    return C, f0, dx, len(sp)

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

and, at the end, the known-answer problems of the reference's Eshelby,
PlateHole and neo-Hookean tests.
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


# ------------------------------------------------------------------
# Known-answer problems of the reference's regression tests, restated on
# this library's grids; the tests and the benchmark's measurements of the
# psi, nonlinear and AMR paths use them.

def _trapz(x, y):
    return float(np.sum(0.5 * (y[1:] + y[:-1]) * (x[1:] - x[:-1])))


# tests/Eshelby/input
ESHELBY_E, ESHELBY_NU = 210.0, 0.3
ESHELBY_AXES = (1.0, 0.75, 0.5)
ESHELBY_EPS = 0.1
ESHELBY_EIGEN = 0.001


def eshelby_fields(xs, ys=None, zs=None):
    """Stiffness (lambda, mu per node) and dilatational eigenstrain of the
    reference's Eshelby inclusion (see eshelby) at the nodes xs x ys x zs
    (ys, zs default to xs)."""
    from scipy.special import erf
    ys = xs if ys is None else ys
    zs = xs if zs is None else zs
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    a = ESHELBY_AXES
    q = (X / a[0]) ** 2 + (Y / a[1]) ** 2 + (Z / a[2]) ** 2
    norm = np.sqrt((X / a[0] ** 2) ** 2 + (Y / a[1] ** 2) ** 2 + (Z / a[2] ** 2) ** 2)
    del X, Y, Z
    with np.errstate(divide="ignore", invalid="ignore"):
        eta = 0.5 - 0.5 * erf((q - 1.0) / ESHELBY_EPS / norm)
    eta[norm == 0.0] = 1.0
    E, nu = ESHELBY_E, ESHELBY_NU
    C = np.empty(eta.shape + (2,))
    C[..., 0] = E * nu / (1 + nu) / (1 - 2 * nu)
    C[..., 1] = E / 2 / (1 + nu)
    return C, ESHELBY_EIGEN * eta



def eshelby_amr_levels(nvs=(63, 63, 95)):
    """tests/Eshelby with four levels on [-8, 8]^3: level 0 65^3 (spacing
    1/4) and boxes about the origin of nvs valid nodes at spacings 1/8, 1/16
    and 1/32, each lo even (the composite solve's rule), their arrays
    covering the box plus one ghost ring.  The finest box's faces lie outside
    the inclusion's diffuse boundary.  Returns (n0, dx0, boxes, Cs, F0s, hw);
    the boundary condition is zero displacement (bc.Constant())."""
    n0, hw = 65, 8.0
    dx0 = 2 * hw / (n0 - 1)
    xs = -hw + dx0 * np.arange(n0)
    C0, F00 = eshelby_fields(xs)
    Cs, F0s, boxes = [C0], [F00], []
    for l, nv in enumerate(nvs, start=1):
        h = dx0 / 2 ** l
        lo = int(round((hw - h * (nv - 1) / 2) / h))
        lo -= lo % 2
        c = -hw + h * (lo - 1 + np.arange(nv + 2))
        C, F0 = eshelby_fields(c)
        Cs.append(C)
        F0s.append(F0)
        boxes.append((lo, nv))
    return n0, dx0, boxes, Cs, F0s, hw


# tests/PlateHole/input: [-16, 16]^2, a circular void of radius 1 (psi from
# the inverted ellipse IC, eps 0.2), E = 1, nu = 0.3 in plane stress,
# TensionTest uniaxial_stress with disp 0.01, elasticop.small 1e-16
PLATEHOLE_HALF = 16.0
PLATEHOLE_EPS = 0.2
PLATEHOLE_SMALL = 1e-16
# far-field stress of tests/PlateHole/test (the value its Kirsch curves use)
PLATEHOLE_SIG0 = 0.0003075


def platehole(nxy, nz):
    """The reference's 2D plane-stress PlateHole test restated in 3D: a plate
    of nxy^2 x nz nodes over [-16, 16]^2 (cubic cells) whose solution does not
    depend on z.  The z faces are displacement rows for u_z (= 0) and
    traction rows for u_x, u_y (sigma_xz = sigma_yz = 0, i.e. du/dz = 0
    one-sided), so every z-plane carries the 2D plane-strain problem; the
    plane-stress Lame constant lambda 2 mu / (lambda + 2 mu)
    (src/Model/Solid/Linear/Isotropic.H:183-184) then makes it the
    reference's plane-stress problem.  psi is the cell field of
    src/IC/Ellipse.H:58-61 with invert: 1/2 + 1/2 erf((r^2 - 1) / eps / r) at
    cell centres, r the distance from the z axis.  Returns (C, psi, bc, dx)."""
    from scipy.special import erf
    from . import bc as B
    hw = PLATEHOLE_HALF
    dx = 2 * hw / (nxy - 1)
    E, nu = 1.0, 0.3
    lam = E * nu / (1 + nu) / (1 - 2 * nu)
    mu = E / 2 / (1 + nu)
    C = np.empty((nz, nxy, nxy, 2))
    C[..., 0] = lam * (1.0 - lam / (2 * mu + lam))
    C[..., 1] = mu
    xc = -hw + dx * (np.arange(nxy - 1) + 0.5)
    Y, X = np.meshgrid(xc, xc, indexing="ij")
    r = np.sqrt(X ** 2 + Y ** 2)
    psi2 = 0.5 + 0.5 * erf((r ** 2 - 1.0) / PLATEHOLE_EPS / r)
    psi = np.ascontiguousarray(np.broadcast_to(psi2, (nz - 1,) + psi2.shape))
    bc = B.TensionTest("uniaxial_stress", disp=0.01)
    for f in B.FACES:
        if "zlo" in f or "zhi" in f:
            bc.set(f, 2, "displacement", 0.0)
    return C, psi, bc, dx


def kirsch(x, y, a=1.0, s0=PLATEHOLE_SIG0):
    """Kirsch's stresses about a circular hole of radius a in an infinite
    plate under uniaxial tension s0 along x (polar components, rotated to
    xx, yy, xy)."""
    r = np.sqrt(x ** 2 + y ** 2)
    t = np.arctan2(y, x)
    q2, q4 = (a / r) ** 2, (a / r) ** 4
    c2, s2 = np.cos(2 * t), np.sin(2 * t)
    srr = 0.5 * s0 * (1 - q2) + 0.5 * s0 * (1 - 4 * q2 + 3 * q4) * c2
    stt = 0.5 * s0 * (1 + q2) - 0.5 * s0 * (1 + 3 * q4) * c2
    srt = -0.5 * s0 * (1 + 2 * q2 - 3 * q4) * s2
    c, s = np.cos(t), np.sin(t)
    sxx = srr * c * c - 2 * srt * c * s + stt * s * s
    syy = srr * s * s + 2 * srt * c * s + stt * c * c
    sxy = (srr - stt) * s * c + (c * c - s * s) * srt
    return sxx, syy, sxy


def platehole_errors(xs, sxx, syy, sxy, y=2.0):
    """tests/PlateHole/test: along the ray at height y over x in [-16, 16],
    the L2 distance of each stress component from Kirsch's (1000 points,
    the numerical curve interpolated onto them) over |integral of the
    numerical sigma_xx|; the test's tolerance is 0.01."""
    xr = np.linspace(-PLATEHOLE_HALF, PLATEHOLE_HALF, 1000)
    ref = kirsch(xr, np.full_like(xr, y))
    norm = abs(_trapz(xs, sxx))
    return np.array([np.sqrt(_trapz(xr, (np.interp(xr, xs, s) - r) ** 2)) / norm
                     for s, r in zip((sxx, syy, sxy), ref)])


def neohookean_twophase(n, seed=5, disp=0.02):
    """A two-phase NeoHookean cube on the unit cube: (mu, kappa) per node,
    mu 3 (kappa 9) in a central sphere of radius 0.3 and 1 (3) outside, mu
    perturbed by 5 % uniform noise; x faces clamped, the x+ face pulled by
    u_x = disp, the other faces traction-free (TensionTest
    uniaxial_stress_clamp).  Returns (model, bc, dx)."""
    from . import bc as B
    rng = np.random.default_rng(seed)
    x = np.arange(n) / (n - 1)
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    inc = ((X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.5) ** 2) < 0.3 ** 2
    model = np.empty((n, n, n, 2))
    model[..., 0] = np.where(inc, 3.0, 1.0) * (1 + 0.05 * rng.uniform(-1, 1, (n, n, n)))
    model[..., 1] = np.where(inc, 9.0, 3.0)
    return model, B.TensionTest("uniaxial_stress_clamp", disp=disp), 1.0 / (n - 1)

"""Problem set-ups shared by the parity tests (inputs only, no solver)."""
import numpy as np

from alamo_gb300 import bc as B
from alamo_gb300 import synth

SEED = 20261203


def c1(n=33):
    """Config 1: isotropic matrix lambda=mu=1, centred inclusion r=0.25 with
    lambda=mu=10 and eigenstrain 0.01 I, zero displacement on all faces."""
    C, F0, dx = synth.inclusion_iso(n)
    return C, F0, B.Constant(), dx


def voronoi_clamp(n=33, nseeds=64, seed=7, disp=0.01):
    """Config 2 shape: cubic Voronoi polycrystal, uniaxial_stress_clamp."""
    C, dx = synth.voronoi_cubic(n, nseeds, seed=seed)
    return C, None, B.TensionTest("uniaxial_stress_clamp", disp=disp), dx


def random_bc(seed):
    """Every region gets a random type among displacement / traction /
    neumann and a random value: exercises all 26 x 3 boundary rows."""
    rng = np.random.default_rng(seed)
    bc = B.Constant()
    bc.type[:, :] = rng.choice([B.DISPLACEMENT, B.TRACTION, B.NEUMANN], size=(26, 3))
    bc.val[:, :] = rng.uniform(-1, 1, size=(26, 3))
    return bc


def random_field(shape, seed=SEED):
    return synth.uniform(seed, shape)


def iso_as_mm(C):
    """The isotropic tensor written as 21 major-minor entries."""
    lam, mu = C[..., 0], C[..., 1]
    out = np.zeros(C.shape[:-1] + (21,))
    # pair order (00,01,02,11,12,22); C_iijj = lam, C_iiii = lam + 2 mu, C_ijij = mu
    ut = {}
    c = 0
    for a in range(6):
        for b in range(a, 6):
            ut[(a, b)] = c
            c += 1
    diag_pairs = [0, 3, 5]
    shear_pairs = [1, 2, 4]
    for a in diag_pairs:
        for b in diag_pairs:
            if a <= b:
                out[..., ut[(a, b)]] = lam + (2 * mu if a == b else 0)
    for a in shear_pairs:
        out[..., ut[(a, a)]] = mu
    return out


# ------------------------------------------------------------------ Eshelby
from alamo_gb300.workloads import (ESHELBY_AXES, ESHELBY_E, ESHELBY_EIGEN, ESHELBY_EPS, ESHELBY_NU,  # noqa: E402,F401
                                   PLATEHOLE_EPS, PLATEHOLE_HALF, PLATEHOLE_SIG0, PLATEHOLE_SMALL, eshelby_fields,
                                   kirsch, platehole, platehole_errors)


def eshelby(n, half_width):
    """The reference's 3D Eshelby inclusion test (tests/Eshelby/input) on a
    uniform grid of n^3 nodes over [-half_width, half_width]^3: an ellipsoid
    with semi-axes (1, 0.75, 0.5) at the origin and a diffuse boundary of width
    0.1, eta = 1/2 - 1/2 erf((x^T A x - 1) / eps / |A x|) with A = diag(1/a^2)
    (src/IC/Ellipse.H:58-61, A from :124; eta = 1 at the centre, where
    |A x| = 0); E = 210
    and nu = 0.3 inside and out, eigenstrain 0.001 I inside, mixed per node as
    eta model1 + (1 - eta) model2 (src/Integrator/Mechanics.H:241-252), so C is
    uniform and F0 = 0.001 eta I; zero displacement on all faces (the default
    constant BC).  Returns (C, F0, bc, dx)."""
    from scipy.special import erf

    dx = 2.0 * half_width / (n - 1)
    xs = -half_width + dx * np.arange(n)
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    a = ESHELBY_AXES
    q = (X / a[0]) ** 2 + (Y / a[1]) ** 2 + (Z / a[2]) ** 2
    norm = np.sqrt((X / a[0] ** 2) ** 2 + (Y / a[1] ** 2) ** 2 + (Z / a[2] ** 2) ** 2)
    del X, Y, Z
    with np.errstate(divide="ignore", invalid="ignore"):
        eta = 0.5 - 0.5 * erf((q - 1.0) / ESHELBY_EPS / norm)
    eta[norm == 0.0] = 1.0
    E, nu = ESHELBY_E, ESHELBY_NU
    C = np.empty((n, n, n, 2))
    C[..., 0] = E * nu / (1 + nu) / (1 - 2 * nu)
    C[..., 1] = E / 2 / (1 + nu)
    return C, ESHELBY_EIGEN * eta, B.Constant(), dx


def _integrate(x, y):
    return float(np.sum(0.5 * (y[1:] + y[:-1]) * (x[1:] - x[:-1])))


def eshelby_errors(golden, u, sig_normal, half_width, dx):
    """The reference test's error norms (tests/Eshelby/test): along the ray
    x = y = 0.25, z in [-2, 2], the relative L2 error of each displacement
    component and the relative L1 error of each normal stress against the
    analytic curves (displacement in units of 1e-4, stress in units of E/1000).
    The nodal fields are interpolated bilinearly in x, y onto the ray at the
    node planes z.  u: (3, nz, ny, nx); sig_normal: three (nz, ny, nx) arrays
    (sigma_xx, sigma_yy, sigma_zz).  Returns (u errors, sigma errors)."""
    n = u.shape[1]
    xs = -half_width + dx * np.arange(n)
    f = (0.25 + half_width) / dx
    i0 = int(np.floor(f))
    t = f - i0
    w = [((1 - t) * (1 - t), i0, i0), (t * (1 - t), i0, i0 + 1), ((1 - t) * t, i0 + 1, i0), (t * t, i0 + 1, i0 + 1)]

    def ray(fld):
        return sum(c * fld[:, j, i] for c, j, i in w)

    sel = np.abs(xs) <= 2.0 + 1e-12
    z = xs[sel]
    ref = np.array([golden["displacement"][k] for k in ["x", "disp1", "disp2", "disp3"]])
    uerr = []
    for c in range(3):
        exact = ref[c + 1] / 1e4
        d = np.interp(z, ref[0], exact) - ray(u[c])[sel]
        uerr.append(np.sqrt(_integrate(z, d * d) / _integrate(ref[0], exact * exact)))
    ref = np.array([golden["sigma_normal"][k] for k in ["x", "sigma11", "sigma22", "sigma33"]])
    serr = []
    for c in range(3):
        exact = ref[c + 1] * ESHELBY_E / 1000
        d = np.interp(z, ref[0], exact) - ray(sig_normal[c])[sel]
        serr.append(_integrate(z, np.abs(d)) / _integrate(ref[0], np.abs(exact)))
    return np.array(uerr), np.array(serr)


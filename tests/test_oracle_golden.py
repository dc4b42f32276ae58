"""The oracle pinned against the reference's own known answers.

- tests/UniaxialTension of the reference: linear displacement and constant
  stress to 1e-8 (finite differences are exact on linear fields);
- tests/Solid/reference/{linear-cubic,affine-cubic,affine-hexagonal,
  transverselyisotropic}.dat:
  trac_xhi_x(t) of the 4^3 cell tension test to the reference test's
  tolerance 1e-4 (fixture tests/golden/solid_trac_xhi.json, made by
  tests/golden/make_golden.py);
- src/Test/Numeric/Stencil.H:58-106: derivative accuracy below 1e-2 on
  cos(pi x/L) cos(pi y/L) cos(pi z/L) with 32 cells;
- tests/Eshelby/reference/Eshelby_{displacement,sigma_normal}.csv: the
  analytic Eshelby inclusion solution along x = y = 0.25 to the reference
  test's tolerance 0.1 (fixture tests/golden/eshelby.json);
- tests/TrigTest: the Laplacian model's trigonometric solution along the
  diagonal to 1e-4, with second-order convergence.
"""
import json
import os

import numpy as np
import pytest

from alamo_gb300 import bc as B

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

UNIAXIAL_BC = {
    "type.xlo": "disp trac trac", "type.xhi": "disp trac trac", "val.xhi": "0.1 0 0",
    "type.ylo": "trac disp trac", "type.yhi": "trac trac trac", "type.zlo": "trac trac disp",
    "type.zhi": "trac trac trac",
    "type.xloylo": "disp trac trac", "type.xloyhi": "disp trac trac", "type.xhiylo": "disp trac trac",
    "type.xhiyhi": "disp trac trac", "val.xhiylo": "0.1 0 0", "val.xhiyhi": "0.1 0 0",
    "type.zloxlo": "disp trac trac", "type.zhixlo": "disp trac trac", "type.zloxhi": "disp trac trac",
    "type.zhixhi": "disp trac trac", "val.zloxhi": "0.1 0 0", "val.zhixhi": "0.1 0 0",
    "type.ylozlo": "trac disp disp", "type.ylozhi": "trac disp trac", "type.yhizlo": "trac trac disp",
    "type.yhizhi": "trac trac trac",
    "type.xloylozlo": "disp disp disp", "type.xloylozhi": "disp disp trac", "type.xloyhizlo": "disp trac disp",
    "type.xloyhizhi": "disp trac trac",
    "type.xhiylozlo": "disp disp disp", "val.xhiylozlo": "0.1 0 0", "type.xhiylozhi": "disp disp trac",
    "val.xhiylozhi": "0.1 0 0", "type.xhiyhizlo": "disp trac disp", "val.xhiyhizlo": "0.1 0 0",
    "type.xhiyhizhi": "disp trac trac", "val.xhiyhizhi": "0.1 0 0",
}


def uniaxial_problem(n=33):
    L = 16.0
    dx = L / (n - 1)
    E, nu = 210.0, 0.3
    lam = E * nu / (1 + nu) / (1 - 2 * nu)
    mu = E / 2 / (1 + nu)
    C = np.empty((n, n, n, 2))
    C[..., 0] = lam
    C[..., 1] = mu
    return C, B.Constant.parse(UNIAXIAL_BC), dx, E


def test_uniaxial_tension_known_answer(oracle):
    n = 33
    C, bc, dx, E = uniaxial_problem(n)
    bt, bv = bc.tables()
    u0 = np.zeros((3, n, n, n))
    b = oracle.bc_init(np.zeros_like(u0), bt, bv)
    rhs = oracle.build_rhs(C, None, bt, u0, b, dx)
    x, rep, _ = oracle.solve(C, bt, rhs, dx, tol_rel=1e-10, max_iter=200)
    assert rep.status == 0
    xs = -8 + dx * np.arange(n)
    ux = x[0, n // 2, n // 2, :]
    exact = (xs + 8) * 0.1 / 16
    assert np.sum((exact - ux) ** 2) / np.sum(exact ** 2) < 1e-8
    s, _, _ = oracle.stress_strain(C, None, x, dx)
    sig = s[n // 2, n // 2, :, 0]
    assert np.sum((sig - E * 0.1 / 16) ** 2) / np.sum(np.full_like(sig, E * 0.1 / 16) ** 2) < 1e-8


def _integrate(x, y):
    return sum(0.5 * (y[i + 1] + y[i]) * (x[i + 1] - x[i]) for i in range(len(x) - 1))


@pytest.mark.parametrize("name,f0", [("linear-cubic", None), ("affine-cubic", 0.001)])
def test_solid_tension_series(oracle, name, f0):
    with open(os.path.join(GOLDEN, "solid_trac_xhi.json")) as f:
        ref = json.load(f)[name]
    rt, rtr = np.array(ref["time"]), np.array(ref["trac_xhi_x"])
    n, dx = 5, 0.25
    C = np.empty((n, n, n, 21))
    C[...] = oracle.cubic(168.3, 1.221, 0.757, np.eye(3))
    F0 = None if f0 is None else np.full((n, n, n), f0)
    u = np.zeros((3, n, n, n))
    times, trac = [], []
    # the reference input: bc.tensiontest.type = uniaxial_stress,
    # bc.tensiontest.disp = (0,1:0,0.01) (tests/Solid/input)
    bc = B.TensionTest("uniaxial_stress", disp="(0,1:0,0.01)")
    for step in range(100):
        t = 0.01 * step
        bt, bv = bc.tables(t)
        b = oracle.bc_init(np.zeros_like(u), bt, bv)
        rhs = oracle.build_rhs(C, F0, bt, u, b, dx)
        du, rep, _ = oracle.solve(C, bt, rhs, dx, tol_rel=1e-8, tol_abs=1e-8, max_iter=30)
        u = u + du
        s, _, _ = oracle.stress_strain(C, F0, u, dx)
        sxx = s[..., 0]
        tot = 0.0
        for k in range(n - 1):
            for j in range(n - 1):
                tot += 0.25 * (sxx[k, j, n - 1] + sxx[k, j + 1, n - 1] + sxx[k + 1, j, n - 1] +
                               sxx[k + 1, j + 1, n - 1]) * dx * dx
        times.append(t)
        trac.append(tot)
    times, trac = np.array(times), np.array(trac)
    diff = np.interp(times, rt, rtr) - trac
    err = np.sqrt(_integrate(times, diff ** 2)) / np.sqrt(_integrate(rt, rtr * rtr))
    assert err < 1e-4, err


def hexagonal_mm(C11, C12, C13, C33, C44):
    """The 21 major-minor values of Model::Solid::Linear::Hexagonal at zero
    Euler angles (src/Model/Solid/Linear/Hexagonal.H:67-111): C1111 = C2222 =
    C11, C3333 = C33, C1122 = C12, C1133 = C2233 = C13, C2323 = C1313 = C44,
    and C1212 = (C11 - C12) / 2 (the class's last-written entry, (1,0,1,0))."""
    pairs = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    val = {(0, 0, 0, 0): C11, (1, 1, 1, 1): C11, (2, 2, 2, 2): C33, (0, 1, 0, 1): 0.5 * (C11 - C12),
           (0, 2, 0, 2): C44, (1, 2, 1, 2): C44, (0, 0, 1, 1): C12, (0, 0, 2, 2): C13, (1, 1, 2, 2): C13}
    return np.array([val.get(pairs[a] + pairs[b], 0.0) for a in range(6) for b in range(a, 6)])


@pytest.mark.parametrize("name,consts,f0", [
    ("affine-hexagonal", (0.597, 0.262, 0.217, 0.617, 0.164), 0.001),
    ("transverselyisotropic", (168.3, 1.221, 1.0, 160.0, 0.757), None)])
def test_solid_hexagonal_series(oracle, name, consts, f0):
    """tests/Solid [affine-hexagonal] (tests/Solid/input:31-44) and
    [linear-transverse] (:108-120): the same tension test with the hexagonal
    model (eigenstrain 0.001 I: a nonzero traction already at t = 0) and the
    transversely isotropic one (Set::Matrix4<3,MajorMinor>::Transverse,
    src/Set/Matrix4_MajorMinor.H:564-611, the same table) -- major-minor
    tensors with five distinct constants -- against their .dat series to
    1e-4 (1.1e-6 and 1.9e-6)."""
    with open(os.path.join(GOLDEN, "solid_trac_xhi.json")) as f:
        ref = json.load(f)[name]
    rt, rtr = np.array(ref["time"]), np.array(ref["trac_xhi_x"])
    n, dx = 5, 0.25
    C = np.empty((n, n, n, 21))
    C[...] = hexagonal_mm(*consts)
    F0 = None if f0 is None else np.full((n, n, n), f0)
    bc = B.TensionTest("uniaxial_stress", disp="(0,1:0,0.01)")
    u = np.zeros((3, n, n, n))
    times, trac = [], []
    for step in range(100):
        t = 0.01 * step
        bt, bv = bc.tables(t)
        b = oracle.bc_init(np.zeros_like(u), bt, bv)
        rhs = oracle.build_rhs(C, F0, bt, u, b, dx)
        du, rep, _ = oracle.solve(C, bt, rhs, dx, tol_rel=1e-8, tol_abs=1e-8, max_iter=30)
        u = u + du
        s, _, _ = oracle.stress_strain(C, F0, u, dx)
        face = s[..., 0][:, :, n - 1]
        times.append(t)
        trac.append(0.25 * dx * dx * float((face[:-1, :-1] + face[1:, :-1] + face[:-1, 1:] + face[1:, 1:]).sum()))
    times, trac = np.array(times), np.array(trac)
    diff = np.interp(times, rt, rtr) - trac
    err = np.sqrt(_integrate(times, diff ** 2)) / np.sqrt(_integrate(rt, rtr * rtr))
    assert err < 1e-4, err


@pytest.mark.parametrize("which", [100, 10, 1, 200, 20, 2, 110, 101, 11])
def test_stencil_accuracy(oracle, which):
    n = 33
    Lb = 1.0
    dx = Lb / (n - 1)
    x = np.arange(n) * dx
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    k = np.pi / Lb
    order = [which // 100, (which // 10) % 10, which % 10]
    f = np.cos(k * X) * np.cos(k * Y) * np.cos(k * Z)
    exact = np.ones_like(f) * k ** sum(order)
    for coord, o in zip([X, Y, Z], order):
        exact = exact * np.cos(k * coord + o * np.pi / 2)
    d = oracle.derivative(which, f, dx)
    s = (slice(1, -1),) * 3
    assert np.abs(d[s] - exact[s]).max() / np.abs(exact[s]).max() < 1e-2


def test_eshelby_known_answer(oracle):
    """The reference's Eshelby test (tests/Eshelby/test): eigenstrain 0.001 I
    in a diffuse ellipsoid, zero displacement far away; displacement (relative
    L2) and normal stress (relative L1) along x = y = 0.25 within 0.1 of the
    analytic solution.  The reference runs [-8, 8]^3 with AMR down to a
    spacing of 1/32 near the inclusion; here a uniform 129^3 grid over
    [-4, 4]^3 (spacing 1/16).  Measured errors: u 0.017 / 0.019 / 0.029,
    sigma 0.076 / 0.069 / 0.084 (sigma_zz is set by the resolution of the
    0.5-wide z semi-axis, sigma_xx and sigma_yy by the clamped faces)."""
    import problems as P
    with open(os.path.join(GOLDEN, "eshelby.json")) as f:
        golden = json.load(f)
    n, hw = 129, 4.0
    C, F0, bc, dx = P.eshelby(n, hw)
    bt, bv = bc.tables()
    u0 = np.zeros((3, n, n, n))
    b = oracle.bc_init(np.zeros_like(u0), bt, bv)
    rhs = oracle.build_rhs(C, F0, bt, u0, b, dx)
    u, rep, _ = oracle.solve(C, bt, rhs, dx, tol_rel=1e-10, max_iter=100)
    assert rep.status == 0
    s, _, _ = oracle.stress_strain(C, F0, u, dx)
    uerr, serr = P.eshelby_errors(golden, u, [s[..., 0], s[..., 4], s[..., 8]], hw, dx)
    assert np.all(uerr < 0.1), uerr
    assert np.all(serr < 0.1), serr
    # the solution is not trivially small: the inclusion's z displacement
    # reaches 0.8 of its analytic peak on the ray
    assert np.abs(u[2]).max() > 0.8 * np.abs(np.array(golden["displacement"]["disp3"])).max() / 1e4


def _trig_error(oracle, n):
    dx = 1.0 / (n - 1)
    xs = dx * np.arange(n)
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    ut = [(P, Q) for P in range(9) for Q in range(P, 9)]
    C = np.zeros((n, n, n, 45))
    for q, (P, Q) in enumerate(ut):
        if P == Q:
            C[..., q] = 1.0
    bc = B.Constant()
    bt, bv = bc.tables()
    body = np.zeros((3, n, n, n))
    body[0] = np.sin(np.pi * X) * np.sin(np.pi * Y) * np.sin(np.pi * Z)
    b = oracle.bc_init(body, bt, bv)
    rhs = oracle.build_rhs(C, None, bt, np.zeros_like(body), b, dx)
    u, rep, _ = oracle.solve(C, bt, rhs, dx, tol_rel=1e-10, max_iter=100)
    assert rep.status == 0
    d = np.arange(n)
    exact = -np.sin(np.pi * xs) ** 3 / np.pi ** 2 / 3.0
    return np.sum((exact - u[0, d, d, d]) ** 2) / np.sum(exact ** 2)


def test_trig_known_answer(oracle):
    """The reference's TrigTest (tests/TrigTest/input, tests/TrigTest/test):
    the Laplacian model (DDW = alpha, alpha = 1) with the body force
    b_x = sin(pi x) sin(pi y) sin(pi z) on the unit cube, zero displacement
    on every face; u_x must match -sin(pi x) sin(pi y) sin(pi z) / (3 pi^2)
    along the diagonal x = y = z with relative squared error < 1e-4.  The
    Laplacian's stiffness C_ijkl = delta_ik delta_jl has major but not minor
    symmetry, so it runs as the 45-value Major tensor with C_PQ = delta_PQ.
    The reference refines two levels on an explicit mesh; here uniform grids
    of 33^3 and 65^3 nodes: errors 6.5e-7 and 4.0e-8, the factor 16 of a
    second-order discretisation in the squared error."""
    e33, e65 = _trig_error(oracle, 33), _trig_error(oracle, 65)
    assert e33 < 1e-4 and e65 < 1e-4, (e33, e65)
    assert 12 < e33 / e65 < 20

"""Finite-deformation Newton path: Operator::Elastic<Sym::Major> (45 stiffness
values per node, Matrix4_Major.H:274-541) and Model::Solid::Finite::NeoHookean
(NeoHookean.H:21-121) inside Solver::Nonlocal::Newton with nriters > 1
(Newton.H:144-266, 319-355).

CPU: the oracle's NeoHookean against finite differences of its own energy and
stress; the Major contraction against the major-minor one on a minor-symmetric
tensor.  GPU: the Major operator at every level and the Newton loop against
the oracle's."""
import numpy as np
import pytest

import problems as P
from alamo_gb300 import bc as B


def mm_to_major(Cmm, oracle):
    """21 major-minor values -> 45 Major values of the same tensor."""
    pair = np.array([[0, 1, 2], [1, 3, 4], [2, 4, 5]])
    ut = np.zeros((6, 6), int)
    c = 0
    for a in range(6):
        for b in range(a, 6):
            ut[a, b] = ut[b, a] = c
            c += 1
    out = np.empty(Cmm.shape[:-1] + (45,))
    q = 0
    for P_ in range(9):
        for Q in range(P_, 9):
            i, j, k, l = P_ // 3, P_ % 3, Q // 3, Q % 3
            out[..., q] = Cmm[..., ut[pair[i, j], pair[k, l]]]
            q += 1
    return out


def random_F(rng, amp=0.1):
    return np.eye(3) + amp * rng.uniform(-1, 1, (3, 3))


def test_neohookean_dw_is_the_gradient_of_w(oracle):
    rng = np.random.default_rng(1)
    h = 1e-6
    for _ in range(5):
        F = random_F(rng)
        mu, kappa = rng.uniform(0.5, 2.0, 2)
        _, dw, _ = oracle.neohookean(mu, kappa, F)
        fd = np.zeros((3, 3))
        for a in range(3):
            for b in range(3):
                Fp, Fm = F.copy(), F.copy()
                Fp[a, b] += h
                Fm[a, b] -= h
                fd[a, b] = (oracle.neohookean(mu, kappa, Fp)[0] - oracle.neohookean(mu, kappa, Fm)[0]) / (2 * h)
        assert np.abs(dw - fd).max() <= 1e-7 * max(1.0, np.abs(dw).max())


def test_neohookean_ddw_is_the_gradient_of_dw(oracle):
    rng = np.random.default_rng(2)
    h = 1e-6
    for _ in range(5):
        F = random_F(rng)
        mu, kappa = rng.uniform(0.5, 2.0, 2)
        _, _, ddw = oracle.neohookean(mu, kappa, F)
        full = np.zeros((3, 3, 3, 3))
        for k in range(3):
            for l in range(3):
                Fp, Fm = F.copy(), F.copy()
                Fp[k, l] += h
                Fm[k, l] -= h
                full[:, :, k, l] = (oracle.neohookean(mu, kappa, Fp)[1] - oracle.neohookean(mu, kappa, Fm)[1]) / (2 * h)
        q = 0
        for P_ in range(9):
            for Q in range(P_, 9):
                i, j, k, l = P_ // 3, P_ % 3, Q // 3, Q % 3
                assert abs(ddw[q] - full[i, j, k, l]) <= 1e-6 * max(1.0, np.abs(full).max()), (q, ddw[q])
                q += 1


def test_neohookean_material_frame_indifference(oracle):
    """Model::Solid::Solid::MaterialFrameIndifference (src/Model/Solid/
    Solid.H:210-268): W(R F) = W(F) for rotations R and det F in [0.5, 2],
    relative to |W(RF) + W(F)| + 1e-4, tolerance 1e-4 (here far below it)."""
    rng = np.random.default_rng(3)
    for _ in range(10):
        F = rng.uniform(-1, 1, (3, 3))
        while not 0.5 <= np.linalg.det(F) <= 2.0:
            F = rng.uniform(-1, 1, (3, 3))
        mu, kappa = rng.uniform(0.5, 2.0, 2)
        w0 = oracle.neohookean(mu, kappa, F)[0]
        for _ in range(10):
            q = rng.normal(size=4)
            q /= np.linalg.norm(q)
            a, b, c, d = q
            R = np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                          [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                          [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])
            w = oracle.neohookean(mu, kappa, R @ F)[0]
            assert abs(w - w0) / abs(w + w0 + 1e-4) <= 1e-10


def test_solid_neo_hookean_series(oracle):
    """The reference's tests/Solid [neo-hookean] case (tests/Solid/input:69-82,
    tests/Solid/test): a 4^3-cell unit cube of NeoHookean material mu = 3.0,
    kappa = 6.5 under the uniaxial_stress tension test with
    bc.tensiontest.disp = (0,1:0,1), 100 steps of 0.01, solver.nriters = 10;
    trac_xhi_x(t) -- the first Piola-Kirchhoff P_xx integrated over the x+
    face -- against tests/Solid/reference/neo-hookean.dat (fixture
    tests/golden/solid_trac_xhi.json) to the reference test's 1e-4: the
    oracle's NeoHookean DW/DDW, Major operator, Newton right-hand side and
    Newton loop reach 9e-7 up to a stretch of 2."""
    import json
    import os
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "solid_trac_xhi.json")) as f:
        ref = json.load(f)["neo-hookean"]
    rt, rtr = np.array(ref["time"]), np.array(ref["trac_xhi_x"])
    n, dx = 5, 0.25
    model = np.empty((n, n, n, 2))
    model[..., 0], model[..., 1] = 3.0, 6.5
    bc = B.TensionTest("uniaxial_stress", disp="(0,1:0,1)")
    u = np.zeros((3, n, n, n))
    times, trac = [], []
    for step in range(100):
        t = 0.01 * step
        bt, bv = bc.tables(t)
        b = oracle.bc_init(np.zeros_like(u), bt, bv)
        du = np.zeros_like(u)
        for _ in range(10):
            dw, ddw = oracle.neohookean_field(model, u, dx)
            rhs = oracle.rhs_dw(dw, bt, u, b, dx)
            du, rep, _ = oracle.solve(np.ascontiguousarray(ddw), bt, rhs, dx, tol_rel=1e-8, tol_abs=1e-8,
                                      max_iter=30, x0=du)
            u = u + du
        pxx = oracle.neohookean_field(model, u, dx)[0][..., 0]
        face = pxx[:, :, n - 1]
        times.append(t)
        trac.append(0.25 * dx * dx * float((face[:-1, :-1] + face[1:, :-1] + face[:-1, 1:] + face[1:, 1:]).sum()))
    times, trac = np.array(times), np.array(trac)

    def integrate(x, y):
        return float(np.sum(0.5 * (y[1:] + y[:-1]) * (x[1:] - x[:-1])))
    diff = np.interp(times, rt, rtr) - trac
    err = np.sqrt(integrate(times, diff ** 2)) / np.sqrt(integrate(rt, rtr * rtr))
    assert err < 1e-4, err


def test_major_operator_equals_major_minor_on_minor_symmetric_tensor(oracle):
    """The same (minor-symmetric) tensor in Major storage gives the major-minor
    operator's rows and diagonal."""
    n = 9
    C, F0, bc, dx = P.voronoi_clamp(n)
    Cmaj = np.ascontiguousarray(mm_to_major(C, oracle))
    bt, _ = P.random_bc(3).tables()
    u = P.random_field((3, n, n, n), 4)
    for f_mm, f_maj in ((oracle.fapply(C, bt, u, dx), oracle.fapply(Cmaj, bt, u, dx)),
                        (oracle.diagonal(C, bt, dx), oracle.diagonal(Cmaj, bt, dx))):
        assert np.abs(f_maj - f_mm).max() <= 1e-12 * np.abs(f_mm).max()
    assert np.abs(mm_to_major(oracle.restrict_C(C), oracle) - oracle.restrict_C(Cmaj)).max() <= 1e-15


def neo_problem(n, seed=5, disp=0.02):
    """A two-phase NeoHookean cube (mu, kappa per node), x faces clamped, x+
    face pulled by u_x = disp, other faces traction-free
    (workloads.neohookean_twophase)."""
    from alamo_gb300.workloads import neohookean_twophase
    return neohookean_twophase(n, seed, disp)


def oracle_newton(oracle, model, bc, dx, nriters, tol=1e-10):
    n = model.shape[0]
    bt, bv = bc.tables()
    u = np.zeros((3, n, n, n))
    b = oracle.bc_init(u, bt, bv)
    hist = []
    for _ in range(nriters):
        dw, ddw = oracle.neohookean_field(model, u, dx)
        rhs = oracle.rhs_dw(dw, bt, u, b, dx)
        du, rep, _ = oracle.solve(np.ascontiguousarray(ddw), bt, rhs, dx, tol_rel=tol, max_iter=200,
                                  bottom_solver=1, max_coarsening_level=oracle.num_levels(n, n, n) - 2)
        assert rep.status == 0
        u = u + du
        hist.append(np.abs(du).max())
    return u, hist


def test_oracle_newton_neohookean_converges(oracle):
    """The Newton increments shrink on a 17^3 two-phase cube.  The tangent is
    the operator with C = DDW (non-divergence form) while the residual
    differentiates the nodal stress DW by central differences, so the
    reference's iteration is an inexact Newton method: linear, not quadratic,
    convergence after the first step."""
    model, bc, dx = neo_problem(17)
    u, hist = oracle_newton(oracle, model, bc, dx, 4)
    assert hist[1] < 0.05 * hist[0], hist
    assert all(b < a for a, b in zip(hist, hist[1:])), hist


@pytest.mark.gpu
def test_gpu_major_operator_all_levels(agb, oracle):
    n = 17
    model, bc, dx = neo_problem(n)
    rng = np.random.default_rng(8)
    u0 = 0.01 * P.random_field((3, n, n, n), 9)
    _, ddw = oracle.neohookean_field(model, u0, dx)
    C = np.ascontiguousarray(ddw)
    bt, _ = P.random_bc(21).tables()
    bcx = P.random_bc(21)
    with agb.Elastic(n, dx, "major") as op:
        op.SetModel(C)
        op.SetBC(bcx)
        op.prepareForSolve()
        Cl, dxl = C, dx
        for lev in range(op.num_levels()):
            if lev > 0:
                Cl = oracle.restrict_C(Cl)
                dxl = 2 * dxl
            nz = Cl.shape[0]
            u = P.random_field((3, nz, nz, nz), 30 + lev)
            f = op.Fapply(u, level=lev)
            ref = oracle.fapply(Cl, bt, u, dxl)
            assert np.abs(f - ref).max() <= 1e-12 * np.abs(ref).max()
            d = op.Diagonal(lev)
            dref = oracle.diagonal(Cl, bt, dxl)
            assert np.abs(d - dref).max() <= 1e-12 * np.abs(dref).max()
        b = P.random_field((3, n, n, n), 40)
        r, _ = op.residual(u0, b)
        rref, _ = oracle.residual(C, bt, u0, b, dx)
        assert np.abs(r - rref).max() <= 1e-12 * np.abs(rref).max()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_newton_neohookean_matches_oracle(agb, oracle, precision):
    """agb_newton_solve_neohookean: each iteration evaluates DW and DDW at
    F = I + grad u on the GPU, solves for the increment and adds it; after
    four iterations the displacement matches the oracle's loop."""
    n = 17
    model, bc, dx = neo_problem(n)
    uo, hist = oracle_newton(oracle, model, bc, dx, 4)
    opts = agb.default_opts(precision=precision, solver="fgmres", bottom_solver="direct", max_coarsening_level=1)
    with agb.Elastic(n, dx, "major", opts) as op:
        op.SetBC(bc)
        b = op.bc_init()
        u = np.zeros((3, n, n, n))
        rep = agb.Newton(op, nriters=4).solve_neohookean(np.ascontiguousarray(model), u, b, tol_rel=1e-10)
    assert np.abs(u - uo).max() <= 1e-7 * np.abs(uo).max()
    assert abs(rep["relnorm"] - hist[-1]) <= 1e-3 * hist[0]

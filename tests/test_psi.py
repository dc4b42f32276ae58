"""psi, the void indicator of Operator::Elastic (Elastic.cpp:118-137,
191-260, 341-363, 839-905) and of the Newton right-hand side
(Newton.H:236-263).

CPU tests pin the oracle's psi terms against numpy restatements built from
its own psi-free operator: with psi, interior rows are
psi_avg * (rows without psi) + (1 - small) (C grad u) grad psi, traction rows
scale by psi_avg, displacement rows do not change, and the coarse-level psi is
the reference's full weighting (low-side boundary forms only).  GPU tests
compare the CUDA path with the oracle at every multigrid level and through
whole solves.
"""
import numpy as np
import pytest

import problems as P
from alamo_gb300 import bc as B

SMALL = 1e-8


def psi_void(n, centre=(0.55, 0.45, 0.5), radius=0.22, width=0.06, floor=0.05):
    """Cell field (n-1)^3 of a smooth spherical void: ~floor inside, 1 outside."""
    h = 1.0 / (n - 1)
    x = (np.arange(n - 1) + 0.5) * h
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    r = np.sqrt((X - centre[0]) ** 2 + (Y - centre[1]) ** 2 + (Z - centre[2]) ** 2)
    return floor + (1 - floor) * (0.5 + 0.5 * np.tanh((r - radius) / width))


def psi_random(shape, seed):
    return np.random.default_rng(seed).uniform(0.1, 1.0, shape)


def _ghosted(psi):
    g = np.ones(tuple(s + 2 for s in psi.shape))
    g[1:-1, 1:-1, 1:-1] = psi
    return g


def node_avg_grad(psi, dx):
    """avg8 and CellGradientOnNode of a cell field at every node (numpy)."""
    g = _ghosted(psi)
    # node (k, j, i) sees ghosted entries [k..k+1, j..j+1, i..i+1]
    c = {}
    for a in (0, 1):
        for b in (0, 1):
            for d in (0, 1):
                c[(a, b, d)] = g[d:d + g.shape[0] - 1, b:b + g.shape[1] - 1, a:a + g.shape[2] - 1]
    avg = sum(c.values()) / 8.0
    gx = 0.25 * sum(c[(1, b, d)] - c[(0, b, d)] for b in (0, 1) for d in (0, 1)) / dx
    gy = 0.25 * sum(c[(a, 1, d)] - c[(a, 0, d)] for a in (0, 1) for d in (0, 1)) / dx
    gz = 0.25 * sum(c[(a, b, 1)] - c[(a, b, 0)] for a in (0, 1) for b in (0, 1)) / dx
    return avg, np.stack([gx, gy, gz])


def coarsen_numpy(pf):
    """The reference's psi coarsening written out independently (dict of
    offsets, no shared code with the oracle)."""
    nzf, nyf, nxf = pf.shape
    nc = ((nzf) // 2, (nyf) // 2, (nxf) // 2)
    out = np.empty(nc)
    w1 = {-1: 1.0, 0: 2.0, 1: 1.0}
    for K in range(nc[0]):
        for J in range(nc[1]):
            for I in range(nc[2]):
                k, j, i = 2 * K, 2 * J, 2 * I
                lo = (I == 0, J == 0, K == 0)
                axes = [d for d in range(3) if not lo[d]]  # axes that are averaged
                tot, wsum = 0.0, 0.0
                for dz in ((-1, 0, 1) if 2 in axes else (0,)):
                    for dy in ((-1, 0, 1) if 1 in axes else (0,)):
                        for dxo in ((-1, 0, 1) if 0 in axes else (0,)):
                            w = w1[dz] * w1[dy] * w1[dxo]
                            tot += w * pf[k + dz, j + dy, i + dxo]
                            wsum += w
                out[K, J, I] = tot / wsum
    return out


def spheres_void(n):
    """Six diffuse-interface isotropic spheres (contrast 10, eigenstrain up
    to 0.02), clamped faces, and the smooth void of psi_void."""
    from alamo_gb300 import synth
    C, F0, dx = synth.spheres_diffuse(n, 6, 3, 0.1, 0.2)[:3]
    return (C, F0, B.Constant(), dx), psi_void(n)


def traction_bc():
    """Traction rows on every boundary region."""
    bc = B.Constant()
    bc.type[:, :] = B.TRACTION
    return bc


def interior(n):
    m = np.zeros((n, n, n), bool)
    m[1:-1, 1:-1, 1:-1] = True
    return m


# ------------------------------------------------------------------ oracle
@pytest.fixture
def psi_oracle(oracle):
    yield oracle
    oracle.set_psi(None)


@pytest.mark.parametrize("mm", [False, True])
def test_oracle_fapply_psi_terms(psi_oracle, mm):
    O = psi_oracle
    n = 13
    C, F0, bc, dx = P.voronoi_clamp(n) if mm else P.c1(n)
    bt, _ = bc.tables()
    u = P.random_field((3, n, n, n), seed=3)
    psi = psi_random((n - 1,) * 3, 4)
    O.set_psi(None)
    f0 = O.fapply(C, bt, u, dx)
    stress, _, _ = O.stress_strain(C, None, u, dx)
    O.set_psi(psi, SMALL)
    f1 = O.fapply(C, bt, u, dx)
    avg, gp = node_avg_grad(psi, dx)
    pa = (1 - SMALL) * avg + SMALL
    sg = stress.reshape(n, n, n, 3, 3)
    extra = np.einsum("zyxrq,qzyx->rzyx", sg, gp) * (1 - SMALL)
    m = interior(n)
    expect = pa * f0 + extra
    assert np.abs(f1[:, m] - expect[:, m]).max() <= 1e-11 * np.abs(expect[:, m]).max()
    # displacement rows ignore psi
    b = ~m
    db, _ = B.Constant().tables()
    O.set_psi(None)
    d0 = O.fapply(C, db, u, dx)
    O.set_psi(psi, SMALL)
    assert np.array_equal(O.fapply(C, db, u, dx)[:, b], d0[:, b])
    # traction rows scale with psi_avg
    tb, _ = traction_bc().tables()
    O.set_psi(None)
    t0 = O.fapply(C, tb, u, dx)
    O.set_psi(psi, SMALL)
    t1 = O.fapply(C, tb, u, dx)
    assert np.abs(t1[:, b] - (pa * t0)[:, b]).max() <= 1e-13 * np.abs(t0[:, b]).max()


def test_oracle_diagonal_psi(psi_oracle):
    O = psi_oracle
    n = 11
    C, F0, _, dx = P.voronoi_clamp(n)
    bc = B.Constant()
    psi = psi_random((n - 1,) * 3, 5)
    avg, _ = node_avg_grad(psi, dx)
    pa = (1 - SMALL) * avg + SMALL
    for bcx in (bc, traction_bc()):
        bt, _ = bcx.tables()
        O.set_psi(None)
        d0 = O.diagonal(C, bt, dx)
        O.set_psi(psi, SMALL)
        d1 = O.diagonal(C, bt, dx)
        m = interior(n)
        assert np.abs(d1[:, m] - pa[m] * d0[:, m]).max() <= 1e-14 * np.abs(d0[:, m]).max()
        if bcx is bc:
            assert np.array_equal(d1[:, ~m], d0[:, ~m])
        else:
            assert np.abs(d1[:, ~m] - (pa * d0)[:, ~m]).max() <= 1e-14 * np.abs(d0[:, ~m]).max()


@pytest.mark.parametrize("cells", [(8, 8, 8), (16, 8, 4), (4, 12, 8)])
def test_oracle_coarsen_psi(psi_oracle, cells):
    pf = psi_random(cells[::-1], 6)
    pc = psi_oracle.coarsen_psi(pf)
    assert np.abs(pc - coarsen_numpy(pf)).max() <= 1e-15
    # every stencil's weights sum to one
    const = np.full(cells[::-1], 0.37)
    assert np.abs(psi_oracle.coarsen_psi(const) - 0.37).max() <= 1e-15


def test_oracle_newton_rhs_psi(psi_oracle):
    O = psi_oracle
    n = 13
    C, F0, bc, dx = P.c1(n)
    bt, bv = bc.tables()
    u = P.random_field((3, n, n, n), seed=8) * 1e-3
    b = O.bc_init(np.zeros((3, n, n, n)), bt, bv)
    psi = psi_random((n - 1,) * 3, 9)
    O.set_psi(None)
    r0 = O.build_rhs(C, F0, bt, u, b, dx)
    stress, _, _ = O.stress_strain(C, F0, u, dx)
    O.set_psi(psi, SMALL)
    r1 = O.build_rhs(C, F0, bt, u, b, dx)
    avg, gp = node_avg_grad(psi, dx)
    m = interior(n)
    divdw = b - r0
    expect = b - (avg * divdw + np.einsum("zyxrq,qzyx->rzyx", stress.reshape(n, n, n, 3, 3), gp))
    assert np.abs(r1[:, m] - expect[:, m]).max() <= 1e-11 * np.abs(expect[:, m]).max()
    assert np.array_equal(r1[:, ~m], r0[:, ~m])


def test_oracle_solve_with_void_converges(psi_oracle):
    """Diffuse-interface stiffness with a void: the reference's V-cycles
    converge about as fast as without psi."""
    O = psi_oracle
    n = 17
    (C, F0, bc, dx), psi = spheres_void(n)
    bt, bv = bc.tables()
    b = O.bc_init(np.zeros((3, n, n, n)), bt, bv)
    iters = []
    for p in (None, psi):
        O.set_psi(p, SMALL)
        rhs = O.build_rhs(C, F0, bt, np.zeros((3, n, n, n)), b, dx)
        x, rep, hist = O.solve(C, bt, rhs, dx, tol_rel=1e-10, max_iter=100)
        assert rep.status == 0, (rep.status, hist[-3:])
        r, _ = O.residual(C, bt, x, rhs, dx)
        assert np.abs(r).max() <= 1e-9 * np.abs(rhs).max()
        iters.append(rep.iters)
    assert iters[1] <= iters[0] + 5, iters


def test_oracle_void_on_sharp_inclusion_diverges(psi_oracle):
    """A sharp 10x stiffness jump (the centred inclusion) with even a 1 %
    psi variation makes the reference's Jacobi-smoothed V-cycle diverge: the
    (C grad u) grad psi rows are first-order terms on top of the
    non-divergence-form operator.  The same void on diffuse stiffness
    converges (previous test)."""
    O = psi_oracle
    n = 17
    C, F0, bc, dx = P.c1(n)
    bt, bv = bc.tables()
    O.set_psi(psi_void(n, floor=0.99), SMALL)
    b = O.bc_init(np.zeros((3, n, n, n)), bt, bv)
    rhs = O.build_rhs(C, F0, bt, np.zeros((3, n, n, n)), b, dx)
    x, rep, hist = O.solve(C, bt, rhs, dx, tol_rel=1e-10, max_iter=40)
    assert rep.status != 0 and hist[-1] > hist[0]


# ------------------------------------------------------------------ GPU
def make_op(agb, C, bc, dx, psi, **kw):
    n = C.shape[2], C.shape[1], C.shape[0]
    op = agb.Elastic(n, dx, "isotropic" if C.shape[-1] == 2 else "majorminor", agb.default_opts(**kw))
    op.SetModel(np.ascontiguousarray(C))
    op.SetBC(bc)
    op.SetPsi(np.ascontiguousarray(psi), SMALL)
    return op


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max()


GCASES = {
    "iso-void": lambda: (P.c1(33), psi_void(33)),
    "spheres-void": lambda: spheres_void(33),
    "mm-random": lambda: (P.voronoi_clamp(33), psi_random((32, 32, 32), 21)),
    "mm-randbc": lambda: ((P.voronoi_clamp(17)[0], None, P.random_bc(12), P.voronoi_clamp(17)[3]),
                          psi_random((16, 16, 16), 22)),
}


@pytest.mark.gpu
@pytest.mark.parametrize("case", list(GCASES))
def test_gpu_psi_operator_all_levels(agb, psi_oracle, case):
    (C, F0, bc, dx), psi = GCASES[case]()
    O = psi_oracle
    bt, _ = bc.tables()
    with make_op(agb, C, bc, dx, psi) as op:
        op.prepareForSolve()
        Cl, dxl, pl = C, dx, psi
        for lev in range(op.num_levels()):
            if lev > 0:
                Cl = O.restrict_C(Cl)
                dxl = 2 * dxl
                pl = O.coarsen_psi(pl)
            O.set_psi(pl, SMALL)
            nz, ny, nx = Cl.shape[:3]
            u = P.random_field((3, nz, ny, nx), seed=30 + lev)
            assert rel(op.Diagonal(lev), O.diagonal(Cl, bt, dxl)) <= 1e-12
            assert rel(op.Fapply(u, level=lev), O.fapply(Cl, bt, u, dxl)) <= 1e-12
            if lev == 0:
                assert rel(op.Fapply_f32(u.astype(np.float32)), O.fapply(Cl, bt, u, dxl)) <= 2e-6
                b = P.random_field((3, nz, ny, nx), seed=40)
                dg = O.diagonal(Cl, bt, dxl)
                x = op.Fsmooth(u.copy(), b, ncalls=2)
                assert rel(x, O.fsmooth(Cl, bt, dg, u, b, dxl, ncalls=2)) <= 1e-12
                r = op.residual(u, b)
                r = r[0] if isinstance(r, tuple) else r
                assert rel(r, O.residual(Cl, bt, u, b, dxl)[0]) <= 1e-12


@pytest.mark.gpu
def test_gpu_psi_newton_rhs(agb, psi_oracle):
    n = 33
    C, F0, bc, dx = P.c1(n)
    psi = psi_void(n)
    bt, bv = bc.tables()
    u = P.random_field((3, n, n, n), seed=50) * 1e-3
    with make_op(agb, C, bc, dx, psi) as op:
        b = op.bc_init()
        rhs = op.build_rhs(u, b, F0)
    psi_oracle.set_psi(psi, SMALL)
    ref = psi_oracle.build_rhs(C, F0, bt, u, b, dx)
    assert rel(rhs, ref) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("precision,solver", [("fp64", "vcycle"), ("mixed", "fgmres")])
def test_gpu_psi_solve_matches_oracle(agb, psi_oracle, precision, solver):
    """Newton step with a void: the GPU solve (the reference's V-cycles in
    FP64, or FGMRES in mixed precision) reaches the oracle's solution."""
    n = 33
    (C, F0, bc, dx), psi = spheres_void(n)
    bt, bv = bc.tables()
    with make_op(agb, C, bc, dx, psi, precision=precision, solver=solver) as op:
        b = op.bc_init()
        u = np.zeros((3, n, n, n))
        agb.Newton(op).solve(u, b, F0, tol_rel=1e-10, tol_abs=0.0)
    O = psi_oracle
    O.set_psi(psi, SMALL)
    rhs = O.build_rhs(C, F0, bt, np.zeros((3, n, n, n)), b, dx)
    x, rep, _ = O.solve(C, bt, rhs, dx, tol_rel=1e-10, max_iter=100)
    assert rep.status == 0
    assert rel(u, x) <= 1e-7
    # the void changes the answer
    O.set_psi(None)
    x0, _, _ = O.solve(C, bt, O.build_rhs(C, F0, bt, np.zeros((3, n, n, n)), b, dx), dx, tol_rel=1e-10)
    assert rel(x0, x) > 1e-3


@pytest.mark.gpu
def test_gpu_psi_cleared_restores_fast_path(agb, oracle):
    """SetPsi(None) returns the operator to the psi-free result (and the FP32
    levels to the z-marching kernels)."""
    n = 33
    C, F0, bc, dx = P.voronoi_clamp(n)
    bt, _ = bc.tables()
    u = P.random_field((3, n, n, n), seed=60)
    with make_op(agb, C, bc, dx, psi_void(n), precision="mixed") as op:
        op.prepareForSolve()
        op.SetPsi(None)
        op.prepareForSolve()
        assert rel(op.Fapply(u), oracle.fapply(C, bt, u, dx)) <= 1e-12
        assert rel(op.Fapply_f32(u.astype(np.float32)), oracle.fapply(C, bt, u, dx)) <= 2e-6


@pytest.mark.gpu
@pytest.mark.parametrize("mm", [False, True])
def test_gpu_operator_stress_strain(agb, psi_oracle, mm):
    """Elastic::Stress = (C grad u) psi_avg and Elastic::Strain = sym grad u
    in the MultiFab layout, 9 components or the reference's Voigt order
    (00, 11, 22, 12, 20, 01), with and without psi."""
    n = 17
    C, F0, bc, dx = P.voronoi_clamp(n) if mm else P.c1(n)
    u = P.random_field((3, n, n, n), seed=70)
    psi = psi_random((n - 1,) * 3, 71)
    stress, strain, _ = psi_oracle.stress_strain(C, None, u, dx)
    sg = stress.reshape(n, n, n, 3, 3)
    ep = strain.reshape(n, n, n, 3, 3)
    avg, _ = node_avg_grad(psi, dx)
    pa = (1 - SMALL) * avg + SMALL
    voigt_idx = [(0, 0), (1, 1), (2, 2), (1, 2), (2, 0), (0, 1)]
    with make_op(agb, C, bc, dx, psi) as op:
        for use_psi in (True, False):
            if not use_psi:
                op.SetPsi(None)
            scale = pa if use_psi else 1.0
            s9 = op.OpStress(u)
            e9 = op.OpStrain(u)
            s6 = op.OpStress(u, voigt=True)
            e6 = op.OpStrain(u, voigt=True)
            for p in range(3):
                for q in range(3):
                    assert rel(s9[3 * p + q], sg[..., p, q] * scale) <= 1e-13
                    assert rel(e9[3 * p + q], ep[..., p, q]) <= 1e-13
            for c, (p, q) in enumerate(voigt_idx):
                assert np.array_equal(s6[c], s9[3 * p + q])
                assert np.array_equal(e6[c], e9[3 * p + q])

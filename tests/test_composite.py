"""The multi-level (AMR) composite solve, restated on the oracle
(oracle/composite.py) and run by the library (agb_composite_*), against the
reference's two AMR known answers:

- tests/UniaxialTension (three levels, a linear displacement and a constant
  stress, relative squared error < 1e-8);
- tests/Eshelby (four levels around the inclusion; displacement and normal
  stress along x = y = 0.25 within 0.1 of the analytic solution): 65^3 over
  [-8, 8]^3 and boxes of 63^3, 63^3 and 95^3 valid nodes at spacings 1/8,
  1/16 and 1/32.

The GPU tests compare the library's composite solution with the oracle's
(the same iteration in FP64) and repeat the known-answer gates on it.
"""
import json
import os
import sys

import numpy as np
import pytest

import problems as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def _cp():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import composite as CP
    return CP


def uniaxial_levels():
    """tests/UniaxialTension: [-8, 8]^3, 32 cells on level 0, two nested
    boxes (31 valid nodes each) at spacings 1/4 and 1/8."""
    from test_oracle_golden import uniaxial_problem
    C0, bc, dx0, E = uniaxial_problem(33)
    boxes = [(16, 31), (48, 31)]
    Cs = [C0]
    for l, (lo, nv) in enumerate(boxes, start=1):
        n = nv + 2
        C = np.empty((n, n, n, 2))
        C[..., 0] = C0[0, 0, 0, 0]
        C[..., 1] = C0[0, 0, 0, 1]
        Cs.append(C)
    return 33, dx0, boxes, Cs, [None] * 3, bc, E


def eshelby_levels(nvs=(63, 63, 95)):
    """tests/Eshelby on [-8, 8]^3 with four levels: level 0 65^3 (spacing
    1/4) and boxes about the origin of 63 valid nodes from -4 (spacing 1/8),
    63 from -2 (1/16) and 95 from -1.5 (1/32) (workloads.eshelby_amr_levels).
    The finest box's faces lie outside the inclusion's diffuse boundary
    (semi-axes 1, 0.75, 0.5, width 0.1), as the reference's gradient tagging
    keeps them."""
    from alamo_gb300 import bc as B
    from alamo_gb300.workloads import eshelby_amr_levels
    n0, dx0, boxes, Cs, F0s, hw = eshelby_amr_levels(nvs)
    return n0, dx0, boxes, Cs, F0s, B.Constant(), hw


def oracle_composite(oracle, n0, dx0, boxes, Cs, F0s, bc, tol, max_iter=80):
    CP = _cp()
    bt, bv = bc.tables()
    from alamo_gb300 import bc as B
    rbt, rbv = B.Constant().tables()
    levels = [CP.Level((n0,) * 3, dx0, None, (n0,) * 3, Cs[0], bt, bv)]
    for l, (lo, nv) in enumerate(boxes, start=1):
        levels.append(CP.Level((nv + 2,) * 3, dx0 / 2 ** l, (lo,) * 3, (nv,) * 3, Cs[l], rbt, rbv))
    opts = oracle.default_opts(max_fmg_iter=0, bottom_solver=1, max_coarsening_level=oracle.num_levels(n0, n0, n0) - 2)
    comp = CP.Composite(levels, F0s=F0s, opts0=opts, optsf=opts)
    u, it, hist = comp.solve(tol_rel=tol, max_iter=max_iter)
    return u, it, hist, levels


def uniaxial_errors(oracle, u, levels, E):
    """Relative squared errors of u_x and sigma_xx along y = z = 0 on every
    level's valid nodes."""
    errs = []
    for l, lev in enumerate(levels):
        xs = -8 + lev.dx * (np.arange(lev.n[0]) + lev.off[0])
        j = int(round(8 / lev.dx)) - lev.off[1]
        sl = slice(1, -1) if l else slice(None)
        ux = u[l][0, j, j, sl]
        exact = (xs[sl] + 8) * 0.1 / 16
        s, _, _ = oracle.stress_strain(lev.C, None, u[l], lev.dx)
        sig = s[j, j, sl, 0]
        errs.append((np.sum((exact - ux) ** 2) / np.sum(exact ** 2),
                     np.sum((sig - E * 0.1 / 16) ** 2) / np.sum(np.full_like(sig, E * 0.1 / 16) ** 2)))
    return errs


def eshelby_ray_errors(oracle, u, levels, Cs, F0s, hw):
    """The reference test's norms along x = y = 0.25, z in [-2, 2], each point
    taken from the finest level whose valid box holds it."""
    with open(os.path.join(GOLDEN, "eshelby.json")) as f:
        golden = json.load(f)
    pts = {}
    for l in range(len(levels) - 1, -1, -1):
        lev = levels[l]
        coords = -hw + lev.dx * (np.arange(lev.n[0]) + lev.off[0])
        ix = int(round((0.25 + hw) / lev.dx)) - lev.off[0]
        s, _, _ = oracle.stress_strain(Cs[l], F0s[l], u[l], lev.dx)
        for k in range(1 if l else 0, lev.n[2] - (1 if l else 0)):
            z = round(coords[k], 9)
            if abs(z) <= 2 + 1e-9 and z not in pts:
                pts[z] = (u[l][:, k, ix, ix], (s[k, ix, ix, 0], s[k, ix, ix, 4], s[k, ix, ix, 8]))
    z = np.array(sorted(pts))
    U = np.array([pts[q][0] for q in z]).T
    S = np.array([pts[q][1] for q in z]).T

    def integ(x, y):
        return float(np.sum(0.5 * (y[1:] + y[:-1]) * (x[1:] - x[:-1])))
    ref = np.array([golden["displacement"][k] for k in ["x", "disp1", "disp2", "disp3"]])
    ue = [np.sqrt(integ(z, (np.interp(z, ref[0], ref[c + 1] / 1e4) - U[c]) ** 2) / integ(ref[0], (ref[c + 1] / 1e4) ** 2))
          for c in range(3)]
    ref = np.array([golden["sigma_normal"][k] for k in ["x", "sigma11", "sigma22", "sigma33"]])
    sc = P.ESHELBY_E / 1000
    se = [integ(z, np.abs(np.interp(z, ref[0], ref[c + 1] * sc) - S[c])) / integ(ref[0], np.abs(ref[c + 1] * sc))
          for c in range(3)]
    return np.array(ue), np.array(se)


def test_composite_oracle_uniaxial_tension(oracle):
    n0, dx0, boxes, Cs, F0s, bc, E = uniaxial_levels()
    u, it, hist, levels = oracle_composite(oracle, n0, dx0, boxes, Cs, F0s, bc, tol=1e-9)
    assert hist[-1] <= 1e-9
    for eu, es in uniaxial_errors(oracle, u, levels, E):
        assert eu < 1e-8 and es < 1e-8


@pytest.mark.slow
def test_composite_oracle_eshelby(oracle):
    n0, dx0, boxes, Cs, F0s, bc, hw = eshelby_levels()
    u, it, hist, levels = oracle_composite(oracle, n0, dx0, boxes, Cs, F0s, bc, tol=1e-7)
    assert hist[-1] <= 1e-7
    ue, se = eshelby_ray_errors(oracle, u, levels, Cs, F0s, hw)
    assert np.all(ue < 0.1), ue
    assert np.all(se < 0.1), se


def _gpu_composite(agb, oracle, n0, dx0, boxes, Cs, F0s, bc, tol):
    """The library's composite solve with the oracle composite's level
    solver settings (FP64 V(2,2), exact 5^3 bottom)."""
    from alamo_gb300.composite import Composite
    opts = agb.default_opts(precision=0, bottom_solver="direct",
                            max_coarsening_level=oracle.num_levels(n0, n0, n0) - 2, max_iter=80)
    with Composite(n0, dx0, boxes, "isotropic", opts) as c:
        c.SetBC(bc)
        for l, C in enumerate(Cs):
            c.SetModel(l, C)
        return c.solve(F0=F0s if any(f is not None for f in F0s) else None, tol_rel=tol)


@pytest.mark.gpu
def test_composite_gpu_uniaxial_tension(agb, oracle):
    n0, dx0, boxes, Cs, F0s, bc, E = uniaxial_levels()
    ug, itg, rn = _gpu_composite(agb, oracle, n0, dx0, boxes, Cs, F0s, bc, 1e-9)
    uo, ito, hist, levels = oracle_composite(oracle, n0, dx0, boxes, Cs, F0s, bc, tol=1e-9)
    assert rn <= 1e-9
    assert abs(itg - ito) <= 1
    for l in range(len(levels)):
        assert np.abs(ug[l] - uo[l]).max() <= 1e-8 * np.abs(uo[l]).max()
    for eu, es in uniaxial_errors(oracle, ug, levels, E):
        assert eu < 1e-8 and es < 1e-8


@pytest.mark.gpu
@pytest.mark.slow
def test_composite_gpu_eshelby(agb, oracle):
    n0, dx0, boxes, Cs, F0s, bc, hw = eshelby_levels()
    ug, itg, rn = _gpu_composite(agb, oracle, n0, dx0, boxes, Cs, F0s, bc, 1e-7)
    uo, ito, hist, levels = oracle_composite(oracle, n0, dx0, boxes, Cs, F0s, bc, tol=1e-7)
    assert rn <= 1e-7
    for l in range(len(levels)):
        assert np.abs(ug[l] - uo[l]).max() <= 1e-6 * np.abs(uo[l]).max()
    ue, se = eshelby_ray_errors(oracle, ug, levels, Cs, F0s, hw)
    assert np.all(ue < 0.1), ue
    assert np.all(se < 0.1), se

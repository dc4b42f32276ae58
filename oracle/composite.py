"""Multi-level (AMR) composite solve restated on the oracle (TEST
INFRASTRUCTURE ONLY: the checker of the library's composite solve).

The reference solves the elastic operator on a hierarchy of AMR levels
through AMReX's MLMG with the ghost-node coarse/fine strategy; alamo's share
of it is the operator's hooks: `reflux` (the coarse residual under a fine
level is the fine residual restricted by nodal full weighting,
src/Operator/Operator.cpp:526-633), `fixUpResidualMask` (:230-251) and
`averageDownCoeffsDifferentAmrLevels` (the coarse stiffness under a fine
level is the fine stiffness restricted by the same weights,
src/Operator/Elastic.cpp:628-742).  AMReX itself is not vendored, so the
composite iteration is restated from its documented behaviour:

* level 0 covers the domain with the user's boundary conditions; level l >= 1
  is one box of valid nodes lo .. lo + nv - 1 (in level-l node indices,
  refinement ratio 2, lo even, nv odd, so the box's faces lie on coarse
  nodes), strictly inside level l-1's valid region;
* a fine level carries one ring of ghost nodes around its box, filled by
  trilinear nodal interpolation of level l-1's solution, and the operator
  applies its interior rows at every valid node, the box's faces included
  (ghost-node strategy);
* coarse nodes covered by a finer box take the finer level's values
  (average down = injection at coincident nodes) and, in the coarse
  correction, the finer level's residual restricted by full weighting
  (reflux); their coarse stiffness is the restricted fine stiffness;
* the converged composite solution satisfies the fine rows at every fine
  valid node and the coarse rows at every uncovered coarse node; the norm
  of those rows is the convergence test.

The iteration (fast adaptive composite, McCormick 1989): per iteration, for
l = 1..L fill the ghosts from level l-1 and run `fine_cycles` V-cycles of
level l's own hierarchy (its ghost rows are displacement rows); average
down l = L..1; form the composite residual and reflux it down to level 0;
one coarse V-cycle on level 0 and its correction interpolated up through
every level.

Arrays: level 0 as the oracle's node fields (3, n, n, n); level l >= 1 on
its extended grid (valid box plus the ghost ring, nv + 2 nodes per axis).
"""
import numpy as np

import oracle as O


def _interp_axis(p):
    """Coarse indices and weights of the nodal linear interpolation at fine
    index p (coarse position p / 2)."""
    if p % 2 == 0:
        return [(p // 2, 1.0)]
    return [((p - 1) // 2, 0.5), ((p + 1) // 2, 0.5)]


def _interp_matrix(off_f, n_f, off_c, n_c):
    """(n_f, n_c) matrix of the 1-D nodal linear interpolation from coarse
    array indices (level index off_c + j) to fine ones (off_f + i)."""
    M = np.zeros((n_f, n_c))
    for i in range(n_f):
        for j, w in _interp_axis(off_f + i):
            M[i, j - off_c] += w
    return M


def interp_block(field_c, off_c, off_f, n_f):
    """Trilinear nodal interpolation of a coarse field (3, nz, ny, nx) whose
    index 0 is coarse node off_c, on the fine block of n_f nodes per axis
    starting at fine level index off_f.  Separable: one 1-D interpolation
    per axis."""
    nc = field_c.shape[1:][::-1]
    Mx = _interp_matrix(off_f[0], n_f[0], off_c[0], nc[0])
    My = _interp_matrix(off_f[1], n_f[1], off_c[1], nc[1])
    Mz = _interp_matrix(off_f[2], n_f[2], off_c[2], nc[2])
    return np.einsum("zk,yj,xi,ckji->czyx", Mz, My, Mx, field_c, optimize=True)


def fw_weights():
    w = np.zeros((3, 3, 3))
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                w[dz + 1, dy + 1, dx + 1] = (0.5 if dx == 0 else 0.25) * (0.5 if dy == 0 else 0.25) * \
                    (0.5 if dz == 0 else 0.25)
    return w


class Level:
    def __init__(self, n, dx, lo, nv, C, bt, bv):
        self.n = n          # nodes per axis of the level's array (extended for l >= 1)
        self.dx = dx
        self.lo = lo        # level index of the first valid node (l >= 1), None for level 0
        self.nv = nv        # valid nodes per axis
        self.C = np.ascontiguousarray(C)
        self.bt, self.bv = bt, bv
        self.off = (0, 0, 0) if lo is None else tuple(v - 1 for v in lo)  # level index of array index 0

    def ring_mask(self):
        m = np.zeros((self.n[2], self.n[1], self.n[0]), bool)
        if self.lo is None:
            return m
        m[0, :, :] = m[-1, :, :] = m[:, 0, :] = m[:, -1, :] = m[:, :, 0] = m[:, :, -1] = True
        return m


def covered_mask(crse, fine):
    """Nodes of the coarse level's array covered by the fine level's box."""
    m = np.zeros((crse.n[2], crse.n[1], crse.n[0]), bool)
    sl = []
    for a in range(3):
        c0 = fine.lo[a] // 2 - crse.off[a]
        c1 = (fine.lo[a] + fine.nv[a] - 1) // 2 - crse.off[a]
        sl.append(slice(c0, c1 + 1))
    m[sl[2], sl[1], sl[0]] = True
    return m, sl


def restrict_fw(field_f, fine, crse, sl):
    """Full-weighting restriction of a fine extended-grid field (k, nz, ny,
    nx) onto the coarse nodes covered by the fine box (returned in the
    shape of those nodes)."""
    w = fw_weights()
    k = field_f.shape[0]
    cz, cy, cx = (sl[2].stop - sl[2].start, sl[1].stop - sl[1].start, sl[0].stop - sl[0].start)
    out = np.zeros((k, cz, cy, cx))
    # coarse covered node c (0-based in the covered block) <-> fine ext index 2 c + 1
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                out += w[dz + 1, dy + 1, dx + 1] * field_f[:, 1 + dz: 1 + dz + 2 * cz: 2, 1 + dy: 1 + dy + 2 * cy: 2,
                                                           1 + dx: 1 + dx + 2 * cx: 2]
    return out


class Composite:
    """levels[0]: Level of the domain; levels[l]: nested boxes.  F0s: per
    level eigenstrain (None, scalar field or 9-component field) on the
    level's array."""

    def __init__(self, levels, F0s=None, opts0=None, optsf=None):
        self.L = levels
        nl = len(levels)
        self.F0s = F0s or [None] * nl
        self.ring = [lev.ring_mask() for lev in levels]
        self.cov = [None] * nl
        for l in range(nl - 1):
            self.cov[l] = covered_mask(levels[l], levels[l + 1])
        # right-hand sides at u = 0 from each level's own model (ghost rows
        # filled each iteration), before the stiffness is averaged down: the
        # reference builds them per level (Newton.H:144-275) before MLMG's
        # prepareForSolve averages the coefficients
        self.rhs = []
        for l, lev in enumerate(levels):
            z = np.zeros((3, lev.n[2], lev.n[1], lev.n[0]))
            b = O.bc_init(z, lev.bt, lev.bv)
            self.rhs.append(O.build_rhs(lev.C, self.F0s[l], lev.bt, z, b, lev.dx))
        # stiffness under a finer box: the restricted finer stiffness
        # (fine to coarse, so a level's restricted values include the finer
        # levels' below it)
        for l in range(nl - 2, -1, -1):
            m, sl = self.cov[l]
            Cf = np.moveaxis(levels[l + 1].C, -1, 0)
            rc = restrict_fw(Cf, levels[l + 1], levels[l], sl)
            C = levels[l].C.copy()
            C[sl[2], sl[1], sl[0], :] = np.moveaxis(rc, 0, -1)
            levels[l].C = np.ascontiguousarray(C)
        self.opts0 = opts0
        self.optsf = optsf

    def fill_ghosts(self, l, u):
        lev, crse = self.L[l], self.L[l - 1]
        vals = interp_block(u[l - 1], crse.off, lev.off, lev.n)[:, self.ring[l]]
        self.rhs[l][:, self.ring[l]] = vals
        u[l][:, self.ring[l]] = vals

    def residuals(self, u):
        """Composite residual per level (covered coarse nodes: the reflux of
        the finer residual; ghost rows: 0) and its inf-norm over the rows of
        the composite system."""
        nl = len(self.L)
        r = [None] * nl
        rn = 0.0
        for l in range(nl - 1, -1, -1):
            lev = self.L[l]
            rl, _ = O.residual(lev.C, lev.bt, u[l], self.rhs[l], lev.dx)
            rl[:, self.ring[l]] = 0.0
            if l < nl - 1:
                m, sl = self.cov[l]
                rn = max(rn, np.abs(rl[:, ~m]).max())
                rl[:, sl[2], sl[1], sl[0]] = restrict_fw(r[l + 1], self.L[l + 1], lev, sl)
            else:
                rn = max(rn, np.abs(rl).max())
            r[l] = rl
        return r, rn

    verbose = False

    def level_norms(self, u):
        out = []
        nl = len(self.L)
        for l, lev in enumerate(self.L):
            rl, _ = O.residual(lev.C, lev.bt, u[l], self.rhs[l], lev.dx)
            m = ~self.ring[l]
            if l < nl - 1:
                m = m & ~self.cov[l][0]
            out.append("%.2e" % np.abs(rl[:, m]).max())
        return out

    def rhs_norm(self):
        nl = len(self.L)
        v = 0.0
        for l in range(nl):
            m = ~self.ring[l]
            if l < nl - 1:
                m = m & ~self.cov[l][0]
            v = max(v, np.abs(self.rhs[l][:, m]).max())
        return v

    def average_down(self, u):
        for l in range(len(self.L) - 1, 0, -1):
            m, sl = self.cov[l - 1]
            u[l - 1][:, sl[2], sl[1], sl[0]] = u[l][:, 1:-1:2, 1:-1:2, 1:-1:2]

    def vcycles(self, l, r, cycles, opts):
        """cycles V-cycles of level l's own hierarchy on A c = r from c = 0
        (ghost rows of r zero, so the ghost values of c stay zero)."""
        lev = self.L[l]
        c = O.vcycle(lev.C, lev.bt, r, lev.dx, opts=opts)
        for _ in range(cycles - 1):
            rr, _ = O.residual(lev.C, lev.bt, c, r, lev.dx)
            c = c + O.vcycle(lev.C, lev.bt, rr, lev.dx, opts=opts)
        return c

    def solve(self, tol_rel=1e-10, max_iter=100, fine_cycles=1, coarse_cycles=1, u=None):
        """Composite iterations in correction form, as MLMG::oneIter runs
        them over AMR levels: the composite residual (reflux under finer
        boxes); down the levels, a correction on each fine level from its
        residual (ghost values zero) and the reflux of what it leaves; the
        coarse correction on level 0; up the levels, the coarser correction
        interpolated (ghosts included) and a correction of the remaining
        residual; then the solution update and the average down."""
        nl = len(self.L)
        if u is None:
            u = [np.zeros((3, lev.n[2], lev.n[1], lev.n[0])) for lev in self.L]
        hist = []
        for l in range(1, nl):
            self.fill_ghosts(l, u)
        bn = self.rhs_norm()
        it = 0
        for it in range(max_iter + 1):
            # covered coarse values from the finer levels, then the ghosts
            # from the coarser ones
            self.average_down(u)
            for l in range(1, nl):
                self.fill_ghosts(l, u)
            r, rn = self.residuals(u)
            hist.append(rn / bn)
            if self.verbose:
                print("composite it %d |r|/|b| %.3e per level %s" % (it, rn / bn, self.level_norms(u)))
            if rn <= tol_rel * bn or it == max_iter:
                break
            c = [None] * nl
            for l in range(nl - 1, 0, -1):
                lev = self.L[l]
                c[l] = self.vcycles(l, r[l], fine_cycles, self.optsf)
                rr, _ = O.residual(lev.C, lev.bt, c[l], r[l], lev.dx)
                rr[:, self.ring[l]] = 0.0
                m, sl = self.cov[l - 1]
                r[l - 1][:, sl[2], sl[1], sl[0]] = restrict_fw(rr, lev, self.L[l - 1], sl)
            c[0] = self.vcycles(0, r[0], coarse_cycles, self.opts0)
            for l in range(1, nl):
                lev = self.L[l]
                c[l] = c[l] + interp_block(c[l - 1], self.L[l - 1].off, lev.off, lev.n)
                rr, _ = O.residual(lev.C, lev.bt, c[l], r[l], lev.dx)
                rr[:, self.ring[l]] = 0.0
                c[l] = c[l] + self.vcycles(l, rr, fine_cycles, self.optsf)
            for l in range(nl):
                u[l] += c[l]
        return u, it, hist

// ============================================================================
// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// A plain C++ (OpenMP) restatement of the reference's CPU path for the nodal
// linear-elastic multigrid solve of alamo (Gopal-B/alamo).  It is the checker
// for the CUDA product in alamo_gb300/: only tests/, __graft_entry__.smoke()
// and bench.py's cpu_baseline / --impl reference leg load this library.  The
// product never links, loads or calls it.
//
// What it restates (reference file:line, paths inside the reference project):
//   stencils          src/Numeric/Stencil.H:41-60 (GetStencil), :70-191 (D1),
//                     :197-243 (D2, zero unless central), :245-301 (mixed),
//                     :588-657 (Divergence of a nodal matrix field),
//                     :742-786 (Gradient), :900-963 (Gradient_Diagonal)
//   stiffness algebra src/Set/Matrix4_Isotropic.H:137-173 (C*gradu, C*gradgradu)
//                     src/Set/Matrix4_MajorMinor.H:327-375 (21-entry index
//                     map), :518-547 (Cubic), :675-691, :709-767
//   Fapply            src/Operator/Elastic.cpp:139-292
//   Diagonal          src/Operator/Elastic.cpp:296-379
//   Fsmooth           src/Operator/Operator.cpp:88-154 (2 damped-Jacobi sweeps)
//   residuals         src/Operator/Operator.cpp:635-657
//   restriction       src/Operator/Operator.cpp:262-363
//   interpolation     src/Operator/Operator.cpp:365-434
//   C coarsening      src/Operator/Elastic.cpp:746-836
//   normalize         src/Operator/Operator.cpp:156-165 (divide by diagonal)
//   BC rows           src/BC/Operator/Elastic/Elastic.H:35-43,79-80;
//                     src/BC/Operator/Elastic/Constant.H:100-194 (Init),
//                     :344-425 (operator(), set)
//   Newton RHS        src/Solver/Nonlocal/Newton.H:144-275
//   stress/strain     src/Integrator/Base/Mechanics.H:210-248,
//                     src/Operator/Elastic.cpp:426-603
//   psi (void)        src/Operator/Elastic.cpp:118-137 (SetPsi), :191-260 and
//                     :341-363 (psi_avg, grad psi terms), :839-905 (psi
//                     coarsening); src/Numeric/Stencil.H:699-715
//                     (CellGradientOnNode), :1390-1405 (CellToNodeAverage);
//                     src/Solver/Nonlocal/Newton.H:236-263 (RHS).  Pinned
//                     against numpy restatements (tests/test_psi.py); the
//                     reference has no known-answer test for psi in 3D.
//   V-cycle driver    behaviour of amrex::MLMG as configured by
//                     src/Solver/Nonlocal/Linear.H:255-290 (AMReX itself is not
//                     vendored in the reference: parity is unpinned at the MLMG
//                     boundary, the loop below restates its published
//                     behaviour: F-cycles (max_fmg_iter = 100000000,
//                     Linear.H:261) or V-cycles on the correction equation,
//                     BiCGStab bottom on the diagonally normalised system,
//                     inf-norm test)
//
// Pinned against the reference's own known answers (tests/test_oracle_golden.py):
//   tests/UniaxialTension (linear exactness, 1e-8), tests/Solid/reference/
//   linear-cubic.dat, affine-cubic.dat, affine-hexagonal.dat,
//   transverselyisotropic.dat and neo-hookean.dat (trac_xhi_x(t), 1e-4;
//   tests/test_neohookean.py for the last),
//   src/Test/Numeric/Stencil.H:58-106 (derivative accuracy, 1e-2),
//   tests/Eshelby (analytic inclusion solution, 0.1) and tests/TrigTest
//   (the Laplacian's trigonometric solution, 1e-4).
//
// Layouts: node grid nx*ny*nz, x fastest; vector fields are SoA per component
// (comp slowest), no ghost nodes.  Stiffness is per node in the reference's
// object layout (AoS): isotropic = {lambda, mu}, major-minor = data[0..20].
// Floating point: built with -ffp-contract=off so the same bits come out on
// x86-64 and aarch64.
// ============================================================================
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <chrono>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum { ISO = 0, MM = 1, MAJ = 2 };
enum { DISP = 0, TRAC = 1, PERIODIC = 2, NEUMANN = 3, NONE = 4 };
enum Sten { LO = 0, HI = 1, CENTRAL = 2 };

// Face order of BC::Operator::Elastic::Elastic::Face (Elastic.H:35-43)
enum Face {
    XLO, YLO, ZLO, XHI, YHI, ZHI,
    YLO_ZLO, YLO_ZHI, YHI_ZLO, YHI_ZHI,
    ZLO_XLO, ZLO_XHI, ZHI_XLO, ZHI_XHI,
    XLO_YLO, XLO_YHI, XHI_YLO, XHI_YHI,
    XLO_YLO_ZLO, XLO_YLO_ZHI, XLO_YHI_ZLO, XLO_YHI_ZHI,
    XHI_YLO_ZLO, XHI_YLO_ZHI, XHI_YHI_ZLO, XHI_YHI_ZHI,
    INTERIOR
};

// Truncated literals of the reference (Elastic.H:79-80)
const double S3 = 0.57735026919;
const double S2 = 0.70710678118;

struct Grid {
    int n[3];
    double dx[3];
    // psi (SetPsi, Elastic.cpp:120-136): cell field stored with one ghost
    // layer, (n0+1)(n1+1)(n2+1) values, entry (a,b,c) = cell (a-1,b-1,c-1);
    // ghosts outside the domain keep the define-time fill 1.0
    // (Elastic.cpp:49-52).  nullptr: psi not set.
    const double* psi = nullptr;
    double psi_small = 0.0;
    int64_t N() const { return (int64_t)n[0] * n[1] * n[2]; }
    int64_t id(int i, int j, int k) const { return i + (int64_t)n[0] * (j + (int64_t)n[1] * k); }
    bool boundary(int i, int j, int k) const {
        return i == 0 || j == 0 || k == 0 || i == n[0] - 1 || j == n[1] - 1 || k == n[2] - 1;
    }
};

inline int nc_of(int sym) { return sym == ISO ? 2 : sym == MM ? 21 : 45; }

// ---------------------------------------------------------------------------
// Stiffness tensors.  Major-minor storage: 6x6 symmetric matrix over the pair
// order (00,01,02,11,12,22), upper triangle row-major = data[0..20]
// (Matrix4_MajorMinor.H:327-375).
// ---------------------------------------------------------------------------
const int PAIR[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
int UT[6][6];  // upper-triangle index table
struct UTInit {
    UTInit() {
        int c = 0;
        for (int a = 0; a < 6; a++)
            for (int b = a; b < 6; b++) { UT[a][b] = c; UT[b][a] = c; c++; }
    }
} ut_init;

inline double mm_get(const double* d, int i, int j, int k, int l) { return d[UT[PAIR[i][j]][PAIR[k][l]]]; }

// Major symmetry only (C_ijkl = C_klij): 9x9 symmetric matrix over the pairs
// P = 3i + j, upper triangle row-major = data[0..44] (Matrix4_Major.H:274-320)
inline int maj_index(int P, int Q) {
    if (P > Q) { const int t = P; P = Q; Q = t; }
    return P * 9 - P * (P - 1) / 2 + (Q - P);
}
inline double maj_get(const double* d, int i, int j, int k, int l) { return d[maj_index(3 * i + j, 3 * k + l)]; }

// sigma = C * g  (Matrix4_Isotropic.H:137-157, Matrix4_MajorMinor.H:675-691)
inline void c_grad(int sym, const double* c, const double g[3][3], double s[3][3]) {
    if (sym == ISO) {
        const double l = c[0], m = c[1];
        s[0][0] = (l + 2. * m) * g[0][0] + l * g[1][1] + l * g[2][2];
        s[1][1] = l * g[0][0] + (l + 2. * m) * g[1][1] + l * g[2][2];
        s[2][2] = l * g[0][0] + l * g[1][1] + (l + 2. * m) * g[2][2];
        s[1][2] = m * (g[1][2] + g[2][1]); s[2][1] = s[1][2];
        s[2][0] = m * (g[2][0] + g[0][2]); s[0][2] = s[2][0];
        s[0][1] = m * (g[0][1] + g[1][0]); s[1][0] = s[0][1];
    } else if (sym == MAJ) {
        // sigma_ij = sum_kl C(3i+j, 3k+l) g_kl (Matrix4_Major.H:510-523)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double acc = 0.0;
                for (int k = 0; k < 3; k++)
                    for (int l = 0; l < 3; l++) acc += maj_get(c, i, j, k, l) * g[k][l];
                s[i][j] = acc;
            }
    } else {
        // symmetric-pair vector of g: (g00, g01+g10, g02+g20, g11, g12+g21, g22)
        const double v[6] = {g[0][0], g[0][1] + g[1][0], g[0][2] + g[2][0], g[1][1], g[1][2] + g[2][1], g[2][2]};
        const int rows[6][2] = {{0, 0}, {1, 1}, {2, 2}, {1, 2}, {2, 0}, {0, 1}};
        for (int r = 0; r < 6; r++) {
            const int a = PAIR[rows[r][0]][rows[r][1]];
            double acc = 0.0;
            for (int b = 0; b < 6; b++) acc += c[UT[a][b]] * v[b];
            s[rows[r][0]][rows[r][1]] = acc;
            s[rows[r][1]][rows[r][0]] = acc;
        }
    }
}

// f = C * gradgradu, b[k][l][j] = u_{k,lj}  (Matrix4_Isotropic.H:163-173,
// Matrix4_MajorMinor.H:709-767: f_i = sum_{jkl} C_ijkl u_{k,lj})
inline void c_hess(int sym, const double* c, const double b[3][3][3], double f[3]) {
    if (sym == ISO) {
        const double l = c[0], m = c[1];
        for (int i = 0; i < 3; i++) {
            double r = 0.0;
            for (int j = 0; j < 3; j++) r += m * (b[i][j][j] + b[j][i][j]) + l * b[j][j][i];
            f[i] = r;
        }
    } else {
        // Matrix4_Major.H:527-541 / Matrix4_MajorMinor.H:709-767
        for (int i = 0; i < 3; i++) {
            double r = 0.0;
            for (int j = 0; j < 3; j++)
                for (int k = 0; k < 3; k++)
                    for (int l = 0; l < 3; l++)
                        r += (sym == MAJ ? maj_get(c, i, j, k, l) : mm_get(c, i, j, k, l)) * b[k][l][j];
            f[i] = r;
        }
    }
}

// ---------------------------------------------------------------------------
// Stencils (Stencil.H)
// ---------------------------------------------------------------------------
inline void get_stencil(const Grid& g, int i, int j, int k, int s[3]) {
    const int p[3] = {i, j, k};
    for (int d = 0; d < 3; d++) s[d] = (p[d] == 0) ? HI : (p[d] == g.n[d] - 1) ? LO : CENTRAL;
}

const int E[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};

inline double at(const Grid& g, const double* f, int i, int j, int k) { return f[g.id(i, j, k)]; }

// first derivative along d with stencil type s (Stencil.H:70-191)
inline double d1(const Grid& g, const double* f, int i, int j, int k, int d, int s) {
    const int a = E[d][0], b = E[d][1], c = E[d][2];
    if (s == LO) return (at(g, f, i, j, k) - at(g, f, i - a, j - b, k - c)) / g.dx[d];
    if (s == HI) return (at(g, f, i + a, j + b, k + c) - at(g, f, i, j, k)) / g.dx[d];
    return (at(g, f, i + a, j + b, k + c) - at(g, f, i - a, j - b, k - c)) * 0.5 / g.dx[d];
}

// pure second derivative, central only (Stencil.H:197-243; callers only use
// it on interior nodes, where the stencil is central)
inline double d2(const Grid& g, const double* f, int i, int j, int k, int d) {
    const int a = E[d][0], b = E[d][1], c = E[d][2];
    return (at(g, f, i + a, j + b, k + c) - 2.0 * at(g, f, i, j, k) + at(g, f, i - a, j - b, k - c)) / g.dx[d] / g.dx[d];
}

// central mixed derivative along d1<d2 (Stencil.H:245-301 with central stencil)
inline double dmix(const Grid& g, const double* f, int i, int j, int k, int p, int q) {
    const int ap = E[p][0], bp = E[p][1], cp = E[p][2];
    const int aq = E[q][0], bq = E[q][1], cq = E[q][2];
    const double fpp = at(g, f, i + ap + aq, j + bp + bq, k + cp + cq);
    const double fmm = at(g, f, i - ap - aq, j - bp - bq, k - cp - cq);
    const double fpm = at(g, f, i + ap - aq, j + bp - bq, k + cp - cq);
    const double fmp = at(g, f, i - ap + aq, j - bp + bq, k - cp + cq);
    return 0.5 * 0.5 * (fpp + fmm - fpm - fmp) / (g.dx[p] * g.dx[q]);
}

// ---------------------------------------------------------------------------
// Boundary rows (Constant.H:344-425): region precedence corners > edges > faces
// ---------------------------------------------------------------------------
inline int region(const Grid& g, int i, int j, int k, double nrm[3]) {
    const bool xl = i == 0, xh = i == g.n[0] - 1, yl = j == 0, yh = j == g.n[1] - 1, zl = k == 0, zh = k == g.n[2] - 1;
    auto set = [&](double a, double b, double c) { nrm[0] = a; nrm[1] = b; nrm[2] = c; };
    if (xl && yl && zl) { set(-S3, -S3, -S3); return XLO_YLO_ZLO; }
    if (xl && yl && zh) { set(-S3, -S3, +S3); return XLO_YLO_ZHI; }
    if (xl && yh && zl) { set(-S3, +S3, -S3); return XLO_YHI_ZLO; }
    if (xl && yh && zh) { set(-S3, +S3, +S3); return XLO_YHI_ZHI; }
    if (xh && yl && zl) { set(+S3, -S3, -S3); return XHI_YLO_ZLO; }
    if (xh && yl && zh) { set(+S3, -S3, +S3); return XHI_YLO_ZHI; }
    if (xh && yh && zl) { set(+S3, +S3, -S3); return XHI_YHI_ZLO; }
    if (xh && yh && zh) { set(+S3, +S3, +S3); return XHI_YHI_ZHI; }
    if (yl && zl) { set(0, -S2, -S2); return YLO_ZLO; }
    if (yl && zh) { set(0, -S2, +S2); return YLO_ZHI; }
    if (yh && zl) { set(0, +S2, -S2); return YHI_ZLO; }
    if (yh && zh) { set(0, +S2, +S2); return YHI_ZHI; }
    if (zl && xl) { set(-S2, 0, -S2); return ZLO_XLO; }
    if (zl && xh) { set(+S2, 0, -S2); return ZLO_XHI; }
    if (zh && xl) { set(-S2, 0, +S2); return ZHI_XLO; }
    if (zh && xh) { set(+S2, 0, +S2); return ZHI_XHI; }
    if (xl && yl) { set(-S2, -S2, 0); return XLO_YLO; }
    if (xl && yh) { set(-S2, +S2, 0); return XLO_YHI; }
    if (xh && yl) { set(+S2, -S2, 0); return XHI_YLO; }
    if (xh && yh) { set(+S2, +S2, 0); return XHI_YHI; }
    if (xl) { set(-1, 0, 0); return XLO; }
    if (xh) { set(+1, 0, 0); return XHI; }
    if (yl) { set(0, -1, 0); return YLO; }
    if (yh) { set(0, +1, 0); return YHI; }
    if (zl) { set(0, 0, -1); return ZLO; }
    if (zh) { set(0, 0, +1); return ZHI; }
    set(0, 0, 0);
    return INTERIOR;
}

inline void bc_row(const int* bc_type, int reg, const double nrm[3], const double u[3], const double gu[3][3],
                   const double s[3][3], double f[3]) {
    for (int i = 0; i < 3; i++) {
        const int t = bc_type[reg * 3 + i];
        if (t == DISP) f[i] = u[i];
        else if (t == TRAC) f[i] = s[i][0] * nrm[0] + s[i][1] * nrm[1] + s[i][2] * nrm[2];
        else if (t == NEUMANN) f[i] = gu[i][0] * nrm[0] + gu[i][1] * nrm[1] + gu[i][2] * nrm[2];
        else f[i] = 0.0;
    }
}

// When false, interior rows drop the sum_q (d_q C : grad u)_{:,q} term (the
// reference's m_uniform = true branch, Elastic.cpp:245).
bool g_grad_c = true;

// psi of the grid the per-call functions below operate on (orc_set_psi)
const double* g_psi = nullptr;
double g_psi_small = 0.0;

inline int64_t psi_id(const Grid& g, int a, int b, int c) {
    return a + (int64_t)(g.n[0] + 1) * (b + (int64_t)(g.n[1] + 1) * c);
}
// Numeric::Interpolate::CellToNodeAverage (Numeric/Stencil.H:1390-1405):
// mean of the 8 cells at a node, summed in the reference's order
inline double psi_cell_avg(const Grid& g, int i, int j, int k) {
    auto P = [&](int a, int b, int c) { return g.psi[psi_id(g, i + 1 + a, j + 1 + b, k + 1 + c)]; };
    return (P(0, 0, 0) + P(-1, 0, 0) + P(0, -1, 0) + P(-1, -1, 0) + P(0, 0, -1) + P(-1, 0, -1) + P(0, -1, -1) +
            P(-1, -1, -1)) * 0.125;
}
// psi_avg of Fapply / Diagonal (Elastic.cpp:191-192)
inline double psi_avg(const Grid& g, int i, int j, int k) {
    if (!g.psi) return 1.0;
    return (1.0 - g.psi_small) * psi_cell_avg(g, i, j, k) + g.psi_small;
}
// Numeric::CellGradientOnNode (Stencil.H:699-715)
inline void psi_grad(const Grid& g, int i, int j, int k, double gp[3]) {
    auto P = [&](int a, int b, int c) { return g.psi[psi_id(g, i + 1 + a, j + 1 + b, k + 1 + c)]; };
    // cell (i + a, j + b, k + c) with a, b, c in {-1, 0}
    gp[0] = 0.25 * (P(0, 0, 0) - P(-1, 0, 0) + P(0, -1, 0) - P(-1, -1, 0) + P(0, 0, -1) - P(-1, 0, -1) + P(0, -1, -1) -
                    P(-1, -1, -1)) / g.dx[0];
    gp[1] = 0.25 * (P(0, 0, 0) - P(0, -1, 0) + P(-1, 0, 0) - P(-1, -1, 0) + P(0, 0, -1) - P(0, -1, -1) + P(-1, 0, -1) -
                    P(-1, -1, -1)) / g.dx[1];
    gp[2] = 0.25 * (P(0, 0, 0) - P(0, 0, -1) + P(-1, 0, 0) - P(-1, 0, -1) + P(0, -1, 0) - P(0, -1, -1) + P(-1, -1, 0) -
                    P(-1, -1, -1)) / g.dx[2];
}

// ---------------------------------------------------------------------------
// Fapply at one node (Elastic.cpp:165-290; psi not set, m_uniform false)
// ---------------------------------------------------------------------------
void fapply_gradc(int sym, const Grid& g, const double* C, const double gu[3][3], double pa, int i, int j, int k,
                  double f[3]);

void fapply_node(int sym, const Grid& g, const double* C, const int* bct, const double* U, int i, int j, int k,
                 double f[3]) {
    const int64_t N = g.N();
    const int64_t id = g.id(i, j, k);
    const int nc = nc_of(sym);
    const double* u0 = U;
    const double* uu[3] = {U, U + N, U + 2 * N};
    (void)u0;
    double u[3] = {uu[0][id], uu[1][id], uu[2][id]};
    int s[3];
    get_stencil(g, i, j, k, s);
    double gu[3][3];
    for (int p = 0; p < 3; p++)
        for (int q = 0; q < 3; q++) gu[p][q] = d1(g, uu[p], i, j, k, q, s[q]);
    const double* c = C + id * nc;
    double sig[3][3];
    c_grad(sym, c, gu, sig);
    const double pa = psi_avg(g, i, j, k);
    if (g.boundary(i, j, k)) {
        double nrm[3];
        const int reg = region(g, i, j, k, nrm);
        double sp[3][3];
        for (int p = 0; p < 3; p++)
            for (int q = 0; q < 3; q++) sp[p][q] = g.psi ? sig[p][q] * pa : sig[p][q];
        bc_row(bct, reg, nrm, u, gu, sp, f);
        return;
    }
    double b[3][3][3];
    for (int p = 0; p < 3; p++) {
        b[p][0][0] = d2(g, uu[p], i, j, k, 0);
        b[p][1][1] = d2(g, uu[p], i, j, k, 1);
        b[p][2][2] = d2(g, uu[p], i, j, k, 2);
        b[p][0][1] = dmix(g, uu[p], i, j, k, 0, 1);
        b[p][1][0] = b[p][0][1];
        b[p][0][2] = dmix(g, uu[p], i, j, k, 0, 2);
        b[p][1][2] = dmix(g, uu[p], i, j, k, 1, 2);
        b[p][2][0] = b[p][0][2];
        b[p][2][1] = b[p][1][2];
    }
    c_hess(sym, c, b, f);
    if (g.psi)
        for (int r = 0; r < 3; r++) f[r] *= pa;
    if (g_grad_c) fapply_gradc(sym, g, C, gu, pa, i, j, k, f);
    if (g.psi) {
        // + (C grad u) grad psi (1 - small) (Elastic.cpp:255-260)
        double gp[3];
        psi_grad(g, i, j, k, gp);
        for (int q = 0; q < 3; q++) gp[q] *= (1.0 - g.psi_small);
        for (int r = 0; r < 3; r++) f[r] += sig[r][0] * gp[0] + sig[r][1] * gp[1] + sig[r][2] * gp[2];
    }
}

// + sum_q (d_q C * gradu)_{:,q} psi_avg: central differences of C (Elastic.cpp:245-254)
void fapply_gradc(int sym, const Grid& g, const double* C, const double gu[3][3], double pa, int i, int j, int k,
                  double f[3]) {
    const int nc = nc_of(sym);
    double col[3][3];
    for (int q = 0; q < 3; q++) {
        const double* cp = C + g.id(i + E[q][0], j + E[q][1], k + E[q][2]) * nc;
        const double* cm = C + g.id(i - E[q][0], j - E[q][1], k - E[q][2]) * nc;
        double dc[45];
        for (int a = 0; a < nc; a++) dc[a] = (cp[a] - cm[a]) * 0.5 / g.dx[q];
        double t[3][3];
        c_grad(sym, dc, gu, t);
        for (int r = 0; r < 3; r++) col[q][r] = t[r][q];
    }
    for (int r = 0; r < 3; r++) f[r] += g.psi ? ((col[0][r] + col[1][r]) + col[2][r]) * pa : (col[0][r] + col[1][r]) + col[2][r];
}

// diagonal at one node (Elastic.cpp:321-373, Stencil.H:900-963)
void diag_node(int sym, const Grid& g, const double* C, const int* bct, int i, int j, int k, double d[3]) {
    const int nc = nc_of(sym);
    const double* c = C + g.id(i, j, k) * nc;
    int s[3];
    get_stencil(g, i, j, k, s);
    const bool bnd = g.boundary(i, j, k);
    for (int p = 0; p < 3; p++) {
        if (bnd) {
            double gu[3][3];
            for (int q = 0; q < 3; q++)
                for (int dd = 0; dd < 3; dd++) {
                    const bool mn = s[dd] == HI, mx = s[dd] == LO;
                    const double one = (p == q) ? 1.0 : 0.0;
                    gu[q][dd] = ((!mx ? 0.0 : one) - (!mn ? 0.0 : one)) / ((mn || mx ? 1.0 : 2.0) * g.dx[dd]);
                }
            double sig[3][3];
            c_grad(sym, c, gu, sig);
            if (g.psi) {
                const double pa = psi_avg(g, i, j, k);
                for (int q = 0; q < 3; q++)
                    for (int dd = 0; dd < 3; dd++) sig[q][dd] *= pa;
            }
            double u[3] = {0, 0, 0};
            u[p] = 1.0;
            double nrm[3], f[3];
            const int reg = region(g, i, j, k, nrm);
            bc_row(bct, reg, nrm, u, gu, sig, f);
            d[p] = f[p];
        } else {
            double b[3][3][3];
            for (int q = 0; q < 3; q++)
                for (int l = 0; l < 3; l++)
                    for (int jj = 0; jj < 3; jj++)
                        b[q][l][jj] = (l == jj && p == q) ? -2.0 / g.dx[l] / g.dx[l] : 0.0;
            double f[3];
            c_hess(sym, c, b, f);
            d[p] = 0.0 + (g.psi ? f[p] * psi_avg(g, i, j, k) : f[p]);
        }
    }
}

template <class F>
void for_nodes(const Grid& g, F fn) {
#pragma omp parallel for schedule(static)
    for (int k = 0; k < g.n[2]; k++)
        for (int j = 0; j < g.n[1]; j++)
            for (int i = 0; i < g.n[0]; i++) fn(i, j, k);
}

void fapply(int sym, const Grid& g, const double* C, const int* bct, const double* u, double* f) {
    const int64_t N = g.N();
    for_nodes(g, [&](int i, int j, int k) {
        double r[3];
        fapply_node(sym, g, C, bct, u, i, j, k, r);
        const int64_t id = g.id(i, j, k);
        f[id] = r[0]; f[N + id] = r[1]; f[2 * N + id] = r[2];
    });
}

void diagonal(int sym, const Grid& g, const double* C, const int* bct, double* dg) {
    const int64_t N = g.N();
    for_nodes(g, [&](int i, int j, int k) {
        double r[3];
        diag_node(sym, g, C, bct, i, j, k, r);
        const int64_t id = g.id(i, j, k);
        dg[id] = r[0]; dg[N + id] = r[1]; dg[2 * N + id] = r[2];
    });
}

// one Fsmooth call = two damped-Jacobi sweeps (Operator.cpp:107-153)
void fsmooth(int sym, const Grid& g, const double* C, const int* bct, const double* dg, double* x, const double* b,
             double omega, std::vector<double>& Ax) {
    const int64_t n3 = 3 * g.N();
    Ax.resize(n3);
    for (int ctr = 0; ctr < 2; ctr++) {
        fapply(sym, g, C, bct, x, Ax.data());
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < n3; q++) {
            const double Dx = x[q] * dg[q];
            const double Rx = Ax[q] - Dx;
            x[q] = (1. - omega) * x[q] + omega * (b[q] - Rx) / dg[q];
        }
    }
}

// Multicolour Gauss-Seidel (no counterpart in the reference, whose only
// smoother is the damped Jacobi above; a colour-ordered smoother is the
// alternative this port offers).  Colour of node (i, j, k) = (i & 1) +
// 2 (j & 1) + 4 (k & 1): every operator row reads u only at offsets with
// components in {-1, 0, 1} and at most two of them non-zero (19 points:
// faces and edges, the one-sided boundary gradients included), so two nodes
// of one colour never read each other and a colour is updated in place, in
// any order.  One sweep visits colours 0..7; a node's three components are
// updated together from the current field, x_p <- x_p + w (b_p - (A x)_p) /
// D_p, with w = 1 on interior rows and w = omega (the Jacobi damping) on
// boundary rows: undamped updates of traction rows make the V-cycle
// diverge on the traction-free faces of the uniaxial tension test.  One
// Fsmooth call = two sweeps, as for Jacobi.
void gs_sweep(int sym, const Grid& g, const double* C, const int* bct, const double* dg, double* x, const double* b,
              double omega_boundary) {
    const int64_t N = g.N();
    for (int c = 0; c < 8; c++) {
        const int pi = c & 1, pj = (c >> 1) & 1, pk = (c >> 2) & 1;
#pragma omp parallel for schedule(static)
        for (int k = pk; k < g.n[2]; k += 2)
            for (int j = pj; j < g.n[1]; j += 2)
                for (int i = pi; i < g.n[0]; i += 2) {
                    double r[3];
                    fapply_node(sym, g, C, bct, x, i, j, k, r);
                    const int64_t id = g.id(i, j, k);
                    const double w = g.boundary(i, j, k) ? omega_boundary : 1.0;
                    for (int p = 0; p < 3; p++) {
                        const int64_t q = p * N + id;
                        x[q] = x[q] + w * (b[q] - r[p]) / dg[q];
                    }
                }
    }
}

void gs_smooth(int sym, const Grid& g, const double* C, const int* bct, const double* dg, double* x, const double* b,
               double omega_boundary) {
    for (int s = 0; s < 2; s++) gs_sweep(sym, g, C, bct, dg, x, b, omega_boundary);
}

// r = b - A x; returns inf-norm of r (Operator.cpp:635-657)
double residual(int sym, const Grid& g, const double* C, const int* bct, const double* x, const double* b, double* r) {
    const int64_t n3 = 3 * g.N();
    fapply(sym, g, C, bct, x, r);
    double mx = 0.0;
    int64_t nans = 0;
#pragma omp parallel for reduction(max : mx) reduction(+ : nans) schedule(static)
    for (int64_t q = 0; q < n3; q++) {
        r[q] = b[q] + (-1.0) * r[q];
        mx = std::max(mx, std::fabs(r[q]));
        nans += std::isnan(r[q]) ? 1 : 0;
    }
    return nans ? std::nan("") : mx;
}

// nodal full weighting with boundary-reduced weights; works on ncomp values
// per node at stride cs between components and es between node entries
// (Operator.cpp:294-352, Elastic.cpp:786-834).  Used both for vector fields
// (SoA: cs = N, es = 1) and stiffness (AoS: cs = 1, es = nc).
void restrict_generic(const Grid& gf, const Grid& gc, const double* fine, double* crse, int ncomp, int64_t fcs,
                      int64_t fes, int64_t ccs, int64_t ces) {
    const int lox = 0, hix = gc.n[0] - 1, loy = 0, hiy = gc.n[1] - 1, loz = 0, hiz = gc.n[2] - 1;
#pragma omp parallel for schedule(static)
    for (int K = 0; K < gc.n[2]; K++)
        for (int J = 0; J < gc.n[1]; J++)
            for (int I = 0; I < gc.n[0]; I++) {
                const int i = 2 * I, j = 2 * J, k = 2 * K;
                for (int n = 0; n < ncomp; n++) {
                    auto F = [&](int a, int b, int c) { return fine[n * fcs + gf.id(a, b, c) * fes]; };
                    double v;
                    const bool ex = (I == lox || I == hix), ey = (J == loy || J == hiy), ez = (K == loz || K == hiz);
                    if (ex && ey && ez) v = F(i, j, k);
                    else if (ey && ez) v = 0.25 * F(i - 1, j, k) + 0.5 * F(i, j, k) + 0.25 * F(i + 1, j, k);
                    else if (ez && ex) v = 0.25 * F(i, j - 1, k) + 0.5 * F(i, j, k) + 0.25 * F(i, j + 1, k);
                    else if (ex && ey) v = 0.25 * F(i, j, k - 1) + 0.5 * F(i, j, k) + 0.25 * F(i, j, k + 1);
                    else if (ex)
                        v = (+F(i, j - 1, k - 1) + 2.0 * F(i, j, k - 1) + F(i, j + 1, k - 1) + 2.0 * F(i, j - 1, k) +
                             4.0 * F(i, j, k) + 2.0 * F(i, j + 1, k) + F(i, j - 1, k + 1) + 2.0 * F(i, j, k + 1) +
                             F(i, j + 1, k + 1)) / 16.0;
                    else if (ey)
                        v = (+F(i - 1, j, k - 1) + 2.0 * F(i - 1, j, k) + F(i - 1, j, k + 1) + 2.0 * F(i, j, k - 1) +
                             4.0 * F(i, j, k) + 2.0 * F(i, j, k + 1) + F(i + 1, j, k - 1) + 2.0 * F(i + 1, j, k) +
                             F(i + 1, j, k + 1)) / 16.0;
                    else if (ez)
                        v = (+F(i - 1, j - 1, k) + 2.0 * F(i, j - 1, k) + F(i + 1, j - 1, k) + 2.0 * F(i - 1, j, k) +
                             4.0 * F(i, j, k) + 2.0 * F(i + 1, j, k) + F(i - 1, j + 1, k) + 2.0 * F(i, j + 1, k) +
                             F(i + 1, j + 1, k)) / 16.0;
                    else
                        v = (F(i - 1, j - 1, k - 1) + F(i - 1, j - 1, k + 1) + F(i - 1, j + 1, k - 1) +
                             F(i - 1, j + 1, k + 1) + F(i + 1, j - 1, k - 1) + F(i + 1, j - 1, k + 1) +
                             F(i + 1, j + 1, k - 1) + F(i + 1, j + 1, k + 1)) / 64.0 +
                            (F(i, j - 1, k - 1) + F(i, j - 1, k + 1) + F(i, j + 1, k - 1) + F(i, j + 1, k + 1) +
                             F(i - 1, j, k - 1) + F(i + 1, j, k - 1) + F(i - 1, j, k + 1) + F(i + 1, j, k + 1) +
                             F(i - 1, j - 1, k) + F(i - 1, j + 1, k) + F(i + 1, j - 1, k) + F(i + 1, j + 1, k)) / 32.0 +
                            (F(i - 1, j, k) + F(i, j - 1, k) + F(i, j, k - 1) + F(i + 1, j, k) + F(i, j + 1, k) +
                             F(i, j, k + 1)) / 16.0 +
                            F(i, j, k) / 8.0;
                    crse[n * ccs + gc.id(I, J, K) * ces] = v;
                }
            }
}

// trilinear prolongation, added to the fine field (Operator.cpp:399-428)
void prolong_add(const Grid& gf, const Grid& gc, const double* crse, double* fine, int ncomp) {
    const int64_t Nf = gf.N(), Nc = gc.N();
#pragma omp parallel for schedule(static)
    for (int k = 0; k < gf.n[2]; k++)
        for (int j = 0; j < gf.n[1]; j++)
            for (int i = 0; i < gf.n[0]; i++)
                for (int n = 0; n < ncomp; n++) {
                    const int I = i / 2, J = j / 2, K = k / 2;
                    auto Cd = [&](int a, int b, int c) { return crse[n * Nc + gc.id(a, b, c)]; };
                    const bool ei = i % 2 == 0, ej = j % 2 == 0, ek = k % 2 == 0;
                    double v;
                    if (ei && ej && ek) v = Cd(I, J, K);
                    else if (ej && ek) v = 0.5 * (Cd(I, J, K) + Cd(I + 1, J, K));
                    else if (ek && ei) v = 0.5 * (Cd(I, J, K) + Cd(I, J + 1, K));
                    else if (ei && ej) v = 0.5 * (Cd(I, J, K) + Cd(I, J, K + 1));
                    else if (ei) v = 0.25 * (Cd(I, J, K) + Cd(I, J + 1, K) + Cd(I, J, K + 1) + Cd(I, J + 1, K + 1));
                    else if (ej) v = 0.25 * (Cd(I, J, K) + Cd(I, J, K + 1) + Cd(I + 1, J, K) + Cd(I + 1, J, K + 1));
                    else if (ek) v = 0.25 * (Cd(I, J, K) + Cd(I + 1, J, K) + Cd(I, J + 1, K) + Cd(I + 1, J + 1, K));
                    else
                        v = 0.125 * (Cd(I, J, K) + Cd(I + 1, J, K) + Cd(I, J + 1, K) + Cd(I, J, K + 1) +
                                     Cd(I, J + 1, K + 1) + Cd(I + 1, J, K + 1) + Cd(I + 1, J + 1, K) +
                                     Cd(I + 1, J + 1, K + 1));
                    fine[n * Nf + gf.id(i, j, k)] += v;
                }
}

// Coarse-level psi from the fine level (Elastic.cpp:839-905): full
// weighting of the fine cells around coarse cell (I,J,K) = fine (2I,2J,2K).
// The boundary cases compare the cell index against the NODE domain bounds,
// so only index 0 (the low side) takes the face, edge and corner stencils;
// the high side keeps the interior stencil.  Ghost entries stay at 1.0.
void coarsen_psi(const Grid& gf, const Grid& gc, const double* pf, double* pc) {
    const int64_t tot = (int64_t)(gc.n[0] + 1) * (gc.n[1] + 1) * (gc.n[2] + 1);
    for (int64_t q = 0; q < tot; q++) pc[q] = 1.0;
    auto F = [&](int i, int j, int k) { return pf[psi_id(gf, i + 1, j + 1, k + 1)]; };
    for (int K = 0; K < gc.n[2] - 1; K++)
        for (int J = 0; J < gc.n[1] - 1; J++)
            for (int I = 0; I < gc.n[0] - 1; I++) {
                const int i = 2 * I, j = 2 * J, k = 2 * K;
                const bool xi = I == 0, yj = J == 0, zk = K == 0;
                double v;
                if (xi && yj && zk) v = F(i, j, k);
                else if (yj && zk) v = F(i - 1, j, k) * 0.25 + F(i, j, k) * 0.5 + F(i + 1, j, k) * 0.25;
                else if (zk && xi) v = F(i, j - 1, k) * 0.25 + F(i, j, k) * 0.5 + F(i, j + 1, k) * 0.25;
                else if (xi && yj) v = F(i, j, k - 1) * 0.25 + F(i, j, k) * 0.5 + F(i, j, k + 1) * 0.25;
                else if (xi)
                    v = (F(i, j - 1, k - 1) + F(i, j, k - 1) * 2.0 + F(i, j + 1, k - 1) + F(i, j - 1, k) * 2.0 +
                         F(i, j, k) * 4.0 + F(i, j + 1, k) * 2.0 + F(i, j - 1, k + 1) + F(i, j, k + 1) * 2.0 +
                         F(i, j + 1, k + 1)) / 16.0;
                else if (yj)
                    v = (F(i - 1, j, k - 1) + F(i - 1, j, k) * 2.0 + F(i - 1, j, k + 1) + F(i, j, k - 1) * 2.0 +
                         F(i, j, k) * 4.0 + F(i, j, k + 1) * 2.0 + F(i + 1, j, k - 1) + F(i + 1, j, k) * 2.0 +
                         F(i + 1, j, k + 1)) / 16.0;
                else if (zk)
                    v = (F(i - 1, j - 1, k) + F(i, j - 1, k) * 2.0 + F(i + 1, j - 1, k) + F(i - 1, j, k) * 2.0 +
                         F(i, j, k) * 4.0 + F(i + 1, j, k) * 2.0 + F(i - 1, j + 1, k) + F(i, j + 1, k) * 2.0 +
                         F(i + 1, j + 1, k)) / 16.0;
                else
                    v = (F(i - 1, j - 1, k - 1) + F(i - 1, j - 1, k + 1) + F(i - 1, j + 1, k - 1) +
                         F(i - 1, j + 1, k + 1) + F(i + 1, j - 1, k - 1) + F(i + 1, j - 1, k + 1) +
                         F(i + 1, j + 1, k - 1) + F(i + 1, j + 1, k + 1)) / 64.0 +
                        (F(i, j - 1, k - 1) + F(i, j - 1, k + 1) + F(i, j + 1, k - 1) + F(i, j + 1, k + 1) +
                         F(i - 1, j, k - 1) + F(i + 1, j, k - 1) + F(i - 1, j, k + 1) + F(i + 1, j, k + 1) +
                         F(i - 1, j - 1, k) + F(i - 1, j + 1, k) + F(i + 1, j - 1, k) + F(i + 1, j + 1, k)) / 32.0 +
                        (F(i - 1, j, k) + F(i, j - 1, k) + F(i, j, k - 1) + F(i + 1, j, k) + F(i, j + 1, k) +
                         F(i, j, k + 1)) / 16.0 +
                        F(i, j, k) / 8.0;
                pc[psi_id(gc, I + 1, J + 1, K + 1)] = v;
            }
}

// max |a|; NaN when any entry is NaN (a max-reduction alone drops NaNs)
double norm_inf(const double* a, int64_t n) {
    double mx = 0.0;
    int64_t nans = 0;
#pragma omp parallel for reduction(max : mx) reduction(+ : nans) schedule(static)
    for (int64_t q = 0; q < n; q++) {
        mx = std::max(mx, std::fabs(a[q]));
        nans += std::isnan(a[q]) ? 1 : 0;
    }
    return nans ? std::nan("") : mx;
}

double dot(const double* a, const double* b, int64_t n) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t q = 0; q < n; q++) s += a[q] * b[q];
    return s;
}

}  // namespace

// ============================================================================
// C ABI of the oracle
// ============================================================================
extern "C" {

struct orc_opts {
    int max_iter;              // MLMG max iterations (AMReX default 200)
    int pre_smooth;            // Fsmooth calls before restriction (2)
    int post_smooth;           // Fsmooth calls after prolongation (2)
    int final_smooth;          // Fsmooth calls when the bottom solve fails (8)
    int bottom_smooth;         // Fsmooth calls after a good bottom solve (0)
    int bottom_max_iter;       // BiCGStab iterations (200)
    double bottom_tol_rel;     // 1e-4
    double bottom_tol_abs;     // -1
    double omega;              // 2/3
    int max_coarsening_level;  // -1 = as deep as possible
    int fixed_iter;            // -1 = run to tolerance
    int verbose;
    int bottom_solver;         // 0 BiCGStab, 1 dense direct (exact), 2 smoother only
    int max_fmg_iter;          // iterations that run an F-cycle before V-cycles take over
                               // (Linear::PrepareMLMG sets 100000000, Linear.H:261)
    int smoother;              // 0 damped Jacobi (the reference's Fsmooth), 1 multicolour Gauss-Seidel
};

struct orc_report {
    int iters;
    int status;  // 0 converged, 1 not converged, 2 nan
    int nlevels;
    int bottom_iters_total;
    double resnorm0, rhsnorm0, final_resnorm, seconds;
    double setup_seconds;  // hierarchy set-up and the first residual
};

static int64_t nsz(int nx, int ny, int nz) { return (int64_t)nx * ny * nz; }

static Grid mkgrid(int nx, int ny, int nz, const double* dx) {
    Grid g;
    g.n[0] = nx; g.n[1] = ny; g.n[2] = nz;
    g.dx[0] = dx[0]; g.dx[1] = dx[1]; g.dx[2] = dx[2];
    g.psi = g_psi;
    g.psi_small = g_psi_small;
    return g;
}

// SetUniform (src/Operator/Elastic.H:104-107): uniform = 1 drops the
// grad-C term of interior rows.
void orc_set_uniform(int uniform) { g_grad_c = uniform == 0; }

// psi for the calls that follow (Elastic::SetPsi, Elastic.cpp:118-137).
// For a node grid nx*ny*nz, psi_ghost holds (nx+1)(ny+1)(nz+1) values: the
// (nx-1)(ny-1)(nz-1) cells with one ghost layer on each side, x fastest,
// entry (a,b,c) = cell (a-1,b-1,c-1).  The ghost entries must be 1.0 (the
// reference fills its psi with 1.0 at define time and SetPsi copies only
// the domain's cells).  nullptr clears psi.
void orc_set_psi(const double* psi_ghost, double small) {
    g_psi = psi_ghost;
    g_psi_small = small;
}

// Coarse-level psi of one multigrid coarsening (Elastic.cpp:839-905); both
// arrays in the ghosted layout of orc_set_psi (fine node grid nxf*nyf*nzf).
void orc_coarsen_psi(int nxf, int nyf, int nzf, const double* pf, double* pc) {
    const double one[3] = {1, 1, 1};
    Grid gf = mkgrid(nxf, nyf, nzf, one);
    Grid gc = mkgrid((nxf - 1) / 2 + 1, (nyf - 1) / 2 + 1, (nzf - 1) / 2 + 1, one);
    coarsen_psi(gf, gc, pf, pc);
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

void orc_fapply(int sym, int nx, int ny, int nz, const double* dx, const double* C, const int* bc_type,
                const double* u, double* f) {
    Grid g = mkgrid(nx, ny, nz, dx);
    fapply(sym, g, C, bc_type, u, f);
}

void orc_diagonal(int sym, int nx, int ny, int nz, const double* dx, const double* C, const int* bc_type,
                  double* diag) {
    Grid g = mkgrid(nx, ny, nz, dx);
    diagonal(sym, g, C, bc_type, diag);
}

void orc_fsmooth(int sym, int nx, int ny, int nz, const double* dx, const double* C, const int* bc_type,
                 const double* diag, double* x, const double* b, double omega, int ncalls) {
    Grid g = mkgrid(nx, ny, nz, dx);
    std::vector<double> Ax;
    for (int c = 0; c < ncalls; c++) fsmooth(sym, g, C, bc_type, diag, x, b, omega, Ax);
}

// ncalls calls of the multicolour Gauss-Seidel smoother (two sweeps each)
void orc_gs_smooth(int sym, int nx, int ny, int nz, const double* dx, const double* C, const int* bc_type,
                   const double* diag, double* x, const double* b, double omega, int ncalls) {
    Grid g = mkgrid(nx, ny, nz, dx);
    for (int c = 0; c < ncalls; c++) gs_smooth(sym, g, C, bc_type, diag, x, b, omega);
}

// one damped-Jacobi sweep (half an Fsmooth call), for sweep-level parity tests
void orc_jacobi_sweep(int sym, int nx, int ny, int nz, const double* dx, const double* C, const int* bc_type,
                      const double* diag, const double* x, const double* b, double omega, double* xout) {
    Grid g = mkgrid(nx, ny, nz, dx);
    const int64_t n3 = 3 * g.N();
    std::vector<double> Ax(n3);
    fapply(sym, g, C, bc_type, x, Ax.data());
    for (int64_t q = 0; q < n3; q++) {
        const double Dx = x[q] * diag[q];
        const double Rx = Ax[q] - Dx;
        xout[q] = (1. - omega) * x[q] + omega * (b[q] - Rx) / diag[q];
    }
}

double orc_residual(int sym, int nx, int ny, int nz, const double* dx, const double* C, const int* bc_type,
                    const double* x, const double* b, double* r) {
    Grid g = mkgrid(nx, ny, nz, dx);
    return residual(sym, g, C, bc_type, x, b, r);
}

// restrict a 3-component SoA field from a fine node grid to its 2x coarser grid
void orc_restrict(int nxf, int nyf, int nzf, const double* fine, double* crse) {
    double one[3] = {1, 1, 1};
    Grid gf = mkgrid(nxf, nyf, nzf, one);
    Grid gc = mkgrid((nxf - 1) / 2 + 1, (nyf - 1) / 2 + 1, (nzf - 1) / 2 + 1, one);
    restrict_generic(gf, gc, fine, crse, 3, gf.N(), 1, gc.N(), 1);
}

// restrict per-node stiffness (AoS, nc values per node)
void orc_restrict_C(int sym, int nxf, int nyf, int nzf, const double* Cf, double* Cc) {
    double one[3] = {1, 1, 1};
    const int nc = nc_of(sym);
    Grid gf = mkgrid(nxf, nyf, nzf, one);
    Grid gc = mkgrid((nxf - 1) / 2 + 1, (nyf - 1) / 2 + 1, (nzf - 1) / 2 + 1, one);
    restrict_generic(gf, gc, Cf, Cc, nc, 1, nc, 1, nc);
}

void orc_prolong_add(int nxf, int nyf, int nzf, const double* crse, double* fine) {
    double one[3] = {1, 1, 1};
    Grid gf = mkgrid(nxf, nyf, nzf, one);
    Grid gc = mkgrid((nxf - 1) / 2 + 1, (nyf - 1) / 2 + 1, (nzf - 1) / 2 + 1, one);
    prolong_add(gf, gc, crse, fine, 3);
}

// BC::Operator::Elastic::Constant::Init: write boundary values into b
// (Constant.H:197-286; non-periodic geometry)
void orc_bc_init(int nx, int ny, int nz, const int* bc_type, const double* bc_val, int homogeneous, double* b) {
    double one[3] = {1, 1, 1};
    Grid g = mkgrid(nx, ny, nz, one);
    const int64_t N = g.N();
    for_nodes(g, [&](int i, int j, int k) {
        if (!g.boundary(i, j, k)) return;
        double nrm[3];
        const int reg = region(g, i, j, k, nrm);
        for (int d = 0; d < 3; d++) {
            if (homogeneous && bc_type[reg * 3 + d] == DISP) b[d * N + g.id(i, j, k)] = 0.0;
            else b[d * N + g.id(i, j, k)] = bc_val[reg * 3 + d];
        }
    });
}

// Newton::prepareForSolve for a gradu-kinematics model with eigenstrain F0
// (Newton.H:144-231, psi unset):  dw = C (grad u - F0);  rhs = b - div dw in
// the interior, rhs = b - BC(u, grad u, dw) on the boundary.
// F0 has f0_ncomp values per node: 0 (none), 1 (F0 = s I) or 9 (row-major).
void rhs_from_dw(const Grid& g, const double* dw, const int* bc_type, const double* u, const double* b,
                 double* rhs);

void orc_build_rhs(int sym, int nx, int ny, int nz, const double* dx, const double* C, const double* F0,
                   int f0_ncomp, const int* bc_type, const double* u, const double* b, double* rhs) {
    Grid g = mkgrid(nx, ny, nz, dx);
    const int64_t N = g.N();
    const int nc = nc_of(sym);
    std::vector<double> dw(9 * N);
    const double* uu[3] = {u, u + N, u + 2 * N};
    for_nodes(g, [&](int i, int j, int k) {
        const int64_t id = g.id(i, j, k);
        int s[3];
        get_stencil(g, i, j, k, s);
        double gu[3][3];
        for (int p = 0; p < 3; p++)
            for (int q = 0; q < 3; q++) gu[p][q] = d1(g, uu[p], i, j, k, q, s[q]);
        if (f0_ncomp == 1) {
            for (int p = 0; p < 3; p++) gu[p][p] = gu[p][p] - F0[id];
        } else if (f0_ncomp == 9) {
            for (int p = 0; p < 3; p++)
                for (int q = 0; q < 3; q++) gu[p][q] = gu[p][q] - F0[id * 9 + p * 3 + q];
        }
        double sg[3][3];
        c_grad(sym, C + id * nc, gu, sg);
        for (int p = 0; p < 3; p++)
            for (int q = 0; q < 3; q++) dw[id * 9 + p * 3 + q] = sg[p][q];
    });
    rhs_from_dw(g, dw.data(), bc_type, u, b, rhs);
}

// rhs = b - div(dw) (interior) / b - BC(u, grad u, dw) (boundary) for a given
// nodal stress field dw (Newton.H:205-266); dw AoS, 9 values row-major
void rhs_from_dw(const Grid& g, const double* dw, const int* bc_type, const double* u, const double* b,
                 double* rhs) {
    const int64_t N = g.N();
    const double* uu[3] = {u, u + N, u + 2 * N};
    for_nodes(g, [&](int i, int j, int k) {
        const int64_t id = g.id(i, j, k);
        int s[3];
        get_stencil(g, i, j, k, s);
        double ret[3];
        if (g.boundary(i, j, k)) {
            double gu[3][3];
            for (int p = 0; p < 3; p++)
                for (int q = 0; q < 3; q++) gu[p][q] = d1(g, uu[p], i, j, k, q, s[q]);
            double uv[3] = {uu[0][id], uu[1][id], uu[2][id]};
            double sg[3][3];
            for (int p = 0; p < 3; p++)
                for (int q = 0; q < 3; q++) sg[p][q] = dw[id * 9 + p * 3 + q];
            double nrm[3];
            const int reg = region(g, i, j, k, nrm);
            bc_row(bc_type, reg, nrm, uv, gu, sg, ret);
        } else {
            // Stencil.H:588-657 with central stencil in every direction
            ret[0] = ret[1] = ret[2] = 0.0;
            for (int d = 0; d < 3; d++) {
                const int64_t ip = g.id(i + E[d][0], j + E[d][1], k + E[d][2]);
                const int64_t im = g.id(i - E[d][0], j - E[d][1], k - E[d][2]);
                for (int c = 0; c < 3; c++) ret[c] += (dw[ip * 9 + c * 3 + d] - dw[im * 9 + c * 3 + d]) / 2. / g.dx[d];
            }
            if (g.psi) {
                // Newton.H:255-261: raw cell average (no psi_small), dw grad psi
                const double pa = psi_cell_avg(g, i, j, k);
                double gp[3];
                psi_grad(g, i, j, k, gp);
                for (int c = 0; c < 3; c++)
                    ret[c] = ret[c] * pa + dw[id * 9 + c * 3 + 0] * gp[0] + dw[id * 9 + c * 3 + 1] * gp[1] +
                             dw[id * 9 + c * 3 + 2] * gp[2];
            }
        }
        for (int d = 0; d < 3; d++) rhs[d * N + id] = b[d * N + id] - ret[d];
    });
}

// Per-node stress sigma = C (grad u - F0) (9 values, row-major) and strain
// eps = sym(grad u) (9 values), one-sided at the domain boundary
// (Mechanics.H:210-248, Elastic.cpp:426-549).  energy = 0.5 sigma:eps.
void orc_stress_strain(int sym, int nx, int ny, int nz, const double* dx, const double* C, const double* F0,
                       int f0_ncomp, const double* u, double* stress, double* strain, double* energy) {
    Grid g = mkgrid(nx, ny, nz, dx);
    const int64_t N = g.N();
    const int nc = nc_of(sym);
    const double* uu[3] = {u, u + N, u + 2 * N};
    for_nodes(g, [&](int i, int j, int k) {
        const int64_t id = g.id(i, j, k);
        int s[3];
        get_stencil(g, i, j, k, s);
        double gu[3][3], ge[3][3];
        for (int p = 0; p < 3; p++)
            for (int q = 0; q < 3; q++) gu[p][q] = d1(g, uu[p], i, j, k, q, s[q]);
        for (int p = 0; p < 3; p++)
            for (int q = 0; q < 3; q++) {
                double f0 = 0.0;
                if (f0_ncomp == 1) f0 = (p == q) ? F0[id] : 0.0;
                else if (f0_ncomp == 9) f0 = F0[id * 9 + p * 3 + q];
                ge[p][q] = gu[p][q] - f0;
            }
        double sg[3][3];
        c_grad(sym, C + id * nc, ge, sg);
        double en = 0.0;
        for (int p = 0; p < 3; p++)
            for (int q = 0; q < 3; q++) {
                const double e = 0.5 * (gu[p][q] + gu[q][p]);
                if (stress) stress[id * 9 + p * 3 + q] = sg[p][q];
                if (strain) strain[id * 9 + p * 3 + q] = e;
                en += .5 * sg[p][q] * e;
            }
        if (energy) energy[id] = en;
    });
}

// One finite-difference derivative of a scalar node field at every interior
// node with the central stencils of Stencil.H (which = 100, 010, 001, 200,
// 020, 002, 110, 101, 011); boundary nodes are set to 0.  Used to restate the
// reference's stencil accuracy test (src/Test/Numeric/Stencil.H:58-106).
void orc_derivative(int which, int nx, int ny, int nz, const double* dx, const double* f, double* out) {
    Grid g = mkgrid(nx, ny, nz, dx);
    for_nodes(g, [&](int i, int j, int k) {
        double v = 0.0;
        if (!g.boundary(i, j, k)) {
            switch (which) {
                case 100: v = d1(g, f, i, j, k, 0, CENTRAL); break;
                case 10: v = d1(g, f, i, j, k, 1, CENTRAL); break;
                case 1: v = d1(g, f, i, j, k, 2, CENTRAL); break;
                case 200: v = d2(g, f, i, j, k, 0); break;
                case 20: v = d2(g, f, i, j, k, 1); break;
                case 2: v = d2(g, f, i, j, k, 2); break;
                case 110: v = dmix(g, f, i, j, k, 0, 1); break;
                case 101: v = dmix(g, f, i, j, k, 0, 2); break;
                case 11: v = dmix(g, f, i, j, k, 1, 2); break;
                default: v = NAN;
            }
        }
        out[g.id(i, j, k)] = v;
    });
}

// Matrix4<3,MajorMinor>::Cubic(C11,C12,C44,R) (Matrix4_MajorMinor.H:518-547):
// rotate the (not minor-symmetrised) cubic table and store each of the 21
// classes with the value of its last-written index tuple in (p,q,s,t) order.
void orc_cubic(double C11, double C12, double C44, const double* R, double* out21) {
    double Ct[3][3][3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++) {
                    if (i == j && j == k && k == l) Ct[i][j][k][l] = C11;
                    else if (i == k && j == l) Ct[i][j][k][l] = C44;
                    else if (i == j && k == l) Ct[i][j][k][l] = C12;
                    else Ct[i][j][k][l] = 0.0;
                }
    auto Rm = [&](int a, int b) { return R[a * 3 + b]; };
    for (int p = 0; p < 3; p++)
        for (int q = 0; q < 3; q++)
            for (int s = 0; s < 3; s++)
                for (int t = 0; t < 3; t++) {
                    double acc = 0.0;
                    for (int i = 0; i < 3; i++)
                        for (int j = 0; j < 3; j++)
                            for (int k = 0; k < 3; k++)
                                for (int l = 0; l < 3; l++) acc += Rm(p, i) * Rm(s, k) * Ct[i][j][k][l] * Rm(q, j) * Rm(t, l);
                    out21[UT[PAIR[p][q]][PAIR[s][t]]] = acc;
                }
}

// ---------------------------------------------------------------------------
// Multigrid solve of A x = rhs on one AMR level, restating amrex::MLMG as
// configured by Solver::Nonlocal::Linear (F-cycles, or V-cycles after
// max_fmg_iter iterations, on the correction equation; BiCGStab bottom on the
// diagonally normalised system).
// ---------------------------------------------------------------------------
namespace {

struct Level {
    Grid g;
    std::vector<double> C, diag, res, cor, rescor, tmp, psi, hold;
};

// psi of level l > 0 coarsened from level l - 1 (prepareForSolve order:
// averageDownCoeffs before Diagonal, Operator.cpp:253-259)
void level_psi(Level& f, Level& c) {
    if (!f.g.psi) { c.g.psi = nullptr; return; }
    c.psi.assign((size_t)(c.g.n[0] + 1) * (c.g.n[1] + 1) * (c.g.n[2] + 1), 1.0);
    coarsen_psi(f.g, c.g, f.g.psi, c.psi.data());
    c.g.psi = c.psi.data();
}

struct Hier {
    int sym;
    const int* bct;
    std::vector<Level> L;
    orc_opts o;
    int bottom_iters = 0;

    void smooth(int l, int ncalls) {
        Level& v = L[l];
        for (int c = 0; c < ncalls; c++) {
            if (o.smoother == 1) gs_smooth(sym, v.g, v.C.data(), bct, v.diag.data(), v.cor.data(), v.res.data(), o.omega);
            else fsmooth(sym, v.g, v.C.data(), bct, v.diag.data(), v.cor.data(), v.res.data(), o.omega, v.tmp);
        }
    }

    // BiCGStab with left Jacobi scaling (alamo's normalize divides by the
    // diagonal); published algorithm (van der Vorst 1992) as MLCGSolver runs it.
    // A NaN residual norm counts as a breakdown (ret 5): the failed-bottom
    // path (zero correction, final_smooth calls) takes over.
    int bicgstab(int l, double* sol, const double* rhs) {
        Level& v = L[l];
        const Grid& g = v.g;
        const int64_t n3 = 3 * g.N();
        std::vector<double> r(n3), rh(n3), p(n3, 0.0), vv(n3, 0.0), s(n3), t(n3);
        const double* dg = v.diag.data();
        // r = rhs - A sol, sol = 0 start
        fapply(sym, g, v.C.data(), bct, sol, r.data());
        for (int64_t q = 0; q < n3; q++) r[q] = (rhs[q] - r[q]) / dg[q];
        std::vector<double> sorig(sol, sol + n3);
        std::fill(sol, sol + n3, 0.0);
        rh = r;
        double rnorm = norm_inf(r.data(), n3);
        const double rnorm0 = rnorm;
        int ret = 0, iter = 1;
        double rho_1 = 0, alpha = 0, omega = 0;
        if (rnorm0 == 0 || rnorm0 < o.bottom_tol_abs) {
            for (int64_t q = 0; q < n3; q++) sol[q] += sorig[q];
            return 0;
        }
        for (; iter <= o.bottom_max_iter; ++iter) {
            const double rho = dot(rh.data(), r.data(), n3);
            if (rho == 0) { ret = 1; break; }
            if (iter == 1) p = r;
            else {
                const double beta = (rho / rho_1) * (alpha / omega);
                for (int64_t q = 0; q < n3; q++) p[q] = r[q] + beta * (p[q] - omega * vv[q]);
            }
            fapply(sym, g, v.C.data(), bct, p.data(), vv.data());
            for (int64_t q = 0; q < n3; q++) vv[q] /= dg[q];
            const double rhTv = dot(rh.data(), vv.data(), n3);
            if (rhTv != 0.0) alpha = rho / rhTv;
            else { ret = 2; break; }
            for (int64_t q = 0; q < n3; q++) { sol[q] += alpha * p[q]; s[q] = r[q] - alpha * vv[q]; }
            rnorm = norm_inf(s.data(), n3);
            if (std::isnan(rnorm)) { ret = 5; break; }
            if (rnorm < o.bottom_tol_rel * rnorm0 || rnorm < o.bottom_tol_abs) break;
            fapply(sym, g, v.C.data(), bct, s.data(), t.data());
            for (int64_t q = 0; q < n3; q++) t[q] /= dg[q];
            const double tt = dot(t.data(), t.data(), n3), ts = dot(t.data(), s.data(), n3);
            if (tt != 0.0) omega = ts / tt;
            else { ret = 3; break; }
            for (int64_t q = 0; q < n3; q++) { sol[q] += omega * s[q]; r[q] = s[q] - omega * t[q]; }
            rnorm = norm_inf(r.data(), n3);
            if (std::isnan(rnorm)) { ret = 5; break; }
            if (rnorm < o.bottom_tol_rel * rnorm0 || rnorm < o.bottom_tol_abs) break;
            if (omega == 0) { ret = 4; break; }
            rho_1 = rho;
        }
        bottom_iters += std::min(iter, o.bottom_max_iter);
        if (ret == 0 && rnorm > o.bottom_tol_rel * rnorm0 && rnorm > o.bottom_tol_abs) ret = 8;
        if ((ret == 0 || ret == 8) && rnorm < rnorm0) {
            for (int64_t q = 0; q < n3; q++) sol[q] += sorig[q];
        } else {
            for (int64_t q = 0; q < n3; q++) sol[q] = sorig[q];
        }
        return ret;
    }

    // dense matrix of the coarsest operator, factorised once (Gaussian
    // elimination with partial pivoting); empty when singular
    std::vector<double> LU;
    std::vector<int> piv;
    bool dense_ok = false, dense_tried = false;

    void build_dense() {
        dense_tried = true;
        Level& v = L.back();
        const int nb = (int)(3 * v.g.N());
        if (nb > 4000) return;
        LU.assign((size_t)nb * nb, 0.0);
        std::vector<double> e(nb, 0.0), col(nb);
        for (int j = 0; j < nb; j++) {
            e[j] = 1.0;
            fapply(sym, v.g, v.C.data(), bct, e.data(), col.data());
            for (int i = 0; i < nb; i++) LU[(size_t)i * nb + j] = col[i];
            e[j] = 0.0;
        }
        double dmax = 0.0;
        for (int i = 0; i < nb; i++) dmax = std::max(dmax, std::fabs(v.diag[i]));
        piv.resize(nb);
        for (int k = 0; k < nb; k++) {
            int p = k;
            for (int i = k + 1; i < nb; i++)
                if (std::fabs(LU[(size_t)i * nb + k]) > std::fabs(LU[(size_t)p * nb + k])) p = i;
            piv[k] = p;
            if (!(std::fabs(LU[(size_t)p * nb + k]) > 1e-12 * dmax)) { LU.clear(); return; }
            if (p != k)
                for (int c = 0; c < nb; c++) std::swap(LU[(size_t)k * nb + c], LU[(size_t)p * nb + c]);
            for (int i = k + 1; i < nb; i++) {
                const double f = LU[(size_t)i * nb + k] / LU[(size_t)k * nb + k];
                LU[(size_t)i * nb + k] = f;
                for (int c = k + 1; c < nb; c++) LU[(size_t)i * nb + c] -= f * LU[(size_t)k * nb + c];
            }
        }
        dense_ok = true;
    }

    void dense_solve(double* x, const double* b) {
        const int nb = (int)piv.size();
        std::vector<double> y(b, b + nb);
        for (int k = 0; k < nb; k++) std::swap(y[k], y[piv[k]]);
        for (int i = 0; i < nb; i++)
            for (int c = 0; c < i; c++) y[i] -= LU[(size_t)i * nb + c] * y[c];
        for (int i = nb - 1; i >= 0; i--) {
            for (int c = i + 1; c < nb; c++) y[i] -= LU[(size_t)i * nb + c] * y[c];
            y[i] /= LU[(size_t)i * nb + i];
        }
        for (int i = 0; i < nb; i++) x[i] = y[i];
    }

    void bottom() {
        const int l = (int)L.size() - 1;
        Level& v = L[l];
        if (o.bottom_solver == 1) {
            if (!dense_tried) build_dense();
            if (dense_ok) { dense_solve(v.cor.data(), v.res.data()); return; }
        }
        std::fill(v.cor.begin(), v.cor.end(), 0.0);
        if (o.bottom_solver == 2) {
            smooth(l, o.final_smooth);
            return;
        }
        const int ret = bicgstab(l, v.cor.data(), v.res.data());
        if (ret != 0) {
            std::fill(v.cor.begin(), v.cor.end(), 0.0);
            smooth(l, o.final_smooth);
        } else {
            smooth(l, o.bottom_smooth);
        }
    }

    // V-cycle on A cor = res of level l0 (MLMG::mgVcycle(amrlev, mglev))
    void vcycle(int l0 = 0) {
        const int nl = (int)L.size();
        if (l0 == nl - 1) { bottom(); return; }
        for (int l = l0; l < nl - 1; l++) {
            Level& v = L[l];
            std::fill(v.cor.begin(), v.cor.end(), 0.0);
            smooth(l, o.pre_smooth);
            // rescor = res - A cor
            residual(sym, v.g, v.C.data(), bct, v.cor.data(), v.res.data(), v.rescor.data());
            Level& c = L[l + 1];
            restrict_generic(v.g, c.g, v.rescor.data(), c.res.data(), 3, v.g.N(), 1, c.g.N(), 1);
        }
        bottom();
        for (int l = nl - 2; l >= l0; l--) {
            Level& v = L[l];
            Level& c = L[l + 1];
            prolong_add(v.g, c.g, c.cor.data(), v.cor.data(), 3);
            smooth(l, o.post_smooth);
        }
    }

    // F-cycle on A cor = res of level 0, as MLMG::mgFcycle runs it for the
    // iterations below max_fmg_iter: the residual restricted to every level,
    // the bottom solve, then on each finer level the interpolated coarse
    // correction as a start (interpAssign), the residual of that correction
    // as the right-hand side of a V-cycle from this level, and the
    // interpolated start added back.  The residual goes down with the
    // operator's restriction (Operator.cpp:262-363), the correction up with
    // its interpolation (:365-434) into a zeroed fine correction.
    void fcycle() {
        const int nl = (int)L.size();
        for (int l = 1; l < nl; l++)
            restrict_generic(L[l - 1].g, L[l].g, L[l - 1].res.data(), L[l].res.data(), 3, L[l - 1].g.N(), 1,
                             L[l].g.N(), 1);
        bottom();
        for (int l = nl - 2; l >= 0; l--) {
            Level& v = L[l];
            Level& c = L[l + 1];
            std::fill(v.cor.begin(), v.cor.end(), 0.0);
            prolong_add(v.g, c.g, c.cor.data(), v.cor.data(), 3);
            residual(sym, v.g, v.C.data(), bct, v.cor.data(), v.res.data(), v.rescor.data());
            std::swap(v.res, v.rescor);
            v.hold.swap(v.cor);
            v.cor.assign(v.hold.size(), 0.0);
            vcycle(l);
            for (size_t q = 0; q < v.cor.size(); q++) v.cor[q] += v.hold[q];
        }
    }

    void cycle(int iter) {
        if (iter < o.max_fmg_iter) fcycle();
        else vcycle();
    }
};

}  // namespace

void orc_default_opts(orc_opts* o) {
    o->max_iter = 200;
    o->pre_smooth = 2;
    o->post_smooth = 2;
    o->final_smooth = 8;
    o->bottom_smooth = 0;
    o->bottom_max_iter = 200;
    o->bottom_tol_rel = 1e-4;
    o->bottom_tol_abs = -1.0;
    o->omega = 2. / 3.;
    o->max_coarsening_level = -1;
    o->fixed_iter = -1;
    o->verbose = 0;
    o->bottom_solver = 0;
    o->max_fmg_iter = 100000000;
    o->smoother = 0;
}

// number of multigrid levels for a node grid (coarsen by 2 while every
// direction keeps at least 2 cells, AMReX's default minimum width)
int orc_num_levels(int nx, int ny, int nz, int max_coarsening_level) {
    int n[3] = {nx, ny, nz};
    int lev = 1;
    while (max_coarsening_level < 0 || lev - 1 < max_coarsening_level) {
        bool ok = true;
        for (int d = 0; d < 3; d++) {
            const int cells = n[d] - 1;
            if (cells % 2 != 0 || cells / 2 < 2) ok = false;
        }
        if (!ok) break;
        for (int d = 0; d < 3; d++) n[d] = (n[d] - 1) / 2 + 1;
        lev++;
    }
    return lev;
}

// One V-cycle on A cor = res from cor = 0 on the fine level (for parity of
// the multigrid cycle itself).
void orc_vcycle(int sym, int nx, int ny, int nz, const double* dx, const double* C, const int* bc_type,
                const orc_opts* opts, const double* res, double* cor) {
    Hier H;
    H.sym = sym;
    H.bct = bc_type;
    H.o = *opts;
    const int nlev = orc_num_levels(nx, ny, nz, opts->max_coarsening_level);
    const int nc = nc_of(sym);
    H.L.resize(nlev);
    for (int l = 0; l < nlev; l++) {
        Level& v = H.L[l];
        if (l == 0) v.g = mkgrid(nx, ny, nz, dx);
        else {
            const Grid& f = H.L[l - 1].g;
            const double cdx[3] = {2 * f.dx[0], 2 * f.dx[1], 2 * f.dx[2]};
            v.g = mkgrid((f.n[0] - 1) / 2 + 1, (f.n[1] - 1) / 2 + 1, (f.n[2] - 1) / 2 + 1, cdx);
        }
        const int64_t N = v.g.N();
        v.C.resize(N * nc);
        if (l == 0) std::memcpy(v.C.data(), C, sizeof(double) * N * nc);
        else {
            restrict_generic(H.L[l - 1].g, v.g, H.L[l - 1].C.data(), v.C.data(), nc, 1, nc, 1, nc);
            level_psi(H.L[l - 1], v);
        }
        v.diag.resize(3 * N);
        diagonal(sym, v.g, v.C.data(), bc_type, v.diag.data());
        v.res.assign(3 * N, 0.0);
        v.cor.assign(3 * N, 0.0);
        v.rescor.assign(3 * N, 0.0);
    }
    const int64_t n3 = 3 * H.L[0].g.N();
    std::memcpy(H.L[0].res.data(), res, sizeof(double) * n3);
    H.vcycle();
    std::memcpy(cor, H.L[0].cor.data(), sizeof(double) * n3);
}

// Solve A sol = rhs (sol holds the initial guess on entry).  res_hist (may be
// null) receives the inf-norm of the residual before each V-cycle and after
// the last one (max_iter+1 entries).
int orc_solve(int sym, int nx, int ny, int nz, const double* dx, const double* C, const int* bc_type,
              const orc_opts* opts, double tol_rel, double tol_abs, double* sol, const double* rhs,
              orc_report* rep, double* res_hist) {
    auto t0 = std::chrono::steady_clock::now();
    Hier H;
    H.sym = sym;
    H.bct = bc_type;
    H.o = *opts;
    const int nlev = orc_num_levels(nx, ny, nz, opts->max_coarsening_level);
    const int nc = nc_of(sym);
    H.L.resize(nlev);
    for (int l = 0; l < nlev; l++) {
        Level& v = H.L[l];
        if (l == 0) v.g = mkgrid(nx, ny, nz, dx);
        else {
            const Grid& f = H.L[l - 1].g;
            const double cdx[3] = {2 * f.dx[0], 2 * f.dx[1], 2 * f.dx[2]};
            v.g = mkgrid((f.n[0] - 1) / 2 + 1, (f.n[1] - 1) / 2 + 1, (f.n[2] - 1) / 2 + 1, cdx);
        }
        const int64_t N = v.g.N();
        v.C.resize(N * nc);
        if (l == 0) std::memcpy(v.C.data(), C, sizeof(double) * N * nc);
        else {
            Level& f = H.L[l - 1];
            restrict_generic(f.g, v.g, f.C.data(), v.C.data(), nc, 1, nc, 1, nc);
            level_psi(f, v);
        }
        v.diag.resize(3 * N);
        diagonal(sym, v.g, v.C.data(), bc_type, v.diag.data());
        v.res.assign(3 * N, 0.0);
        v.cor.assign(3 * N, 0.0);
        v.rescor.assign(3 * N, 0.0);
    }
    Level& top = H.L[0];
    const int64_t n3 = 3 * top.g.N();
    double resnorm0 = residual(sym, top.g, top.C.data(), bc_type, sol, rhs, top.res.data());
    const double rhsnorm0 = norm_inf(rhs, n3);
    const double t_setup = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    const double max_norm = (rhsnorm0 >= resnorm0) ? rhsnorm0 : resnorm0;
    const double target = std::max(tol_abs, std::max(tol_rel, 1.e-16) * max_norm);
    int status = 1, it = 0;
    double rn = resnorm0;
    if (res_hist) res_hist[0] = rn;
    const int maxit = opts->fixed_iter > 0 ? opts->fixed_iter : opts->max_iter;
    if (rn <= target && opts->fixed_iter <= 0) status = 0;
    else {
        for (it = 0; it < maxit; it++) {
            H.cycle(it);
            for (int64_t q = 0; q < n3; q++) sol[q] += top.cor[q];
            rn = residual(sym, top.g, top.C.data(), bc_type, sol, rhs, top.res.data());
            if (res_hist) res_hist[it + 1] = rn;
            if (std::isnan(rn)) { status = 2; it++; break; }
            if (rn <= target && opts->fixed_iter <= 0) { status = 0; it++; break; }
        }
        if (opts->fixed_iter > 0 && status != 2) status = 0;
    }
    if (rep) {
        rep->iters = it;
        rep->status = status;
        rep->nlevels = nlev;
        rep->bottom_iters_total = H.bottom_iters;
        rep->resnorm0 = resnorm0;
        rep->rhsnorm0 = rhsnorm0;
        rep->final_resnorm = rn;
        rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        rep->setup_seconds = t_setup;
    }
    return status;
}

}  // extern "C"


// ---------------------------------------------------------------------------
// Model::Solid::Finite::NeoHookean (src/Model/Solid/Finite/NeoHookean.H:21-121):
// W(F) = mu/2 (tr(F F^T) / J^(2/3) - 3) + kappa/2 (J - 1)^2, DW, DDW (Major
// symmetry, 45 values written in the reference's loop order).
// ---------------------------------------------------------------------------
static void inv3(const double F[3][3], double* J, double Fi[3][3]) {
    const double c00 = F[1][1] * F[2][2] - F[1][2] * F[2][1];
    const double c01 = F[1][2] * F[2][0] - F[1][0] * F[2][2];
    const double c02 = F[1][0] * F[2][1] - F[1][1] * F[2][0];
    const double det = F[0][0] * c00 + F[0][1] * c01 + F[0][2] * c02;
    const double id = 1.0 / det;
    Fi[0][0] = c00 * id;
    Fi[1][0] = c01 * id;
    Fi[2][0] = c02 * id;
    Fi[0][1] = (F[0][2] * F[2][1] - F[0][1] * F[2][2]) * id;
    Fi[1][1] = (F[0][0] * F[2][2] - F[0][2] * F[2][0]) * id;
    Fi[2][1] = (F[0][1] * F[2][0] - F[0][0] * F[2][1]) * id;
    Fi[0][2] = (F[0][1] * F[1][2] - F[0][2] * F[1][1]) * id;
    Fi[1][2] = (F[0][2] * F[1][0] - F[0][0] * F[1][2]) * id;
    Fi[2][2] = (F[0][0] * F[1][1] - F[0][1] * F[1][0]) * id;
    *J = det;
}

extern "C" {

void orc_neohookean(double mu, double kappa, const double* F9, double* W, double* dw9, double* ddw45) {
    double F[3][3], Fi[3][3], J;
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) F[a][b] = F9[3 * a + b];
    inv3(F, &J, Fi);
    double FinvT[3][3];
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) FinvT[a][b] = Fi[b][a];
    double tr = 0.0;  // tr(F F^T)
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) tr += F[a][b] * F[a][b];
    const double J23 = std::pow(std::fabs(J), 2. / 3.);
    if (W) *W = 0.5 * mu * (tr / J23 - 3.) + 0.5 * kappa * (J - 1.0) * (J - 1.0);
    if (dw9)
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++)
                dw9[3 * a + b] = mu * (F[a][b] / J23 - tr * FinvT[a][b] / (3. * J23)) + kappa * (J - 1) * J * FinvT[a][b];
    if (ddw45)
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                for (int k = 0; k < 3; k++)
                    for (int l = 0; l < 3; l++) {
                        double t1 = 0.0, t2 = 0.0;
                        if (i == k && j == l) t1 += 1.0;
                        t1 -= (2. / 3.) * F[i][j] * FinvT[k][l];
                        t1 -= (2. / 3.) * FinvT[i][j] * F[k][l];
                        t1 += (2. / 9.) * tr * FinvT[i][j] * FinvT[k][l];
                        t1 += (1. / 3.) * tr * FinvT[i][l] * FinvT[k][j];
                        t2 += (2. * J - 1.) * FinvT[i][j] * FinvT[k][l];
                        t2 += (1. - J) * FinvT[i][l] * FinvT[k][j];
                        ddw45[maj_index(3 * i + j, 3 * k + l)] = (mu / J23) * t1 + kappa * J * t2;
                    }
}

// Newton::prepareForSolve for a NeoHookean medium (Newton.H:144-196): per
// node F = I + grad u (one-sided on the faces), dw = DW(F) (AoS, 9) and
// ddw = DDW(F) (AoS, 45); model = (mu, kappa) per node
void orc_neohookean_field(int nx, int ny, int nz, const double* dx, const double* model, const double* u, double* dw,
                          double* ddw) {
    Grid g = mkgrid(nx, ny, nz, dx);
    const int64_t N = g.N();
    const double* uu[3] = {u, u + N, u + 2 * N};
    for_nodes(g, [&](int i, int j, int k) {
        const int64_t id = g.id(i, j, k);
        int st[3];
        get_stencil(g, i, j, k, st);
        double F[9];
        for (int p = 0; p < 3; p++)
            for (int q = 0; q < 3; q++) F[3 * p + q] = d1(g, uu[p], i, j, k, q, st[q]) + (p == q ? 1.0 : 0.0);
        orc_neohookean(model[2 * id], model[2 * id + 1], F, nullptr, dw + 9 * id, ddw + 45 * id);
    });
}

// rhs = b - div(dw) / b - BC(u, grad u, dw) for a given stress field dw (AoS, 9)
void orc_rhs_dw(int nx, int ny, int nz, const double* dx, const double* dw, const int* bc_type, const double* u,
                const double* b, double* rhs) {
    Grid g = mkgrid(nx, ny, nz, dx);
    rhs_from_dw(g, dw, bc_type, u, b, rhs);
}

}  // extern "C"

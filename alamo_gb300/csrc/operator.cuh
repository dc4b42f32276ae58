// Per-node arithmetic of the nodal linear-elastic operator, shared by every
// kernel of the library (Fapply, damped Jacobi, residual, diagonal, bottom
// solver).  Templated on the arithmetic type T (double for the FP64 path,
// float for the FP32 inner cycle of the mixed-precision solve) and on the
// stiffness symmetry (isotropic: lambda, mu per node; major-minor: 21 values
// per node).
//
// The operator is the one of Operator::Elastic<SYM>::Fapply
// (src/Operator/Elastic.cpp:165-290 of the reference):
//   interior node : f = C : grad grad u + sum_q (d_q C : grad u)_{:,q}
//                   (central differences; C differentiated over the 6 face
//                   neighbours), psi terms absent;
//   boundary node : f = BC row of the node's region (displacement u_i,
//                   traction (sigma n)_i or neumann (grad u n)_i) with
//                   first-order one-sided gradients at the domain faces
//                   (src/BC/Operator/Elastic/Constant.H:344-425).
// The contraction order differs from the reference's Eigen code; the results
// agree to rounding (the parity tests hold them to 1e-12 relative in FP64).
#pragma once
#include <cstdint>
#include "agb_types.h"

namespace agb {

// Truncated unit normals of the reference (Elastic.H:79-80)
#define AGB_S3 0.57735026919
#define AGB_S2 0.70710678118

// Region of a boundary node and its outward normal, with the reference's
// precedence: corners, then edges (yz, zx, xy), then faces
// (src/BC/Operator/Elastic/Constant.H:373-400).
template <typename T>
__device__ __forceinline__ int boundary_region(int cx, int cy, int cz, T n[3]) {
    const int cnt = (cx != 0) + (cy != 0) + (cz != 0);
    if (cnt == 3) {
        n[0] = T(cx * AGB_S3); n[1] = T(cy * AGB_S3); n[2] = T(cz * AGB_S3);
        return 18 + (cx > 0) * 4 + (cy > 0) * 2 + (cz > 0);
    }
    if (cnt == 2) {
        n[0] = T(cx * AGB_S2); n[1] = T(cy * AGB_S2); n[2] = T(cz * AGB_S2);
        if (cy && cz) return 6 + (cy > 0) * 2 + (cz > 0);
        if (cz && cx) return 10 + (cz > 0) * 2 + (cx > 0);
        return 14 + (cx > 0) * 2 + (cy > 0);
    }
    n[0] = T(cx); n[1] = T(cy); n[2] = T(cz);
    if (cx) return cx < 0 ? 0 : 3;
    if (cy) return cy < 0 ? 1 : 4;
    return cz < 0 ? 2 : 5;
}

// sigma = C : g for a per-node stiffness read through `c(k)` (k = 0..nc-1)
template <typename T, int SYM, typename CF>
__device__ __forceinline__ void stress_of(CF c, const T g[3][3], T s[3][3]) {
    if (SYM == SYM_ISO) {
        const T l = c(0), m = c(1);
        const T tr = g[0][0] + g[1][1] + g[2][2];
        const T m2 = m + m;
        s[0][0] = l * tr + m2 * g[0][0];
        s[1][1] = l * tr + m2 * g[1][1];
        s[2][2] = l * tr + m2 * g[2][2];
        s[0][1] = s[1][0] = m * (g[0][1] + g[1][0]);
        s[0][2] = s[2][0] = m * (g[0][2] + g[2][0]);
        s[1][2] = s[2][1] = m * (g[1][2] + g[2][1]);
    } else if (SYM == SYM_MAJ) {
        // sigma_ij = sum_kl C_ijkl g_kl (src/Set/Matrix4_Major.H:510-523)
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                T acc = T(0);
#pragma unroll
                for (int k = 0; k < 3; k++)
#pragma unroll
                    for (int l = 0; l < 3; l++) acc += c(maj_of(i, j, k, l)) * g[k][l];
                s[i][j] = acc;
            }
    } else {
        const T v[6] = {g[0][0], g[0][1] + g[1][0], g[0][2] + g[2][0], g[1][1], g[1][2] + g[2][1], g[2][2]};
        T w[6];
#pragma unroll
        for (int a = 0; a < 6; a++) {
            T acc = c(mm_ut(a, 0)) * v[0];
#pragma unroll
            for (int b = 1; b < 6; b++) acc += c(mm_ut(a, b)) * v[b];
            w[a] = acc;
        }
        s[0][0] = w[0]; s[1][1] = w[3]; s[2][2] = w[5];
        s[0][1] = s[1][0] = w[1];
        s[0][2] = s[2][0] = w[2];
        s[1][2] = s[2][1] = w[4];
    }
}

// Row r of the boundary condition for region `reg`; bt: the 78-entry type
// table (region * 3 + component)
template <typename T>
__device__ __forceinline__ T bc_component(const unsigned char* bt, int reg, int r, T ur, const T g[3][3],
                                          const T s[3][3], const T n[3]) {
    const int t = bt[reg * 3 + r];
    if (t == BC_DISP) return ur;
    if (t == BC_TRAC) return s[r][0] * n[0] + s[r][1] * n[1] + s[r][2] * n[2];
    if (t == BC_NEUMANN) return g[r][0] * n[0] + g[r][1] * n[1] + g[r][2] * n[2];
    return T(0);
}

// One-sided (first-order) or central first derivative at a node along one
// axis (src/Numeric/Stencil.H:41-60, :70-191): forward at the low face,
// backward at the high face.  fp, f0, fm: the values at +1, 0, -1.
template <typename T>
__device__ __forceinline__ T d1_of(T fp, T f0, T fm, int pos, int n, T h, T inv) {
    if (pos == 0) return (fp - f0) * inv;
    if (pos == n - 1) return (f0 - fm) * inv;
    return (fp - fm) * h;
}

// Gradient g[p][q] = du_p/dx_q with the boundary-aware stencil, from global
// memory
template <typename T>
__device__ __forceinline__ void grad_at(const T* __restrict__ u, const LevelGeom<T>& G, int i, int j, int k, int64_t id,
                                        T g[3][3]) {
    const int64_t sy = G.sy, sz = G.sz;
#pragma unroll
    for (int p = 0; p < 3; p++) {
        const T* f = u + p * G.N + id;
        const T f0 = f[0];
        g[p][0] = d1_of(i < G.nx - 1 ? f[1] : f0, f0, i > 0 ? f[-1] : f0, i, G.nx, G.h[0], G.inv[0]);
        g[p][1] = d1_of(j < G.ny - 1 ? f[sy] : f0, f0, j > 0 ? f[-sy] : f0, j, G.ny, G.h[1], G.inv[1]);
        g[p][2] = d1_of(k < G.nz - 1 ? f[sz] : f0, f0, k > 0 ? f[-sz] : f0, k, G.nz, G.h[2], G.inv[2]);
    }
}

// BC rows of a boundary node (i, j, k).  U(p, a, b, c): component p of the
// displacement at offset (a, b, c) from the node; c(e): stiffness entry e of
// the node.  Offsets that leave the grid are never requested.
template <typename T, int SYM, typename UA, typename CF>
__device__ __forceinline__ void boundary_rows(UA U, CF c, const LevelGeom<T>& G, const unsigned char* bt, int i,
                                              int j, int k, T f[3], T pa = T(1)) {
    T g[3][3], s[3][3], n[3];
    const int cx = (i == 0) ? -1 : (i == G.nx - 1) ? 1 : 0;
    const int cy = (j == 0) ? -1 : (j == G.ny - 1) ? 1 : 0;
    const int cz = (k == 0) ? -1 : (k == G.nz - 1) ? 1 : 0;
    const int reg = boundary_region<T>(cx, cy, cz, n);
    const int t0 = bt[reg * 3], t1 = bt[reg * 3 + 1], t2 = bt[reg * 3 + 2];
    // displacement (and periodic / none) rows read neither the gradient nor
    // the stiffness: a region without traction or Neumann rows skips both
    if (!(t0 == BC_TRAC || t0 == BC_NEUMANN || t1 == BC_TRAC || t1 == BC_NEUMANN || t2 == BC_TRAC ||
          t2 == BC_NEUMANN)) {
#pragma unroll
        for (int r = 0; r < 3; r++) f[r] = bt[reg * 3 + r] == BC_DISP ? U(r, 0, 0, 0) : T(0);
        return;
    }
#pragma unroll
    for (int p = 0; p < 3; p++) {
        const T u0 = U(p, 0, 0, 0);
        g[p][0] = d1_of(i < G.nx - 1 ? U(p, 1, 0, 0) : u0, u0, i > 0 ? U(p, -1, 0, 0) : u0, i, G.nx, G.h[0], G.inv[0]);
        g[p][1] = d1_of(j < G.ny - 1 ? U(p, 0, 1, 0) : u0, u0, j > 0 ? U(p, 0, -1, 0) : u0, j, G.ny, G.h[1], G.inv[1]);
        g[p][2] = d1_of(k < G.nz - 1 ? U(p, 0, 0, 1) : u0, u0, k > 0 ? U(p, 0, 0, -1) : u0, k, G.nz, G.h[2], G.inv[2]);
    }
    if (t0 == BC_TRAC || t1 == BC_TRAC || t2 == BC_TRAC) {
        stress_of<T, SYM>(c, g, s);
        // sigma psi_avg (Elastic.cpp:195); pa = 1 without psi leaves s unchanged
#pragma unroll
        for (int p = 0; p < 3; p++)
#pragma unroll
            for (int q = 0; q < 3; q++) s[p][q] *= pa;
    } else {
#pragma unroll
        for (int p = 0; p < 3; p++)
#pragma unroll
            for (int q = 0; q < 3; q++) s[p][q] = T(0);
    }
#pragma unroll
    for (int r = 0; r < 3; r++) f[r] = bc_component<T>(bt, reg, r, U(r, 0, 0, 0), g, s, n);
}

// Apply the operator at a boundary node (i, j, k) reading global memory
template <typename T, int SYM, typename CF>
__device__ __forceinline__ void apply_boundary(const T* __restrict__ u, const LevelGeom<T>& G, const BcTable& bc, CF c,
                                               int i, int j, int k, int64_t id, T f[3], T pa = T(1)) {
    const int64_t N = G.N, sy = G.sy, sz = G.sz;
    auto U = [&](int p, int a, int b, int cc) { return u[p * N + id + a + sy * b + sz * cc]; };
    boundary_rows<T, SYM>(U, c, G, bc.t, i, j, k, f, pa);
}

// psi at node (i, j, k): the mean of its 8 cells in the order of
// Numeric::Interpolate::CellToNodeAverage (src/Numeric/Stencil.H:1390-1405)
// and, when gp is given, Numeric::CellGradientOnNode (src/Numeric/
// Stencil.H:699-715).  Entry (i, j, k) of the ghosted field is cell
// (i-1, j-1, k-1), so P(a, b, c) below is cell (i+a, j+b, k+c).
template <typename T>
__device__ __forceinline__ T psi_node(const LevelGeom<T>& G, int i, int j, int k, T* gp) {
    const T* base = G.psi + (i + 1) + G.psy * (j + 1) + G.psz * (k + 1);
    const int64_t py = G.psy, pz = G.psz;
    auto P = [&](int a, int b, int c) { return base[a + py * b + pz * c]; };
    const T p000 = P(0, 0, 0), p100 = P(-1, 0, 0), p010 = P(0, -1, 0), p110 = P(-1, -1, 0);
    const T p001 = P(0, 0, -1), p101 = P(-1, 0, -1), p011 = P(0, -1, -1), p111 = P(-1, -1, -1);
    if (gp) {
        gp[0] = T(0.25) * (p000 - p100 + p010 - p110 + p001 - p101 + p011 - p111) * G.inv[0];
        gp[1] = T(0.25) * (p000 - p010 + p100 - p110 + p001 - p011 + p101 - p111) * G.inv[1];
        gp[2] = T(0.25) * (p000 - p001 + p100 - p101 + p010 - p011 + p110 - p111) * G.inv[2];
    }
    return (p000 + p100 + p010 + p110 + p001 + p101 + p011 + p111) * T(0.125);
}

// psi_avg = (1 - small) avg8(psi) + small (Elastic.cpp:191-192)
template <typename T>
__device__ __forceinline__ T psi_avg_of(const LevelGeom<T>& G, T avg) {
    return (T(1) - G.psi_small) * avg + G.psi_small;
}

// Interior rows with psi (Elastic.cpp:243-260): f (the rows without psi)
// becomes f psi_avg + (C grad u) grad psi (1 - small).
template <typename T, int SYM>
__device__ __forceinline__ void psi_interior(const T* __restrict__ u, const T* __restrict__ C,
                                             const LevelGeom<T>& G, int i, int j, int k, int64_t id, T f[3]) {
    T gp[3];
    const T pa = psi_avg_of(G, psi_node(G, i, j, k, gp));
    const T w = T(1) - G.psi_small;
#pragma unroll
    for (int q = 0; q < 3; q++) gp[q] *= w;
    const int64_t N = G.N;
    const int64_t off[3] = {1, G.sy, G.sz};
    T g[3][3], s[3][3];
#pragma unroll
    for (int p = 0; p < 3; p++)
#pragma unroll
        for (int q = 0; q < 3; q++) g[p][q] = (u[p * N + id + off[q]] - u[p * N + id - off[q]]) * G.h[q];
    auto cf = [&](int a) { return C[a * N + id]; };
    stress_of<T, SYM>(cf, g, s);
#pragma unroll
    for (int r = 0; r < 3; r++) f[r] = f[r] * pa + (s[r][0] * gp[0] + s[r][1] * gp[1] + s[r][2] * gp[2]);
}

// Interior-node arithmetic with the displacement and the stiffness read
// through accessors: U(p, a, b, c) is component p of u at node offset
// (a, b, c) in {-1, 0, 1}^3 and Cf(e, a, b, c) is stiffness entry e at an
// offset with at most one non-zero axis.  Offsets and entries are
// compile-time constants once the loops unroll, so the accessors cost nothing
// beyond their loads.
template <typename T, int SYM, typename UA, typename CA>
__device__ __forceinline__ void interior_rows(UA U, CA Cf, const LevelGeom<T>& G, T f[3]) {
    T g[3][3];
    // Hessian of each component: xx, yy, zz, xy, xz, yz
    T H[3][6];
#pragma unroll
    for (int p = 0; p < 3; p++) {
        const T c0 = U(p, 0, 0, 0);
        const T xp = U(p, 1, 0, 0), xm = U(p, -1, 0, 0), yp = U(p, 0, 1, 0), ym = U(p, 0, -1, 0);
        const T zp = U(p, 0, 0, 1), zm = U(p, 0, 0, -1);
        g[p][0] = (xp - xm) * G.h[0];
        g[p][1] = (yp - ym) * G.h[1];
        g[p][2] = (zp - zm) * G.h[2];
        const T c2 = c0 + c0;
        H[p][0] = ((xp + xm) - c2) * G.i2[0];
        H[p][1] = ((yp + ym) - c2) * G.i2[1];
        H[p][2] = ((zp + zm) - c2) * G.i2[2];
        H[p][3] = ((U(p, 1, 1, 0) + U(p, -1, -1, 0)) - (U(p, 1, -1, 0) + U(p, -1, 1, 0))) * G.q[0];
        H[p][4] = ((U(p, 1, 0, 1) + U(p, -1, 0, -1)) - (U(p, 1, 0, -1) + U(p, -1, 0, 1))) * G.q[1];
        H[p][5] = ((U(p, 0, 1, 1) + U(p, 0, -1, -1)) - (U(p, 0, 1, -1) + U(p, 0, -1, 1))) * G.q[2];
    }
    enum { XX = 0, YY = 1, ZZ = 2, XY = 3, XZ = 4, YZ = 5 };
    if (SYM == SYM_ISO) {
        const T l = Cf(0, 0, 0, 0), m = Cf(1, 0, 0, 0);
        const T lm = l + m;
        f[0] = m * (H[0][XX] + H[0][YY] + H[0][ZZ]) + lm * (H[0][XX] + H[1][XY] + H[2][XZ]);
        f[1] = m * (H[1][XX] + H[1][YY] + H[1][ZZ]) + lm * (H[0][XY] + H[1][YY] + H[2][YZ]);
        f[2] = m * (H[2][XX] + H[2][YY] + H[2][ZZ]) + lm * (H[0][XZ] + H[1][YZ] + H[2][ZZ]);
        // grad C term: f_i += dl_i tr(g) + sum_q dm_q (g_iq + g_qi)
        const T tr = g[0][0] + g[1][1] + g[2][2];
        const T dl[3] = {(Cf(0, 1, 0, 0) - Cf(0, -1, 0, 0)) * G.h[0], (Cf(0, 0, 1, 0) - Cf(0, 0, -1, 0)) * G.h[1],
                         (Cf(0, 0, 0, 1) - Cf(0, 0, 0, -1)) * G.h[2]};
        const T dm[3] = {(Cf(1, 1, 0, 0) - Cf(1, -1, 0, 0)) * G.h[0], (Cf(1, 0, 1, 0) - Cf(1, 0, -1, 0)) * G.h[1],
                         (Cf(1, 0, 0, 1) - Cf(1, 0, 0, -1)) * G.h[2]};
#pragma unroll
        for (int i = 0; i < 3; i++) {
            T t = dl[i] * tr;
#pragma unroll
            for (int q = 0; q < 3; q++) t += dm[q] * (g[i][q] + g[q][i]);
            f[i] += t;
        }
    } else if (SYM == SYM_MAJ) {
        // f_i = sum_{jkl} C_ijkl u_{k,lj} (src/Set/Matrix4_Major.H:527-541)
        // with the Hessian pairs (l, j) of component k
        auto hs = [&](int k, int l, int j) -> T {
            if (l == j) return H[k][l];
            const int a = l < j ? l : j, b = l < j ? j : l;
            return H[k][a == 0 ? (b == 1 ? XY : XZ) : YZ];
        };
#pragma unroll
        for (int i = 0; i < 3; i++) {
            T acc = T(0);
#pragma unroll
            for (int j = 0; j < 3; j++)
#pragma unroll
                for (int k = 0; k < 3; k++)
#pragma unroll
                    for (int l = 0; l < 3; l++) acc += Cf(maj_of(i, j, k, l), 0, 0, 0) * hs(k, l, j);
            f[i] = acc;
        }
        // grad C term: f_i += sum_q ((d_q C) grad u)_{iq}, d_q C central
        T col[3][3];
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const int ox = q == 0, oy = q == 1, oz = q == 2;
#pragma unroll
            for (int i = 0; i < 3; i++) {
                T acc = T(0);
#pragma unroll
                for (int k = 0; k < 3; k++)
#pragma unroll
                    for (int l = 0; l < 3; l++) {
                        const int e = maj_of(i, q, k, l);
                        acc += (Cf(e, ox, oy, oz) - Cf(e, -ox, -oy, -oz)) * g[k][l];
                    }
                col[q][i] = acc * G.h[q];
            }
        }
#pragma unroll
        for (int i = 0; i < 3; i++) f[i] += (col[0][i] + col[1][i]) + col[2][i];
    } else {
        T d[21];
#pragma unroll
        for (int a = 0; a < 21; a++) d[a] = Cf(a, 0, 0, 0);
        // C : grad grad u (the grouping of src/Set/Matrix4_MajorMinor.H:709-767)
        f[0] = d[0] * H[0][XX] + d[1] * (H[0][XY] + H[0][XY] + H[1][XX]) + d[2] * (H[0][XZ] + H[0][XZ] + H[2][XX]) +
               d[3] * H[1][XY] + d[4] * (H[1][XZ] + H[2][XY]) + d[5] * H[2][XZ] + d[6] * (H[0][YY] + H[1][XY]) +
               d[7] * (H[0][YZ] + H[0][YZ] + H[2][XY] + H[1][XZ]) + d[8] * H[1][YY] + d[9] * (H[1][YZ] + H[2][YY]) +
               d[10] * H[2][YZ] + d[11] * (H[0][ZZ] + H[2][XZ]) + d[12] * H[1][YZ] + d[13] * (H[1][ZZ] + H[2][YZ]) +
               d[14] * H[2][ZZ];
        f[1] = d[1] * H[0][XX] + d[4] * H[0][XZ] + d[3] * H[0][XY] + d[6] * (H[0][XY] + H[1][XX]) +
               d[7] * (H[0][XZ] + H[2][XX]) + d[8] * (H[1][XY] + H[1][XY] + H[0][YY]) +
               d[9] * (H[1][XZ] + H[1][XZ] + H[2][XY] + H[0][YZ]) + d[10] * H[2][XZ] + d[12] * (H[0][YZ] + H[2][XY]) +
               d[13] * (H[0][ZZ] + H[2][XZ]) + d[15] * H[1][YY] + d[16] * (H[1][YZ] + H[1][YZ] + H[2][YY]) +
               d[17] * H[2][YZ] + d[18] * (H[1][ZZ] + H[2][YZ]) + d[19] * H[2][ZZ];
        f[2] = d[2] * H[0][XX] + d[4] * H[0][XY] + d[5] * H[0][XZ] + d[7] * (H[0][XY] + H[1][XX]) +
               d[9] * (H[0][YY] + H[1][XY]) + d[10] * (H[0][YZ] + H[1][XZ]) + d[11] * (H[0][XZ] + H[2][XX]) +
               d[12] * H[1][XY] + d[13] * (H[1][XZ] + H[2][XY] + H[2][XY] + H[0][YZ]) +
               d[14] * (H[2][XZ] + H[2][XZ] + H[0][ZZ]) + d[16] * H[1][YY] + d[17] * H[1][YZ] +
               d[18] * (H[1][YZ] + H[2][YY]) + d[19] * (H[2][YZ] + H[2][YZ] + H[1][ZZ]) + d[20] * H[2][ZZ];
        // grad C term: f_i += sum_q sum_b dC_q[pair(i,q)][b] v_b, dC_q central
        const T v[6] = {g[0][0], g[0][1] + g[1][0], g[0][2] + g[2][0], g[1][1], g[1][2] + g[2][1], g[2][2]};
        T col[3][3];
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const int ox = q == 0, oy = q == 1, oz = q == 2;
#pragma unroll
            for (int i = 0; i < 3; i++) {
                const int a = pair_of(i, q);
                T acc = T(0);
#pragma unroll
                for (int bb = 0; bb < 6; bb++) {
                    const int e = mm_ut(a, bb);
                    acc += (Cf(e, ox, oy, oz) - Cf(e, -ox, -oy, -oz)) * v[bb];
                }
                col[q][i] = acc * G.h[q];
            }
        }
#pragma unroll
        for (int i = 0; i < 3; i++) f[i] += (col[0][i] + col[1][i]) + col[2][i];
    }
}

// Apply the operator at an interior node, everything read from global
// memory.  C is SoA: C[k * N + node].
template <typename T, int SYM>
__device__ __forceinline__ void apply_interior(const T* __restrict__ u, const T* __restrict__ C, const LevelGeom<T>& G,
                                               int64_t id, T f[3]) {
    const int64_t N = G.N, sy = G.sy, sz = G.sz;
    auto U = [&](int p, int a, int b, int c) { return u[p * N + id + a + sy * b + sz * c]; };
    auto Cf = [&](int e, int a, int b, int c) { return C[e * N + id + a + sy * b + sz * c]; };
    interior_rows<T, SYM>(U, Cf, G, f);
}

// Apply the operator at any node.  PSI = false compiles the psi terms out
// (the kernels instantiate both and pick by G.psi, so the common case keeps
// its register budget).
template <typename T, int SYM, bool PSI = true>
__device__ __forceinline__ void apply_node(const T* __restrict__ u, const T* __restrict__ C, const LevelGeom<T>& G,
                                           const BcTable& bc, int i, int j, int k, int64_t id, T f[3]) {
    const bool bnd = (i == 0) | (j == 0) | (k == 0) | (i == G.nx - 1) | (j == G.ny - 1) | (k == G.nz - 1);
    if (bnd) {
        const int64_t N = G.N;
        auto cf = [&](int a) { return C[a * N + id]; };
        const T pa = (PSI && G.psi) ? psi_avg_of(G, psi_node<T>(G, i, j, k, nullptr)) : T(1);
        apply_boundary<T, SYM>(u, G, bc, cf, i, j, k, id, f, pa);
    } else {
        apply_interior<T, SYM>(u, C, G, id, f);
        if (PSI && G.psi) psi_interior<T, SYM>(u, C, G, i, j, k, id, f);
    }
}

// Diagonal of the operator at a node (src/Operator/Elastic.cpp:321-373 with
// Gradient_Diagonal, src/Numeric/Stencil.H:900-963)
template <typename T, int SYM>
__device__ __forceinline__ void diag_node(const T* __restrict__ C, const LevelGeom<T>& G, const BcTable& bc, int i,
                                          int j, int k, int64_t id, T dg[3]) {
    const int64_t N = G.N;
    auto cf = [&](int a) { return C[a * N + id]; };
    const bool bnd = (i == 0) | (j == 0) | (k == 0) | (i == G.nx - 1) | (j == G.ny - 1) | (k == G.nz - 1);
    if (bnd) {
        const int pos[3] = {i, j, k};
        const int nn[3] = {G.nx, G.ny, G.nz};
        const int cx = (i == 0) ? -1 : (i == G.nx - 1) ? 1 : 0;
        const int cy = (j == 0) ? -1 : (j == G.ny - 1) ? 1 : 0;
        const int cz = (k == 0) ? -1 : (k == G.nz - 1) ? 1 : 0;
        T n[3];
        const int reg = boundary_region<T>(cx, cy, cz, n);
        const T pa = G.psi ? psi_avg_of(G, psi_node<T>(G, i, j, k, nullptr)) : T(1);
#pragma unroll
        for (int p = 0; p < 3; p++) {
            T g[3][3], s[3][3];
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    T v = T(0);
                    if (a == p) {
                        if (pos[d] == 0) v = -G.inv[d];
                        else if (pos[d] == nn[d] - 1) v = G.inv[d];
                    }
                    g[a][d] = v;
                }
            stress_of<T, SYM>(cf, g, s);
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int d = 0; d < 3; d++) s[a][d] *= pa;
            dg[p] = bc_component<T>(bc.t, reg, p, T(1), g, s, n);
        }
    } else {
        // (C : dgradgradu/du_p)_p with d2/dx_l^2 -> -2/dx_l^2 for component p
        if (SYM == SYM_ISO) {
            const T l = cf(0), m = cf(1);
            const T s2 = -(G.i2[0] + G.i2[1] + G.i2[2]) * T(2);
#pragma unroll
            for (int p = 0; p < 3; p++) dg[p] = m * s2 + (l + m) * (T(-2) * G.i2[p]);
        } else if (SYM == SYM_MAJ) {
#pragma unroll
            for (int p = 0; p < 3; p++) {
                T acc = T(0);
#pragma unroll
                for (int l = 0; l < 3; l++) acc += cf(maj_of(p, l, p, l)) * (T(-2) * G.i2[l]);
                dg[p] = acc;
            }
        } else {
#pragma unroll
            for (int p = 0; p < 3; p++) {
                T acc = T(0);
#pragma unroll
                for (int l = 0; l < 3; l++) acc += cf(mm_ut(pair_of(p, l), pair_of(p, l))) * (T(-2) * G.i2[l]);
                dg[p] = acc;
            }
        }
        // Elastic.cpp:363: the interior diagonal times psi_avg
        if (G.psi) {
            const T pa = psi_avg_of(G, psi_node<T>(G, i, j, k, nullptr));
#pragma unroll
            for (int p = 0; p < 3; p++) dg[p] *= pa;
        }
    }
}

}  // namespace agb

// Plain data types shared by the host driver (compiled by g++) and the CUDA
// kernels (compiled by nvcc).
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define AGB_HD __host__ __device__
#else
#define AGB_HD
#endif

namespace agb {

enum { SYM_ISO = 0, SYM_MM = 1, SYM_MAJ = 2 };
enum { BC_DISP = 0, BC_TRAC = 1, BC_PERIODIC = 2, BC_NEUMANN = 3, BC_NONE = 4 };

// Boundary-condition types: region * 3 + component, region order of the
// reference's Face enum (src/BC/Operator/Elastic/Elastic.H:35-43).
struct BcTable {
    unsigned char t[78];
};

// One multigrid level's geometry and the scaling constants derived from dx.
template <typename T>
struct LevelGeom {
    int nx, ny, nz;
    int64_t N;       // nodes
    int64_t sy, sz;  // strides of j and k
    T h[3];          // 0.5 / dx  (central first derivative)
    T inv[3];        // 1 / dx    (one-sided first derivative)
    T i2[3];         // 1 / dx^2  (second derivative)
    T q[3];          // 0.25 / (dx_a dx_b) for the pairs xy, xz, yz
    // psi of Operator::Elastic (void indicator, Elastic.cpp:191-192): cell
    // field with one ghost layer, (nx+1)(ny+1)(nz+1) values, entry (a,b,c) =
    // cell (a-1,b-1,c-1), strides psy = nx+1 and psz = (nx+1)(ny+1).
    // nullptr when no psi is set.
    const T* psi;
    T psi_small;
    int64_t psy, psz;
};

// index of the 21 major-minor entries by Voigt-pair (00,01,02,11,12,22) rows
// and columns: upper triangle of the symmetric 6x6 matrix, row-major
// (src/Set/Matrix4_MajorMinor.H:327-375)
AGB_HD constexpr int mm_ut(int a, int b) {
    return a <= b ? (a * 11 - a * a) / 2 + b : (b * 11 - b * b) / 2 + a;
}
// index of the 45 Major-symmetry entries: upper triangle, row-major, of the
// symmetric 9 x 9 matrix over the pairs P = 3 i + j (src/Set/Matrix4_Major.H:
// 274-320)
AGB_HD constexpr int maj_ut(int P, int Q) {
    return P <= Q ? P * 9 - P * (P - 1) / 2 + (Q - P) : Q * 9 - Q * (Q - 1) / 2 + (P - Q);
}
AGB_HD constexpr int maj_of(int i, int j, int k, int l) { return maj_ut(3 * i + j, 3 * k + l); }
AGB_HD constexpr int pair_of(int i, int j) {
    return (i == j) ? (i == 0 ? 0 : i == 1 ? 3 : 5) : ((i + j) == 1 ? 1 : (i + j) == 2 ? 2 : 4);
}

}  // namespace agb

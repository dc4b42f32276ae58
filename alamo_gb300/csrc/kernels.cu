// Field kernels of the nodal elastic multigrid path, sm_103a.
//
// All node fields are SoA per component with x fastest and no ghost nodes;
// boundary nodes of the domain carry the boundary-condition rows, so every
// stencil stays inside the grid.  One thread owns one node; blocks are
// 32 x 4 x 2 nodes so a warp reads 32 consecutive x-nodes (coalesced
// 256-byte rows in FP64) and the y/z neighbours of a block hit L1/L2.
#include <cuda_runtime.h>
#include <cmath>
#include "agb_launch.h"
#include "operator.cuh"

namespace agb {

static constexpr int BX = 32, BY = 4, BZ = 2;

static inline dim3 grid3(int nx, int ny, int nz) { return dim3((nx + BX - 1) / BX, (ny + BY - 1) / BY, (nz + BZ - 1) / BZ); }

template <typename T>
LevelGeom<T> make_geom(int nx, int ny, int nz, const double dx[3]) {
    LevelGeom<T> G;
    G.nx = nx; G.ny = ny; G.nz = nz;
    G.sy = nx;
    G.sz = (int64_t)nx * ny;
    G.N = G.sz * nz;
    for (int d = 0; d < 3; d++) {
        G.h[d] = T(0.5 / dx[d]);
        G.inv[d] = T(1.0 / dx[d]);
        G.i2[d] = T(1.0 / (dx[d] * dx[d]));
    }
    G.q[0] = T(0.25 / (dx[0] * dx[1]));
    G.q[1] = T(0.25 / (dx[0] * dx[2]));
    G.q[2] = T(0.25 / (dx[1] * dx[2]));
    G.psi = nullptr;
    G.psi_small = T(0);
    G.psy = nx + 1;
    G.psz = (int64_t)(nx + 1) * (ny + 1);
    return G;
}
template LevelGeom<double> make_geom<double>(int, int, int, const double*);
template LevelGeom<float> make_geom<float>(int, int, int, const double*);

#define AGB_NODE_INDEX                                    \
    const int i = blockIdx.x * BX + threadIdx.x;          \
    const int j = blockIdx.y * BY + threadIdx.y;          \
    const int k = blockIdx.z * BZ + threadIdx.z;          \
    const bool live = (i < G.nx) & (j < G.ny) & (k < G.nz); \
    const int64_t id = i + G.sy * j + G.sz * k;

// ---------------------------------------------------------------- Fapply
template <typename T, int SYM, bool PSI>
__global__ void __launch_bounds__(256) k_fapply(const T* __restrict__ u, const T* __restrict__ C, LevelGeom<T> G,
                                                BcTable bc, T* __restrict__ f) {
    AGB_NODE_INDEX
    if (!live) return;
    T r[3];
    apply_node<T, SYM, PSI>(u, C, G, bc, i, j, k, id, r);
    f[id] = r[0];
    f[G.N + id] = r[1];
    f[2 * G.N + id] = r[2];
}

template <typename T>
cudaError_t launch_fapply(int sym, const T* u, const T* C, const LevelGeom<T>& G, const BcTable& bc, T* f,
                          cudaStream_t s) {
    dim3 blk(BX, BY, BZ), grd = grid3(G.nx, G.ny, G.nz);
    if (G.psi) {
        if (sym == SYM_ISO) k_fapply<T, SYM_ISO, true><<<grd, blk, 0, s>>>(u, C, G, bc, f);
        else if (sym == SYM_MAJ) k_fapply<T, SYM_MAJ, true><<<grd, blk, 0, s>>>(u, C, G, bc, f);
        else k_fapply<T, SYM_MM, true><<<grd, blk, 0, s>>>(u, C, G, bc, f);
    } else {
        if (sym == SYM_ISO) k_fapply<T, SYM_ISO, false><<<grd, blk, 0, s>>>(u, C, G, bc, f);
        else if (sym == SYM_MAJ) k_fapply<T, SYM_MAJ, false><<<grd, blk, 0, s>>>(u, C, G, bc, f);
        else k_fapply<T, SYM_MM, false><<<grd, blk, 0, s>>>(u, C, G, bc, f);
    }
    return cudaGetLastError();
}
template cudaError_t launch_fapply<double>(int, const double*, const double*, const LevelGeom<double>&, const BcTable&,
                                           double*, cudaStream_t);
template cudaError_t launch_fapply<float>(int, const float*, const float*, const LevelGeom<float>&, const BcTable&,
                                          float*, cudaStream_t);

// ---------------------------------------------------------------- Diagonal
template <typename T, int SYM>
__global__ void __launch_bounds__(256) k_diag(const T* __restrict__ C, LevelGeom<T> G, BcTable bc, T* __restrict__ dg) {
    AGB_NODE_INDEX
    if (!live) return;
    T r[3];
    diag_node<T, SYM>(C, G, bc, i, j, k, id, r);
    dg[id] = r[0];
    dg[G.N + id] = r[1];
    dg[2 * G.N + id] = r[2];
}

template <typename T>
cudaError_t launch_diagonal(int sym, const T* C, const LevelGeom<T>& G, const BcTable& bc, T* diag, cudaStream_t s) {
    dim3 blk(BX, BY, BZ), grd = grid3(G.nx, G.ny, G.nz);
    if (sym == SYM_ISO) k_diag<T, SYM_ISO><<<grd, blk, 0, s>>>(C, G, bc, diag);
    else if (sym == SYM_MAJ) k_diag<T, SYM_MAJ><<<grd, blk, 0, s>>>(C, G, bc, diag);
    else k_diag<T, SYM_MM><<<grd, blk, 0, s>>>(C, G, bc, diag);
    return cudaGetLastError();
}
template cudaError_t launch_diagonal<double>(int, const double*, const LevelGeom<double>&, const BcTable&, double*,
                                             cudaStream_t);
template cudaError_t launch_diagonal<float>(int, const float*, const LevelGeom<float>&, const BcTable&, float*,
                                            cudaStream_t);

// ---------------------------------------------------------------- Jacobi
// One damped-Jacobi sweep of Operator<Grid::Node>::Fsmooth
// (src/Operator/Operator.cpp:109-146) fused with the operator application:
// Ax is never written to memory.
template <typename T, int SYM, bool PSI>
__global__ void __launch_bounds__(256) k_jacobi(const T* __restrict__ x, const T* __restrict__ b,
                                                const T* __restrict__ dg, const T* __restrict__ C, LevelGeom<T> G,
                                                BcTable bc, T omega, T* __restrict__ xo) {
    AGB_NODE_INDEX
    if (!live) return;
    T ax[3];
    apply_node<T, SYM, PSI>(x, C, G, bc, i, j, k, id, ax);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const int64_t q = c * G.N + id;
        const T xv = x[q], d = dg[q];
        const T rx = ax[c] - xv * d;
        xo[q] = (T(1) - omega) * xv + omega * (b[q] - rx) / d;
    }
}

// first sweep from a zero guess: A 0 = 0, so x = w b / diag
template <typename T>
__global__ void k_jacobi_zero(const T* __restrict__ b, const T* __restrict__ dg, T omega, T* __restrict__ xo,
                              int64_t n) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        xo[q] = omega * (b[q] - T(0)) / dg[q];
}

static inline int flat_blocks(int64_t n) {
    int64_t b = (n + 255) / 256;
    return (int)(b < 152 * 16 ? (b < 1 ? 1 : b) : 152 * 16);
}

template <typename T>
cudaError_t launch_jacobi(int sym, const T* x, const T* b, const T* diag, const T* C, const LevelGeom<T>& G,
                          const BcTable& bc, T omega, T* xout, cudaStream_t s) {
    if (x == nullptr) {
        const int64_t n = 3 * G.N;
        k_jacobi_zero<T><<<flat_blocks(n), 256, 0, s>>>(b, diag, omega, xout, n);
        return cudaGetLastError();
    }
    dim3 blk(BX, BY, BZ), grd = grid3(G.nx, G.ny, G.nz);
    if (G.psi) {
        if (sym == SYM_ISO) k_jacobi<T, SYM_ISO, true><<<grd, blk, 0, s>>>(x, b, diag, C, G, bc, omega, xout);
        else if (sym == SYM_MAJ) k_jacobi<T, SYM_MAJ, true><<<grd, blk, 0, s>>>(x, b, diag, C, G, bc, omega, xout);
        else k_jacobi<T, SYM_MM, true><<<grd, blk, 0, s>>>(x, b, diag, C, G, bc, omega, xout);
    } else {
        if (sym == SYM_ISO) k_jacobi<T, SYM_ISO, false><<<grd, blk, 0, s>>>(x, b, diag, C, G, bc, omega, xout);
        else if (sym == SYM_MAJ) k_jacobi<T, SYM_MAJ, false><<<grd, blk, 0, s>>>(x, b, diag, C, G, bc, omega, xout);
        else k_jacobi<T, SYM_MM, false><<<grd, blk, 0, s>>>(x, b, diag, C, G, bc, omega, xout);
    }
    return cudaGetLastError();
}
template cudaError_t launch_jacobi<double>(int, const double*, const double*, const double*, const double*,
                                           const LevelGeom<double>&, const BcTable&, double, double*, cudaStream_t);
template cudaError_t launch_jacobi<float>(int, const float*, const float*, const float*, const float*,
                                          const LevelGeom<float>&, const BcTable&, float, float*, cudaStream_t);

// ---------------------------------------------------------------- Gauss-Seidel
// One colour of the multicolour Gauss-Seidel sweep (no counterpart in the
// reference, whose smoother is the damped Jacobi above).  Colour c =
// (i & 1) + 2 (j & 1) + 4 (k & 1); a row reads u only at offsets in the
// 19-point set (components in {-1, 0, 1}, at most two non-zero), so nodes of
// one colour never read each other and x is updated in place.  One thread
// per node of the colour: x_p += w (b_p - (A x)_p) / D_p, w = 1 on interior
// rows and the Jacobi damping on boundary rows.
template <typename T, int SYM, bool PSI>
__global__ void __launch_bounds__(256) k_gs_colour(T* x, const T* __restrict__ b, const T* __restrict__ dg,
                                                   const T* __restrict__ C, LevelGeom<T> G, BcTable bc,
                                                   T omega_b, int colour) {
    const int i = 2 * (blockIdx.x * BX + threadIdx.x) + (colour & 1);
    const int j = 2 * (blockIdx.y * BY + threadIdx.y) + ((colour >> 1) & 1);
    const int k = 2 * (blockIdx.z * BZ + threadIdx.z) + ((colour >> 2) & 1);
    if (i >= G.nx || j >= G.ny || k >= G.nz) return;
    const int64_t id = i + G.sy * j + G.sz * k;
    T ax[3];
    apply_node<T, SYM, PSI>(x, C, G, bc, i, j, k, id, ax);
    const bool bnd = i == 0 || j == 0 || k == 0 || i == G.nx - 1 || j == G.ny - 1 || k == G.nz - 1;
    const T w = bnd ? omega_b : T(1);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const int64_t q = c * G.N + id;
        x[q] = x[q] + w * (b[q] - ax[c]) / dg[q];
    }
}

template <typename T>
cudaError_t launch_gs_colour(int sym, T* x, const T* b, const T* diag, const T* C, const LevelGeom<T>& G,
                             const BcTable& bc, T omega_b, int colour, cudaStream_t s) {
    const int hx = (G.nx - (colour & 1) + 1) / 2, hy = (G.ny - ((colour >> 1) & 1) + 1) / 2,
              hz = (G.nz - ((colour >> 2) & 1) + 1) / 2;
    if (hx <= 0 || hy <= 0 || hz <= 0) return cudaSuccess;
    dim3 blk(BX, BY, BZ), grd = grid3(hx, hy, hz);
    if (G.psi) {
        if (sym == SYM_ISO) k_gs_colour<T, SYM_ISO, true><<<grd, blk, 0, s>>>(x, b, diag, C, G, bc, omega_b, colour);
        else if (sym == SYM_MAJ) k_gs_colour<T, SYM_MAJ, true><<<grd, blk, 0, s>>>(x, b, diag, C, G, bc, omega_b, colour);
        else k_gs_colour<T, SYM_MM, true><<<grd, blk, 0, s>>>(x, b, diag, C, G, bc, omega_b, colour);
    } else {
        if (sym == SYM_ISO) k_gs_colour<T, SYM_ISO, false><<<grd, blk, 0, s>>>(x, b, diag, C, G, bc, omega_b, colour);
        else if (sym == SYM_MAJ) k_gs_colour<T, SYM_MAJ, false><<<grd, blk, 0, s>>>(x, b, diag, C, G, bc, omega_b, colour);
        else k_gs_colour<T, SYM_MM, false><<<grd, blk, 0, s>>>(x, b, diag, C, G, bc, omega_b, colour);
    }
    return cudaGetLastError();
}
template cudaError_t launch_gs_colour<double>(int, double*, const double*, const double*, const double*,
                                              const LevelGeom<double>&, const BcTable&, double, int, cudaStream_t);
template cudaError_t launch_gs_colour<float>(int, float*, const float*, const float*, const float*,
                                             const LevelGeom<float>&, const BcTable&, float, int, cudaStream_t);

// ---------------------------------------------------------------- residual
// Block reduction of (max, sum) pairs: warp shuffles, then one warp over the
// per-warp results.  Deterministic for a fixed launch shape.
__device__ __forceinline__ void block_max_sum(double& mx, double& sm, double* out) {
    __shared__ double smx[32], ssm[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        sm += __shfl_xor_sync(0xffffffffu, sm, o);
    }
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nthr = blockDim.x * blockDim.y * blockDim.z;
    const int w = tid >> 5, l = tid & 31, nw = (nthr + 31) >> 5;
    if (l == 0) { smx[w] = mx; ssm[w] = sm; }
    __syncthreads();
    if (w == 0) {
        mx = (l < nw) ? smx[l] : 0.0;
        sm = (l < nw) ? ssm[l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            sm += __shfl_xor_sync(0xffffffffu, sm, o);
        }
        if (l == 0) { out[0] = mx; out[1] = sm; }
    }
}

template <typename T, int SYM, bool PSI>
__global__ void __launch_bounds__(256) k_residual(const T* __restrict__ x, const T* __restrict__ b,
                                                  const T* __restrict__ C, LevelGeom<T> G, BcTable bc,
                                                  T* __restrict__ r, double* __restrict__ partials) {
    AGB_NODE_INDEX
    double mx = 0.0, sm = 0.0;
    if (live) {
        T ax[3];
        apply_node<T, SYM, PSI>(x, C, G, bc, i, j, k, id, ax);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const int64_t q = c * G.N + id;
            const T rv = b[q] - ax[c];
            r[q] = rv;
            const double a = fabs((double)rv);
            mx = fmax(mx, a);
            sm += a * a;
        }
    }
    if (partials) {
        const int blk = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
        block_max_sum(mx, sm, partials + 2 * blk);
    }
}

int residual_blocks(int nx, int ny, int nz) {
    dim3 g = grid3(nx, ny, nz);
    return (int)(g.x * g.y * g.z);
}

template <typename T>
cudaError_t launch_residual(int sym, const T* x, const T* b, const T* C, const LevelGeom<T>& G, const BcTable& bc,
                            T* r, double* partials, int* nblocks_out, cudaStream_t s) {
    dim3 blk(BX, BY, BZ), grd = grid3(G.nx, G.ny, G.nz);
    if (nblocks_out) *nblocks_out = (int)(grd.x * grd.y * grd.z);
    if (G.psi) {
        if (sym == SYM_ISO) k_residual<T, SYM_ISO, true><<<grd, blk, 0, s>>>(x, b, C, G, bc, r, partials);
        else if (sym == SYM_MAJ) k_residual<T, SYM_MAJ, true><<<grd, blk, 0, s>>>(x, b, C, G, bc, r, partials);
        else k_residual<T, SYM_MM, true><<<grd, blk, 0, s>>>(x, b, C, G, bc, r, partials);
    } else {
        if (sym == SYM_ISO) k_residual<T, SYM_ISO, false><<<grd, blk, 0, s>>>(x, b, C, G, bc, r, partials);
        else if (sym == SYM_MAJ) k_residual<T, SYM_MAJ, false><<<grd, blk, 0, s>>>(x, b, C, G, bc, r, partials);
        else k_residual<T, SYM_MM, false><<<grd, blk, 0, s>>>(x, b, C, G, bc, r, partials);
    }
    return cudaGetLastError();
}
template cudaError_t launch_residual<double>(int, const double*, const double*, const double*,
                                             const LevelGeom<double>&, const BcTable&, double*, double*, int*,
                                             cudaStream_t);
template cudaError_t launch_residual<float>(int, const float*, const float*, const float*, const LevelGeom<float>&,
                                            const BcTable&, float*, double*, int*, cudaStream_t);

__global__ void __launch_bounds__(1024) k_reduce_norms(const double* __restrict__ p, int nb, double* __restrict__ out) {
    double mx = 0.0, sm = 0.0;
    for (int q = threadIdx.x; q < nb; q += blockDim.x) {
        mx = fmax(mx, p[2 * q]);
        sm += p[2 * q + 1];
    }
    __shared__ double o[2];
    block_max_sum(mx, sm, o);
    __syncthreads();
    if (threadIdx.x == 0) { out[0] = o[0]; out[1] = sqrt(o[1]); }
}

cudaError_t launch_reduce_norms(const double* partials, int nblocks, double* norms, cudaStream_t s) {
    k_reduce_norms<<<1, 1024, 0, s>>>(partials, nblocks, norms);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256) k_vec_partials(const double* __restrict__ v, int64_t n, double* __restrict__ p) {
    double mx = 0.0, sm = 0.0;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const double a = fabs(v[q]);
        mx = fmax(mx, a);
        sm += a * a;
    }
    block_max_sum(mx, sm, p + 2 * blockIdx.x);
}

cudaError_t launch_vec_norms(const double* v, int64_t n, double* partials, int nblocks, double* norms,
                             cudaStream_t s) {
    k_vec_partials<<<nblocks, 256, 0, s>>>(v, n, partials);
    k_reduce_norms<<<1, 1024, 0, s>>>(partials, nblocks, norms);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- transfer
// Nodal full weighting with boundary-reduced weights
// (src/Operator/Operator.cpp:294-352): corners injected, edges 1/4-1/2-1/4,
// faces the 9-point /16 stencil, interior the 27-point 1/8-1/16-1/32-1/64.
template <typename T, typename F>
__device__ __forceinline__ T restrict_point(F f, int I, int J, int K, int ncx, int ncy, int ncz) {
    const bool ex = (I == 0) | (I == ncx - 1), ey = (J == 0) | (J == ncy - 1), ez = (K == 0) | (K == ncz - 1);
    if (ex & ey & ez) return f(0, 0, 0);
    if (ey & ez) return T(0.25) * f(-1, 0, 0) + T(0.5) * f(0, 0, 0) + T(0.25) * f(1, 0, 0);
    if (ez & ex) return T(0.25) * f(0, -1, 0) + T(0.5) * f(0, 0, 0) + T(0.25) * f(0, 1, 0);
    if (ex & ey) return T(0.25) * f(0, 0, -1) + T(0.5) * f(0, 0, 0) + T(0.25) * f(0, 0, 1);
    if (ex)
        return (f(0, -1, -1) + T(2) * f(0, 0, -1) + f(0, 1, -1) + T(2) * f(0, -1, 0) + T(4) * f(0, 0, 0) +
                T(2) * f(0, 1, 0) + f(0, -1, 1) + T(2) * f(0, 0, 1) + f(0, 1, 1)) * T(1.0 / 16.0);
    if (ey)
        return (f(-1, 0, -1) + T(2) * f(-1, 0, 0) + f(-1, 0, 1) + T(2) * f(0, 0, -1) + T(4) * f(0, 0, 0) +
                T(2) * f(0, 0, 1) + f(1, 0, -1) + T(2) * f(1, 0, 0) + f(1, 0, 1)) * T(1.0 / 16.0);
    if (ez)
        return (f(-1, -1, 0) + T(2) * f(0, -1, 0) + f(1, -1, 0) + T(2) * f(-1, 0, 0) + T(4) * f(0, 0, 0) +
                T(2) * f(1, 0, 0) + f(-1, 1, 0) + T(2) * f(0, 1, 0) + f(1, 1, 0)) * T(1.0 / 16.0);
    const T corners = f(-1, -1, -1) + f(-1, -1, 1) + f(-1, 1, -1) + f(-1, 1, 1) + f(1, -1, -1) + f(1, -1, 1) +
                      f(1, 1, -1) + f(1, 1, 1);
    const T edges = f(0, -1, -1) + f(0, -1, 1) + f(0, 1, -1) + f(0, 1, 1) + f(-1, 0, -1) + f(1, 0, -1) + f(-1, 0, 1) +
                    f(1, 0, 1) + f(-1, -1, 0) + f(-1, 1, 0) + f(1, -1, 0) + f(1, 1, 0);
    const T faces = f(-1, 0, 0) + f(0, -1, 0) + f(0, 0, -1) + f(1, 0, 0) + f(0, 1, 0) + f(0, 0, 1);
    return corners * T(1.0 / 64.0) + edges * T(1.0 / 32.0) + faces * T(1.0 / 16.0) + f(0, 0, 0) * T(1.0 / 8.0);
}

// xout (optional): the coarse level's first Jacobi sweep from a zero
// correction, xout = omega crse / diag (k_jacobi_zero fused in)
template <typename T>
__global__ void __launch_bounds__(256) k_restrict(const T* __restrict__ fine, LevelGeom<T> Gf, T* __restrict__ crse,
                                                  LevelGeom<T> G, const T* __restrict__ dg, T omega,
                                                  T* __restrict__ xout) {
    AGB_NODE_INDEX
    if (!live) return;
    const int64_t fid = 2 * i + Gf.sy * (2 * j) + Gf.sz * (2 * k);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const T* fc = fine + c * Gf.N + fid;
        auto f = [&](int a, int b, int d) { return fc[a + Gf.sy * b + Gf.sz * d]; };
        const T v = restrict_point<T>(f, i, j, k, G.nx, G.ny, G.nz);
        crse[c * G.N + id] = v;
        if (xout) xout[c * G.N + id] = omega * (v - T(0)) / dg[c * G.N + id];
    }
}

template <typename T>
cudaError_t launch_restrict(const T* fine, const LevelGeom<T>& Gf, T* crse, const LevelGeom<T>& Gc, cudaStream_t s) {
    dim3 blk(BX, BY, BZ), grd = grid3(Gc.nx, Gc.ny, Gc.nz);
    k_restrict<T><<<grd, blk, 0, s>>>(fine, Gf, crse, Gc, nullptr, T(0), nullptr);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_restrict_jacobi(const T* fine, const LevelGeom<T>& Gf, T* crse, const LevelGeom<T>& Gc,
                                   const T* diag, T omega, T* xout, cudaStream_t s) {
    dim3 blk(BX, BY, BZ), grd = grid3(Gc.nx, Gc.ny, Gc.nz);
    k_restrict<T><<<grd, blk, 0, s>>>(fine, Gf, crse, Gc, diag, omega, xout);
    return cudaGetLastError();
}
template cudaError_t launch_restrict_jacobi<double>(const double*, const LevelGeom<double>&, double*,
                                                    const LevelGeom<double>&, const double*, double, double*,
                                                    cudaStream_t);
template cudaError_t launch_restrict_jacobi<float>(const float*, const LevelGeom<float>&, float*,
                                                   const LevelGeom<float>&, const float*, float, float*, cudaStream_t);
template cudaError_t launch_restrict<double>(const double*, const LevelGeom<double>&, double*,
                                             const LevelGeom<double>&, cudaStream_t);
template cudaError_t launch_restrict<float>(const float*, const LevelGeom<float>&, float*, const LevelGeom<float>&,
                                            cudaStream_t);

// C coarsening (src/Operator/Elastic.cpp:786-834): same weights per entry
template <typename T>
__global__ void __launch_bounds__(256) k_restrict_C(const T* __restrict__ Cf, LevelGeom<T> Gf, T* __restrict__ Cc,
                                                    LevelGeom<T> G, int nc) {
    AGB_NODE_INDEX
    if (!live) return;
    const int64_t fid = 2 * i + Gf.sy * (2 * j) + Gf.sz * (2 * k);
    for (int c = 0; c < nc; c++) {
        const T* fc = Cf + c * Gf.N + fid;
        auto f = [&](int a, int b, int d) { return fc[a + Gf.sy * b + Gf.sz * d]; };
        Cc[c * G.N + id] = restrict_point<T>(f, i, j, k, G.nx, G.ny, G.nz);
    }
}

cudaError_t launch_restrict_C(const double* Cf, const LevelGeom<double>& Gf, double* Cc, const LevelGeom<double>& Gc,
                              int nc, cudaStream_t s) {
    dim3 blk(BX, BY, BZ), grd = grid3(Gc.nx, Gc.ny, Gc.nz);
    k_restrict_C<double><<<grd, blk, 0, s>>>(Cf, Gf, Cc, Gc, nc);
    return cudaGetLastError();
}
cudaError_t launch_restrict_C(const float* Cf, const LevelGeom<float>& Gf, float* Cc, const LevelGeom<float>& Gc,
                              int nc, cudaStream_t s) {
    dim3 blk(BX, BY, BZ), grd = grid3(Gc.nx, Gc.ny, Gc.nz);
    k_restrict_C<float><<<grd, blk, 0, s>>>(Cf, Gf, Cc, Gc, nc);
    return cudaGetLastError();
}

// trilinear prolongation added to the fine field
// (src/Operator/Operator.cpp:399-428)
template <typename T>
__global__ void __launch_bounds__(256) k_prolong_add(const T* __restrict__ crse, LevelGeom<T> Gc, T* __restrict__ fine,
                                                     LevelGeom<T> G) {
    // one thread per coarse column I and fine row (j, k): fine nodes 2I
    // (weight 1 at I) and 2I+1 (1/2 at I and I+1) along x; the (j, k) parity
    // picks the coarse rows averaged first, uniform across a warp.  R(I+1)
    // comes from the next lane (the warp's last lane reads it).
    const int I = blockIdx.x * BX + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int k = blockIdx.z * BZ + threadIdx.z;
    const bool live = (I < Gc.nx) & (j < G.ny) & (k < G.nz);
    const int J = j >> 1, K = k >> 1, oj = j & 1, ok = k & 1;
    const int64_t dy = oj ? Gc.sy : 0, dz = ok ? Gc.sz : 0;
    auto rowavg = [&](const T* cc) -> T {
        if (oj & ok) return T(0.25) * ((cc[0] + cc[dy]) + (cc[dz] + cc[dy + dz]));
        if (oj | ok) return T(0.5) * (cc[0] + cc[dy + dz]);
        return cc[0];
    };
    const int64_t cid = (int64_t)I + Gc.sy * J + Gc.sz * K;
    const int64_t fid = 2 * (int64_t)I + G.sy * j + G.sz * (int64_t)k;
    const bool odd = live && (I + 1 < Gc.nx);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const T* cc = crse + c * Gc.N + cid;
        const T R = live ? rowavg(cc) : T(0);
        T Rn = __shfl_down_sync(0xffffffffu, R, 1);
        if (threadIdx.x == BX - 1 && odd) Rn = rowavg(cc + 1);
        if (live) {
            T* f = fine + c * G.N + fid;
            f[0] += R;
            if (odd) f[1] += T(0.5) * (R + Rn);
        }
    }
}

template <typename T>
cudaError_t launch_prolong_add(const T* crse, const LevelGeom<T>& Gc, T* fine, const LevelGeom<T>& Gf,
                               cudaStream_t s) {
    dim3 blk(BX, BY, BZ), grd = grid3(Gc.nx, Gf.ny, Gf.nz);
    k_prolong_add<T><<<grd, blk, 0, s>>>(crse, Gc, fine, Gf);
    return cudaGetLastError();
}
template cudaError_t launch_prolong_add<double>(const double*, const LevelGeom<double>&, double*,
                                                const LevelGeom<double>&, cudaStream_t);
template cudaError_t launch_prolong_add<float>(const float*, const LevelGeom<float>&, float*, const LevelGeom<float>&,
                                               cudaStream_t);

// ---------------------------------------------------------------- helpers
// AoS (N, nc) -> SoA (nc, N) through shared memory: a tile of 128 nodes is
// read as one contiguous run and written as nc contiguous runs, both
// coalesced (nc <= 21; the stride-nc shared reads are conflict-free per
// half-warp for odd nc)
static constexpr int TR_NODES = 128;
__global__ void __launch_bounds__(256) k_aos_to_soa(const double* __restrict__ a, double* __restrict__ s, int64_t N,
                                                    int nc) {
    __shared__ double t[TR_NODES * 21];
    const int64_t ntiles = (N + TR_NODES - 1) / TR_NODES;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t n0 = tile * TR_NODES;
        const int nn = (int)(N - n0 < TR_NODES ? N - n0 : TR_NODES);
        const double* src = a + n0 * nc;
        for (int q = threadIdx.x; q < nn * nc; q += blockDim.x) t[q] = src[q];
        __syncthreads();
        for (int q = threadIdx.x; q < nn * nc; q += blockDim.x) {
            const int c = q / nn, node = q - c * nn;
            s[c * N + n0 + node] = t[node * nc + c];
        }
        __syncthreads();
    }
}
__global__ void k_soa_to_aos(const double* __restrict__ s, double* __restrict__ a, int64_t N, int nc) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < N * nc; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t node = q / nc;
        const int c = (int)(q - node * nc);
        a[q] = s[c * N + node];
    }
}
// (lambda, mu, F0) per node for the learned initial guess: the isotropic
// entries, or the Voigt average of a major-minor tensor (K = (C11 + C22 + C33
// + 2 (C12 + C13 + C23)) / 9, mu = (C11 + C22 + C33 - C12 - C13 - C23 + 3 (C44
// + C55 + C66)) / 15, lambda = K - 2 mu / 3); F0 scalar or trace / 3
__global__ void k_guess_features(int sym, const double* __restrict__ C, int64_t N, const double* __restrict__ F0,
                                 int f0n, double* __restrict__ out) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < N; q += (int64_t)gridDim.x * blockDim.x) {
        double lam, mu;
        if (sym == SYM_ISO) {
            lam = C[q];
            mu = C[N + q];
        } else {
            auto c = [&](int a, int b) { return C[mm_ut(a, b) * N + q]; };
            const double d = c(0, 0) + c(3, 3) + c(5, 5);
            const double o = c(0, 3) + c(0, 5) + c(3, 5);
            const double sh = c(4, 4) + c(2, 2) + c(1, 1);
            const double K = (d + 2.0 * o) / 9.0;
            mu = (d - o + 3.0 * sh) / 15.0;
            lam = K - 2.0 * mu / 3.0;
        }
        double f = 0.0;
        if (f0n == 1) f = F0[q];
        else if (f0n == 9) f = (F0[9 * q] + F0[9 * q + 4] + F0[9 * q + 8]) / 3.0;
        out[q] = lam;
        out[N + q] = mu;
        out[2 * N + q] = f;
    }
}
cudaError_t launch_guess_features(int sym, const double* C, int64_t N, const double* F0, int f0n, double* out,
                                  cudaStream_t s) {
    k_guess_features<<<flat_blocks(N), 256, 0, s>>>(sym, C, N, F0, f0n, out);
    return cudaGetLastError();
}

// wider records (the 45 Major-symmetry entries): one strided pass
__global__ void k_aos_to_soa_wide(const double* __restrict__ a, double* __restrict__ s, int64_t N, int nc) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < N * nc; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = q / N, node = q - c * N;
        s[q] = a[node * nc + c];
    }
}

cudaError_t launch_aos_to_soa(const double* aos, double* soa, int64_t N, int nc, cudaStream_t s) {
    if (nc > 21) {
        k_aos_to_soa_wide<<<flat_blocks(N * nc), 256, 0, s>>>(aos, soa, N, nc);
        return cudaGetLastError();
    }
    const int64_t tiles = (N + TR_NODES - 1) / TR_NODES;
    k_aos_to_soa<<<(int)(tiles < 152 * 8 ? tiles : 152 * 8), 256, 0, s>>>(aos, soa, N, nc);
    return cudaGetLastError();
}
cudaError_t launch_soa_to_aos(const double* soa, double* aos, int64_t N, int nc, cudaStream_t s) {
    k_soa_to_aos<<<flat_blocks(N * nc), 256, 0, s>>>(soa, aos, N, nc);
    return cudaGetLastError();
}

__global__ void k_recip(const float* __restrict__ in, float* __restrict__ out, int64_t n) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        out[q] = 1.f / in[q];
}

cudaError_t launch_recip(const float* in, float* out, int64_t n, cudaStream_t s) {
    k_recip<<<flat_blocks(n), 256, 0, s>>>(in, out, n);
    return cudaGetLastError();
}

__global__ void k_to_float(const double* __restrict__ in, float* __restrict__ out, int64_t n, double scale) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        out[q] = (float)(in[q] * scale);
}
cudaError_t launch_to_float(const double* in, float* out, int64_t n, double scale, cudaStream_t s) {
    k_to_float<<<flat_blocks(n), 256, 0, s>>>(in, out, n, scale);
    return cudaGetLastError();
}

__global__ void k_add_float(const float* __restrict__ in, double* __restrict__ out, int64_t n, double scale) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        out[q] += scale * (double)in[q];
}
cudaError_t launch_add_float(const float* in, double* out, int64_t n, double scale, cudaStream_t s) {
    k_add_float<<<flat_blocks(n), 256, 0, s>>>(in, out, n, scale);
    return cudaGetLastError();
}

template <typename T>
__global__ void k_axpy(T a, const T* __restrict__ x, T* __restrict__ y, int64_t n) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        y[q] += a * x[q];
}
cudaError_t launch_axpy(double a, const double* x, double* y, int64_t n, cudaStream_t s) {
    k_axpy<double><<<flat_blocks(n), 256, 0, s>>>(a, x, y, n);
    return cudaGetLastError();
}
cudaError_t launch_axpy(float a, const float* x, float* y, int64_t n, cudaStream_t s) {
    k_axpy<float><<<flat_blocks(n), 256, 0, s>>>(a, x, y, n);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- BC init
// BC::Operator::Elastic::Constant::Init (src/BC/Operator/Elastic/Constant.H:
// 197-286): every boundary node of b gets its region's value (0 for
// displacement rows when homogeneous).
__global__ void __launch_bounds__(256) k_bc_init(double* __restrict__ b, LevelGeom<double> G, BcTable bc,
                                                 const double* __restrict__ val, int homogeneous) {
    AGB_NODE_INDEX
    if (!live) return;
    const int cx = (i == 0) ? -1 : (i == G.nx - 1) ? 1 : 0;
    const int cy = (j == 0) ? -1 : (j == G.ny - 1) ? 1 : 0;
    const int cz = (k == 0) ? -1 : (k == G.nz - 1) ? 1 : 0;
    if (!(cx | cy | cz)) return;
    double n[3];
    const int reg = boundary_region<double>(cx, cy, cz, n);
#pragma unroll
    for (int d = 0; d < 3; d++)
        b[d * G.N + id] = (homogeneous && bc.t[reg * 3 + d] == BC_DISP) ? 0.0 : val[reg * 3 + d];
}

cudaError_t launch_bc_init(double* b, const LevelGeom<double>& G, const BcTable& bc, const double* bcval_dev,
                           int homogeneous, cudaStream_t s) {
    dim3 blk(BX, BY, BZ), grd = grid3(G.nx, G.ny, G.nz);
    k_bc_init<<<grd, blk, 0, s>>>(b, G, bc, bcval_dev, homogeneous);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- RHS
__device__ __forceinline__ double f0_at(const double* F0, int f0n, int64_t id, int p, int q) {
    if (f0n == 1) return p == q ? F0[id] : 0.0;
    if (f0n == 9) return F0[id * 9 + p * 3 + q];
    return 0.0;
}

// dw = C (grad u - F0), stored SoA as 9 components (row-major p*3+q);
// ZERO_U: u = 0 (the Newton step from zero), no displacement is read
template <int SYM, bool ZERO_U>
__global__ void __launch_bounds__(256) k_dw(const double* __restrict__ u, const double* __restrict__ F0, int f0n,
                                            const double* __restrict__ C, LevelGeom<double> G,
                                            double* __restrict__ dw) {
    AGB_NODE_INDEX
    if (!live) return;
    double g[3][3], s[3][3];
    if (ZERO_U) {
#pragma unroll
        for (int p = 0; p < 3; p++)
#pragma unroll
            for (int q = 0; q < 3; q++) g[p][q] = 0.0;
    } else {
        grad_at(u, G, i, j, k, id, g);
    }
#pragma unroll
    for (int p = 0; p < 3; p++)
#pragma unroll
        for (int q = 0; q < 3; q++) g[p][q] -= f0_at(F0, f0n, id, p, q);
    const int64_t N = G.N;
    auto cf = [&](int a) { return C[a * N + id]; };
    stress_of<double, SYM>(cf, g, s);
#pragma unroll
    for (int p = 0; p < 3; p++)
#pragma unroll
        for (int q = 0; q < 3; q++) dw[(p * 3 + q) * N + id] = s[p][q];
}

template <bool ZERO_U>
__global__ void __launch_bounds__(256) k_rhs(const double* __restrict__ u, const double* __restrict__ b,
                                             const double* __restrict__ dw, LevelGeom<double> G, BcTable bc,
                                             double* __restrict__ rhs) {
    AGB_NODE_INDEX
    if (!live) return;
    const int64_t N = G.N;
    const int cx = (i == 0) ? -1 : (i == G.nx - 1) ? 1 : 0;
    const int cy = (j == 0) ? -1 : (j == G.ny - 1) ? 1 : 0;
    const int cz = (k == 0) ? -1 : (k == G.nz - 1) ? 1 : 0;
    double ret[3];
    if (cx | cy | cz) {
        double g[3][3], s[3][3], n[3];
        if (ZERO_U) {
#pragma unroll
            for (int p = 0; p < 3; p++)
#pragma unroll
                for (int q = 0; q < 3; q++) g[p][q] = 0.0;
        } else {
            grad_at(u, G, i, j, k, id, g);
        }
#pragma unroll
        for (int p = 0; p < 3; p++)
#pragma unroll
            for (int q = 0; q < 3; q++) s[p][q] = dw[(p * 3 + q) * N + id];
        const int reg = boundary_region<double>(cx, cy, cz, n);
#pragma unroll
        for (int r = 0; r < 3; r++) ret[r] = bc_component<double>(bc.t, reg, r, ZERO_U ? 0.0 : u[r * N + id], g, s, n);
    } else {
        // div dw with central differences (src/Numeric/Stencil.H:588-657)
        const int64_t off[3] = {1, G.sy, G.sz};
#pragma unroll
        for (int c = 0; c < 3; c++) {
            double acc = 0.0;
#pragma unroll
            for (int d = 0; d < 3; d++) {
                const double* w = dw + (c * 3 + d) * N + id;
                acc += (w[off[d]] - w[-off[d]]) * G.h[d];
            }
            ret[c] = acc;
        }
        if (G.psi) {
            // Newton.H:255-261: div(dw) avg8(psi) + dw grad psi (no psi_small)
            double gp[3];
            const double avg = psi_node<double>(G, i, j, k, gp);
#pragma unroll
            for (int c = 0; c < 3; c++)
                ret[c] = ret[c] * avg + (dw[(c * 3 + 0) * N + id] * gp[0] + dw[(c * 3 + 1) * N + id] * gp[1] +
                                         dw[(c * 3 + 2) * N + id] * gp[2]);
        }
    }
#pragma unroll
    for (int c = 0; c < 3; c++) rhs[c * N + id] = b[c * N + id] - ret[c];
}

cudaError_t launch_build_rhs(int sym, const double* u, const double* b, const double* F0, int f0_ncomp,
                             const double* C, const LevelGeom<double>& G, const BcTable& bc, double* dw, double* rhs,
                             cudaStream_t s) {
    dim3 blk(BX, BY, BZ), grd = grid3(G.nx, G.ny, G.nz);
    if (u == nullptr && f0_ncomp == 0) {
        // u = 0 and no eigenstrain: dw = 0, every row of b - (BC rows / div dw)
        // subtracts an exact zero, so rhs = b
        if (rhs == b) return cudaSuccess;
        return cudaMemcpyAsync(rhs, b, sizeof(double) * 3 * G.N, cudaMemcpyDeviceToDevice, s);
    }
    if (u == nullptr) {
        if (sym == SYM_ISO) k_dw<SYM_ISO, true><<<grd, blk, 0, s>>>(u, F0, f0_ncomp, C, G, dw);
        else if (sym == SYM_MAJ) k_dw<SYM_MAJ, true><<<grd, blk, 0, s>>>(u, F0, f0_ncomp, C, G, dw);
        else k_dw<SYM_MM, true><<<grd, blk, 0, s>>>(u, F0, f0_ncomp, C, G, dw);
    } else {
        if (sym == SYM_ISO) k_dw<SYM_ISO, false><<<grd, blk, 0, s>>>(u, F0, f0_ncomp, C, G, dw);
        else if (sym == SYM_MAJ) k_dw<SYM_MAJ, false><<<grd, blk, 0, s>>>(u, F0, f0_ncomp, C, G, dw);
        else k_dw<SYM_MM, false><<<grd, blk, 0, s>>>(u, F0, f0_ncomp, C, G, dw);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (u == nullptr) k_rhs<true><<<grd, blk, 0, s>>>(u, b, dw, G, bc, rhs);
    else k_rhs<false><<<grd, blk, 0, s>>>(u, b, dw, G, bc, rhs);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- NeoHookean
// Newton::prepareForSolve for Model::Solid::Finite::NeoHookean
// (src/Solver/Nonlocal/Newton.H:144-196, src/Model/Solid/Finite/NeoHookean.H:
// 21-121): per node F = I + grad u (one-sided on the faces), dw = DW(F)
// (SoA 9, row-major) and C = DDW(F) (SoA 45, Major symmetry; every entry is
// written by both of its index pairs in the reference's loop order, the
// later one kept).  model: SoA (mu, kappa).
__global__ void __launch_bounds__(256) k_neohookean(const double* __restrict__ model, const double* __restrict__ u,
                                                    LevelGeom<double> G, double* __restrict__ dw,
                                                    double* __restrict__ C) {
    AGB_NODE_INDEX
    if (!live) return;
    const int64_t N = G.N;
    double F[3][3];
    grad_at(u, G, i, j, k, id, F);
#pragma unroll
    for (int a = 0; a < 3; a++) F[a][a] += 1.0;
    const double mu = model[id], kappa = model[N + id];
    // inverse by cofactors, det by the first row
    const double c00 = F[1][1] * F[2][2] - F[1][2] * F[2][1];
    const double c01 = F[1][2] * F[2][0] - F[1][0] * F[2][2];
    const double c02 = F[1][0] * F[2][1] - F[1][1] * F[2][0];
    const double J = F[0][0] * c00 + F[0][1] * c01 + F[0][2] * c02;
    const double iJ = 1.0 / J;
    double FiT[3][3];  // (F^-1)^T
    FiT[0][0] = c00 * iJ;
    FiT[0][1] = c01 * iJ;
    FiT[0][2] = c02 * iJ;
    FiT[1][0] = (F[0][2] * F[2][1] - F[0][1] * F[2][2]) * iJ;
    FiT[1][1] = (F[0][0] * F[2][2] - F[0][2] * F[2][0]) * iJ;
    FiT[1][2] = (F[0][1] * F[2][0] - F[0][0] * F[2][1]) * iJ;
    FiT[2][0] = (F[0][1] * F[1][2] - F[0][2] * F[1][1]) * iJ;
    FiT[2][1] = (F[0][2] * F[1][0] - F[0][0] * F[1][2]) * iJ;
    FiT[2][2] = (F[0][0] * F[1][1] - F[0][1] * F[1][0]) * iJ;
    double tr = 0.0;
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b2 = 0; b2 < 3; b2++) tr += F[a][b2] * F[a][b2];
    const double J23 = pow(fabs(J), 2. / 3.);
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b2 = 0; b2 < 3; b2++)
            dw[(a * 3 + b2) * N + id] =
                mu * (F[a][b2] / J23 - tr * FiT[a][b2] / (3. * J23)) + kappa * (J - 1) * J * FiT[a][b2];
#pragma unroll
    for (int ii = 0; ii < 3; ii++)
#pragma unroll
        for (int jj = 0; jj < 3; jj++)
#pragma unroll
            for (int kk = 0; kk < 3; kk++)
#pragma unroll
                for (int ll = 0; ll < 3; ll++) {
                    // only the later of the two writes of an entry is kept
                    if (3 * ii + jj < 3 * kk + ll) continue;
                    double t1 = 0.0, t2 = 0.0;
                    if (ii == kk && jj == ll) t1 += 1.0;
                    t1 -= (2. / 3.) * F[ii][jj] * FiT[kk][ll];
                    t1 -= (2. / 3.) * FiT[ii][jj] * F[kk][ll];
                    t1 += (2. / 9.) * tr * FiT[ii][jj] * FiT[kk][ll];
                    t1 += (1. / 3.) * tr * FiT[ii][ll] * FiT[kk][jj];
                    t2 += (2. * J - 1.) * FiT[ii][jj] * FiT[kk][ll];
                    t2 += (1. - J) * FiT[ii][ll] * FiT[kk][jj];
                    C[maj_of(ii, jj, kk, ll) * N + id] = (mu / J23) * t1 + kappa * J * t2;
                }
}

cudaError_t launch_neohookean(const double* model, const double* u, const LevelGeom<double>& G, double* dw,
                              double* C, cudaStream_t s) {
    dim3 blk(BX, BY, BZ), grd = grid3(G.nx, G.ny, G.nz);
    k_neohookean<<<grd, blk, 0, s>>>(model, u, G, dw, C);
    return cudaGetLastError();
}

cudaError_t launch_rhs_from_dw(const double* u, const double* b, const double* dw, const LevelGeom<double>& G,
                               const BcTable& bc, double* rhs, cudaStream_t s) {
    dim3 blk(BX, BY, BZ), grd = grid3(G.nx, G.ny, G.nz);
    k_rhs<false><<<grd, blk, 0, s>>>(u, b, dw, G, bc, rhs);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- psi
// Ghosted psi of the fine level from the caller's (nx-1)(ny-1)(nz-1) cells;
// ghost entries 1.0 (the reference's define-time fill, Elastic.cpp:49-52).
__global__ void k_psi_embed(const double* __restrict__ cells, LevelGeom<double> G, double* __restrict__ psi) {
    const int64_t tot = G.psz * (G.nz + 1);
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < tot; q += (int64_t)gridDim.x * blockDim.x) {
        const int a = (int)(q % G.psy);
        const int b = (int)((q / G.psy) % (G.ny + 1));
        const int c = (int)(q / G.psz);
        const bool ghost = a == 0 || b == 0 || c == 0 || a == G.nx || b == G.ny || c == G.nz;
        psi[q] = ghost ? 1.0 : cells[(a - 1) + (int64_t)(G.nx - 1) * ((b - 1) + (int64_t)(G.ny - 1) * (c - 1))];
    }
}

cudaError_t launch_psi_embed(const double* cells, const LevelGeom<double>& G, double* psi, cudaStream_t s) {
    k_psi_embed<<<flat_blocks(G.psz * (G.nz + 1)), 256, 0, s>>>(cells, G, psi);
    return cudaGetLastError();
}

// Coarse-level psi (Elastic.cpp:839-905): full weighting around fine cell
// (2I, 2J, 2K).  The boundary cases compare the cell index against the node
// domain's bounds, so only index 0 takes the face, edge and corner forms;
// the last cell keeps the interior form (its fine neighbours 2I+1 are in the
// domain).  Ghost entries 1.0.
__global__ void k_coarsen_psi(const double* __restrict__ pf, LevelGeom<double> Gf, double* __restrict__ pc,
                              LevelGeom<double> Gc) {
    const int64_t tot = Gc.psz * (Gc.nz + 1);
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < tot; q += (int64_t)gridDim.x * blockDim.x) {
        const int a = (int)(q % Gc.psy);
        const int b = (int)((q / Gc.psy) % (Gc.ny + 1));
        const int c = (int)(q / Gc.psz);
        if (a == 0 || b == 0 || c == 0 || a == Gc.nx || b == Gc.ny || c == Gc.nz) {
            pc[q] = 1.0;
            continue;
        }
        const int I = a - 1, J = b - 1, K = c - 1;
        const double* base = pf + (2 * I + 1) + Gf.psy * (2 * J + 1) + Gf.psz * (2 * K + 1);
        const int64_t py = Gf.psy, pz = Gf.psz;
        auto F = [&](int x, int y, int z) { return base[x + py * y + pz * z]; };
        const bool xi = I == 0, yj = J == 0, zk = K == 0;
        double v;
        if (xi && yj && zk) v = F(0, 0, 0);
        else if (yj && zk) v = F(-1, 0, 0) * 0.25 + F(0, 0, 0) * 0.5 + F(1, 0, 0) * 0.25;
        else if (zk && xi) v = F(0, -1, 0) * 0.25 + F(0, 0, 0) * 0.5 + F(0, 1, 0) * 0.25;
        else if (xi && yj) v = F(0, 0, -1) * 0.25 + F(0, 0, 0) * 0.5 + F(0, 0, 1) * 0.25;
        else if (xi)
            v = (F(0, -1, -1) + F(0, 0, -1) * 2.0 + F(0, 1, -1) + F(0, -1, 0) * 2.0 + F(0, 0, 0) * 4.0 +
                 F(0, 1, 0) * 2.0 + F(0, -1, 1) + F(0, 0, 1) * 2.0 + F(0, 1, 1)) / 16.0;
        else if (yj)
            v = (F(-1, 0, -1) + F(-1, 0, 0) * 2.0 + F(-1, 0, 1) + F(0, 0, -1) * 2.0 + F(0, 0, 0) * 4.0 +
                 F(0, 0, 1) * 2.0 + F(1, 0, -1) + F(1, 0, 0) * 2.0 + F(1, 0, 1)) / 16.0;
        else if (zk)
            v = (F(-1, -1, 0) + F(0, -1, 0) * 2.0 + F(1, -1, 0) + F(-1, 0, 0) * 2.0 + F(0, 0, 0) * 4.0 +
                 F(1, 0, 0) * 2.0 + F(-1, 1, 0) + F(0, 1, 0) * 2.0 + F(1, 1, 0)) / 16.0;
        else
            v = (F(-1, -1, -1) + F(-1, -1, 1) + F(-1, 1, -1) + F(-1, 1, 1) + F(1, -1, -1) + F(1, -1, 1) +
                 F(1, 1, -1) + F(1, 1, 1)) / 64.0 +
                (F(0, -1, -1) + F(0, -1, 1) + F(0, 1, -1) + F(0, 1, 1) + F(-1, 0, -1) + F(1, 0, -1) +
                 F(-1, 0, 1) + F(1, 0, 1) + F(-1, -1, 0) + F(-1, 1, 0) + F(1, -1, 0) + F(1, 1, 0)) / 32.0 +
                (F(-1, 0, 0) + F(0, -1, 0) + F(0, 0, -1) + F(1, 0, 0) + F(0, 1, 0) + F(0, 0, 1)) / 16.0 +
                F(0, 0, 0) / 8.0;
        pc[q] = v;
    }
}

cudaError_t launch_coarsen_psi(const double* pf, const LevelGeom<double>& Gf, double* pc, const LevelGeom<double>& Gc,
                               cudaStream_t s) {
    k_coarsen_psi<<<flat_blocks(Gc.psz * (Gc.nz + 1)), 256, 0, s>>>(pf, Gf, pc, Gc);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- stress
template <int SYM>
__global__ void __launch_bounds__(256) k_stress_strain(const double* __restrict__ u, const double* __restrict__ F0,
                                                       int f0n, const double* __restrict__ C, LevelGeom<double> G,
                                                       double* __restrict__ stress, double* __restrict__ strain,
                                                       double* __restrict__ energy) {
    AGB_NODE_INDEX
    if (!live) return;
    double g[3][3], ge[3][3], s[3][3];
    grad_at(u, G, i, j, k, id, g);
#pragma unroll
    for (int p = 0; p < 3; p++)
#pragma unroll
        for (int q = 0; q < 3; q++) ge[p][q] = g[p][q] - f0_at(F0, f0n, id, p, q);
    const int64_t N = G.N;
    auto cf = [&](int a) { return C[a * N + id]; };
    stress_of<double, SYM>(cf, ge, s);
    double en = 0.0;
#pragma unroll
    for (int p = 0; p < 3; p++)
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const double e = 0.5 * (g[p][q] + g[q][p]);
            if (stress) stress[id * 9 + p * 3 + q] = s[p][q];
            if (strain) strain[id * 9 + p * 3 + q] = e;
            en += 0.5 * s[p][q] * e;
        }
    if (energy) energy[id] = en;
}

cudaError_t launch_stress_strain(int sym, const double* u, const double* F0, int f0_ncomp, const double* C,
                                 const LevelGeom<double>& G, double* stress, double* strain, double* energy,
                                 cudaStream_t s) {
    dim3 blk(BX, BY, BZ), grd = grid3(G.nx, G.ny, G.nz);
    if (sym == SYM_ISO) k_stress_strain<SYM_ISO><<<grd, blk, 0, s>>>(u, F0, f0_ncomp, C, G, stress, strain, energy);
    else if (sym == SYM_MAJ) k_stress_strain<SYM_MAJ><<<grd, blk, 0, s>>>(u, F0, f0_ncomp, C, G, stress, strain, energy);
    else k_stress_strain<SYM_MM><<<grd, blk, 0, s>>>(u, F0, f0_ncomp, C, G, stress, strain, energy);
    return cudaGetLastError();
}

// Operator-level Stress / Strain (src/Operator/Elastic.cpp:426-549): which 0
// sigma = (C grad u) psi_avg, 1 eps = sym grad u; one-sided gradients at the
// domain boundary.  Output SoA per component (the MultiFab layout): voigt
// 6 components (00, 11, 22, 12, 20, 01), else 9 row-major.
template <int SYM>
__global__ void __launch_bounds__(256) k_op_tensor(const double* __restrict__ u, const double* __restrict__ C,
                                                   LevelGeom<double> G, int which, int voigt,
                                                   double* __restrict__ out) {
    AGB_NODE_INDEX
    if (!live) return;
    double g[3][3], t[3][3];
    grad_at(u, G, i, j, k, id, g);
    const int64_t N = G.N;
    if (which == 0) {
        auto cf = [&](int a) { return C[a * N + id]; };
        stress_of<double, SYM>(cf, g, t);
        if (G.psi) {
            const double pa = psi_avg_of(G, psi_node<double>(G, i, j, k, nullptr));
#pragma unroll
            for (int p = 0; p < 3; p++)
#pragma unroll
                for (int q = 0; q < 3; q++) t[p][q] *= pa;
        }
    } else {
#pragma unroll
        for (int p = 0; p < 3; p++)
#pragma unroll
            for (int q = 0; q < 3; q++) t[p][q] = 0.5 * (g[p][q] + g[q][p]);
    }
    if (voigt) {
        out[0 * N + id] = t[0][0];
        out[1 * N + id] = t[1][1];
        out[2 * N + id] = t[2][2];
        out[3 * N + id] = t[1][2];
        out[4 * N + id] = t[2][0];
        out[5 * N + id] = t[0][1];
    } else {
#pragma unroll
        for (int p = 0; p < 3; p++)
#pragma unroll
            for (int q = 0; q < 3; q++) out[(p * 3 + q) * N + id] = t[p][q];
    }
}

cudaError_t launch_op_tensor(int sym, const double* u, const double* C, const LevelGeom<double>& G, int which,
                             int voigt, double* out, cudaStream_t s) {
    dim3 blk(BX, BY, BZ), grd = grid3(G.nx, G.ny, G.nz);
    if (sym == SYM_ISO) k_op_tensor<SYM_ISO><<<grd, blk, 0, s>>>(u, C, G, which, voigt, out);
    else if (sym == SYM_MAJ) k_op_tensor<SYM_MAJ><<<grd, blk, 0, s>>>(u, C, G, which, voigt, out);
    else k_op_tensor<SYM_MM><<<grd, blk, 0, s>>>(u, C, G, which, voigt, out);
    return cudaGetLastError();
}

}  // namespace agb

namespace agb {

// ---------------------------------------------------------------- Krylov
// Sum of products in the vectors' own type.  For FP32 the products' rounding
// errors (exact through an FMA) and the additions' errors (TwoSum, Knuth) are
// carried in a second FP32 word, so the result is about as accurate as FP64
// accumulation while every operation runs on the FP32 pipe.
template <typename T>
struct Acc {
    T s = T(0);
    __device__ __forceinline__ void add(T a, T b) { s = fma(a, b, s); }
    __device__ __forceinline__ T value() const { return s; }
    __device__ __forceinline__ double dvalue() const { return (double)s; }
};
template <>
struct Acc<float> {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float a, float b) {
        const float p = a * b;
        const float pe = fmaf(a, b, -p);
        const float t = s + p;
        const float z = t - s;
        const float e = (s - (t - z)) + (p - z);
        s = t;
        c += e + pe;
    }
    __device__ __forceinline__ float value() const { return s + c; }
    __device__ __forceinline__ double dvalue() const { return (double)s + (double)c; }
};

// 16-byte vector view of a T array: float4 / double2.  Every Krylov vector
// is its own cudaMalloc allocation, so its base is 16-byte aligned; the
// n % W tail is handled element by element.
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
    using V = float4;
    static constexpr int W = 4;
    __device__ static __forceinline__ float get(const float4& v, int c) {
        return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w;
    }
    __device__ static __forceinline__ void set(float4& v, int c, float x) {
        if (c == 0) v.x = x; else if (c == 1) v.y = x; else if (c == 2) v.z = x; else v.w = x;
    }
};
template <>
struct Vec16<double> {
    using V = double2;
    static constexpr int W = 2;
    __device__ static __forceinline__ double get(const double2& v, int c) { return c == 0 ? v.x : v.y; }
    __device__ static __forceinline__ void set(double2& v, int c, double x) {
        if (c == 0) v.x = x; else v.y = x;
    }
};

// Block sum of one double per thread into part[blockIdx.x * KMAX + col].
static constexpr int KMAX = 40;
__device__ __forceinline__ void block_sum_to(double v, double* part, int col) {
    __shared__ double sh[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += sh[q];
        part[(int64_t)blockIdx.x * KMAX + col] = t;
    }
}

// out[i] = sum_q V_i[q] * w[q] for i < k, two passes: per-block partial sums,
// then one block per i over the partials.  Blocks are organised as (element
// range) x (chunk of 8 vectors) so the 8 accumulators of a thread stay in
// registers.  Each thread streams 16-byte loads of two element groups per
// iteration, which keeps (k+1) x 1 KB in flight per warp: the loads, not
// the arithmetic, set the pace.
static constexpr int KCH = 8;

// Per-thread sums run in the vectors' own type (FP32 vectors: compensated
// FP32, the 1/64-rate FP64 pipe of GB300 would bound the kernel); the
// cross-thread and cross-block reductions run in FP64.
template <typename T>
__global__ void __launch_bounds__(256, 4) k_multidot_partial(const T* const* __restrict__ V, int k,
                                                             const T* __restrict__ w, int64_t n,
                                                             double* __restrict__ part) {
    using VT = Vec16<T>;
    using V4 = typename VT::V;
    constexpr int W = VT::W;
    const int c0 = blockIdx.y * KCH;
    const int kk = min(KCH, k - c0);
    const V4* vp[KCH];
#pragma unroll
    for (int i = 0; i < KCH; i++) vp[i] = reinterpret_cast<const V4*>(i < kk ? V[c0 + i] : V[c0]);
    const V4* w4 = reinterpret_cast<const V4*>(w);
    Acc<T> acc[KCH];
    const int64_t n4 = n / W;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n4; q += 2 * stride) {
        const int64_t q2 = q + stride;
        const bool two = q2 < n4;
        const V4 wa = w4[q];
        V4 wb = wa;
        if (two) wb = w4[q2];
#pragma unroll
        for (int i = 0; i < KCH; i++) {
            if (i < kk) {
                const V4 va = vp[i][q];
#pragma unroll
                for (int c = 0; c < W; c++) acc[i].add(VT::get(va, c), VT::get(wa, c));
                if (two) {
                    const V4 vb = vp[i][q2];
#pragma unroll
                    for (int c = 0; c < W; c++) acc[i].add(VT::get(vb, c), VT::get(wb, c));
                }
            }
        }
    }
    // tail elements n4*W .. n-1
    for (int64_t q = n4 * W + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += stride) {
        const T wq = w[q];
#pragma unroll
        for (int i = 0; i < KCH; i++)
            if (i < kk) acc[i].add(V[c0 + i][q], wq);
    }
    __shared__ double sh[8][KCH];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < KCH; i++) {
        double v = acc[i].dvalue();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sh[wid][i] = v;
    }
    __syncthreads();
    if (threadIdx.x < kk) {
        double t = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += sh[q][threadIdx.x];
        part[(int64_t)blockIdx.x * KMAX + c0 + threadIdx.x] = t;
    }
}

__global__ void k_multidot_final(const double* __restrict__ part, int nb, int k, double* __restrict__ out) {
    const int i = blockIdx.x;
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += part[(int64_t)b * KMAX + i];
    __shared__ double sh[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) t += sh[q];
        out[i] = t;
    }
}

int multidot_blocks() { return 152 * 4; }

template <typename T>
cudaError_t launch_multidot(const T* const* V, int k, const T* w, int64_t n, double* part, double* out,
                            cudaStream_t s) {
    if (k < 1 || k > KMAX) return cudaErrorInvalidValue;
    const int nb = multidot_blocks();
    dim3 grd(nb, (k + KCH - 1) / KCH);
    k_multidot_partial<T><<<grd, 256, 0, s>>>(V, k, w, n, part);
    k_multidot_final<<<k, 256, 0, s>>>(part, nb, k, out);
    return cudaGetLastError();
}
template cudaError_t launch_multidot<double>(const double* const*, int, const double*, int64_t, double*, double*,
                                             cudaStream_t);
template cudaError_t launch_multidot<float>(const float* const*, int, const float*, int64_t, double*, double*,
                                            cudaStream_t);

// w = beta * w + sum_i coef[i] * scale * V_i  (coef in device memory), one
// 16-byte group per thread and step, the loop over the vectors unrolled by 4
// so four loads are in flight; coefficients and the pointer table in shared
// memory, compensated arithmetic in the vectors' type.  With part non-null
// the block sums of w_new^2 go to part[blockIdx.x * KMAX] (the norm of the
// result without another pass over it).
template <typename T>
__global__ void __launch_bounds__(256, 4) k_multiaxpy(T* __restrict__ w, double beta, const T* const* __restrict__ V,
                                                      const double* __restrict__ coef, double scale, int k, int64_t n,
                                                      double* __restrict__ part) {
    using VT = Vec16<T>;
    using V4 = typename VT::V;
    constexpr int W = VT::W;
    __shared__ T c[KMAX];
    __shared__ const V4* vp[KMAX];
    for (int i = threadIdx.x; i < k; i += blockDim.x) {
        c[i] = (T)(coef[i] * scale);
        vp[i] = reinterpret_cast<const V4*>(V[i]);
    }
    __syncthreads();
    const T bt = (T)beta;
    V4* w4 = reinterpret_cast<V4*>(w);
    const int64_t n4 = n / W;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    Acc<T> nrm;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n4; q += stride) {
        Acc<T> a[W];
        if (beta != 0.0) {
            const V4 x = w4[q];
#pragma unroll
            for (int e = 0; e < W; e++) a[e].add(bt, VT::get(x, e));
        }
#pragma unroll 4
        for (int i = 0; i < k; i++) {
            const V4 v = vp[i][q];
            const T ci = c[i];
#pragma unroll
            for (int e = 0; e < W; e++) a[e].add(ci, VT::get(v, e));
        }
        V4 o;
#pragma unroll
        for (int e = 0; e < W; e++) {
            const T r = a[e].value();
            VT::set(o, e, r);
            nrm.add(r, r);
        }
        w4[q] = o;
    }
    for (int64_t q = n4 * W + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += stride) {
        Acc<T> a;
        if (beta != 0.0) a.add(bt, w[q]);
        for (int i = 0; i < k; i++) a.add(c[i], V[i][q]);
        const T r = a.value();
        w[q] = r;
        nrm.add(r, r);
    }
    if (part) block_sum_to(nrm.dvalue(), part, 0);
}

template <typename T>
cudaError_t launch_multiaxpy(T* w, double beta, const T* const* V, const double* coef, double scale, int k, int64_t n,
                             cudaStream_t s) {
    if (k < 0 || k > KMAX) return cudaErrorInvalidValue;
    k_multiaxpy<T><<<multidot_blocks(), 256, 0, s>>>(w, beta, V, coef, scale, k, n, nullptr);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_multiaxpy_norm(T* w, double beta, const T* const* V, const double* coef, double scale, int k,
                                  int64_t n, double* part, double* norm2, cudaStream_t s) {
    if (k < 0 || k > KMAX) return cudaErrorInvalidValue;
    const int nb = multidot_blocks();
    k_multiaxpy<T><<<nb, 256, 0, s>>>(w, beta, V, coef, scale, k, n, part);
    k_multidot_final<<<1, 256, 0, s>>>(part, nb, 1, norm2);
    return cudaGetLastError();
}
template cudaError_t launch_multiaxpy<double>(double*, double, const double* const*, const double*, double, int,
                                              int64_t, cudaStream_t);
template cudaError_t launch_multiaxpy<float>(float*, double, const float* const*, const double*, double, int, int64_t,
                                             cudaStream_t);
template cudaError_t launch_multiaxpy_norm<double>(double*, double, const double* const*, const double*, double, int,
                                                   int64_t, double*, double*, cudaStream_t);
template cudaError_t launch_multiaxpy_norm<float>(float*, double, const float* const*, const double*, double, int,
                                                  int64_t, double*, double*, cudaStream_t);

// dst = a * src, 16-byte groups (both arrays are cudaMalloc bases)
template <typename T>
__global__ void __launch_bounds__(256) k_scale_copy(const T* __restrict__ src, T* __restrict__ dst, double a,
                                                    int64_t n) {
    using VT = Vec16<T>;
    using V4 = typename VT::V;
    constexpr int W = VT::W;
    const int64_t n4 = n / W;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const T at = (T)a;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n4; q += stride) {
        const V4 v = reinterpret_cast<const V4*>(src)[q];
        V4 o;
#pragma unroll
        for (int e = 0; e < W; e++) VT::set(o, e, at * VT::get(v, e));
        reinterpret_cast<V4*>(dst)[q] = o;
    }
    for (int64_t q = n4 * W + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += stride) dst[q] = at * src[q];
}
template <typename T>
cudaError_t launch_scale_copy(const T* src, T* dst, int64_t n, double a, cudaStream_t s) {
    k_scale_copy<T><<<flat_blocks(n), 256, 0, s>>>(src, dst, a, n);
    return cudaGetLastError();
}
template cudaError_t launch_scale_copy<double>(const double*, double*, int64_t, double, cudaStream_t);
template cudaError_t launch_scale_copy<float>(const float*, float*, int64_t, double, cudaStream_t);

// out(double) = scale * in(double or float) added with weight: y += a * x (mixed types)
template <typename TI>
__global__ void k_axpy_to_double(const TI* __restrict__ x, double* __restrict__ y, double a, int64_t n) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        y[q] += a * (double)x[q];
}
template <typename TI>
cudaError_t launch_axpy_to_double(const TI* x, double* y, int64_t n, double a, cudaStream_t s) {
    k_axpy_to_double<TI><<<flat_blocks(n), 256, 0, s>>>(x, y, a, n);
    return cudaGetLastError();
}
template cudaError_t launch_axpy_to_double<double>(const double*, double*, int64_t, double, cudaStream_t);
template cudaError_t launch_axpy_to_double<float>(const float*, double*, int64_t, double, cudaStream_t);

// out(T) = scale * in(double)
template <typename TO>
__global__ void k_from_double(const double* __restrict__ in, TO* __restrict__ out, double a, int64_t n) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        out[q] = (TO)(a * in[q]);
}
template <typename TO>
cudaError_t launch_from_double(const double* in, TO* out, int64_t n, double a, cudaStream_t s) {
    k_from_double<TO><<<flat_blocks(n), 256, 0, s>>>(in, out, a, n);
    return cudaGetLastError();
}
template cudaError_t launch_from_double<double>(const double*, double*, int64_t, double, cudaStream_t);
template cudaError_t launch_from_double<float>(const double*, float*, int64_t, double, cudaStream_t);

}  // namespace agb

// The outer residual of the mixed-precision solve in double-float
// arithmetic (dfloat.cuh): r = b - A x with x, b and the stiffness held as
// hi + lo FP32 pairs, evaluated by the same stencil code as the FP64 kernels
// (operator.cuh instantiated on dfloat) on the FP32 pipe.  The FP64 residual
// of Operator<Grid::Node>::solutionResidual (src/Operator/Operator.cpp:
// 635-657) costs about 300 FP64 operations per major-minor node, and GB300
// issues FP64 at 1/64 of its FP32 rate, so the FP64 kernel is bound by the
// FP64 pipe at a few percent of the HBM bandwidth; the double-float kernel
// keeps about 48 significant bits (relative error near 1e-14 of the row's
// terms) at FP32 speed.  It writes the residual rounded to FP32 (the inner
// FP32 solve's input) and per-block partial norms (max |r|, sum r^2, in
// FP64), and the solution update x += a e is done in double-float too.
#include <cuda_runtime.h>

#include "agb_launch.h"
#include "dfloat.cuh"
#include "operator.cuh"

namespace agb {

namespace {

constexpr int DX = 32, DY = 4, DZ = 2;

inline dim3 dgrid(int nx, int ny, int nz) { return dim3((nx + DX - 1) / DX, (ny + DY - 1) / DY, (nz + DZ - 1) / DZ); }

// block (max, sum) of per-thread FP32 values: warp shuffles in FP32 (the
// FP64 pipe runs at 1/64 of the FP32 rate; a warp's 32 squares summed in
// FP32 keep the 2-norm to about 1e-7, and the max is exact), then the
// warps' results in FP64.  NaNs propagate.
__device__ __forceinline__ void blk_max_sum_f(float mx, float sm, double* out) {
    __shared__ double smx[32], ssm[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float y = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = (y > mx || y != y) ? y : mx;
        sm += __shfl_xor_sync(0xffffffffu, sm, o);
    }
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nthr = blockDim.x * blockDim.y * blockDim.z;
    const int w = tid >> 5, l = tid & 31, nw = (nthr + 31) >> 5;
    if (l == 0) { smx[w] = (double)mx; ssm[w] = (double)sm; }
    __syncthreads();
    if (tid == 0) {
        double m = 0.0, t = 0.0;
        for (int q = 0; q < nw; q++) {
            m = (smx[q] > m || smx[q] != smx[q]) ? smx[q] : m;
            t += ssm[q];
        }
        out[0] = m;
        out[1] = t;
    }
}

// WIDE: r is written in FP64 (hi + lo), else rounded to FP32
template <int SYM, bool WIDE>
__global__ void __launch_bounds__(256) k_residual_df(const dfloat* __restrict__ x, const dfloat* __restrict__ b,
                                                     const dfloat* __restrict__ C, LevelGeom<dfloat> G, BcTable bc,
                                                     float* __restrict__ r, double* __restrict__ r64,
                                                     double* __restrict__ partials) {
    const int i = blockIdx.x * DX + threadIdx.x;
    const int j = blockIdx.y * DY + threadIdx.y;
    const int k = blockIdx.z * DZ + threadIdx.z;
    const bool live = (i < G.nx) & (j < G.ny) & (k < G.nz);
    const int64_t id = i + G.sy * j + G.sz * k;
    float mx = 0.f, sm = 0.f;
    if (live) {
        dfloat ax[3];
        apply_node<dfloat, SYM, false>(x, C, G, bc, i, j, k, id, ax);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const int64_t q = c * G.N + id;
            const dfloat rv = b[q] - ax[c];
            const float rf = df_float(rv);
            if (WIDE) r64[q] = df_double(rv);
            else r[q] = rf;
            const float a = fabsf(rf);
            mx = (a > mx || a != a) ? a : mx;
            sm = __fmaf_rn(a, a, sm);
        }
    }
    const int blk = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    blk_max_sum_f(mx, sm, partials + 2 * blk);
}

__global__ void k_to_df(const double* __restrict__ src, dfloat* __restrict__ dst, int64_t n) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        dst[q] = dfloat(src[q]);
}

__global__ void k_df_to_double(const dfloat* __restrict__ src, double* __restrict__ dst, int64_t n) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        dst[q] = df_double(src[q]);
    }
}

// x += a e, e an FP32 correction, a a double-float scale
__global__ void k_df_axpy(const float* __restrict__ e, dfloat a, dfloat* __restrict__ x, int64_t n) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    {
        // stored normalised: the iterate is updated many times
        const dfloat v = x[q] + a * dfloat(e[q]);
        x[q] = df_fast_two_sum(v.hi, v.lo);
    }
}

__global__ void k_scale_f32(float* __restrict__ v, float a, int64_t n) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        v[q] *= a;
}

inline int flat(int64_t n) {
    int64_t b = (n + 255) / 256;
    return (int)(b < 152 * 16 ? (b < 1 ? 1 : b) : 152 * 16);
}

}  // namespace

static LevelGeom<dfloat> geom_df(const LevelGeom<double>& g) {
    LevelGeom<dfloat> d;
    d.nx = g.nx; d.ny = g.ny; d.nz = g.nz;
    d.N = g.N; d.sy = g.sy; d.sz = g.sz;
    for (int a = 0; a < 3; a++) {
        d.h[a] = dfloat(g.h[a]);
        d.inv[a] = dfloat(g.inv[a]);
        d.i2[a] = dfloat(g.i2[a]);
        d.q[a] = dfloat(g.q[a]);
    }
    d.psi = nullptr;
    d.psi_small = dfloat(0);
    d.psy = g.psy; d.psz = g.psz;
    return d;
}

cudaError_t launch_residual_df(int sym, const dfloat* x, const dfloat* b, const dfloat* C,
                               const LevelGeom<double>& G64, const BcTable& bc, float* r, double* r64,
                               double* partials, int* nblocks_out, cudaStream_t s) {
    const LevelGeom<dfloat> G = geom_df(G64);
    dim3 blk(DX, DY, DZ), grd = dgrid(G.nx, G.ny, G.nz);
    if (nblocks_out) *nblocks_out = (int)(grd.x * grd.y * grd.z);
    if (r64) {
        if (sym == SYM_ISO) k_residual_df<SYM_ISO, true><<<grd, blk, 0, s>>>(x, b, C, G, bc, r, r64, partials);
        else if (sym == SYM_MAJ) k_residual_df<SYM_MAJ, true><<<grd, blk, 0, s>>>(x, b, C, G, bc, r, r64, partials);
        else k_residual_df<SYM_MM, true><<<grd, blk, 0, s>>>(x, b, C, G, bc, r, r64, partials);
    } else {
        if (sym == SYM_ISO) k_residual_df<SYM_ISO, false><<<grd, blk, 0, s>>>(x, b, C, G, bc, r, r64, partials);
        else if (sym == SYM_MAJ) k_residual_df<SYM_MAJ, false><<<grd, blk, 0, s>>>(x, b, C, G, bc, r, r64, partials);
        else k_residual_df<SYM_MM, false><<<grd, blk, 0, s>>>(x, b, C, G, bc, r, r64, partials);
    }
    return cudaGetLastError();
}

int residual_df_blocks(int nx, int ny, int nz) {
    const dim3 g = dgrid(nx, ny, nz);
    return (int)(g.x * g.y * g.z);
}

cudaError_t launch_to_df(const double* src, dfloat* dst, int64_t n, cudaStream_t s) {
    k_to_df<<<flat(n), 256, 0, s>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_df_to_double(const dfloat* src, double* dst, int64_t n, cudaStream_t s) {
    k_df_to_double<<<flat(n), 256, 0, s>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_df_axpy(const float* e, double a, dfloat* x, int64_t n, cudaStream_t s) {
    k_df_axpy<<<flat(n), 256, 0, s>>>(e, dfloat(a), x, n);
    return cudaGetLastError();
}

cudaError_t launch_scale_f32(float* v, float a, int64_t n, cudaStream_t s) {
    k_scale_f32<<<flat(n), 256, 0, s>>>(v, a, n);
    return cudaGetLastError();
}

}  // namespace agb

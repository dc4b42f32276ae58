// Bottom solve of the V-cycle on the coarsest multigrid level, in ONE thread
// block so a V-cycle never waits on the host.
//
// The reference runs amrex::MLMG with the BiCGStab bottom solver
// (src/Solver/Nonlocal/Linear.H:258); MLCGSolver applies the operator's
// normalize() after every residual and operator application, which alamo
// defines as division by the diagonal (src/Operator/Operator.cpp:156-165), so
// BiCGStab runs on D^-1 A x = D^-1 b.  The iteration below is the published
// BiCGStab (van der Vorst 1992) with inf-norm stopping tests against the
// initial normalised residual.  When it breaks down, the correction is reset
// to zero and `final_smooth` Fsmooth calls follow; after a good solve,
// `bottom_smooth` calls follow (MLMG's bottom behaviour; AMReX is not part of
// the reference tree, so this restates its documented behaviour).
#include <cuda_runtime.h>
#include "agb_launch.h"
#include "operator.cuh"

namespace agb {

static constexpr int BOT_THREADS = 512;

__device__ __forceinline__ double blk_sum(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) r += sh[q];
    return r;
}
// max that keeps a NaN (fmax drops it): a NaN anywhere in the bottom
// iteration must reach the breakdown test
__device__ __forceinline__ double nan_max(double a, double b) { return a != a ? a : (b != b ? b : fmax(a, b)); }
__device__ __forceinline__ double blk_max(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = nan_max(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) r = nan_max(r, sh[q]);
    return r;
}

template <int SYM>
__device__ void bot_apply(const double* x, double* y, const double* C, const double* dg, const LevelGeom<double>& G,
                          const BcTable& bc) {
    __syncthreads();
    for (int64_t node = threadIdx.x; node < G.N; node += blockDim.x) {
        const int k = (int)(node / G.sz);
        const int64_t rem = node - (int64_t)k * G.sz;
        const int j = (int)(rem / G.nx);
        const int i = (int)(rem - (int64_t)j * G.nx);
        double f[3];
        apply_node<double, SYM>(x, C, G, bc, i, j, k, node, f);
        y[node] = f[0] / dg[node];
        y[G.N + node] = f[1] / dg[G.N + node];
        y[2 * G.N + node] = f[2] / dg[2 * G.N + node];
    }
    __syncthreads();
}

// ncalls Fsmooth calls (2 damped-Jacobi sweeps each) on x with rhs b
template <int SYM>
__device__ void bot_smooth(double* x, const double* b, double* tmp, const double* C, const double* dg,
                           const LevelGeom<double>& G, const BcTable& bc, int ncalls, double omega) {
    const int64_t n3 = 3 * G.N;
    for (int s = 0; s < 2 * ncalls; s++) {
        __syncthreads();
        for (int64_t node = threadIdx.x; node < G.N; node += blockDim.x) {
            const int k = (int)(node / G.sz);
            const int64_t rem = node - (int64_t)k * G.sz;
            const int j = (int)(rem / G.nx);
            const int i = (int)(rem - (int64_t)j * G.nx);
            double f[3];
            apply_node<double, SYM>(x, C, G, bc, i, j, k, node, f);
            for (int c = 0; c < 3; c++) {
                const int64_t q = c * G.N + node;
                const double rx = f[c] - x[q] * dg[q];
                tmp[q] = (1. - omega) * x[q] + omega * (b[q] - rx) / dg[q];
            }
        }
        __syncthreads();
        for (int64_t q = threadIdx.x; q < n3; q += blockDim.x) x[q] = tmp[q];
    }
    __syncthreads();
}

template <int SYM>
__global__ void __launch_bounds__(BOT_THREADS) k_bottom(const double* __restrict__ C, const double* __restrict__ dg,
                                                        LevelGeom<double> G, BcTable bc, const double* __restrict__ rhs,
                                                        double* __restrict__ sol, double* __restrict__ work,
                                                        int max_iter, double eps_rel, double eps_abs, int nsmooth_ok,
                                                        int nsmooth_fail, double omega, int* __restrict__ info) {
    __shared__ double sh[32];
    const int64_t n3 = 3 * G.N;
    double* r = work;
    double* rh = work + n3;
    double* p = work + 2 * n3;
    double* v = work + 3 * n3;
    double* s = work + 4 * n3;
    double* t = work + 5 * n3;
    double* so = work + 6 * n3;
    const int tid = threadIdx.x, nt = blockDim.x;

    // r = D^-1 (rhs - A sol); keep sol as sorig and restart from zero
    bot_apply<SYM>(sol, t, C, dg, G, bc);
    double lm = 0.0;
    for (int64_t q = tid; q < n3; q += nt) {
        const double rv = rhs[q] / dg[q] - t[q];
        r[q] = rv; rh[q] = rv; so[q] = sol[q]; sol[q] = 0.0; p[q] = 0.0; v[q] = 0.0;
        lm = nan_max(lm, fabs(rv));
    }
    const double rnorm0 = blk_max(lm, sh);
    double rnorm = rnorm0;
    int ret = 0, iter = 1;
    double rho_1 = 0.0, alpha = 0.0, omg = 0.0;
    if (rnorm0 == 0.0 || rnorm0 < eps_abs) {
        for (int64_t q = tid; q < n3; q += nt) sol[q] += so[q];
        if (tid == 0) { info[0] = 0; info[1] = 0; }
        return;
    }
    for (; iter <= max_iter; ++iter) {
        double ls = 0.0;
        for (int64_t q = tid; q < n3; q += nt) ls += rh[q] * r[q];
        const double rho = blk_sum(ls, sh);
        if (rho == 0.0) { ret = 1; break; }
        if (iter == 1) {
            for (int64_t q = tid; q < n3; q += nt) p[q] = r[q];
        } else {
            const double beta = (rho / rho_1) * (alpha / omg);
            for (int64_t q = tid; q < n3; q += nt) p[q] = r[q] + beta * (p[q] - omg * v[q]);
        }
        bot_apply<SYM>(p, v, C, dg, G, bc);
        ls = 0.0;
        for (int64_t q = tid; q < n3; q += nt) ls += rh[q] * v[q];
        const double rhTv = blk_sum(ls, sh);
        if (rhTv != 0.0) alpha = rho / rhTv;
        else { ret = 2; break; }
        lm = 0.0;
        for (int64_t q = tid; q < n3; q += nt) {
            sol[q] += alpha * p[q];
            const double sv = r[q] - alpha * v[q];
            s[q] = sv;
            lm = nan_max(lm, fabs(sv));
        }
        rnorm = blk_max(lm, sh);
        if (rnorm != rnorm) { ret = 5; break; }
        if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
        bot_apply<SYM>(s, t, C, dg, G, bc);
        double ltt = 0.0, lts = 0.0;
        for (int64_t q = tid; q < n3; q += nt) { ltt += t[q] * t[q]; lts += t[q] * s[q]; }
        const double tt = blk_sum(ltt, sh);
        const double ts = blk_sum(lts, sh);
        if (tt != 0.0) omg = ts / tt;
        else { ret = 3; break; }
        lm = 0.0;
        for (int64_t q = tid; q < n3; q += nt) {
            sol[q] += omg * s[q];
            const double rv = s[q] - omg * t[q];
            r[q] = rv;
            lm = nan_max(lm, fabs(rv));
        }
        rnorm = blk_max(lm, sh);
        if (rnorm != rnorm) { ret = 5; break; }
        if (rnorm < eps_rel * rnorm0 || rnorm < eps_abs) break;
        if (omg == 0.0) { ret = 4; break; }
        rho_1 = rho;
    }
    if (ret == 0 && rnorm > eps_rel * rnorm0 && rnorm > eps_abs) ret = 8;
    __syncthreads();
    if ((ret == 0 || ret == 8) && rnorm < rnorm0) {
        for (int64_t q = tid; q < n3; q += nt) sol[q] += so[q];
    } else {
        for (int64_t q = tid; q < n3; q += nt) sol[q] = so[q];
    }
    __syncthreads();
    if (ret != 0) {
        // failed bottom solve: zero correction, then final smoothing
        for (int64_t q = tid; q < n3; q += nt) sol[q] = 0.0;
        bot_smooth<SYM>(sol, rhs, t, C, dg, G, bc, nsmooth_fail, omega);
    } else if (nsmooth_ok > 0) {
        bot_smooth<SYM>(sol, rhs, t, C, dg, G, bc, nsmooth_ok, omega);
    }
    if (tid == 0) { info[0] = ret; info[1] = iter < max_iter ? iter : max_iter; }
}

cudaError_t launch_bottom_bicgstab_ex(int sym, const double* C, const double* diag, const LevelGeom<double>& G,
                                      const BcTable& bc, const double* rhs, double* sol, double* work, int max_iter,
                                      double tol_rel, double tol_abs, int nsmooth_ok, int nsmooth_fail, double omega,
                                      int* info, cudaStream_t s) {
    if (sym == SYM_ISO)
        k_bottom<SYM_ISO><<<1, BOT_THREADS, 0, s>>>(C, diag, G, bc, rhs, sol, work, max_iter, tol_rel, tol_abs,
                                                     nsmooth_ok, nsmooth_fail, omega, info);
    else if (sym == SYM_MAJ)
        k_bottom<SYM_MAJ><<<1, BOT_THREADS, 0, s>>>(C, diag, G, bc, rhs, sol, work, max_iter, tol_rel, tol_abs,
                                                     nsmooth_ok, nsmooth_fail, omega, info);
    else
        k_bottom<SYM_MM><<<1, BOT_THREADS, 0, s>>>(C, diag, G, bc, rhs, sol, work, max_iter, tol_rel, tol_abs,
                                                    nsmooth_ok, nsmooth_fail, omega, info);
    return cudaGetLastError();
}

cudaError_t launch_bottom_bicgstab(int sym, const double* C, const double* diag, const LevelGeom<double>& G,
                                   const BcTable& bc, const double* rhs, double* sol, double* work, int max_iter,
                                   double tol_rel, double tol_abs, int* info, cudaStream_t s) {
    return launch_bottom_bicgstab_ex(sym, C, diag, G, bc, rhs, sol, work, max_iter, tol_rel, tol_abs, 0, 8, 2. / 3.,
                                     info, s);
}

}  // namespace agb

namespace agb {

// ---------------------------------------------------------------------------
// Direct bottom solve: the coarsest level's operator is assembled as a dense
// matrix (column j = A e_j, probing the same per-node arithmetic as Fapply),
// inverted once per prepareForSolve by Gauss-Jordan elimination with partial
// pivoting, and every bottom solve is then one dense matrix-vector product.
// ---------------------------------------------------------------------------

// Acol[j * nb + i] = (A e_j)_i ; E is nb*nb scratch holding the unit vectors
template <int SYM>
__global__ void __launch_bounds__(256) k_assemble(const double* __restrict__ C, LevelGeom<double> G, BcTable bc,
                                                  double* __restrict__ E, double* __restrict__ Acol, int nb) {
    const int j = blockIdx.y;
    double* u = E + (int64_t)j * nb;
    // every block builds its own unit vector, then applies the operator
    for (int q = threadIdx.x; q < nb; q += blockDim.x) u[q] = (q == j) ? 1.0 : 0.0;
    __syncthreads();
    for (int64_t node = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; node < G.N;
         node += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(node / G.sz);
        const int64_t rem = node - (int64_t)k * G.sz;
        const int jj = (int)(rem / G.nx);
        const int i = (int)(rem - (int64_t)jj * G.nx);
        double f[3];
        apply_node<double, SYM>(u, C, G, bc, i, jj, k, node, f);
        for (int c = 0; c < 3; c++) Acol[(int64_t)j * nb + c * G.N + node] = f[c];
    }
}

// W = [A | I], row-major nb x 2nb, from the column-major probe result
__global__ void k_gj_init(const double* __restrict__ Acol, double* __restrict__ W, int nb, int* __restrict__ used) {
    const int64_t tot = (int64_t)nb * 2 * nb;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < tot; q += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(q / (2 * nb)), c = (int)(q - (int64_t)r * 2 * nb);
        W[q] = (c < nb) ? Acol[(int64_t)c * nb + r] : ((c - nb) == r ? 1.0 : 0.0);
    }
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nb; r += gridDim.x * blockDim.x) used[r] = 0;
}

// Grid-wide barrier of the cooperative Gauss-Jordan kernel (all blocks are
// co-resident under cudaLaunchCooperativeKernel).  bar[0] counts arrivals,
// bar[1] is the generation.  The wait is bounded: past the limit the block
// records flag = 2 and every block leaves the elimination loop.
__device__ __forceinline__ bool gj_grid_barrier(unsigned* bar, unsigned nblocks, int* stop_sh, int* flag) {
    __syncthreads();
    if (threadIdx.x == 0 && !*stop_sh) {
        __threadfence();
        const unsigned gen = atomicAdd(&bar[1], 0u);
        const unsigned arrived = atomicAdd(&bar[0], 1u);
        if (arrived == nblocks - 1) {
            atomicExch(&bar[0], 0u);
            __threadfence();
            atomicAdd(&bar[1], 1u);
        } else {
            unsigned it = 0;
            while (atomicAdd(&bar[1], 0u) == gen) {
                if (++it > (1u << 22)) {
                    atomicExch(flag, 2);
                    *stop_sh = 1;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *stop_sh == 0;
}

// Gauss-Jordan elimination with partial pivoting on W = [A | I] (row-major
// nb x 2nb) in one cooperative launch: per column k every block finds the
// same pivot (same data, same reduction order, own copy of the used-row
// flags), eliminates column k from its rows (rows r = blockIdx.x mod
// gridDim.x) with the unscaled pivot row, and meets the others at a grid
// barrier.  Pivot rows are never scaled during the loop (no block writes the
// row every block reads); the extraction divides by the pivots.  Global
// reads of W go through L2 (ld.global.cg): other blocks wrote them.
__global__ void __launch_bounds__(256) k_gj_coop(double* __restrict__ W, int nb, int* __restrict__ perm,
                                                 int* __restrict__ flag, const double* __restrict__ tiny_p,
                                                 unsigned* __restrict__ bar) {
    extern __shared__ unsigned char used_sh[];
    __shared__ double bv[8];
    __shared__ int bi[8];
    __shared__ int p_sh, stop_sh;
    __shared__ double piv_sh;
    const double tiny = tiny_p[0];
    const int64_t ld = 2 * (int64_t)nb;
    for (int r = threadIdx.x; r < nb; r += blockDim.x) used_sh[r] = 0;
    if (threadIdx.x == 0) stop_sh = 0;
    __syncthreads();
    for (int k = 0; k < nb; k++) {
        double best = -1.0;
        int bidx = -1;
        for (int r = threadIdx.x; r < nb; r += blockDim.x) {
            if (used_sh[r]) continue;
            const double a = fabs(__ldcg(W + r * ld + k));
            if (a > best) { best = a; bidx = r; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
            if (ob > best || (ob == best && oi >= 0 && (bidx < 0 || oi < bidx))) { best = ob; bidx = oi; }
        }
        if ((threadIdx.x & 31) == 0) { bv[threadIdx.x >> 5] = best; bi[threadIdx.x >> 5] = bidx; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double b = -1.0;
            int p = -1;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++)
                if (bv[w] > b || (bv[w] == b && bi[w] >= 0 && (p < 0 || bi[w] < p))) { b = bv[w]; p = bi[w]; }
            if (p < 0 || !(b > tiny)) {
                if (blockIdx.x == 0) atomicExch(flag, 1);
                p = (p < 0) ? 0 : p;
            }
            used_sh[p] = 1;
            if (blockIdx.x == 0) perm[k] = p;
            p_sh = p;
            piv_sh = __ldcg(W + p * ld + k);
        }
        __syncthreads();
        const int p = p_sh;
        const double inv = (piv_sh != 0.0) ? 1.0 / piv_sh : 0.0;
        const double* prow = W + p * ld;
        for (int r = blockIdx.x; r < nb; r += gridDim.x) {
            if (r == p) continue;
            double* row = W + r * ld;
            const double f = __ldcg(row + k);
            if (f == 0.0) continue;
            for (int64_t c = k + 1 + threadIdx.x; c < ld; c += blockDim.x) row[c] -= f * (__ldcg(prow + c) * inv);
        }
        // column k of the eliminated rows is zero; written once every thread
        // of the block has read its multiplier f from it
        __syncthreads();
        for (int r = blockIdx.x + gridDim.x * threadIdx.x; r < nb; r += gridDim.x * blockDim.x)
            if (r != p) W[r * ld + k] = 0.0;
        if (!gj_grid_barrier(bar, gridDim.x, &stop_sh, flag)) break;
    }
}

// Ainv[k][j] = W[perm[k]][nb + j] / W[perm[k]][k] (the pivot rows were left
// unscaled by the elimination)
__global__ void k_gj_extract(const double* __restrict__ W, const int* __restrict__ perm, double* __restrict__ Ainv,
                             int nb) {
    const int64_t tot = (int64_t)nb * nb;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < tot; q += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(q / nb), j = (int)(q - (int64_t)k * nb);
        const double* row = W + (int64_t)perm[k] * 2 * nb;
        Ainv[q] = row[nb + j] / row[k];
    }
}

// tiny[0] = rel * max |diag|: the pivot threshold
__global__ void __launch_bounds__(1024) k_pivot_threshold(const double* __restrict__ diag, int nb, double rel,
                                                          double* __restrict__ tiny) {
    __shared__ double sh[32];
    double m = 0.0;
    for (int r = threadIdx.x; r < nb; r += blockDim.x) m = fmax(m, fabs(diag[r]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t = fmax(t, sh[w]);
        tiny[0] = rel * t;
    }
}

cudaError_t build_dense_inverse(int sym, const double* C, const double* diag, const LevelGeom<double>& G,
                                const BcTable& bc, double* Ainv, double* work, int* iwork, int* flag, double* tiny,
                                cudaStream_t s) {
    const int nb = (int)(3 * G.N);
    double* E = work;                          // nb*nb
    double* Acol = work + (int64_t)nb * nb;    // nb*nb
    double* W = work + 2 * (int64_t)nb * nb;   // 2*nb*nb
    int* used = iwork;
    int* perm = iwork + nb;
    unsigned* bar = reinterpret_cast<unsigned*>(work + 4 * (int64_t)nb * nb);  // 2 counters
    dim3 grd((unsigned)((G.N + 255) / 256), (unsigned)nb);
    if (sym == SYM_ISO) k_assemble<SYM_ISO><<<grd, 256, 0, s>>>(C, G, bc, E, Acol, nb);
    else if (sym == SYM_MAJ) k_assemble<SYM_MAJ><<<grd, 256, 0, s>>>(C, G, bc, E, Acol, nb);
    else k_assemble<SYM_MM><<<grd, 256, 0, s>>>(C, G, bc, E, Acol, nb);
    k_gj_init<<<152 * 4, 256, 0, s>>>(Acol, W, nb, used);
    k_pivot_threshold<<<1, 1024, 0, s>>>(diag, nb, 1e-12, tiny);
    cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    // co-resident blocks for the grid barrier: at most one per SM, at most 64
    int dev = 0, sms = 0, per_sm = 0, coop = 0;
    const size_t smem = (size_t)nb;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gj_coop, 256, smem)) != cudaSuccess) return e;
    if (!coop || per_sm < 1) return cudaErrorNotSupported;
    int blocks = sms < 64 ? sms : 64;
    if (blocks > nb) blocks = nb;
    void* args[] = {&W, (void*)&nb, &perm, &flag, &tiny, &bar};
    e = cudaLaunchCooperativeKernel((const void*)k_gj_coop, dim3(blocks), dim3(256), args, smem, s);
    if (e != cudaSuccess) return e;
    k_gj_extract<<<152 * 4, 256, 0, s>>>(W, perm, Ainv, nb);
    return cudaGetLastError();
}

// sol = Ainv * rhs, one warp per row
__global__ void __launch_bounds__(256) k_dense_matvec(const double* __restrict__ Ainv, const double* __restrict__ b,
                                                      double* __restrict__ x, int nb) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= nb) return;
    const double* row = Ainv + (int64_t)warp * nb;
    double acc = 0.0;
    for (int j = lane; j < nb; j += 32) acc += row[j] * b[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) x[warp] = acc;
}

cudaError_t launch_dense_bottom(const double* Ainv, const double* rhs, double* sol, int nb, cudaStream_t s) {
    k_dense_matvec<<<(nb * 32 + 255) / 256, 256, 0, s>>>(Ainv, rhs, sol, nb);
    return cudaGetLastError();
}

}  // namespace agb

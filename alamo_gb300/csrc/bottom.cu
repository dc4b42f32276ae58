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
__device__ __forceinline__ double blk_max(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) r = fmax(r, sh[q]);
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
        lm = fmax(lm, fabs(rv));
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
            lm = fmax(lm, fabs(sv));
        }
        rnorm = blk_max(lm, sh);
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
            lm = fmax(lm, fabs(rv));
        }
        rnorm = blk_max(lm, sh);
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

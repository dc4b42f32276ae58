// z-marching stencil kernels for the fine multigrid level.
//
// A 32 x 8 thread block owns 32 x 8 node columns and walks them through a
// chunk of z-planes.  The displacement planes k-1, k, k+1 (3 components, with
// a one-node x/y halo) live in a 4-slot shared-memory ring; plane k+2 is
// loaded into registers at the top of step k and stored into the free slot
// after the step's arithmetic, so its latency hides behind the compute.  The
// stiffness of the thread's own column is kept in registers for planes k-1,
// k, k+1 (the z-derivative of C comes from registers; plane k+1 is loaded at
// the top of step k and consumed last); its x/y neighbours for the in-plane derivatives of C are read
// through L1, where the neighbouring threads' loads of the same step put
// them.  Every array is therefore read from HBM about once per sweep.
//
// Epilogues (fused, the operator result never goes to memory):
//   FAPPLY    out = A x
//   JACOBI    out = (1-w) x + w (b - (A x - diag x)) / diag   (one Fsmooth sweep)
//   RESIDUAL  out = b - A x
// Boundary nodes (BC rows) take the general per-node path with global reads.
#include <cuda_runtime.h>

#include "agb_launch.h"
#include "operator.cuh"

namespace agb {

static constexpr int ZX = 32, ZY = 8, ZS = 4;
static constexpr int HX = ZX + 2, HY = ZY + 2;
static constexpr int PLANE = 3 * HY * HX;                     // values per staged plane
static constexpr int PER_T = (PLANE + ZX * ZY - 1) / (ZX * ZY);  // loads per thread per plane

template <int SYM>
struct NCof {
    enum { v = SYM == SYM_ISO ? 2 : 21 };
};

template <typename T, int SYM, int MODE>
__global__ void __launch_bounds__(ZX * ZY, 2)
    k_zmarch(const T* __restrict__ x, const T* __restrict__ C, LevelGeom<T> G, BcTable bc, const T* __restrict__ b,
             const T* __restrict__ dg, T omega, T* __restrict__ out, int kchunk) {
    constexpr int NC = NCof<SYM>::v;
    __shared__ T su[ZS][3][HY][HX];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * ZX + tx;
    const int x0 = blockIdx.x * ZX, y0 = blockIdx.y * ZY;
    const int i = x0 + tx, j = y0 + ty;
    const int k0 = blockIdx.z * kchunk;
    const int k1 = min(k0 + kchunk, G.nz);
    const bool col = (i < G.nx) & (j < G.ny);
    const int64_t N = G.N, sy = G.sy, sz = G.sz;

    // global index and in-range flag of this thread's share of a staged plane
    int soff[PER_T];
    int64_t goff[PER_T];
    bool gval[PER_T];
#pragma unroll
    for (int r = 0; r < PER_T; r++) {
        const int q = tid + r * ZX * ZY;
        const int p = q / (HY * HX), rem = q - p * (HY * HX), yy = rem / HX, xx = rem - yy * HX;
        const int gx = x0 - 1 + xx, gy = y0 - 1 + yy;
        soff[r] = q;
        gval[r] = (q < PLANE) & (gx >= 0) & (gx < G.nx) & (gy >= 0) & (gy < G.ny);
        goff[r] = p * N + gx + sy * gy;
    }
    auto fetch = [&](int kk, T v[PER_T]) {
        const bool kin = (kk >= 0) & (kk < G.nz);
#pragma unroll
        for (int r = 0; r < PER_T; r++) v[r] = (kin && gval[r]) ? x[goff[r] + sz * (int64_t)kk] : T(0);
    };
    auto stash = [&](int kk, const T v[PER_T]) {
        T* dst = &su[(kk + ZS) % ZS][0][0][0];
#pragma unroll
        for (int r = 0; r < PER_T; r++)
            if (soff[r] < PLANE) dst[soff[r]] = v[r];
    };
    auto cload = [&](int kk, T c[NC]) {
        const bool ok = col & (kk >= 0) & (kk < G.nz);
        const int64_t id = i + sy * j + sz * (int64_t)kk;
#pragma unroll
        for (int e = 0; e < NC; e++) c[e] = ok ? C[e * N + id] : T(0);
    };

    {
        T v[PER_T];
        fetch(k0 - 1, v); stash(k0 - 1, v);
        fetch(k0, v); stash(k0, v);
        fetch(k0 + 1, v); stash(k0 + 1, v);
    }
    T Cp[NC], Cc[NC], Cn[NC];
    cload(k0 - 1, Cp);
    cload(k0, Cc);
    __syncthreads();

    for (int k = k0; k < k1; k++) {
        T pre[PER_T];
        fetch(k + 2, pre);
        // stiffness of plane k+1: needed last (z-derivative of C), so its
        // latency overlaps the Hessian and x/y terms
        cload(k + 1, Cn);
        if (col) {
            const int64_t id = i + sy * j + sz * (int64_t)k;
            const bool bnd = (i == 0) | (j == 0) | (k == 0) | (i == G.nx - 1) | (j == G.ny - 1) | (k == G.nz - 1);
            T r[3];
            if (bnd) {
                auto cf = [&](int a) { return C[a * N + id]; };
                apply_boundary<T, SYM>(x, G, bc, cf, i, j, k, id, r);
            } else {
                const int s0 = k % ZS, sm = (k + ZS - 1) % ZS, sp = (k + 1) % ZS;
                auto U = [&](int p, int a, int bb, int c) {
                    const int sl = c == 0 ? s0 : (c < 0 ? sm : sp);
                    return su[sl][p][ty + 1 + bb][tx + 1 + a];
                };
                auto Cf = [&](int e, int a, int bb, int c) -> T {
                    if (c > 0) return Cn[e];
                    if (c < 0) return Cp[e];
                    if (a == 0 && bb == 0) return Cc[e];
                    return C[e * N + id + a + sy * bb];
                };
                interior_rows<T, SYM>(U, Cf, G, r);
            }
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const int64_t q = c * N + id;
                if (MODE == 0) {
                    out[q] = r[c];
                } else if (MODE == 1) {
                    const T xv = su[k % ZS][c][ty + 1][tx + 1];
                    const T d = dg[q];
                    const T rx = r[c] - xv * d;
                    out[q] = (T(1) - omega) * xv + omega * (b[q] - rx) / d;
                } else {
                    out[q] = b[q] - r[c];
                }
            }
        }
        stash(k + 2, pre);
#pragma unroll
        for (int e = 0; e < NC; e++) { Cp[e] = Cc[e]; Cc[e] = Cn[e]; }
        __syncthreads();
    }
}

static int zm_kchunk(int nz) { return nz >= 64 ? 32 : 16; }

template <typename T>
cudaError_t launch_zmarch(int mode, int sym, const T* x, const T* C, const LevelGeom<T>& G, const BcTable& bc,
                          const T* b, const T* dg, T omega, T* out, cudaStream_t s) {
    if (sym == SYM_MAJ) return cudaErrorInvalidValue;  // per-node kernels only
    const int kc = zm_kchunk(G.nz);
    dim3 blk(ZX, ZY, 1), grd((G.nx + ZX - 1) / ZX, (G.ny + ZY - 1) / ZY, (G.nz + kc - 1) / kc);
#define AGB_ZM_CASE(SY, MO) \
    k_zmarch<T, SY, MO><<<grd, blk, 0, s>>>(x, C, G, bc, b, dg, omega, out, kc)
    if (sym == SYM_ISO) {
        if (mode == 0) AGB_ZM_CASE(SYM_ISO, 0);
        else if (mode == 1) AGB_ZM_CASE(SYM_ISO, 1);
        else AGB_ZM_CASE(SYM_ISO, 2);
    } else {
        if (mode == 0) AGB_ZM_CASE(SYM_MM, 0);
        else if (mode == 1) AGB_ZM_CASE(SYM_MM, 1);
        else AGB_ZM_CASE(SYM_MM, 2);
    }
#undef AGB_ZM_CASE
    return cudaGetLastError();
}
template cudaError_t launch_zmarch<float>(int, int, const float*, const float*, const LevelGeom<float>&,
                                          const BcTable&, const float*, const float*, float, float*, cudaStream_t);
template cudaError_t launch_zmarch<double>(int, int, const double*, const double*, const LevelGeom<double>&,
                                           const BcTable&, const double*, const double*, double, double*,
                                           cudaStream_t);

}  // namespace agb

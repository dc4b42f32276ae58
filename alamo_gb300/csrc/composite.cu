// Field transfers of the multi-level (AMR) composite solve between one AMR
// level and the next finer one (refinement ratio 2, one box per level).
// Node arrays are SoA per component, x fastest.  A fine level's array is its
// box of valid nodes plus one ring of ghost nodes; "off" is the level index
// of an array's node 0.
//   * interp:   fine (all nodes, or the ghost ring only) = / += trilinear
//               nodal interpolation of the coarse field (the ghost fill of
//               the ghost-node coarse/fine strategy and the interpolated
//               coarse correction);
//   * restrict: coarse nodes covered by the fine box = nodal full weighting
//               (27 points, 1/8 .. 1/64) of the fine field, for residuals
//               (Operator<Grid::Node>::reflux, src/Operator/Operator.cpp:
//               526-633) and stiffness entries (Elastic::
//               averageDownCoeffsDifferentAmrLevels, src/Operator/
//               Elastic.cpp:628-742); the fine box lies inside the domain,
//               so the reference's domain-boundary weights never apply;
//   * inject:   coarse nodes covered by the fine box = the coincident fine
//               nodes (average down of the solution);
//   * masked max: max |v| over the nodes of a level that carry rows of the
//               composite system (neither ghost nor covered).
#include <cuda_runtime.h>

#include <cstdint>

#include "composite.h"

namespace agb {

namespace {

struct Box3 {
    int n[3];    // array nodes per axis
    int off[3];  // level index of array node 0
};

__device__ __forceinline__ void interp_axis(int p, int& j0, int& j1, double& w0, double& w1) {
    if ((p & 1) == 0) {
        j0 = j1 = p >> 1;
        w0 = 1.0;
        w1 = 0.0;
    } else {
        j0 = (p - 1) >> 1;
        j1 = j0 + 1;
        w0 = w1 = 0.5;
    }
}

// mode 0: fine = I(crse); 1: fine += I(crse); 2: fine ring = I(crse)
__global__ void k_interp(const double* __restrict__ c, Box3 cb, double* __restrict__ f, Box3 fb, int ncomp,
                         int mode) {
    const int64_t nf = (int64_t)fb.n[0] * fb.n[1] * fb.n[2];
    const int64_t nc = (int64_t)cb.n[0] * cb.n[1] * cb.n[2];
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nf; q += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(q % fb.n[0]);
        const int j = (int)((q / fb.n[0]) % fb.n[1]);
        const int k = (int)(q / ((int64_t)fb.n[0] * fb.n[1]));
        const bool ring = i == 0 || j == 0 || k == 0 || i == fb.n[0] - 1 || j == fb.n[1] - 1 || k == fb.n[2] - 1;
        if (mode == 2 && !ring) continue;
        int x0, x1, y0, y1, z0, z1;
        double wx0, wx1, wy0, wy1, wz0, wz1;
        interp_axis(i + fb.off[0], x0, x1, wx0, wx1);
        interp_axis(j + fb.off[1], y0, y1, wy0, wy1);
        interp_axis(k + fb.off[2], z0, z1, wz0, wz1);
        x0 -= cb.off[0]; x1 -= cb.off[0];
        y0 -= cb.off[1]; y1 -= cb.off[1];
        z0 -= cb.off[2]; z1 -= cb.off[2];
        const int64_t sy = cb.n[0], sz = (int64_t)cb.n[0] * cb.n[1];
        for (int comp = 0; comp < ncomp; comp++) {
            const double* cc = c + comp * nc;
            const double v = wz0 * (wy0 * (wx0 * cc[x0 + sy * y0 + sz * z0] + wx1 * cc[x1 + sy * y0 + sz * z0]) +
                                    wy1 * (wx0 * cc[x0 + sy * y1 + sz * z0] + wx1 * cc[x1 + sy * y1 + sz * z0])) +
                             wz1 * (wy0 * (wx0 * cc[x0 + sy * y0 + sz * z1] + wx1 * cc[x1 + sy * y0 + sz * z1]) +
                                    wy1 * (wx0 * cc[x0 + sy * y1 + sz * z1] + wx1 * cc[x1 + sy * y1 + sz * z1]));
            double* ff = f + comp * nf + q;
            if (mode == 1) *ff += v;
            else *ff = v;
        }
    }
}

// coarse node (covered block index a, b, c) <-> fine array node 2 (a, b, c) + 1
__global__ void k_restrict_box(const double* __restrict__ f, Box3 fb, int64_t fcs, int64_t fes,
                               double* __restrict__ c, Box3 cb, int64_t ccs, int64_t ces, const int* c0, const int* cn,
                               int ncomp, int inject) {
    const int64_t ncov = (int64_t)cn[0] * cn[1] * cn[2];
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < ncov; q += (int64_t)gridDim.x * blockDim.x) {
        const int a = (int)(q % cn[0]);
        const int b = (int)((q / cn[0]) % cn[1]);
        const int cc = (int)(q / ((int64_t)cn[0] * cn[1]));
        const int64_t fsy = fb.n[0], fsz = (int64_t)fb.n[0] * fb.n[1];
        const int64_t fid = (2 * a + 1) + fsy * (2 * b + 1) + fsz * (2 * cc + 1);
        const int64_t cid = (c0[0] + a) + (int64_t)cb.n[0] * (c0[1] + b) + (int64_t)cb.n[0] * cb.n[1] * (c0[2] + cc);
        for (int comp = 0; comp < ncomp; comp++) {
            const double* ff = f + comp * fcs;
            double v;
            if (inject) {
                v = ff[fid * fes];
            } else {
                v = 0.0;
                for (int dz = -1; dz <= 1; dz++)
                    for (int dy = -1; dy <= 1; dy++)
                        for (int dx = -1; dx <= 1; dx++) {
                            const double w = (dx == 0 ? 0.5 : 0.25) * (dy == 0 ? 0.5 : 0.25) * (dz == 0 ? 0.5 : 0.25);
                            v += w * ff[(fid + dx + fsy * dy + fsz * dz) * fes];
                        }
            }
            c[comp * ccs + cid * ces] = v;
        }
    }
}

__global__ void k_zero_ring(double* __restrict__ v, Box3 b, int ncomp) {
    const int64_t n = (int64_t)b.n[0] * b.n[1] * b.n[2];
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(q % b.n[0]);
        const int j = (int)((q / b.n[0]) % b.n[1]);
        const int k = (int)(q / ((int64_t)b.n[0] * b.n[1]));
        if (i == 0 || j == 0 || k == 0 || i == b.n[0] - 1 || j == b.n[1] - 1 || k == b.n[2] - 1)
            for (int comp = 0; comp < ncomp; comp++) v[comp * n + q] = 0.0;
    }
}

// max |v| over the rows of the composite system; a non-negative double's
// bit pattern orders like the value, so the block maxima combine with an
// integer atomicMax (a NaN's pattern exceeds every finite one)
__global__ void k_masked_max(const double* __restrict__ v, Box3 b, int ring, const int* c0, const int* cn, int ncomp,
                             unsigned long long* out) {
    const int64_t n = (int64_t)b.n[0] * b.n[1] * b.n[2];
    double mx = 0.0;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(q % b.n[0]);
        const int j = (int)((q / b.n[0]) % b.n[1]);
        const int k = (int)(q / ((int64_t)b.n[0] * b.n[1]));
        if (ring && (i == 0 || j == 0 || k == 0 || i == b.n[0] - 1 || j == b.n[1] - 1 || k == b.n[2] - 1)) continue;
        if (cn && i >= c0[0] && i < c0[0] + cn[0] && j >= c0[1] && j < c0[1] + cn[1] && k >= c0[2] &&
            k < c0[2] + cn[2])
            continue;
        for (int comp = 0; comp < ncomp; comp++) {
            const double a = fabs(v[comp * n + q]);
            mx = (a > mx || a != a) ? a : mx;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double y = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = (y > mx || y != y) ? y : mx;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(mx));
}

inline int blocks_for(int64_t n) {
    int64_t b = (n + 255) / 256;
    return (int)(b < 1 ? 1 : (b > 152 * 8 ? 152 * 8 : b));
}

Box3 box3(const int n[3], const int off[3]) {
    Box3 b;
    for (int a = 0; a < 3; a++) { b.n[a] = n[a]; b.off[a] = off[a]; }
    return b;
}

}  // namespace

cudaError_t launch_interp(const double* c, const int cn[3], const int coff[3], double* f, const int fn[3],
                          const int foff[3], int ncomp, int mode, cudaStream_t s) {
    const int64_t nf = (int64_t)fn[0] * fn[1] * fn[2];
    k_interp<<<blocks_for(nf), 256, 0, s>>>(c, box3(cn, coff), f, box3(fn, foff), ncomp, mode);
    return cudaGetLastError();
}

cudaError_t launch_restrict_box(const double* f, const int fn[3], int64_t fcs, int64_t fes, double* c, const int cn[3],
                                int64_t ccs, int64_t ces, const int* c0_dev, const int* cnt_dev, int64_t ncov,
                                int ncomp, int inject, cudaStream_t s) {
    const int zero[3] = {0, 0, 0};
    k_restrict_box<<<blocks_for(ncov), 256, 0, s>>>(f, box3(fn, zero), fcs, fes, c, box3(cn, zero), ccs, ces, c0_dev,
                                                     cnt_dev, ncomp, inject);
    return cudaGetLastError();
}

cudaError_t launch_zero_ring(double* v, const int n[3], int ncomp, cudaStream_t s) {
    const int zero[3] = {0, 0, 0};
    k_zero_ring<<<blocks_for((int64_t)n[0] * n[1] * n[2]), 256, 0, s>>>(v, box3(n, zero), ncomp);
    return cudaGetLastError();
}

cudaError_t launch_masked_max(const double* v, const int n[3], int ring, const int* c0_dev, const int* cnt_dev,
                              int ncomp, unsigned long long* out, cudaStream_t s) {
    const int zero[3] = {0, 0, 0};
    k_masked_max<<<blocks_for((int64_t)n[0] * n[1] * n[2]), 256, 0, s>>>(v, box3(n, zero), ring, c0_dev, cnt_dev,
                                                                         ncomp, out);
    return cudaGetLastError();
}

}  // namespace agb

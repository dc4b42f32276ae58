// Multi-level (AMR) composite solve: the MLMG iteration over AMR levels
// that Solver::Nonlocal::Linear drives for an AMR hierarchy
// (src/Solver/Nonlocal/Linear.H:131-168), with alamo's operator hooks for
// it: reflux (src/Operator/Operator.cpp:526-633), fixUpResidualMask
// (:230-251) and averageDownCoeffsDifferentAmrLevels
// (src/Operator/Elastic.cpp:628-742).
//
// Level 0 covers the domain with the caller's boundary conditions; level
// l >= 1 is one box of valid nodes lo .. lo + nv - 1 in level-l node indices
// (refinement ratio 2; lo even and nv odd, so the box faces lie on coarse
// nodes; the box and its ghost ring strictly inside level l-1's valid
// nodes).  A fine level's arrays hold the box plus one ring of ghost nodes;
// each level is an agb_elastic handle over its array, the fine ones with
// displacement rows on the ring (so the ring rows hold the ghost values and
// every valid node, the box faces included, carries the interior row: the
// ghost-node coarse/fine strategy).  Per iteration (correction form, as
// MLMG::oneIter): average down the solution (covered coarse nodes take the
// coincident fine values), fill the ghosts from the next coarser level
// (trilinear nodal interpolation), the composite residual (under a finer
// box: the finer residual restricted by full weighting), its norm over the
// rows of the composite system; down the levels a correction from each fine
// level's residual (its own V-cycles, ghost values zero) and the reflux of
// what it leaves; the coarse correction on level 0; up the levels the
// coarser correction interpolated (ghosts included) and a correction of the
// remaining residual; the solution update.  Everything stays on the device
// and goes through the level handles' C ABI and the transfer kernels of
// composite.cu.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/agb.h"
#include "agb_launch.h"
#include "composite.h"

namespace agb {
void set_last_error(const char* msg);
}

struct agb_composite {
    int nlev = 0;
    int sym = 0;
    int nc = 0;
    agb_solver_opts opts{};
    struct Level {
        agb_elastic* h = nullptr;
        int n[3] = {0, 0, 0};    // array nodes per axis
        int off[3] = {0, 0, 0};  // level index of array node 0
        int lo[3] = {0, 0, 0}, nv[3] = {0, 0, 0};
        double dx[3] = {0, 0, 0};
        int64_t N = 0;
        double *u = nullptr, *rhs = nullptr, *r = nullptr, *c = nullptr, *t = nullptr, *t2 = nullptr;
        double* C = nullptr;  // AoS stiffness as given (per node nc doubles)
        double* Cavg = nullptr;  // with the finer levels' stiffness averaged down
        bool model = false;
        // coarse nodes covered by the next finer box: block start and counts
        int* cov_dev = nullptr;  // c0[3], cnt[3]
        int c0[3] = {0, 0, 0}, cnt[3] = {0, 0, 0};
        int64_t ncov = 0;
    };
    std::vector<Level> L;
    unsigned long long* maxbits = nullptr;
    cudaStream_t stream = nullptr;
};

namespace {

using Comp = agb_composite;

agb_status cfail(agb_status st, const std::string& msg) {
    agb::set_last_error(msg.c_str());
    return st;
}

#define CCK(x)                                                                                   \
    do {                                                                                         \
        cudaError_t e_ = (x);                                                                    \
        if (e_ != cudaSuccess) return cfail(AGB_CUDA_ERROR, std::string(#x ": ") + cudaGetErrorString(e_)); \
    } while (0)
#define CTRY(x)                       \
    do {                              \
        agb_status s_ = (x);          \
        if (s_ != AGB_OK) return s_;  \
    } while (0)

double max_norm(Comp* c, const double* v, const int n[3], int ring, const int* cov, int ncomp) {
    cudaMemsetAsync(c->maxbits, 0, sizeof(unsigned long long), c->stream);
    agb::launch_masked_max(v, n, ring, cov, cov ? cov + 3 : nullptr, ncomp, c->maxbits, c->stream);
    unsigned long long bits = 0;
    cudaMemcpyAsync(&bits, c->maxbits, sizeof(bits), cudaMemcpyDeviceToHost, c->stream);
    cudaStreamSynchronize(c->stream);
    double d;
    std::memcpy(&d, &bits, sizeof(d));
    return d;
}

// r = rhs - A u on level l (the level handle's FP64 residual), ring rows 0
agb_status level_residual(Comp* c, int l, const double* u, const double* rhs, double* r) {
    Comp::Level& v = c->L[l];
    CTRY(agb_elastic_residual(v.h, 0, u, rhs, r, nullptr, AGB_MEM_DEVICE));
    if (l > 0) CCK(agb::launch_zero_ring(r, v.n, 3, c->stream));
    return AGB_OK;
}

// covered nodes of level l = full weighting (or injection) of level l+1's field
agb_status restrict_down(Comp* c, int l, const double* fine, double* crse, int inject) {
    Comp::Level& v = c->L[l];
    Comp::Level& f = c->L[l + 1];
    CCK(agb::launch_restrict_box(fine, f.n, f.N, 1, crse, v.n, v.N, 1, v.cov_dev, v.cov_dev + 3, v.ncov, 3, inject,
                                 c->stream));
    return AGB_OK;
}

// `cycles` V-cycles of level l's own hierarchy on A e = r from e = 0
agb_status level_vcycles(Comp* c, int l, const double* r, double* e, int cycles) {
    Comp::Level& v = c->L[l];
    const size_t bytes = sizeof(double) * 3 * v.N;
    CTRY(agb_elastic_vcycle(v.h, r, e, c->opts.precision, AGB_MEM_DEVICE));
    for (int k = 1; k < cycles; k++) {
        CTRY(agb_elastic_residual(v.h, 0, e, r, v.t2, nullptr, AGB_MEM_DEVICE));
        if (l > 0) CCK(agb::launch_zero_ring(v.t2, v.n, 3, c->stream));
        CTRY(agb_elastic_vcycle(v.h, v.t2, v.t, c->opts.precision, AGB_MEM_DEVICE));
        CCK(agb::launch_axpy(1.0, v.t, e, 3 * v.N, c->stream));
    }
    (void)bytes;
    return AGB_OK;
}

}  // namespace

extern "C" {

agb_status agb_composite_create(agb_composite** out, int nlev, const int n0[3], const double dx0[3], int sym,
                                const int* lo, const int* nv, const agb_solver_opts* opts) {
    if (!out || nlev < 1 || nlev > 16 || !n0 || !dx0 || (nlev > 1 && (!lo || !nv)))
        return cfail(AGB_BAD_ARG, "agb_composite_create: bad argument");
    if (sym != AGB_SYM_ISOTROPIC && sym != AGB_SYM_MAJORMINOR)
        return cfail(AGB_BAD_ARG, "agb_composite_create: isotropic or major-minor stiffness only");
    Comp* c = new Comp();
    auto bail = [&](agb_status st) { agb_composite_destroy(c); return st; };
    c->nlev = nlev;
    c->sym = sym;
    c->nc = sym == AGB_SYM_ISOTROPIC ? 2 : 21;
    if (opts) c->opts = *opts;
    else agb_default_opts(&c->opts);
    c->L.resize(nlev);
    for (int l = 0; l < nlev; l++) {
        Comp::Level& v = c->L[l];
        for (int a = 0; a < 3; a++) {
            v.dx[a] = dx0[a] / (double)(1 << l);
            if (l == 0) {
                v.n[a] = n0[a];
                v.off[a] = 0;
                v.lo[a] = 0;
                v.nv[a] = n0[a];
            } else {
                v.lo[a] = lo[3 * l + a];
                v.nv[a] = nv[3 * l + a];
                v.n[a] = v.nv[a] + 2;
                v.off[a] = v.lo[a] - 1;
                if (v.lo[a] % 2 != 0 || v.nv[a] % 2 != 1 || v.nv[a] < 3)
                    return bail(cfail(AGB_BAD_ARG, "agb_composite_create: a box needs an even lo and an odd nv >= 3"));
                // the box and its ghost ring inside the coarser level's valid
                // nodes: the ghost interpolation reads valid coarse nodes only
                const Comp::Level& p = c->L[l - 1];
                const int g0 = v.lo[a] - 1, g1 = v.lo[a] + v.nv[a];  // ghost nodes (level l)
                if ((g0 - 1) / 2 < p.lo[a] || (g1 + 1) / 2 > p.lo[a] + p.nv[a] - 1)
                    return bail(cfail(AGB_BAD_ARG,
                                      "agb_composite_create: a box and its ghost ring must lie inside the coarser "
                                      "level's valid nodes"));
            }
        }
        v.N = (int64_t)v.n[0] * v.n[1] * v.n[2];
        agb_status st = agb_elastic_create(&v.h, v.n[0], v.n[1], v.n[2], v.dx, sym, &c->opts);
        if (st != AGB_OK) return bail(st);
        if (l > 0) {
            // ghost ring rows: displacement rows holding the ghost values
            int t[78];
            double val[78];
            for (int q = 0; q < 78; q++) { t[q] = AGB_BC_DISPLACEMENT; val[q] = 0.0; }
            st = agb_elastic_set_bc(v.h, t, val);
            if (st != AGB_OK) return bail(st);
        }
        const size_t vb = sizeof(double) * 3 * v.N;
        if (cudaMalloc(&v.u, vb) != cudaSuccess || cudaMalloc(&v.rhs, vb) != cudaSuccess ||
            cudaMalloc(&v.r, vb) != cudaSuccess || cudaMalloc(&v.c, vb) != cudaSuccess ||
            cudaMalloc(&v.t, vb) != cudaSuccess || cudaMalloc(&v.t2, vb) != cudaSuccess ||
            cudaMalloc(&v.C, sizeof(double) * c->nc * v.N) != cudaSuccess ||
            cudaMalloc(&v.Cavg, sizeof(double) * c->nc * v.N) != cudaSuccess ||
            cudaMalloc(&v.cov_dev, 6 * sizeof(int)) != cudaSuccess)
            return bail(cfail(AGB_OUT_OF_MEMORY, "agb_composite_create: allocation failed"));
    }
    for (int l = 0; l + 1 < nlev; l++) {
        Comp::Level& v = c->L[l];
        const Comp::Level& f = c->L[l + 1];
        v.ncov = 1;
        for (int a = 0; a < 3; a++) {
            v.c0[a] = f.lo[a] / 2 - v.off[a];
            v.cnt[a] = (f.nv[a] - 1) / 2 + 1;
            v.ncov *= v.cnt[a];
        }
        int h6[6] = {v.c0[0], v.c0[1], v.c0[2], v.cnt[0], v.cnt[1], v.cnt[2]};
        if (cudaMemcpy(v.cov_dev, h6, sizeof(h6), cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(cfail(AGB_CUDA_ERROR, "agb_composite_create: copy failed"));
    }
    if (cudaMalloc(&c->maxbits, sizeof(unsigned long long)) != cudaSuccess)
        return bail(cfail(AGB_OUT_OF_MEMORY, "agb_composite_create: allocation failed"));
    // one stream for every level handle and the transfer kernels: their
    // launches stay in order without further synchronisation
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(cfail(AGB_CUDA_ERROR, "agb_composite_create: cudaStreamCreate failed"));
    for (auto& v : c->L) {
        const agb_status st = agb_elastic_set_stream(v.h, c->stream);
        if (st != AGB_OK) return bail(st);
    }
    *out = c;
    return AGB_OK;
}

agb_status agb_composite_destroy(agb_composite* c) {
    if (!c) return AGB_OK;
    cudaDeviceSynchronize();
    for (auto& v : c->L) {
        if (v.h) agb_elastic_destroy(v.h);
        cudaFree(v.u); cudaFree(v.rhs); cudaFree(v.r); cudaFree(v.c); cudaFree(v.t); cudaFree(v.t2);
        cudaFree(v.C); cudaFree(v.Cavg); cudaFree(v.cov_dev);
    }
    cudaFree(c->maxbits);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return AGB_OK;
}

agb_status agb_composite_level_dims(agb_composite* c, int level, int dims[3]) {
    if (!c || !dims || level < 0 || level >= c->nlev) return cfail(AGB_BAD_ARG, "bad argument");
    for (int a = 0; a < 3; a++) dims[a] = c->L[level].n[a];
    return AGB_OK;
}

agb_status agb_composite_set_bc(agb_composite* c, const int* type, const double* val) {
    if (!c) return cfail(AGB_BAD_ARG, "null handle");
    return agb_elastic_set_bc(c->L[0].h, type, val);
}

agb_status agb_composite_set_model(agb_composite* c, int level, const double* C, int where) {
    if (!c || !C || level < 0 || level >= c->nlev) return cfail(AGB_BAD_ARG, "bad argument");
    Comp::Level& v = c->L[level];
    const size_t bytes = sizeof(double) * c->nc * v.N;
    CCK(cudaMemcpyAsync(v.C, C, bytes, where == AGB_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                        c->stream));
    CCK(cudaStreamSynchronize(c->stream));
    v.model = true;
    return AGB_OK;
}

agb_status agb_composite_solve(agb_composite* c, double* const* u, const double* const* F0, int f0_ncomp,
                               double tol_rel, double tol_abs, int* iters, double* relnorm, int where) {
    if (!c || !u) return cfail(AGB_BAD_ARG, "null argument");
    const int nl = c->nlev;
    for (int l = 0; l < nl; l++)
        if (!c->L[l].model) return cfail(AGB_NOT_READY, "agb_composite_solve: a level has no model");
    cudaStream_t s = c->stream;
    // right-hand sides from each level's own model at u = 0 (the reference
    // builds them per level before MLMG averages the coefficients down)
    for (int l = 0; l < nl; l++) {
        Comp::Level& v = c->L[l];
        CTRY(agb_elastic_set_model(v.h, v.C, AGB_MEM_DEVICE));
        CCK(cudaMemsetAsync(v.u, 0, sizeof(double) * 3 * v.N, s));
        CTRY(agb_elastic_bc_init(v.h, v.t, 0, AGB_MEM_DEVICE));
        const double* f0 = nullptr;
        double* f0dev = nullptr;
        if (F0 && F0[l] && f0_ncomp > 0) {
            const size_t fb = sizeof(double) * f0_ncomp * v.N;
            if (where == AGB_MEM_HOST) {
                CCK(cudaMalloc(&f0dev, fb));
                CCK(cudaMemcpyAsync(f0dev, F0[l], fb, cudaMemcpyHostToDevice, s));
                f0 = f0dev;
            } else {
                f0 = F0[l];
            }
        }
        const agb_status st = agb_elastic_build_rhs(v.h, v.u, v.t, f0, f0 ? f0_ncomp : 0, v.rhs, AGB_MEM_DEVICE);
        cudaFree(f0dev);
        if (st != AGB_OK) return st;
    }
    // the stiffness under finer boxes: the finer stiffness restricted
    // (finest first, so each level passes down what it received)
    for (int l = nl - 1; l >= 0; l--) {
        Comp::Level& v = c->L[l];
        CCK(cudaMemcpyAsync(v.Cavg, v.C, sizeof(double) * c->nc * v.N, cudaMemcpyDeviceToDevice, s));
        if (l + 1 < nl) {
            Comp::Level& f = c->L[l + 1];
            CCK(agb::launch_restrict_box(f.Cavg, f.n, 1, c->nc, v.Cavg, v.n, 1, c->nc, v.cov_dev, v.cov_dev + 3,
                                         v.ncov, c->nc, 0, s));
        }
        CTRY(agb_elastic_set_model(v.h, v.Cavg, AGB_MEM_DEVICE));
    }
    // norm of the composite right-hand side
    double bn = 0.0;
    for (int l = 0; l < nl; l++) {
        Comp::Level& v = c->L[l];
        bn = std::fmax(bn, max_norm(c, v.rhs, v.n, l > 0, l + 1 < nl ? v.cov_dev : nullptr, 3));
    }
    const double target = std::fmax(tol_abs, tol_rel * bn);
    const int maxit = c->opts.max_iter > 0 ? c->opts.max_iter : 200;
    const int fine_cycles = 1, coarse_cycles = 1;
    int it = 0;
    double rn = 0.0;
    agb_status status = AGB_NOT_CONVERGED;
    for (;; it++) {
        // covered coarse values from the finer levels, ghosts from the coarser
        for (int l = nl - 1; l >= 1; l--) CTRY(restrict_down(c, l - 1, c->L[l].u, c->L[l - 1].u, 1));
        for (int l = 1; l < nl; l++) {
            Comp::Level& v = c->L[l];
            Comp::Level& p = c->L[l - 1];
            CCK(agb::launch_interp(p.u, p.n, p.off, v.u, v.n, v.off, 3, 2, s));
            CCK(agb::launch_interp(p.u, p.n, p.off, v.rhs, v.n, v.off, 3, 2, s));
        }
        // composite residual, finest first (covered nodes: reflux)
        rn = 0.0;
        for (int l = nl - 1; l >= 0; l--) {
            Comp::Level& v = c->L[l];
            CTRY(level_residual(c, l, v.u, v.rhs, v.r));
            rn = std::fmax(rn, max_norm(c, v.r, v.n, l > 0, l + 1 < nl ? v.cov_dev : nullptr, 3));
            if (l + 1 < nl) CTRY(restrict_down(c, l, c->L[l + 1].r, v.r, 0));
        }
        if (c->opts.verbose > 0) std::fprintf(stderr, "agb composite: iteration %d |r|/|b| = %.6e\n", it, rn / bn);
        if (std::isnan(rn)) { status = AGB_NAN; break; }
        if (rn <= target) { status = AGB_OK; break; }
        if (it >= maxit) break;
        // down the levels
        for (int l = nl - 1; l >= 1; l--) {
            Comp::Level& v = c->L[l];
            CTRY(level_vcycles(c, l, v.r, v.c, fine_cycles));
            CTRY(level_residual(c, l, v.c, v.r, v.t2));
            CTRY(restrict_down(c, l - 1, v.t2, c->L[l - 1].r, 0));
        }
        CTRY(level_vcycles(c, 0, c->L[0].r, c->L[0].c, coarse_cycles));
        // up the levels
        for (int l = 1; l < nl; l++) {
            Comp::Level& v = c->L[l];
            Comp::Level& p = c->L[l - 1];
            CCK(agb::launch_interp(p.c, p.n, p.off, v.c, v.n, v.off, 3, 1, s));
            CTRY(level_residual(c, l, v.c, v.r, v.t2));
            CTRY(level_vcycles(c, l, v.t2, v.t, fine_cycles));
            CCK(agb::launch_axpy(1.0, v.t, v.c, 3 * v.N, s));
        }
        for (int l = 0; l < nl; l++) {
            Comp::Level& v = c->L[l];
            CCK(agb::launch_axpy(1.0, v.c, v.u, 3 * v.N, s));
        }
    }
    // results
    for (int l = 0; l < nl; l++) {
        Comp::Level& v = c->L[l];
        if (!u[l]) continue;
        CCK(cudaMemcpyAsync(u[l], v.u, sizeof(double) * 3 * v.N,
                            where == AGB_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s));
    }
    CCK(cudaStreamSynchronize(s));
    if (iters) *iters = it;
    if (relnorm) *relnorm = bn > 0 ? rn / bn : rn;
    if (status == AGB_NOT_CONVERGED)
        agb::set_last_error("agb_composite_solve: the composite iteration did not reach the tolerance");
    if (status == AGB_NAN) agb::set_last_error("agb_composite_solve: NaN in the composite residual");
    return status;
}

}  // extern "C"

// Host driver of alamo_gb300: the C ABI of include/agb.h, the multigrid
// hierarchy, the multigrid cycles and the solves.
//
// Mapping to the reference (Gopal-B/alamo):
//   agb_elastic            Operator::Elastic<SYM> + Solver::Nonlocal::Linear
//                          (one AMR level, every multigrid level on one GPU)
//   prepare()              Operator<Grid::Node>::prepareForSolve
//                          (src/Operator/Operator.cpp:253-260)
//   vcycle<T>()            the MLMG V-cycle that calls the operator's hooks
//                          (Fsmooth, correctionResidual, restriction,
//                          interpolation, bottom BiCGStab)
//   fcycle64()             the MLMG F-cycle (max_fmg_iter iterations; the
//                          reference sets 100000000, Linear.H:261)
//   solve_fp64 / mixed     Linear::solve (src/Solver/Nonlocal/Linear.H:131)
//   agb_newton_solve       Newton::solve, nriters = 1
//                          (src/Solver/Nonlocal/Newton.H:279-358)
// Nothing here falls back to the CPU: every array operation is a CUDA kernel.
#include "../../include/agb.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "agb_launch.h"
#include "zmarch_tma.h"
#include "unet_net.h"

using namespace agb;

namespace {

thread_local std::string g_last_error;

agb_status fail(agb_status st, const std::string& msg) {
    g_last_error = msg;
    return st;
}

#define CK(call)                                                                                         \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess) {                                                                         \
            return fail(e_ == cudaErrorMemoryAllocation ? AGB_OUT_OF_MEMORY : AGB_CUDA_ERROR,            \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                             \
        }                                                                                                \
    } while (0)

#define TRY(call)                        \
    do {                                 \
        agb_status s_ = (call);          \
        if (s_ != AGB_OK) return s_;     \
    } while (0)

template <typename T>
struct Lev {
    LevelGeom<T> G;
    T* C = nullptr;       // SoA stiffness (nc * N)
    T* diag = nullptr;    // 3N
    T* res = nullptr;     // right-hand side of the level's correction equation
    T* cor = nullptr;     // correction
    T* rescor = nullptr;  // res - A cor
    T* tmp = nullptr;     // Jacobi ping-pong buffer
    // FP32 levels swept by the TMA stencil kernels: stiffness with the x
    // pitch padded to 4 values and its tensor map
    T* Cpad = nullptr;
    CUtensorMap map{};
    bool tma = false;
    // psi of this level (ghosted, LevelGeom::psi layout), owned; the FP64
    // fine level uses the handle's psi_fine instead
    T* psi = nullptr;
    // 1 / diag of FP32 levels swept by the TMA kernels (their Jacobi form)
    T* dinv = nullptr;
    // the F-cycle's interpolated start correction, kept while the V-cycle
    // from this level runs (allocated by the first F-cycle)
    T* hold = nullptr;
};

// Krylov space of the flexible GMRES: Arnoldi basis V (m+1 vectors), the
// preconditioned directions Z (m vectors), work vector w and correction e,
// all fine-level sized, plus device pointer tables for the fused kernels.
template <typename T>
struct Krylov {
    int m = 0;
    int64_t n = 0;
    std::vector<T*> V, Z;
    T** Vdev = nullptr;
    T** Zdev = nullptr;
    T** Wdev = nullptr;  // {w}
    T* w = nullptr;
    T* e = nullptr;
    double* part = nullptr;
    double* dots = nullptr;  // 3 * 40 device doubles
    double* hdots = nullptr; // pinned host mirror
    void release() {
        for (T* p : V) cudaFree(p);
        for (T* p : Z) cudaFree(p);
        V.clear(); Z.clear();
        cudaFree(Vdev); cudaFree(Zdev); cudaFree(Wdev); cudaFree(w); cudaFree(e); cudaFree(part); cudaFree(dots);
        if (hdots) cudaFreeHost(hdots);
        Vdev = Zdev = Wdev = nullptr; w = e = nullptr; part = dots = hdots = nullptr;
        m = 0; n = 0;
    }
};

}  // namespace

struct agb_elastic {
    int sym = 0, nc = 2;
    int n[3] = {0, 0, 0};
    double dx[3] = {1, 1, 1};
    agb_solver_opts opts{};
    BcTable bc{};
    double bcval[78] = {0};
    bool model_set = false, bc_set = true, prepared = false, have_f32 = false;
    int device = 0;
    std::vector<Lev<double>> L64;
    std::vector<Lev<float>> L32;
    std::vector<double> ldx;  // cell sizes per level (3 each)
    cudaStream_t stream = nullptr, own_stream = nullptr;
    double* partials = nullptr;
    int partials_cap = 0;
    double* norms_dev = nullptr;
    double* norms_host = nullptr;  // pinned
    double* bottom_work = nullptr;
    int* bottom_info = nullptr;
    double* bcval_dev = nullptr;
    // staging buffers for host-pointer calls and scratch (allocated on demand)
    double* io[4] = {nullptr, nullptr, nullptr, nullptr};
    size_t io_cap[4] = {0, 0, 0, 0};
    double* dw = nullptr;  // 9N scratch of the Newton RHS
    // psi (Elastic::SetPsi): ghosted fine-level field, m_psi_small
    double* psi_fine = nullptr;
    double psi_small = 1e-8;
    bool psi_set = false;
    // NeoHookean model (mu, kappa) SoA of the finite-deformation Newton path
    double* nh_model = nullptr;
    // double-float outer residual of the mixed solve (opts.outer_residual):
    // the fine stiffness, solution and right-hand side as hi + lo FP32 pairs
    dfloat* df_C = nullptr;
    dfloat* df_x = nullptr;
    dfloat* df_b = nullptr;
    bool have_df = false;
    Krylov<double> K64;
    Krylov<float> K32;
    // dense direct bottom solve
    double* bot_inv = nullptr;
    // which coarsest operator the inverse was built from: 0 none (stale),
    // 64 the FP64 hierarchy, 32 the FP32 hierarchy widened to FP64
    int bot_src = 0;
    int bot_nb = 0;
    bool bot_dense = false;
    // buffers of its build (assembly + one cooperative Gauss-Jordan launch)
    double* bot_work = nullptr;  // 4 nb^2 + 2 nb + 1 (threshold)
    int* bot_iwork = nullptr;    // 2 nb + 1 (flag)
    // profiling
    bool prof = false;
    int64_t prof_count[AGB_K_NFAMILIES] = {0};
    double prof_ms[AGB_K_NFAMILIES] = {0};
    double prof_bytes[AGB_K_NFAMILIES] = {0};  // algorithmic bytes of the timed launches
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
    size_t ev_used = 0;
    int64_t launches = 0;
};

namespace {

int64_t nodes(const agb_elastic* h) { return (int64_t)h->n[0] * h->n[1] * h->n[2]; }

agb_status ensure_io(agb_elastic* h, int slot, size_t bytes) {
    if (h->io_cap[slot] >= bytes) return AGB_OK;
    if (h->io[slot]) cudaFree(h->io[slot]);
    h->io[slot] = nullptr;
    h->io_cap[slot] = 0;
    CK(cudaMalloc(&h->io[slot], bytes));
    h->io_cap[slot] = bytes;
    return AGB_OK;
}

// ---------------------------------------------------------------- profiling
struct ProfScope {
    agb_elastic* h;
    int fam;
    cudaEvent_t a = nullptr, b = nullptr;
    ProfScope(agb_elastic* hh, int f, bool on, double bytes = 0.0) : h(hh), fam(f) {
        if (!on || !h->prof) { h = nullptr; return; }
        h->prof_bytes[f] += bytes;
        if (h->ev_used + 2 > h->ev_pool.size()) {
            for (int q = 0; q < 64; q++) {
                cudaEvent_t e;
                cudaEventCreate(&e);
                h->ev_pool.push_back(e);
            }
        }
        a = h->ev_pool[h->ev_used++];
        b = h->ev_pool[h->ev_used++];
        cudaEventRecord(a, h->stream);
    }
    ~ProfScope() {
        if (!h) return;
        cudaEventRecord(b, h->stream);
        h->ev_pending.push_back({fam, {a, b}});
    }
};

void prof_collect(agb_elastic* h) {
    if (h->ev_pending.empty()) return;
    cudaStreamSynchronize(h->stream);
    for (auto& p : h->ev_pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.second.first, p.second.second) == cudaSuccess) {
            h->prof_count[p.first] += 1;
            h->prof_ms[p.first] += ms;
        }
    }
    h->ev_pending.clear();
    h->ev_used = 0;
}

// ---------------------------------------------------------------- buffers
template <typename T>
void free_levels(std::vector<Lev<T>>& L) {
    for (auto& l : L) {
        cudaFree(l.C); cudaFree(l.diag); cudaFree(l.res); cudaFree(l.cor); cudaFree(l.rescor); cudaFree(l.tmp);
        cudaFree(l.Cpad);
        cudaFree(l.psi);
        cudaFree(l.dinv);
        cudaFree(l.hold);
    }
    L.clear();
}

int num_levels(const int n0[3], int max_coarsening_level) {
    int n[3] = {n0[0], n0[1], n0[2]};
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

agb_status alloc_levels64(agb_elastic* h) {
    free_levels(h->L64);
    const int nl = num_levels(h->n, h->opts.max_coarsening_level);
    h->ldx.assign(3 * nl, 0.0);
    int n[3] = {h->n[0], h->n[1], h->n[2]};
    double dx[3] = {h->dx[0], h->dx[1], h->dx[2]};
    h->L64.resize(nl);
    int maxblocks = 0;
    for (int l = 0; l < nl; l++) {
        Lev<double>& v = h->L64[l];
        v.G = make_geom<double>(n[0], n[1], n[2], dx);
        for (int d = 0; d < 3; d++) h->ldx[3 * l + d] = dx[d];
        const size_t N = (size_t)v.G.N;
        CK(cudaMalloc(&v.C, sizeof(double) * N * h->nc));
        CK(cudaMalloc(&v.diag, sizeof(double) * 3 * N));
        CK(cudaMalloc(&v.res, sizeof(double) * 3 * N));
        CK(cudaMalloc(&v.cor, sizeof(double) * 3 * N));
        CK(cudaMalloc(&v.rescor, sizeof(double) * 3 * N));
        CK(cudaMalloc(&v.tmp, sizeof(double) * 3 * N));
        maxblocks = std::max(maxblocks, residual_blocks(n[0], n[1], n[2]));
        for (int d = 0; d < 3; d++) { n[d] = (n[d] - 1) / 2 + 1; dx[d] *= 2; }
    }
    maxblocks = std::max(maxblocks, 152 * 16);
    if (h->partials_cap < maxblocks) {
        cudaFree(h->partials);
        h->partials = nullptr;
        CK(cudaMalloc(&h->partials, sizeof(double) * 2 * maxblocks));
        h->partials_cap = maxblocks;
    }
    if (h->psi_set) {
        h->L64[0].G.psi = h->psi_fine;
        h->L64[0].G.psi_small = h->psi_small;
    }
    const Lev<double>& b = h->L64.back();
    cudaFree(h->bottom_work);
    h->bottom_work = nullptr;
    CK(cudaMalloc(&h->bottom_work, sizeof(double) * 7 * 3 * (size_t)b.G.N));
    return AGB_OK;
}

agb_status alloc_levels32(agb_elastic* h) {
    free_levels(h->L32);
    const int nl = (int)h->L64.size();
    h->L32.resize(nl);
    for (int l = 0; l < nl; l++) {
        Lev<float>& v = h->L32[l];
        v.G = make_geom<float>(h->L64[l].G.nx, h->L64[l].G.ny, h->L64[l].G.nz, &h->ldx[3 * l]);
        const size_t N = (size_t)v.G.N;
        CK(cudaMalloc(&v.C, sizeof(float) * N * h->nc));
        CK(cudaMalloc(&v.diag, sizeof(float) * 3 * N));
        CK(cudaMalloc(&v.res, sizeof(float) * 3 * N));
        CK(cudaMalloc(&v.cor, sizeof(float) * 3 * N));
        CK(cudaMalloc(&v.rescor, sizeof(float) * 3 * N));
        CK(cudaMalloc(&v.tmp, sizeof(float) * 3 * N));
    }
    return AGB_OK;
}


// Explicit inverse of the coarsest level's operator for the direct bottom
// solve; falls back to BiCGStab (bot_dense = false) when it is too large or
// singular to working precision.

agb_status build_bottom_dense(agb_elastic* h) {
    Lev<double>& b = h->L64.back();
    const int nb = (int)(3 * b.G.N);
    if (nb > 4000) return AGB_OK;
    if (h->bot_nb != nb) {
        cudaFree(h->bot_inv);
        cudaFree(h->bot_work);
        cudaFree(h->bot_iwork);
        h->bot_inv = nullptr;
        h->bot_work = nullptr;
        h->bot_iwork = nullptr;
        h->bot_nb = 0;
        CK(cudaMalloc(&h->bot_inv, sizeof(double) * (size_t)nb * nb));
        CK(cudaMalloc(&h->bot_work, sizeof(double) * (4 * (size_t)nb * nb + 2 * (size_t)nb + 1)));
        CK(cudaMalloc(&h->bot_iwork, sizeof(int) * (2 * (size_t)nb + 1)));
        h->bot_nb = nb;
    }
    int* flag = h->bot_iwork + 2 * nb;
    double* tiny = h->bot_work + 4 * (size_t)nb * nb + 2 * (size_t)nb;
    CK(build_dense_inverse(h->sym, b.C, b.diag, b.G, h->bc, h->bot_inv, h->bot_work, h->bot_iwork, flag, tiny,
                           h->stream));
    h->launches += 5;
    int hflag = 0;
    CK(cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->bot_dense = (hflag == 0);
    return AGB_OK;
}

// ---------------------------------------------------------------- prepare
// levels at least this large (nodes) are swept by the TMA stencil kernels;
// on smaller ones the per-node kernels, one launch instead of two, are
// faster
static constexpr int64_t TMA_MIN_NODES = 30000;  // default of agb_solver_opts::tma_min_nodes

// FP32 copies of every level's stiffness and diagonal; for the levels the
// TMA stencil kernels sweep also the padded copy and its tensor map
// FP32 hierarchy.  With the FP64 hierarchy built (h->prepared) every level
// is its FP64 stiffness rounded; otherwise (the mixed-precision solve on its
// own) level 0 is rounded and the coarser levels are coarsened in FP32 --
// the preconditioner's coarse operators then differ from the FP64 ones by
// FP32 rounding, and the FP64 hierarchy, whose coarsening is FP64-pipe
// bound, is built only when an FP64 operation needs it.
agb_status build_f32(agb_elastic* h) {
    const int nl = (int)h->L64.size();
    if (h->L32.size() != h->L64.size()) TRY(alloc_levels32(h));
    for (int l = 0; l < nl; l++) {
        Lev<float>& v = h->L32[l];
        if (h->prepared || l == 0)
            CK(launch_to_float(h->L64[l].C, v.C, h->L64[l].G.N * h->nc, 1.0, h->stream));
        else
            CK(launch_restrict_C(h->L32[l - 1].C, h->L32[l - 1].G, v.C, v.G, h->nc, h->stream));
        h->launches++;
        if (h->psi_set) {
            const int64_t np = v.G.psz * (v.G.nz + 1);
            if (!v.psi) CK(cudaMalloc(&v.psi, sizeof(float) * np));
            CK(launch_to_float(h->L64[l].G.psi, v.psi, np, 1.0, h->stream));
            h->launches++;
            v.G.psi = v.psi;
            v.G.psi_small = (float)h->psi_small;
        } else {
            v.G.psi = nullptr;
        }
        CK(launch_diagonal<float>(h->sym, v.C, v.G, h->bc, v.diag, h->stream));
        h->launches++;
        const LevelGeom<float>& G = v.G;
        // the z-marching kernels carry no psi terms: psi runs on the per-node ones
        const int64_t min_nodes = h->opts.tma_min_nodes > 0 ? h->opts.tma_min_nodes : TMA_MIN_NODES;
        const bool want = h->opts.fine_kernel == 0 && !h->psi_set && h->sym != SYM_MAJ && G.N >= min_nodes &&
                          zmarch_tma_supported(G.nx, G.ny, G.nz);
        if (!want) {
            cudaFree(v.Cpad);
            v.Cpad = nullptr;
            v.tma = false;
            continue;
        }
        if (!v.Cpad) {
            const size_t bytes = sizeof(float) * h->nc * (size_t)G.nz * G.ny * zmarch_tma_pitch(G.nx);
            if (cudaMalloc(&v.Cpad, bytes) != cudaSuccess) {
                v.Cpad = nullptr;
                cudaGetLastError();
                return fail(AGB_OUT_OF_MEMORY, "allocation of the padded FP32 stiffness failed");
            }
            v.tma = false;
        }
        CK(launch_pad_stiffness(v.C, v.Cpad, G.nx, G.ny, G.nz, h->nc, h->stream));
        if (!v.dinv) CK(cudaMalloc(&v.dinv, sizeof(float) * 3 * G.N));
        CK(launch_recip(v.diag, v.dinv, 3 * G.N, h->stream));
        h->launches += 2;
        if (!v.tma) {
            CK(make_stiffness_map(v.Cpad, G.nx, G.ny, G.nz, h->nc, &v.map));
            v.tma = true;
        }
    }
    h->have_f32 = true;
    return AGB_OK;
}

// psi on every level (Elastic::averageDownCoeffsSameAmrLevel,
// src/Operator/Elastic.cpp:839-905), before the diagonals that use it
agb_status prepare_psi(agb_elastic* h) {
    const int nl = (int)h->L64.size();
    for (int l = 0; l < nl; l++) {
        Lev<double>& v = h->L64[l];
        if (!h->psi_set) {
            v.G.psi = nullptr;
            continue;
        }
        if (l == 0) {
            v.G.psi = h->psi_fine;
        } else {
            if (!v.psi) CK(cudaMalloc(&v.psi, sizeof(double) * v.G.psz * (v.G.nz + 1)));
            CK(launch_coarsen_psi(h->L64[l - 1].G.psi, h->L64[l - 1].G, v.psi, v.G, h->stream));
            h->launches++;
            v.G.psi = v.psi;
        }
        v.G.psi_small = h->psi_small;
    }
    return AGB_OK;
}

// Operator<Grid::Node>::prepareForSolve (src/Operator/Operator.cpp:253-260)
// in FP64: stiffness and psi on every level, every level's diagonal, and the
// direct bottom's inverse from the FP64 coarsest operator
agb_status prepare(agb_elastic* h) {
    if (h->prepared) return AGB_OK;
    if (!h->model_set) return fail(AGB_NOT_READY, "model not set (agb_elastic_set_model)");
    const int nl = (int)h->L64.size();
    for (int l = 1; l < nl; l++) {
        CK(launch_restrict_C(h->L64[l - 1].C, h->L64[l - 1].G, h->L64[l].C, h->L64[l].G, h->nc, h->stream));
        h->launches++;
    }
    TRY(prepare_psi(h));
    for (int l = 0; l < nl; l++) {
        CK(launch_diagonal<double>(h->sym, h->L64[l].C, h->L64[l].G, h->bc, h->L64[l].diag, h->stream));
        h->launches++;
    }
    if (h->opts.bottom_solver != AGB_BOTTOM_DIRECT) {
        h->bot_dense = false;
    } else if (h->bot_src != 64) {
        h->bot_dense = false;
        TRY(build_bottom_dense(h));
        h->bot_src = 64;
    }
    CK(cudaStreamSynchronize(h->stream));
    h->prepared = true;
    return AGB_OK;
}

// The FP32 hierarchy of the mixed-precision cycles.  Without the FP64
// hierarchy, the FP64 coarsest level (the bottom solve's, which stays FP64)
// is the FP32 one widened, with its FP64 diagonal.
agb_status ensure_f32(agb_elastic* h) {
    if (h->have_f32) return AGB_OK;
    if (!h->model_set) return fail(AGB_NOT_READY, "model not set (agb_elastic_set_model)");
    if (!h->prepared) TRY(prepare_psi(h));
    TRY(build_f32(h));
    if (!h->prepared) {
        Lev<double>& d = h->L64.back();
        const Lev<float>& f = h->L32.back();
        CK(cudaMemsetAsync(d.C, 0, sizeof(double) * d.G.N * h->nc, h->stream));
        CK(launch_add_float(f.C, d.C, d.G.N * h->nc, 1.0, h->stream));
        CK(launch_diagonal<double>(h->sym, d.C, d.G, h->bc, d.diag, h->stream));
        h->launches += 2;
        if (h->opts.bottom_solver != AGB_BOTTOM_DIRECT) {
            h->bot_dense = false;
        } else if (h->bot_src == 0) {
            h->bot_dense = false;
            TRY(build_bottom_dense(h));
            h->bot_src = 32;
        }
    }
    CK(cudaStreamSynchronize(h->stream));
    return AGB_OK;
}

// ---------------------------------------------------------------- cycle
template <typename T>
struct Fam;
template <>
struct Fam<double> { enum { J = AGB_K_JACOBI_F64, R = AGB_K_RESIDUAL_F64 }; };
template <>
struct Fam<float> { enum { J = AGB_K_JACOBI_F32, R = AGB_K_RESIDUAL_F32 }; };

// the z-marching kernels serve FP32 levels (FP64 stays on the per-node
// kernels: it is FP64-pipe bound): fine_kernel 0: the TMA-staged kernels on
// every level large enough (see build_f32); 1: none
template <typename T>
bool use_zm(const agb_elastic*, const Lev<T>&, int) { return false; }
template <>
bool use_zm<float>(const agb_elastic* h, const Lev<float>& v, int) {
    if (h->psi_set || h->sym == SYM_MAJ) return false;
    return h->opts.fine_kernel == 0 && v.tma;
}

// FP32 z-marching stencil on a level: mode 0 out = A x, 1 one Jacobi sweep,
// 2 residual
template <typename T>
cudaError_t level_zm(agb_elastic* h, const Lev<T>& v, int mode, const T* x, const T* b, const T* dg, T omega, T* out);
template <>
cudaError_t level_zm<float>(agb_elastic* h, const Lev<float>& v, int mode, const float* x, const float* b,
                            const float* dg, float omega, float* out) {
    // faces and interior on the library's stream: running the faces on a
    // second stream beside the interior sweep measured slower (the face
    // blocks take SM slots the marching blocks need)
    h->launches++;  // interior + faces
    // the TMA kernels' Jacobi form takes the inverse diagonal
    return launch_zmarch_tma(mode, h->sym, v.map, x, v.C, v.G, h->bc, b, mode == 1 ? v.dinv : dg, omega, out,
                             h->bottom_info + 3, h->stream, nullptr);
}
template <>
cudaError_t level_zm<double>(agb_elastic*, const Lev<double>&, int, const double*, const double*, const double*,
                             double, double*) {
    return cudaErrorNotSupported;  // never selected: use_zm<double> is false
}

// ncalls Fsmooth calls (2 sweeps each) on level l; cor_zero: cor is known 0
template <typename T>
agb_status smooth(agb_elastic* h, std::vector<Lev<T>>& L, int l, int ncalls, bool cor_zero,
                  bool first_done = false) {
    Lev<T>& v = L[l];
    const T w = (T)h->opts.omega;
    const int sweeps = 2 * ncalls;
    if (sweeps == 0 && cor_zero) {
        CK(cudaMemsetAsync(v.cor, 0, sizeof(T) * 3 * v.G.N, h->stream));
        return AGB_OK;
    }
    if (h->opts.smoother == AGB_SMOOTHER_GS) {
        // multicolour Gauss-Seidel: in place on cor, eight colours per sweep
        if (cor_zero) CK(cudaMemsetAsync(v.cor, 0, sizeof(T) * 3 * v.G.N, h->stream));
        for (int s = 0; s < sweeps; s++) {
            ProfScope ps(h, Fam<T>::J, l == 0);
            for (int c = 0; c < 8; c++)
                CK(launch_gs_colour<T>(h->sym, v.cor, v.res, v.diag, v.C, v.G, h->bc, w, c, h->stream));
            h->launches += 8;
        }
        return AGB_OK;
    }
    for (int s = 0; s < sweeps; s++) {
        if (s == 0 && cor_zero && first_done) {
            // the sweep from zero was written into tmp by the restriction
            std::swap(v.cor, v.tmp);
            continue;
        }
        {
            ProfScope ps(h, Fam<T>::J, l == 0 && !(cor_zero && s == 0));
            if (use_zm<T>(h, v, l) && !(cor_zero && s == 0))
                CK(level_zm<T>(h, v, 1, v.cor, v.res, v.diag, w, v.tmp));
            else
                CK(launch_jacobi<T>(h->sym, (cor_zero && s == 0) ? nullptr : v.cor, v.res, v.diag, v.C, v.G, h->bc,
                                    w, v.tmp, h->stream));
        }
        h->launches++;
        std::swap(v.cor, v.tmp);
    }
    return AGB_OK;
}

agb_status bottom64(agb_elastic* h, Lev<double>& b) {
    ProfScope ps(h, AGB_K_BOTTOM, true);
    if (h->opts.bottom_solver == AGB_BOTTOM_DIRECT && h->bot_dense) {
        CK(launch_dense_bottom(h->bot_inv, b.res, b.cor, h->bot_nb, h->stream));
        h->launches++;
        return AGB_OK;
    }
    CK(cudaMemsetAsync(b.cor, 0, sizeof(double) * 3 * b.G.N, h->stream));
    // the smoother as bottom solver: no BiCGStab iteration, straight to the
    // zeroed correction and final_smooth Fsmooth calls
    const int bmax = h->opts.bottom_solver == AGB_BOTTOM_SMOOTHER ? 0 : h->opts.bottom_max_iter;
    CK(launch_bottom_bicgstab_ex(h->sym, b.C, b.diag, b.G, h->bc, b.res, b.cor, h->bottom_work,
                                 bmax, h->opts.bottom_tol_rel, h->opts.bottom_tol_abs,
                                 h->opts.bottom_smooth, h->opts.final_smooth, h->opts.omega, h->bottom_info,
                                 h->stream));
    h->launches++;
    return AGB_OK;
}

template <typename T>
agb_status bottom(agb_elastic* h, std::vector<Lev<T>>& L);
template <>
agb_status bottom<double>(agb_elastic* h, std::vector<Lev<double>>& L) {
    return bottom64(h, L.back());
}
template <>
agb_status bottom<float>(agb_elastic* h, std::vector<Lev<float>>& L) {
    // the bottom solve stays FP64: widen the coarse residual, solve, narrow
    Lev<float>& f = L.back();
    Lev<double>& d = h->L64.back();
    const int64_t n3 = 3 * f.G.N;
    CK(cudaMemsetAsync(d.res, 0, sizeof(double) * n3, h->stream));
    CK(launch_add_float(f.res, d.res, n3, 1.0, h->stream));
    TRY(bottom64(h, d));
    CK(launch_to_float(d.cor, f.cor, n3, 1.0, h->stream));
    h->launches += 2;
    return AGB_OK;
}

// One V-cycle on the correction equation A cor = res of level l0
// (MLMG::mgVcycle(amrlev, mglev) as driven by the reference's hooks).
template <typename T>
agb_status vcycle(agb_elastic* h, std::vector<Lev<T>>& L, int l0 = 0) {
    const int nl = (int)L.size();
    if (l0 == nl - 1) return bottom<T>(h, L);
    // levels below l0 receive their first pre-smoothing sweep (from a zero
    // correction) from the restriction that fills their right-hand side
    const bool fuse = h->opts.pre_smooth > 0 && h->opts.smoother == AGB_SMOOTHER_JACOBI;
    for (int l = l0; l < nl - 1; l++) {
        Lev<T>& v = L[l];
        TRY(smooth<T>(h, L, l, h->opts.pre_smooth, true, fuse && l > l0));
        {
            ProfScope ps(h, Fam<T>::R, l == 0);
            if (use_zm<T>(h, v, l))
                CK(level_zm<T>(h, v, 2, v.cor, v.res, nullptr, T(0), v.rescor));
            else
                CK(launch_residual<T>(h->sym, v.cor, v.res, v.C, v.G, h->bc, v.rescor, nullptr, nullptr, h->stream));
        }
        {
            ProfScope ps(h, AGB_K_RESTRICT, l == 0);
            Lev<T>& c = L[l + 1];
            if (fuse && l + 1 < nl - 1)
                CK(launch_restrict_jacobi<T>(v.rescor, v.G, c.res, c.G, c.diag, (T)h->opts.omega, c.tmp, h->stream));
            else
                CK(launch_restrict<T>(v.rescor, v.G, c.res, c.G, h->stream));
        }
        h->launches += 2;
    }
    TRY(bottom<T>(h, L));
    for (int l = nl - 2; l >= l0; l--) {
        {
            ProfScope ps(h, AGB_K_PROLONG, l == 0);
            CK(launch_prolong_add<T>(L[l + 1].cor, L[l + 1].G, L[l].cor, L[l].G, h->stream));
        }
        h->launches++;
        TRY(smooth<T>(h, L, l, h->opts.post_smooth, false));
    }
    return AGB_OK;
}

// One F-cycle on A cor = res of the fine level, as MLMG::mgFcycle runs it
// for the iterations below max_fmg_iter: the residual restricted to every
// level, the bottom solve, then on each finer level the interpolated coarse
// correction as a start (interpAssign: prolongation into a zeroed
// correction), the residual of that start as the right-hand side of a
// V-cycle from this level, and the start added back.  The FP64 iteration
// runs it on L64; FGMRES may run it on its hierarchy as the preconditioner
// (opts.precond_cycle).  It leaves each level's res/rescor and cor/hold
// pointers swapped.
template <typename T>
agb_status fcycle(agb_elastic* h, std::vector<Lev<T>>& L) {
    const int nl = (int)L.size();
    for (int l = 1; l < nl; l++) {
        {
            ProfScope ps(h, AGB_K_RESTRICT, l == 1);
            CK(launch_restrict<T>(L[l - 1].res, L[l - 1].G, L[l].res, L[l].G, h->stream));
        }
        h->launches++;
    }
    TRY(bottom<T>(h, L));
    for (int l = nl - 2; l >= 0; l--) {
        Lev<T>& v = L[l];
        Lev<T>& c = L[l + 1];
        const int64_t n3 = 3 * v.G.N;
        if (!v.hold) CK(cudaMalloc(&v.hold, sizeof(T) * n3));
        CK(cudaMemsetAsync(v.cor, 0, sizeof(T) * n3, h->stream));
        {
            ProfScope ps(h, AGB_K_PROLONG, l == 0);
            CK(launch_prolong_add<T>(c.cor, c.G, v.cor, v.G, h->stream));
        }
        {
            ProfScope ps(h, Fam<T>::R, l == 0);
            if (use_zm<T>(h, v, l))
                CK(level_zm<T>(h, v, 2, v.cor, v.res, nullptr, T(0), v.rescor));
            else
                CK(launch_residual<T>(h->sym, v.cor, v.res, v.C, v.G, h->bc, v.rescor, nullptr, nullptr, h->stream));
        }
        h->launches += 2;
        // res <- res - A start; keep the start; V-cycle; add the start back
        std::swap(v.res, v.rescor);
        std::swap(v.cor, v.hold);
        TRY(vcycle<T>(h, L, l));
        CK(launch_axpy(T(1), v.hold, v.cor, n3, h->stream));
        h->launches++;
    }
    return AGB_OK;
}

agb_status fcycle64(agb_elastic* h) { return fcycle<double>(h, h->L64); }

// FP64 residual of level 0 into L64[0].res and its norms (host copy)
// double-float state of the mixed solve: the fine stiffness as hi + lo
// pairs (rebuilt when the model changes) and room for the solution and the
// right-hand side
agb_status ensure_df(agb_elastic* h) {
    const Lev<double>& top = h->L64[0];
    const int64_t N = top.G.N;
    if (!h->df_C) CK(cudaMalloc(&h->df_C, (size_t)DFLOAT_BYTES * N * h->nc));
    if (!h->df_x) CK(cudaMalloc(&h->df_x, (size_t)DFLOAT_BYTES * 3 * N));
    if (!h->df_b) CK(cudaMalloc(&h->df_b, (size_t)DFLOAT_BYTES * 3 * N));
    if (!h->have_df) {
        CK(launch_to_df(top.C, h->df_C, N * h->nc, h->stream));
        h->launches++;
        h->have_df = true;
    }
    return AGB_OK;
}

// double-float residual of df_x against df_b into the fine FP32 level's
// rescor (unscaled, rounded to FP32) and its norms (host copy)
agb_status residual_df(agb_elastic* h, double out[2]) {
    const Lev<double>& top = h->L64[0];
    int nb = 0;
    {
        // x, b (3 pairs each), the stiffness pairs in; r (3 floats) out
        const double bytes = (double)top.G.N * (DFLOAT_BYTES * (6 + h->nc) + 12);
        ProfScope ps(h, AGB_K_RESIDUAL_DF, true, bytes);
        CK(launch_residual_df(h->sym, h->df_x, h->df_b, h->df_C, top.G, h->bc, h->L32[0].rescor, nullptr,
                              h->partials, &nb, h->stream));
    }
    CK(launch_reduce_norms(h->partials, nb, h->norms_dev, h->stream));
    h->launches += 2;
    CK(cudaMemcpyAsync(h->norms_host, h->norms_dev, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    out[0] = h->norms_host[0];
    out[1] = h->norms_host[1];
    return AGB_OK;
}

agb_status residual64(agb_elastic* h, const double* x, const double* rhs, double out[2]) {
    Lev<double>& v = h->L64[0];
    int nb = 0;
    {
        ProfScope ps(h, AGB_K_RESIDUAL_F64, true);
        CK(launch_residual<double>(h->sym, x, rhs, v.C, v.G, h->bc, v.res, h->partials, &nb, h->stream));
    }
    CK(launch_reduce_norms(h->partials, nb, h->norms_dev, h->stream));
    h->launches += 2;
    CK(cudaMemcpyAsync(h->norms_host, h->norms_dev, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    out[0] = h->norms_host[0];
    out[1] = h->norms_host[1];
    return AGB_OK;
}

agb_status vec_norms(agb_elastic* h, const double* v, int64_t n, double out[2]) {
    CK(launch_vec_norms(v, n, h->partials, std::min(h->partials_cap, 152 * 8), h->norms_dev, h->stream));
    h->launches += 2;
    CK(cudaMemcpyAsync(h->norms_host, h->norms_dev, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    out[0] = h->norms_host[0];
    out[1] = h->norms_host[1];
    return AGB_OK;
}


template <typename T>
Krylov<T>& krylov_of(agb_elastic* h);
template <>
Krylov<double>& krylov_of<double>(agb_elastic* h) { return h->K64; }
template <>
Krylov<float>& krylov_of<float>(agb_elastic* h) { return h->K32; }

template <typename T>
agb_status ensure_krylov(agb_elastic* h, int m, int64_t n) {
    Krylov<T>& K = krylov_of<T>(h);
    if (K.m >= m && K.n == n) return AGB_OK;
    K.release();
    K.V.assign(m + 1, nullptr);
    K.Z.assign(m, nullptr);
    for (int i = 0; i <= m; i++) CK(cudaMalloc(&K.V[i], sizeof(T) * n));
    for (int i = 0; i < m; i++) CK(cudaMalloc(&K.Z[i], sizeof(T) * n));
    CK(cudaMalloc(&K.w, sizeof(T) * n));
    CK(cudaMalloc(&K.e, sizeof(T) * n));
    CK(cudaMalloc(&K.Vdev, sizeof(T*) * (m + 1)));
    CK(cudaMalloc(&K.Zdev, sizeof(T*) * m));
    CK(cudaMalloc(&K.Wdev, sizeof(T*)));
    CK(cudaMalloc(&K.part, sizeof(double) * multidot_blocks() * 40));
    CK(cudaMalloc(&K.dots, sizeof(double) * 3 * 40));
    CK(cudaMallocHost(&K.hdots, sizeof(double) * 3 * 40));
    CK(cudaMemcpy(K.Vdev, K.V.data(), sizeof(T*) * (m + 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(K.Zdev, K.Z.data(), sizeof(T*) * m, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(K.Wdev, &K.w, sizeof(T*), cudaMemcpyHostToDevice));
    K.m = m;
    K.n = n;
    return AGB_OK;
}

// One cycle of flexible GMRES (Saad 1993) on A e = r for the fine level of
// the hierarchy L, right-preconditioned by one V-cycle, classical
// Gram-Schmidt with one re-orthogonalisation; stops when the Arnoldi
// residual estimate falls below rel_tol * ||r||_2 or after m steps.
// Result in K.e; its = V-cycles applied; est = estimated relative residual.
template <typename T>
agb_status fgmres_cycle(agb_elastic* h, std::vector<Lev<T>>& L, const T* r, double rel_tol, int maxit, int* its,
                        double* est) {
    Lev<T>& top = L[0];
    const int64_t n = 3 * top.G.N;
    const int m = std::min(h->opts.krylov_dim, std::max(1, maxit));
    TRY(ensure_krylov<T>(h, h->opts.krylov_dim, n));
    Krylov<T>& K = krylov_of<T>(h);
    cudaStream_t st = h->stream;
    // beta = ||r||_2
    const double vb = (double)sizeof(T) * n;  // bytes of one Krylov vector
    CK(cudaMemcpyAsync(K.w, r, sizeof(T) * n, cudaMemcpyDeviceToDevice, st));
    {
        ProfScope ps(h, AGB_K_KRYLOV, true, vb);
        CK(launch_multidot<T>(K.Wdev, 1, K.w, n, K.part, K.dots, st));
    }
    CK(cudaMemcpyAsync(K.hdots, K.dots, sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    h->launches += 2;
    const double beta = std::sqrt(K.hdots[0]);
    *its = 0;
    *est = 0.0;
    if (!(beta > 0.0)) {
        CK(cudaMemsetAsync(K.e, 0, sizeof(T) * n, st));
        return AGB_OK;
    }
    {
        ProfScope ps(h, AGB_K_KRYLOV, true, 2 * vb);
        CK(launch_scale_copy<T>(r, K.V[0], n, 1.0 / beta, st));
    }
    h->launches++;
    std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m, 0.0), sn(m, 0.0), g(m + 1, 0.0);
    g[0] = beta;
    int j = 0;
    double resid = beta;
    for (; j < m; j++) {
        // Z_j = M^-1 V_j (one V-cycle on the correction equation).  The
        // cycle reads the fine right-hand side in place and builds the fine
        // correction in Z_j directly (the smoother ping-pongs cor and tmp, so
        // an odd sweep count leaves it in the other buffer: copied back).
        {
            const bool fc = h->opts.precond_cycle == AGB_PRECOND_F;
            if (fc && !top.hold) CK(cudaMalloc(&top.hold, sizeof(T) * n));
            T* res0 = top.res;
            T* cor0 = top.cor;
            T* tmp0 = top.tmp;
            T* rescor0 = top.rescor;
            T* hold0 = top.hold;
            // the V-cycle only reads its right-hand side, so it reads V_j in
            // place; the F-cycle's V-cycle from the fine level writes where
            // the right-hand side was (it swaps res and rescor), so it gets
            // a copy of V_j
            if (fc) CK(cudaMemcpyAsync(res0, K.V[j], sizeof(T) * n, cudaMemcpyDeviceToDevice, st));
            else top.res = K.V[j];
            top.cor = K.Z[j];
            const agb_status vs = fc ? fcycle<T>(h, L) : vcycle<T>(h, L);
            T* out = top.cor;
            // the F-cycle also swaps cor and hold, so Z_j passes through the
            // level's work pointers; the level gets its own buffers back (the
            // result is in one of them or in Z_j)
            top.res = res0;
            top.cor = cor0;
            top.tmp = tmp0;
            top.rescor = rescor0;
            top.hold = hold0;
            TRY(vs);
            if (out != K.Z[j]) CK(cudaMemcpyAsync(K.Z[j], out, sizeof(T) * n, cudaMemcpyDeviceToDevice, st));
        }
        // w = A Z_j
        if (use_zm<T>(h, top, 0))
            CK(level_zm<T>(h, top, 0, K.Z[j], nullptr, nullptr, T(0), K.w));
        else
            CK(launch_fapply<T>(h->sym, K.Z[j], top.C, top.G, h->bc, K.w, st));
        // classical Gram-Schmidt, re-orthogonalised once unless krylov_reorth = 0
        // (the last projection also leaves ||w||^2 in dots[80])
        const bool reorth = h->opts.krylov_reorth != 0;
        {
            // algorithmic bytes: each pass of dots reads V_0..V_j and w; each
            // projection reads them and writes w
            const double gs_bytes = (reorth ? 2 : 1) * ((j + 2) + (j + 3)) * vb;
            ProfScope ps(h, AGB_K_KRYLOV, true, gs_bytes);
            CK(launch_multidot<T>(K.Vdev, j + 1, K.w, n, K.part, K.dots, st));
            if (reorth) {
                CK(launch_multiaxpy<T>(K.w, 1.0, K.Vdev, K.dots, -1.0, j + 1, n, st));
                CK(launch_multidot<T>(K.Vdev, j + 1, K.w, n, K.part, K.dots + 40, st));
                CK(launch_multiaxpy_norm<T>(K.w, 1.0, K.Vdev, K.dots + 40, -1.0, j + 1, n, K.part, K.dots + 80,
                                            st));
            } else {
                CK(launch_multiaxpy_norm<T>(K.w, 1.0, K.Vdev, K.dots, -1.0, j + 1, n, K.part, K.dots + 80, st));
            }
        }
        CK(cudaMemcpyAsync(K.hdots, K.dots, sizeof(double) * 120, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        h->launches += reorth ? 8 : 5;
        for (int i = 0; i <= j; i++) H[(size_t)i * m + j] = K.hdots[i] + (reorth ? K.hdots[40 + i] : 0.0);
        const double hn = std::sqrt(std::max(K.hdots[80], 0.0));
        H[(size_t)(j + 1) * m + j] = hn;
        if (hn > 0.0) {
            ProfScope ps(h, AGB_K_KRYLOV, true, 2 * vb);
            CK(launch_scale_copy<T>(K.w, K.V[j + 1], n, 1.0 / hn, st));
            h->launches++;
        }
        // Givens rotations on column j
        for (int i = 0; i < j; i++) {
            const double a = H[(size_t)i * m + j], b = H[(size_t)(i + 1) * m + j];
            H[(size_t)i * m + j] = cs[i] * a + sn[i] * b;
            H[(size_t)(i + 1) * m + j] = -sn[i] * a + cs[i] * b;
        }
        const double a = H[(size_t)j * m + j], b = H[(size_t)(j + 1) * m + j];
        const double rr = std::hypot(a, b);
        cs[j] = rr > 0 ? a / rr : 1.0;
        sn[j] = rr > 0 ? b / rr : 0.0;
        H[(size_t)j * m + j] = rr;
        H[(size_t)(j + 1) * m + j] = 0.0;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        resid = std::fabs(g[j + 1]);
        if (resid <= rel_tol * beta || !(hn > 0.0)) { j++; break; }
    }
    const int k = std::min(j, m);
    // y = H^-1 g (upper triangular k x k), e = Z y
    std::vector<double> y(k, 0.0);
    for (int i = k - 1; i >= 0; i--) {
        double t = g[i];
        for (int q = i + 1; q < k; q++) t -= H[(size_t)i * m + q] * y[q];
        y[i] = H[(size_t)i * m + i] != 0.0 ? t / H[(size_t)i * m + i] : 0.0;
    }
    std::memcpy(K.hdots, y.data(), sizeof(double) * k);
    CK(cudaMemcpyAsync(K.dots, K.hdots, sizeof(double) * k, cudaMemcpyHostToDevice, st));
    {
        ProfScope ps(h, AGB_K_KRYLOV, true, (k + 1) * vb);
        CK(launch_multiaxpy<T>(K.e, 0.0, K.Zdev, K.dots, 1.0, k, n, st));
    }
    h->launches++;
    *its = k;
    *est = resid / beta;
    return AGB_OK;
}

// Linear::solve on device pointers.
// x_zero: x is known to be 0 on entry, so the initial residual is rhs itself
// (b - A 0 = b exactly) and is copied instead of computed
// r32_init (mixed precision, x not zero): the FP32 residual of x already
// computed on the fine FP32 level (the learned guess's fallback test); the
// first refinement step starts from it instead of an FP64 residual, and
// convergence is only declared on an FP64 residual
// target_from_rhs: the relative tolerance refers to the right-hand side
// alone (the solve from a learned guess must meet the tolerance of the
// solve from zero), not to max(|rhs|, |r0|) as MLMG's test does
agb_status solve_dev(agb_elastic* h, double* x, const double* rhs, double tol_rel, double tol_abs,
                     agb_solve_report* rep, bool x_zero = false, const float* r32_init = nullptr,
                     bool target_from_rhs = false) {
    auto t0 = std::chrono::steady_clock::now();
    const bool mixed = h->opts.precision == AGB_PRECISION_MIXED;
    // the mixed solve needs the FP32 hierarchy and the fine FP64 stiffness
    // only; the FP64 one needs the FP64 hierarchy
    if (mixed) TRY(ensure_f32(h));
    else TRY(prepare(h));
    Lev<double>& top = h->L64[0];
    const int64_t n3 = 3 * top.G.N;
    double r[2], bn[2];
    TRY(vec_norms(h, rhs, n3, bn));
    if (!x_zero) {
        // an all-zero initial iterate (e.g. a learned guess that fell back)
        // needs no FP64 residual: one max-norm pass instead of an operator
        double xn[2];
        TRY(vec_norms(h, x, n3, xn));
        x_zero = xn[0] == 0.0;
    }
    int fp64_res = 0;
    bool r_exact = true;  // r is an FP64 residual (or rhs itself)
    // double-float outer residual and update (mixed FGMRES without psi): the
    // iterate lives in df_x during the solve and x receives it at the end;
    // r_f32: the current residual is in the fine FP32 level's rescor
    // (unscaled) instead of the FP64 level's res
    const bool use_df = mixed && h->opts.solver == AGB_SOLVER_FGMRES &&
                        h->opts.outer_residual == AGB_OUTER_DFLOAT && !h->psi_set;
    bool r_f32 = false;
    if (use_df) {
        TRY(ensure_df(h));
        CK(launch_to_df(rhs, h->df_b, n3, h->stream));
        if (x_zero) CK(cudaMemsetAsync(h->df_x, 0, (size_t)DFLOAT_BYTES * n3, h->stream));
        else CK(launch_to_df(x, h->df_x, n3, h->stream));
        h->launches += 2;
    }
    if (x_zero) {
        if (use_df) {
            CK(launch_from_double<float>(rhs, h->L32[0].rescor, n3, 1.0, h->stream));
            h->launches++;
            r_f32 = true;
        } else {
            CK(cudaMemcpyAsync(top.res, rhs, sizeof(double) * n3, cudaMemcpyDeviceToDevice, h->stream));
        }
        r[0] = bn[0];
        r[1] = bn[1];
    } else if (use_df && !r32_init) {
        TRY(residual_df(h, r));
        fp64_res = 1;
        r_f32 = true;
    } else if (mixed && r32_init) {
        CK(cudaMemsetAsync(top.res, 0, sizeof(double) * n3, h->stream));
        CK(launch_add_float(r32_init, top.res, n3, 1.0, h->stream));
        h->launches++;
        TRY(vec_norms(h, top.res, n3, r));
        r_exact = false;
    } else {
        TRY(residual64(h, x, rhs, r));
        fp64_res = 1;
    }
    const double resnorm0 = r[0];
    const double max_norm = (target_from_rhs || bn[0] >= resnorm0) ? bn[0] : resnorm0;
    const double target = std::max(tol_abs, std::max(tol_rel, 1.e-16) * max_norm);
    const bool fixed = h->opts.fixed_iter > 0;
    const int maxit = fixed ? h->opts.fixed_iter : h->opts.max_iter;
    int status = AGB_NOT_CONVERGED, it = 0;
    if (std::isnan(r[0]) || std::isnan(r[1])) status = AGB_NAN;
    else if (r[0] <= target && !fixed && r_exact) status = AGB_OK;
    else {
        while (it < maxit) {
            if (h->opts.solver == AGB_SOLVER_FGMRES) {
                int its = 0;
                double est = 0.0;
                if (mixed) {
                    // FP32 FGMRES(V-cycle) on the scaled FP64 residual, FP64 update.
                    // The inner solve reduces by inner_tol, or by less when the
                    // FP64 residual is already within that factor of the target
                    // (aiming a decade below it: the FP32 estimate is not exact)
                    const double s = (r[0] > 0.0) ? 1.0 / r[0] : 1.0;
                    const double need = 0.1 * target / std::max(r[0], 1e-300);
                    const double rel = std::min(std::max(h->opts.inner_tol, need), 0.5);
                    Lev<float>& t32 = h->L32[0];
                    if (r_f32) CK(launch_scale_f32(t32.rescor, (float)s, n3, h->stream));
                    else CK(launch_from_double<float>(top.res, t32.rescor, n3, s, h->stream));
                    h->launches++;
                    TRY(fgmres_cycle<float>(h, h->L32, t32.rescor, rel, maxit - it, &its, &est));
                    if (use_df) CK(launch_df_axpy(h->K32.e, 1.0 / s, h->df_x, n3, h->stream));
                    else CK(launch_axpy_to_double<float>(h->K32.e, x, n3, 1.0 / s, h->stream));
                } else {
                    // FP64 FGMRES(V-cycle); aim a little below the target, the true residual decides
                    const double rt = std::max(0.5 * target / std::max(r[0], 1e-300), 1e-15);
                    TRY(fgmres_cycle<double>(h, h->L64, top.res, std::min(rt, 0.5), maxit - it, &its, &est));
                    CK(launch_axpy_to_double<double>(h->K64.e, x, n3, 1.0, h->stream));
                }
                h->launches++;
                it += std::max(its, 1);
            } else if (!mixed) {
                if (it < h->opts.max_fmg_iter) TRY(fcycle64(h));
                else TRY(vcycle<double>(h, h->L64));
                CK(launch_axpy(1.0, top.cor, x, n3, h->stream));
                h->launches++;
                it++;
            } else {
                // FP32 cycles on the scaled FP64 residual, FP64 update
                const double s = (r[0] > 0.0) ? 1.0 / r[0] : 1.0;
                Lev<float>& t32 = h->L32[0];
                CK(launch_to_float(top.res, t32.res, n3, s, h->stream));
                h->launches++;
                const int inner = std::max(1, h->opts.inner_cycles);
                for (int c = 0; c < inner && it < maxit; c++) {
                    TRY(vcycle<float>(h, h->L32));
                    CK(launch_add_float(t32.cor, x, n3, 1.0 / s, h->stream));
                    h->launches++;
                    it++;
                    if (c + 1 < inner && it < maxit) {
                        // next FP32 cycle works on res - A cor of the scaled correction equation
                        ProfScope ps(h, AGB_K_RESIDUAL_F32, true);
                        CK(launch_residual<float>(h->sym, t32.cor, t32.res, t32.C, t32.G, h->bc, t32.rescor, nullptr,
                                                  nullptr, h->stream));
                        h->launches++;
                        std::swap(t32.res, t32.rescor);
                    }
                }
            }
            if (use_df) {
                TRY(residual_df(h, r));
                r_f32 = true;
            } else {
                TRY(residual64(h, x, rhs, r));
            }
            fp64_res++;
            if (h->opts.verbose > 0) std::fprintf(stderr, "agb: cycle %d |r|_inf = %.6e\n", it, r[0]);
            if (std::isnan(r[0]) || std::isnan(r[1])) { status = AGB_NAN; break; }
            if (r[0] <= target && !fixed) { status = AGB_OK; break; }
        }
        if (fixed && status != AGB_NAN) status = AGB_OK;
    }
    if (use_df) {
        CK(launch_df_to_double(h->df_x, x, n3, h->stream));
        h->launches++;
    }
    int binfo[4] = {0, 0, 0, 0};
    CK(cudaMemcpyAsync(h->norms_host, h->bottom_info, 4 * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    std::memcpy(binfo, h->norms_host, 4 * sizeof(int));
    if (binfo[3] != 0) {
        CK(cudaMemsetAsync(h->bottom_info + 3, 0, sizeof(int), h->stream));
        CK(cudaStreamSynchronize(h->stream));
        return fail(AGB_CUDA_ERROR, "a TMA load of the fine-level stencil kernel did not complete in time");
    }
    prof_collect(h);
    if (rep) {
        rep->status = status;
        rep->iters = it;
        rep->nlevels = (int)h->L64.size();
        rep->bottom_iters = binfo[1];
        rep->fp64_residuals = fp64_res;
        rep->resnorm0 = resnorm0;
        rep->rhsnorm0 = bn[0];
        rep->final_resnorm = r[0];
        rep->final_resnorm_l2 = r[1];
        rep->rhsnorm_l2 = bn[1];
        rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    if (status == AGB_NOT_CONVERGED) g_last_error = "multigrid did not reach the tolerance within max_iter cycles";
    if (status == AGB_NAN) g_last_error = "NaN in the residual";
    return (agb_status)status;
}

// copy a host or device input of `bytes` into a device pointer
agb_status dev_in(agb_elastic* h, int slot, const void* src, size_t bytes, int where, const void** out) {
    if (where == AGB_MEM_DEVICE) { *out = src; return AGB_OK; }
    if (where != AGB_MEM_HOST) return fail(AGB_BAD_ARG, "where must be AGB_MEM_HOST or AGB_MEM_DEVICE");
    TRY(ensure_io(h, slot, bytes));
    CK(cudaMemcpyAsync(h->io[slot], src, bytes, cudaMemcpyHostToDevice, h->stream));
    *out = h->io[slot];
    return AGB_OK;
}
// device pointer an output lands in before it is copied back to `dst`
agb_status dev_out(agb_elastic* h, int slot, void* dst, size_t bytes, int where, void** out) {
    if (where == AGB_MEM_DEVICE) { *out = dst; return AGB_OK; }
    if (where != AGB_MEM_HOST) return fail(AGB_BAD_ARG, "where must be AGB_MEM_HOST or AGB_MEM_DEVICE");
    TRY(ensure_io(h, slot, bytes));
    *out = h->io[slot];
    return AGB_OK;
}
agb_status finish_out(agb_elastic* h, void* dst, const void* dev, size_t bytes, int where) {
    if (where == AGB_MEM_HOST) CK(cudaMemcpyAsync(dst, dev, bytes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return AGB_OK;
}

agb_status check_level(agb_elastic* h, int level) {
    if (!h) return fail(AGB_BAD_ARG, "null handle");
    if (level < 0 || level >= (int)h->L64.size()) return fail(AGB_BAD_ARG, "level out of range");
    if (level > 0 || !h->model_set) TRY(prepare(h));
    return AGB_OK;
}

}  // namespace

namespace agb {
void set_last_error(const char* msg) { g_last_error = msg ? msg : ""; }
}  // namespace agb

// ============================================================================
extern "C" {

agb_status agb_default_opts(agb_solver_opts* o) {
    if (!o) return fail(AGB_BAD_ARG, "null opts");
    o->max_iter = 200;
    o->pre_smooth = 2;
    o->post_smooth = 2;
    o->final_smooth = 8;
    o->bottom_smooth = 0;
    o->bottom_max_iter = 200;
    o->bottom_tol_rel = 1e-4;
    o->bottom_tol_abs = -1.0;
    o->omega = 2.0 / 3.0;
    o->max_coarsening_level = -1;
    o->fixed_iter = -1;
    o->verbose = 0;
    o->precision = AGB_PRECISION_FP64;
    o->inner_cycles = 1;
    o->solver = AGB_SOLVER_VCYCLE;
    o->krylov_dim = 20;
    o->inner_tol = 1e-4;
    o->bottom_solver = AGB_BOTTOM_BICGSTAB;
    o->fine_kernel = 0;
    o->krylov_reorth = 0;
    o->tma_min_nodes = 0;
    o->max_fmg_iter = 100000000;
    o->smoother = AGB_SMOOTHER_JACOBI;
    o->outer_residual = AGB_OUTER_FP64;
    o->precond_cycle = AGB_PRECOND_V;
    return AGB_OK;
}

static agb_status check_opts(const agb_solver_opts* o) {
    if (o->pre_smooth < 0 || o->post_smooth < 0 || o->final_smooth < 0 || o->bottom_smooth < 0 ||
        o->bottom_max_iter < 0 || o->max_iter < 0)
        return fail(AGB_BAD_ARG, "negative iteration count in opts");
    if (!(o->omega > 0.0) || !(o->omega <= 2.0)) return fail(AGB_BAD_ARG, "omega must lie in (0, 2]");
    if (o->precision != AGB_PRECISION_FP64 && o->precision != AGB_PRECISION_MIXED)
        return fail(AGB_BAD_ARG, "unknown precision");
    if (o->solver != AGB_SOLVER_VCYCLE && o->solver != AGB_SOLVER_FGMRES) return fail(AGB_BAD_ARG, "unknown solver");
    if (o->bottom_solver < AGB_BOTTOM_BICGSTAB || o->bottom_solver > AGB_BOTTOM_SMOOTHER)
        return fail(AGB_BAD_ARG, "unknown bottom solver");
    if (o->fine_kernel < 0 || o->fine_kernel > 1) return fail(AGB_BAD_ARG, "fine_kernel must be 0 or 1");
    if (o->tma_min_nodes < 0) return fail(AGB_BAD_ARG, "tma_min_nodes must be >= 0");
    if (o->smoother != AGB_SMOOTHER_JACOBI && o->smoother != AGB_SMOOTHER_GS)
        return fail(AGB_BAD_ARG, "unknown smoother");
    if (o->outer_residual != AGB_OUTER_FP64 && o->outer_residual != AGB_OUTER_DFLOAT)
        return fail(AGB_BAD_ARG, "unknown outer_residual");
    if (o->precond_cycle != AGB_PRECOND_V && o->precond_cycle != AGB_PRECOND_F)
        return fail(AGB_BAD_ARG, "unknown precond_cycle");
    if (o->solver == AGB_SOLVER_FGMRES && (o->krylov_dim < 1 || o->krylov_dim > 39))
        return fail(AGB_BAD_ARG, "krylov_dim must lie in [1, 39]");
    if (o->solver == AGB_SOLVER_FGMRES && !(o->inner_tol > 0.0 && o->inner_tol < 1.0))
        return fail(AGB_BAD_ARG, "inner_tol must lie in (0, 1)");
    return AGB_OK;
}

agb_status agb_elastic_create(agb_elastic** out, int nx, int ny, int nz, const double dx[3], int sym,
                              const agb_solver_opts* opts) {
    if (!out) return fail(AGB_BAD_ARG, "null output handle");
    *out = nullptr;
    if (nx < 3 || ny < 3 || nz < 3) return fail(AGB_BAD_ARG, "grid needs at least 3 nodes per axis");
    if (!dx || !(dx[0] > 0) || !(dx[1] > 0) || !(dx[2] > 0)) return fail(AGB_BAD_ARG, "dx must be positive");
    if (sym != AGB_SYM_ISOTROPIC && sym != AGB_SYM_MAJORMINOR && sym != AGB_SYM_MAJOR)
        return fail(AGB_BAD_ARG, "unknown symmetry");
    agb_elastic* h = new agb_elastic();
    h->sym = sym;
    h->nc = sym == AGB_SYM_ISOTROPIC ? 2 : sym == AGB_SYM_MAJORMINOR ? 21 : 45;
    h->n[0] = nx; h->n[1] = ny; h->n[2] = nz;
    for (int d = 0; d < 3; d++) h->dx[d] = dx[d];
    if (opts) {
        agb_status st = check_opts(opts);
        if (st != AGB_OK) { delete h; return st; }
        h->opts = *opts;
    } else {
        agb_default_opts(&h->opts);
    }
    // default BC: displacement 0 everywhere (Constant.H:36-45)
    for (int q = 0; q < 78; q++) { h->bc.t[q] = BC_DISP; h->bcval[q] = 0.0; }
    auto bail = [&](agb_status st) { agb_elastic_destroy(h); return st; };
    if (cudaGetDevice(&h->device) != cudaSuccess) return bail(fail(AGB_CUDA_ERROR, "no CUDA device"));
    if (cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(AGB_CUDA_ERROR, "cudaStreamCreate failed"));
    h->stream = h->own_stream;
    agb_status st = alloc_levels64(h);
    if (st != AGB_OK) return bail(st);
    if (cudaMalloc(&h->norms_dev, 4 * sizeof(double)) != cudaSuccess ||
        cudaMallocHost(&h->norms_host, 4 * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&h->bottom_info, 4 * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&h->bcval_dev, 78 * sizeof(double)) != cudaSuccess)
        return bail(fail(AGB_OUT_OF_MEMORY, "allocation of small buffers failed"));
    cudaMemset(h->bottom_info, 0, 4 * sizeof(int));
    *out = h;
    return AGB_OK;
}

agb_status agb_elastic_destroy(agb_elastic* h) {
    if (!h) return AGB_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_levels(h->L64);
    free_levels(h->L32);
    cudaFree(h->partials);
    cudaFree(h->norms_dev);
    if (h->norms_host) cudaFreeHost(h->norms_host);
    cudaFree(h->bottom_work);
    cudaFree(h->bottom_info);
    cudaFree(h->bcval_dev);
    cudaFree(h->dw);
    cudaFree(h->psi_fine);
    cudaFree(h->nh_model);
    cudaFree(h->df_C);
    cudaFree(h->df_x);
    cudaFree(h->df_b);
    h->K64.release();
    h->K32.release();
    cudaFree(h->bot_inv);
    cudaFree(h->bot_work);
    cudaFree(h->bot_iwork);
    for (int s = 0; s < 4; s++) cudaFree(h->io[s]);
    for (auto e : h->ev_pool) cudaEventDestroy(e);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
    return AGB_OK;
}

agb_status agb_elastic_set_opts(agb_elastic* h, const agb_solver_opts* o) {
    if (!h || !o) return fail(AGB_BAD_ARG, "null argument");
    TRY(check_opts(o));
    const bool relevel = o->max_coarsening_level != h->opts.max_coarsening_level;
    h->opts = *o;
    if (relevel) {
        // keep the fine-level stiffness across the re-allocation
        const int64_t N = nodes(h);
        double* keep = nullptr;
        if (h->model_set) {
            CK(cudaMalloc(&keep, sizeof(double) * N * h->nc));
            CK(cudaMemcpyAsync(keep, h->L64[0].C, sizeof(double) * N * h->nc, cudaMemcpyDeviceToDevice, h->stream));
            CK(cudaStreamSynchronize(h->stream));
        }
        free_levels(h->L32);
        h->have_f32 = false;
        h->have_df = false;
        agb_status st = alloc_levels64(h);
        if (st == AGB_OK && keep)
            st = (cudaMemcpy(h->L64[0].C, keep, sizeof(double) * N * h->nc, cudaMemcpyDeviceToDevice) == cudaSuccess)
                     ? AGB_OK
                     : fail(AGB_CUDA_ERROR, "copy of the stiffness failed");
        cudaFree(keep);
        if (st != AGB_OK) return st;
    }
    h->prepared = false;
    h->have_f32 = false;
    h->have_df = false;
    h->bot_src = 0;
    return AGB_OK;
}

agb_status agb_elastic_set_stream(agb_elastic* h, void* s) {
    if (!h) return fail(AGB_BAD_ARG, "null handle");
    CK(cudaStreamSynchronize(h->stream));
    h->stream = s ? (cudaStream_t)s : h->own_stream;
    return AGB_OK;
}

agb_status agb_elastic_set_model(agb_elastic* h, const double* C, int where) {
    if (!h || !C) return fail(AGB_BAD_ARG, "null argument");
    const int64_t N = nodes(h);
    const size_t bytes = sizeof(double) * N * h->nc;
    const void* src = nullptr;
    if (where == AGB_MEM_HOST) {
        // stage through the handle's persistent staging buffer (no
        // allocation per call), then AoS -> SoA
        TRY(ensure_io(h, 0, bytes));
        double* tmp = h->io[0];
        CK(cudaMemcpyAsync(tmp, C, bytes, cudaMemcpyHostToDevice, h->stream));
        CK(launch_aos_to_soa(tmp, h->L64[0].C, N, h->nc, h->stream));
    } else if (where == AGB_MEM_DEVICE) {
        src = C;
        CK(launch_aos_to_soa((const double*)src, h->L64[0].C, N, h->nc, h->stream));
    } else {
        return fail(AGB_BAD_ARG, "where must be AGB_MEM_HOST or AGB_MEM_DEVICE");
    }
    h->launches++;
    CK(cudaStreamSynchronize(h->stream));
    h->model_set = true;
    h->prepared = false;
    h->have_f32 = false;
    h->have_df = false;
    h->bot_src = 0;
    return AGB_OK;
}

agb_status agb_elastic_get_model(agb_elastic* h, int level, double* C, int where) {
    TRY(check_level(h, level));
    if (!C) return fail(AGB_BAD_ARG, "null output");
    Lev<double>& v = h->L64[level];
    const size_t bytes = sizeof(double) * v.G.N * h->nc;
    void* d = nullptr;
    TRY(dev_out(h, 0, C, bytes, where, &d));
    CK(launch_soa_to_aos(v.C, (double*)d, v.G.N, h->nc, h->stream));
    h->launches++;
    return finish_out(h, C, d, bytes, where);
}

agb_status agb_elastic_set_bc(agb_elastic* h, const int* type, const double* val) {
    if (!h || !type || !val) return fail(AGB_BAD_ARG, "null argument");
    for (int q = 0; q < 78; q++) {
        if (type[q] < AGB_BC_DISPLACEMENT || type[q] > AGB_BC_NONE) return fail(AGB_BAD_ARG, "unknown BC type");
    }
    for (int q = 0; q < 78; q++) { h->bc.t[q] = (unsigned char)type[q]; h->bcval[q] = val[q]; }
    h->bc_set = true;
    h->prepared = false;
    h->have_f32 = false;
    h->have_df = false;
    h->bot_src = 0;
    return AGB_OK;
}

agb_status agb_elastic_prepare(agb_elastic* h) {
    if (!h) return fail(AGB_BAD_ARG, "null handle");
    return prepare(h);
}

agb_status agb_elastic_set_psi(agb_elastic* h, const double* psi, double small, int where) {
    if (!h) return fail(AGB_BAD_ARG, "null handle");
    if (!psi) {
        h->psi_set = false;
        for (auto& v : h->L64) v.G.psi = nullptr;
        for (auto& v : h->L32) v.G.psi = nullptr;
    } else {
        if (!(small >= 0.0 && small < 1.0)) return fail(AGB_BAD_ARG, "psi_small must be in [0, 1)");
        const LevelGeom<double>& G = h->L64[0].G;
        const size_t cells = (size_t)(G.nx - 1) * (G.ny - 1) * (G.nz - 1);
        if (!h->psi_fine) CK(cudaMalloc(&h->psi_fine, sizeof(double) * G.psz * (G.nz + 1)));
        if (where == AGB_MEM_HOST) {
            double* tmp = nullptr;
            CK(cudaMallocAsync((void**)&tmp, sizeof(double) * cells, h->stream));
            CK(cudaMemcpyAsync(tmp, psi, sizeof(double) * cells, cudaMemcpyHostToDevice, h->stream));
            CK(launch_psi_embed(tmp, G, h->psi_fine, h->stream));
            CK(cudaFreeAsync(tmp, h->stream));
        } else if (where == AGB_MEM_DEVICE) {
            CK(launch_psi_embed(psi, G, h->psi_fine, h->stream));
        } else {
            return fail(AGB_BAD_ARG, "where must be AGB_MEM_HOST or AGB_MEM_DEVICE");
        }
        h->launches++;
        CK(cudaStreamSynchronize(h->stream));
        h->psi_set = true;
        h->psi_small = small;
        h->L64[0].G.psi = h->psi_fine;
        h->L64[0].G.psi_small = small;
    }
    h->prepared = false;
    h->have_f32 = false;
    h->have_df = false;
    h->bot_src = 0;
    return AGB_OK;
}

agb_status agb_elastic_num_levels(agb_elastic* h, int* nl) {
    if (!h || !nl) return fail(AGB_BAD_ARG, "null argument");
    *nl = (int)h->L64.size();
    return AGB_OK;
}

agb_status agb_elastic_level_dims(agb_elastic* h, int level, int dims[3]) {
    if (!h || !dims) return fail(AGB_BAD_ARG, "null argument");
    if (level < 0 || level >= (int)h->L64.size()) return fail(AGB_BAD_ARG, "level out of range");
    dims[0] = h->L64[level].G.nx; dims[1] = h->L64[level].G.ny; dims[2] = h->L64[level].G.nz;
    return AGB_OK;
}

agb_status agb_elastic_fapply(agb_elastic* h, int level, const double* u, double* f, int where) {
    TRY(check_level(h, level));
    if (!u || !f) return fail(AGB_BAD_ARG, "null argument");
    Lev<double>& v = h->L64[level];
    const size_t bytes = sizeof(double) * 3 * v.G.N;
    const void* du = nullptr;
    void* df = nullptr;
    TRY(dev_in(h, 0, u, bytes, where, &du));
    TRY(dev_out(h, 1, f, bytes, where, &df));
    {
        ProfScope ps(h, AGB_K_FAPPLY_F64, level == 0);
        CK(launch_fapply<double>(h->sym, (const double*)du, v.C, v.G, h->bc, (double*)df, h->stream));
    }
    h->launches++;
    TRY(finish_out(h, f, df, bytes, where));
    prof_collect(h);
    return AGB_OK;
}

agb_status agb_elastic_fapply_f32(agb_elastic* h, int level, const float* u, float* f, int where) {
    TRY(check_level(h, level));
    if (!u || !f) return fail(AGB_BAD_ARG, "null argument");
    TRY(ensure_f32(h));
    Lev<float>& v = h->L32[level];
    const size_t bytes = sizeof(float) * 3 * v.G.N;
    const void* du = nullptr;
    void* df = nullptr;
    TRY(dev_in(h, 0, u, bytes, where, &du));
    TRY(dev_out(h, 1, f, bytes, where, &df));
    {
        ProfScope ps(h, AGB_K_FAPPLY_F32, level == 0);
        if (use_zm<float>(h, v, level))
            CK(level_zm<float>(h, v, 0, (const float*)du, nullptr, nullptr, 0.f, (float*)df));
        else
            CK(launch_fapply<float>(h->sym, (const float*)du, v.C, v.G, h->bc, (float*)df, h->stream));
    }
    h->launches++;
    TRY(finish_out(h, f, df, bytes, where));
    prof_collect(h);
    return AGB_OK;
}

agb_status agb_elastic_diagonal(agb_elastic* h, int level, double* diag, int where) {
    TRY(check_level(h, level));
    TRY(prepare(h));
    if (!diag) return fail(AGB_BAD_ARG, "null argument");
    Lev<double>& v = h->L64[level];
    const size_t bytes = sizeof(double) * 3 * v.G.N;
    if (where == AGB_MEM_HOST) CK(cudaMemcpyAsync(diag, v.diag, bytes, cudaMemcpyDeviceToHost, h->stream));
    else CK(cudaMemcpyAsync(diag, v.diag, bytes, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return AGB_OK;
}

agb_status agb_elastic_fsmooth(agb_elastic* h, int level, double* x, const double* b, int ncalls, int where) {
    TRY(check_level(h, level));
    TRY(prepare(h));
    if (!x || !b || ncalls < 0) return fail(AGB_BAD_ARG, "bad argument");
    Lev<double>& v = h->L64[level];
    const size_t bytes = sizeof(double) * 3 * v.G.N;
    const void* dx0 = nullptr;
    const void* db = nullptr;
    TRY(dev_in(h, 0, x, bytes, where, &dx0));
    TRY(dev_in(h, 1, b, bytes, where, &db));
    // the level's cor/res buffers hold the iterate and the rhs
    CK(cudaMemcpyAsync(v.cor, dx0, bytes, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(v.res, db, bytes, cudaMemcpyDeviceToDevice, h->stream));
    TRY(smooth<double>(h, h->L64, level, ncalls, false));
    if (where == AGB_MEM_HOST) CK(cudaMemcpyAsync(x, v.cor, bytes, cudaMemcpyDeviceToHost, h->stream));
    else CK(cudaMemcpyAsync(x, v.cor, bytes, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    prof_collect(h);
    return AGB_OK;
}

agb_status agb_elastic_residual(agb_elastic* h, int level, const double* x, const double* b, double* r,
                                double norms[2], int where) {
    TRY(check_level(h, level));
    if (!x || !b || !r) return fail(AGB_BAD_ARG, "null argument");
    Lev<double>& v = h->L64[level];
    const size_t bytes = sizeof(double) * 3 * v.G.N;
    const void* dx0 = nullptr;
    const void* db = nullptr;
    void* dr = nullptr;
    TRY(dev_in(h, 0, x, bytes, where, &dx0));
    TRY(dev_in(h, 1, b, bytes, where, &db));
    TRY(dev_out(h, 2, r, bytes, where, &dr));
    int nb = 0;
    {
        ProfScope ps(h, AGB_K_RESIDUAL_F64, level == 0);
        CK(launch_residual<double>(h->sym, (const double*)dx0, (const double*)db, v.C, v.G, h->bc, (double*)dr,
                                   h->partials, &nb, h->stream));
    }
    CK(launch_reduce_norms(h->partials, nb, h->norms_dev, h->stream));
    h->launches += 2;
    CK(cudaMemcpyAsync(h->norms_host, h->norms_dev, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    TRY(finish_out(h, r, dr, bytes, where));
    if (norms) { norms[0] = h->norms_host[0]; norms[1] = h->norms_host[1]; }
    prof_collect(h);
    return AGB_OK;
}

agb_status agb_elastic_fsmooth_f32(agb_elastic* h, int level, float* x, const float* b, int ncalls, int where) {
    TRY(check_level(h, level));
    if (!x || !b || ncalls < 0) return fail(AGB_BAD_ARG, "bad argument");
    TRY(ensure_f32(h));
    Lev<float>& v = h->L32[level];
    const size_t bytes = sizeof(float) * 3 * v.G.N;
    const void* dx0 = nullptr;
    const void* db = nullptr;
    TRY(dev_in(h, 0, x, bytes, where, &dx0));
    TRY(dev_in(h, 1, b, bytes, where, &db));
    CK(cudaMemcpyAsync(v.cor, dx0, bytes, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(v.res, db, bytes, cudaMemcpyDeviceToDevice, h->stream));
    TRY(smooth<float>(h, h->L32, level, ncalls, false));
    if (where == AGB_MEM_HOST) CK(cudaMemcpyAsync(x, v.cor, bytes, cudaMemcpyDeviceToHost, h->stream));
    else CK(cudaMemcpyAsync(x, v.cor, bytes, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    prof_collect(h);
    return AGB_OK;
}

agb_status agb_elastic_residual_f32(agb_elastic* h, int level, const float* x, const float* b, float* r, int where) {
    TRY(check_level(h, level));
    if (!x || !b || !r) return fail(AGB_BAD_ARG, "null argument");
    TRY(ensure_f32(h));
    Lev<float>& v = h->L32[level];
    const size_t bytes = sizeof(float) * 3 * v.G.N;
    const void* dx0 = nullptr;
    const void* db = nullptr;
    void* dr = nullptr;
    TRY(dev_in(h, 0, x, bytes, where, &dx0));
    TRY(dev_in(h, 1, b, bytes, where, &db));
    TRY(dev_out(h, 2, r, bytes, where, &dr));
    {
        ProfScope ps(h, AGB_K_RESIDUAL_F32, level == 0);
        if (use_zm<float>(h, v, level))
            CK(level_zm<float>(h, v, 2, (const float*)dx0, (const float*)db, nullptr, 0.f, (float*)dr));
        else
            CK(launch_residual<float>(h->sym, (const float*)dx0, (const float*)db, v.C, v.G, h->bc, (float*)dr,
                                      nullptr, nullptr, h->stream));
    }
    h->launches++;
    TRY(finish_out(h, r, dr, bytes, where));
    prof_collect(h);
    return AGB_OK;
}

agb_status agb_elastic_residual_dfloat(agb_elastic* h, const double* x, const double* b, double* r, double norms[2],
                                       int where) {
    TRY(check_level(h, 0));
    if (!x || !b || !r) return fail(AGB_BAD_ARG, "null argument");
    if (h->psi_set) return fail(AGB_BAD_ARG, "the double-float residual has no psi terms");
    if (!h->model_set) return fail(AGB_NOT_READY, "model not set (agb_elastic_set_model)");
    TRY(ensure_df(h));
    Lev<double>& v = h->L64[0];
    const int64_t n3 = 3 * v.G.N;
    const size_t bytes = sizeof(double) * n3;
    const void* dx0 = nullptr;
    const void* db = nullptr;
    void* dr = nullptr;
    TRY(dev_in(h, 0, x, bytes, where, &dx0));
    TRY(dev_in(h, 1, b, bytes, where, &db));
    TRY(dev_out(h, 2, r, bytes, where, &dr));
    CK(launch_to_df((const double*)dx0, h->df_x, n3, h->stream));
    CK(launch_to_df((const double*)db, h->df_b, n3, h->stream));
    int nb = 0;
    {
        ProfScope ps(h, AGB_K_RESIDUAL_DF, true, (double)v.G.N * (DFLOAT_BYTES * (6 + h->nc) + 24));
        CK(launch_residual_df(h->sym, h->df_x, h->df_b, h->df_C, v.G, h->bc, nullptr, (double*)dr, h->partials, &nb,
                              h->stream));
    }
    CK(launch_reduce_norms(h->partials, nb, h->norms_dev, h->stream));
    h->launches += 4;
    CK(cudaMemcpyAsync(h->norms_host, h->norms_dev, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    TRY(finish_out(h, r, dr, bytes, where));
    if (norms) { norms[0] = h->norms_host[0]; norms[1] = h->norms_host[1]; }
    prof_collect(h);
    return AGB_OK;
}

agb_status agb_elastic_restrict(agb_elastic* h, int crse_level, const double* fine, double* crse, int where) {
    if (!h) return fail(AGB_BAD_ARG, "null handle");
    if (crse_level < 1 || crse_level >= (int)h->L64.size()) return fail(AGB_BAD_ARG, "level out of range");
    if (!fine || !crse) return fail(AGB_BAD_ARG, "null argument");
    Lev<double>& f = h->L64[crse_level - 1];
    Lev<double>& c = h->L64[crse_level];
    const void* df = nullptr;
    void* dc = nullptr;
    TRY(dev_in(h, 0, fine, sizeof(double) * 3 * f.G.N, where, &df));
    TRY(dev_out(h, 1, crse, sizeof(double) * 3 * c.G.N, where, &dc));
    CK(launch_restrict<double>((const double*)df, f.G, (double*)dc, c.G, h->stream));
    h->launches++;
    return finish_out(h, crse, dc, sizeof(double) * 3 * c.G.N, where);
}

agb_status agb_elastic_prolong_add(agb_elastic* h, int fine_level, const double* crse, double* fine, int where) {
    if (!h) return fail(AGB_BAD_ARG, "null handle");
    if (fine_level < 0 || fine_level + 1 >= (int)h->L64.size()) return fail(AGB_BAD_ARG, "level out of range");
    if (!fine || !crse) return fail(AGB_BAD_ARG, "null argument");
    Lev<double>& f = h->L64[fine_level];
    Lev<double>& c = h->L64[fine_level + 1];
    const size_t fb = sizeof(double) * 3 * f.G.N;
    const void* dc = nullptr;
    const void* df0 = nullptr;
    TRY(dev_in(h, 0, crse, sizeof(double) * 3 * c.G.N, where, &dc));
    TRY(dev_in(h, 1, fine, fb, where, &df0));
    CK(launch_prolong_add<double>((const double*)dc, c.G, (double*)df0, f.G, h->stream));
    h->launches++;
    return finish_out(h, fine, df0, fb, where);
}

agb_status agb_elastic_vcycle(agb_elastic* h, const double* res, double* cor, int precision, int where) {
    TRY(check_level(h, 0));
    TRY(prepare(h));
    if (!res || !cor) return fail(AGB_BAD_ARG, "null argument");
    if (precision != AGB_PRECISION_FP64 && precision != AGB_PRECISION_MIXED) return fail(AGB_BAD_ARG, "bad precision");
    Lev<double>& top = h->L64[0];
    const int64_t n3 = 3 * top.G.N;
    const size_t bytes = sizeof(double) * n3;
    const void* dr = nullptr;
    void* dc = nullptr;
    TRY(dev_in(h, 0, res, bytes, where, &dr));
    TRY(dev_out(h, 1, cor, bytes, where, &dc));
    if (precision == AGB_PRECISION_FP64) {
        CK(cudaMemcpyAsync(top.res, dr, bytes, cudaMemcpyDeviceToDevice, h->stream));
        TRY(vcycle<double>(h, h->L64));
        CK(cudaMemcpyAsync(dc, top.cor, bytes, cudaMemcpyDeviceToDevice, h->stream));
    } else {
        TRY(ensure_f32(h));
        Lev<float>& t32 = h->L32[0];
        CK(launch_from_double<float>((const double*)dr, t32.res, n3, 1.0, h->stream));
        TRY(vcycle<float>(h, h->L32));
        CK(cudaMemsetAsync(dc, 0, bytes, h->stream));
        CK(launch_axpy_to_double<float>(t32.cor, (double*)dc, n3, 1.0, h->stream));
        h->launches += 2;
    }
    TRY(finish_out(h, cor, dc, bytes, where));
    prof_collect(h);
    return AGB_OK;
}

agb_status agb_elastic_bc_init(agb_elastic* h, double* b, int homogeneous, int where) {
    if (!h || !b) return fail(AGB_BAD_ARG, "null argument");
    const size_t bytes = sizeof(double) * 3 * nodes(h);
    const void* db = nullptr;
    TRY(dev_in(h, 0, b, bytes, where, &db));
    CK(cudaMemcpyAsync(h->bcval_dev, h->bcval, sizeof(h->bcval), cudaMemcpyHostToDevice, h->stream));
    CK(launch_bc_init((double*)db, h->L64[0].G, h->bc, h->bcval_dev, homogeneous, h->stream));
    h->launches++;
    return finish_out(h, b, db, bytes, where);
}

static agb_status build_rhs_dev(agb_elastic* h, const double* u, const double* b, const double* F0, int f0n,
                                double* rhs) {
    const int64_t N = nodes(h);
    if (!h->dw) CK(cudaMalloc(&h->dw, sizeof(double) * 9 * N));
    CK(launch_build_rhs(h->sym, u, b, F0, f0n, h->L64[0].C, h->L64[0].G, h->bc, h->dw, rhs, h->stream));
    h->launches += (u || f0n) ? 2 : 0;  // u = 0 without F0: a device copy
    return AGB_OK;
}

agb_status agb_elastic_build_rhs(agb_elastic* h, const double* u, const double* b, const double* F0, int f0_ncomp,
                                 double* rhs, int where) {
    if (!h || !u || !b || !rhs) return fail(AGB_BAD_ARG, "null argument");
    if (!(f0_ncomp == 0 || f0_ncomp == 1 || f0_ncomp == 9) || (f0_ncomp && !F0))
        return fail(AGB_BAD_ARG, "f0_ncomp must be 0, 1 or 9 (with F0 given)");
    if (!h->model_set) return fail(AGB_NOT_READY, "model not set");
    const int64_t N = nodes(h);
    const size_t bytes = sizeof(double) * 3 * N;
    const void *du = nullptr, *db = nullptr, *dF = nullptr;
    void* dr = nullptr;
    TRY(dev_in(h, 0, u, bytes, where, &du));
    TRY(dev_in(h, 1, b, bytes, where, &db));
    if (f0_ncomp) TRY(dev_in(h, 3, F0, sizeof(double) * f0_ncomp * N, where, &dF));
    TRY(dev_out(h, 2, rhs, bytes, where, &dr));
    TRY(build_rhs_dev(h, (const double*)du, (const double*)db, (const double*)dF, f0_ncomp, (double*)dr));
    return finish_out(h, rhs, dr, bytes, where);
}

agb_status agb_linear_solve(agb_elastic* h, double* sol, const double* rhs, double tol_rel, double tol_abs,
                            agb_solve_report* rep, int where) {
    if (!h || !sol || !rhs) return fail(AGB_BAD_ARG, "null argument");
    const size_t bytes = sizeof(double) * 3 * nodes(h);
    const void *dx0 = nullptr, *dr = nullptr;
    TRY(dev_in(h, 0, sol, bytes, where, &dx0));
    TRY(dev_in(h, 1, rhs, bytes, where, &dr));
    agb_status st = solve_dev(h, (double*)dx0, (const double*)dr, tol_rel, tol_abs, rep);
    if (st == AGB_OK || st == AGB_NOT_CONVERGED || st == AGB_NAN) {
        agb_status s2 = finish_out(h, sol, dx0, bytes, where);
        if (s2 != AGB_OK) return s2;
    }
    return st;
}

agb_status agb_newton_solve_n(agb_elastic* h, double* u, const double* b, const double* F0, int f0_ncomp,
                              double tol_rel, double tol_abs, int nriters, double nrtolerance, agb_solve_report* rep,
                              double* relnorm, int where) {
    if (!h || !u || !b) return fail(AGB_BAD_ARG, "null argument");
    if (nriters < 1) return fail(AGB_BAD_ARG, "nriters must be at least 1");
    if (!(f0_ncomp == 0 || f0_ncomp == 1 || f0_ncomp == 9) || (f0_ncomp && !F0))
        return fail(AGB_BAD_ARG, "f0_ncomp must be 0, 1 or 9 (with F0 given)");
    if (!h->model_set) return fail(AGB_NOT_READY, "model not set");
    auto t0 = std::chrono::steady_clock::now();
    const int64_t N = nodes(h);
    const size_t bytes = sizeof(double) * 3 * N;
    const void *du = nullptr, *db = nullptr, *dF = nullptr;
    TRY(dev_in(h, 0, u, bytes, where, &du));
    TRY(dev_in(h, 1, b, bytes, where, &db));
    if (f0_ncomp) TRY(dev_in(h, 3, F0, sizeof(double) * f0_ncomp * N, where, &dF));
    TRY(ensure_io(h, 2, 2 * bytes));
    double* rhs = h->io[2];
    double* dsol = h->io[2] + 3 * N;
    CK(cudaMemsetAsync(dsol, 0, bytes, h->stream));
    agb_status st = AGB_OK;
    double rn = 0.0;
    for (int it = 0; it < nriters; it++) {
        TRY(build_rhs_dev(h, (const double*)du, (const double*)db, (const double*)dF, f0_ncomp, rhs));
        st = solve_dev(h, dsol, rhs, tol_rel, tol_abs, rep, it == 0);
        if (st != AGB_OK && st != AGB_NOT_CONVERGED) return st;
        double n2[2];
        TRY(vec_norms(h, dsol, 3 * N, n2));
        rn = n2[0];
        CK(launch_axpy(1.0, dsol, (double*)du, 3 * N, h->stream));
        h->launches++;
        if (rn < nrtolerance) break;
    }
    if (relnorm) *relnorm = rn;
    agb_status s2 = finish_out(h, u, du, bytes, where);
    if (s2 != AGB_OK) return s2;
    if (rep) rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return st;
}

agb_status agb_newton_solve(agb_elastic* h, double* u, const double* b, const double* F0, int f0_ncomp,
                            double tol_rel, double tol_abs, agb_solve_report* rep, int where) {
    return agb_newton_solve_n(h, u, b, F0, f0_ncomp, tol_rel, tol_abs, 1, 0.0, rep, nullptr, where);
}

// The learned guess on device data: the guess ends in the fine level's cor
// buffer (zero when the fallback fires), the Newton right-hand side at zero
// in io[2] (first 3N doubles); io[2] is scratch, slots 1 and 3 untouched.
static agb_status learned_guess_dev(agb_elastic* h, agb_unet* net, const void* db, const void* dF, int f0_ncomp,
                                    double norms[2], int* used, double** rhs_out) {
    if (h->sym == SYM_MAJ) return fail(AGB_BAD_ARG, "the learned guess takes isotropic or major-minor models");
    const int ng = unet_grid(net);
    int lg = -1;
    for (int l = 0; l < (int)h->L64.size(); l++) {
        const LevelGeom<double>& G = h->L64[l].G;
        if (G.nx == ng && G.ny == ng && G.nz == ng) { lg = l; break; }
    }
    if (lg < 0) return fail(AGB_BAD_ARG, "no multigrid level of the handle has the network's grid");
    const int64_t N = nodes(h);
    const size_t bytes = sizeof(double) * 3 * N;
    // features on the fine level, restricted to the network's level (the
    // levels' rescor buffers are free outside a solve); prediction in cor
    std::vector<Lev<double>>& L = h->L64;
    CK(launch_guess_features(h->sym, L[0].C, N, (const double*)dF, f0_ncomp, L[0].rescor, h->stream));
    for (int l = 0; l < lg; l++) CK(launch_restrict<double>(L[l].rescor, L[l].G, L[l + 1].rescor, L[l + 1].G, h->stream));
    h->launches += 1 + lg;
    TRY(unet_predict_dev(net, L[lg].rescor, L[lg].cor, h->stream));
    for (int l = lg - 1; l >= 0; l--) {
        CK(cudaMemsetAsync(L[l].cor, 0, sizeof(double) * 3 * L[l].G.N, h->stream));
        CK(launch_prolong_add<double>(L[l + 1].cor, L[l + 1].G, L[l].cor, L[l].G, h->stream));
        h->launches++;
    }
    // the linear system of the Newton step from zero: A x = rhs0,
    // rhs0 = b - (interior: div of the stress of F0; boundary: BC rows at 0)
    TRY(ensure_io(h, 2, 2 * bytes));
    double* rhs0 = h->io[2];
    double* rg = h->io[2] + 3 * N;
    TRY(build_rhs_dev(h, nullptr, (const double*)db, (const double*)dF, f0_ncomp, rhs0));
    // fallback test: rhs0 - A x at the guess against rhs0 (x = 0), both
    // restricted to the network's level -- the smooth part of the residual,
    // which the cycles reduce slowly and a coarse guess can reduce; the
    // smoother removes the rest in a sweep or two
    auto coarse_norms = [&](const double* src, double out[2]) -> agb_status {
        for (int l = 0; l < lg; l++) {
            CK(launch_restrict<double>(src, L[l].G, L[l + 1].res, L[l + 1].G, h->stream));
            src = L[l + 1].res;
        }
        h->launches += lg;
        return vec_norms(h, src, 3 * L[lg].G.N, out);
    };
    double ng_[2], nz_[2];
    if (h->opts.precision == AGB_PRECISION_MIXED) {
        // the test is a heuristic: the FP32 residual kernels (a 20th of the
        // FP64 residual's time on a major-minor model) are accurate enough
        TRY(ensure_f32(h));
        std::vector<Lev<float>>& F = h->L32;
        Lev<float>& f = F[0];
        CK(launch_from_double<float>(L[0].cor, f.cor, 3 * N, 1.0, h->stream));
        CK(launch_from_double<float>(rhs0, f.res, 3 * N, 1.0, h->stream));
        if (use_zm<float>(h, f, 0)) CK(level_zm<float>(h, f, 2, f.cor, f.res, nullptr, 0.f, f.rescor));
        else CK(launch_residual<float>(h->sym, f.cor, f.res, f.C, f.G, h->bc, f.rescor, nullptr, nullptr, h->stream));
        const float* src = f.rescor;
        for (int l = 0; l < lg; l++) {
            CK(launch_restrict<float>(src, F[l].G, F[l + 1].res, F[l + 1].G, h->stream));
            src = F[l + 1].res;
        }
        const int64_t nc = 3 * L[lg].G.N;
        CK(cudaMemsetAsync(L[lg].res, 0, sizeof(double) * nc, h->stream));
        CK(launch_axpy_to_double<float>(src, L[lg].res, nc, 1.0, h->stream));
        h->launches += 5 + lg;
        TRY(vec_norms(h, L[lg].res, nc, ng_));
    } else {
        CK(launch_residual<double>(h->sym, L[0].cor, rhs0, L[0].C, L[0].G, h->bc, rg, nullptr, nullptr, h->stream));
        h->launches++;
        TRY(coarse_norms(rg, ng_));
    }
    TRY(coarse_norms(rhs0, nz_));
    const bool ok = std::isfinite(ng_[1]) && ng_[1] <= nz_[1];
    if (norms) { norms[0] = ng_[1]; norms[1] = nz_[1]; }
    if (used) *used = ok ? 1 : 0;
    if (!ok) CK(cudaMemsetAsync(L[0].cor, 0, bytes, h->stream));
    *rhs_out = rhs0;
    return AGB_OK;
}

static agb_status check_guess_args(agb_elastic* h, agb_unet* net, const double* b, const double* u, const double* F0,
                                   int f0_ncomp) {
    if (!h || !net || !b || !u) return fail(AGB_BAD_ARG, "null argument");
    if (!(f0_ncomp == 0 || f0_ncomp == 1 || f0_ncomp == 9) || (f0_ncomp && !F0))
        return fail(AGB_BAD_ARG, "f0_ncomp must be 0, 1 or 9 (with F0 given)");
    if (!h->model_set) return fail(AGB_NOT_READY, "model not set");
    return AGB_OK;
}

agb_status agb_elastic_learned_guess(agb_elastic* h, agb_unet* net, const double* b, const double* F0, int f0_ncomp,
                                     double* u, double* rhs, double norms[2], int* used, int where) {
    TRY(check_guess_args(h, net, b, u, F0, f0_ncomp));
    const int64_t N = nodes(h);
    const size_t bytes = sizeof(double) * 3 * N;
    const void *db = nullptr, *dF = nullptr;
    TRY(dev_in(h, 1, b, bytes, where, &db));
    if (f0_ncomp) TRY(dev_in(h, 3, F0, sizeof(double) * f0_ncomp * N, where, &dF));
    double* rhs0 = nullptr;
    TRY(learned_guess_dev(h, net, db, dF, f0_ncomp, norms, used, &rhs0));
    const cudaMemcpyKind kind = where == AGB_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    CK(cudaMemcpyAsync(u, h->L64[0].cor, bytes, kind, h->stream));
    if (rhs) CK(cudaMemcpyAsync(rhs, rhs0, bytes, kind, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return AGB_OK;
}

agb_status agb_newton_solve_guess(agb_elastic* h, agb_unet* net, double* u, const double* b, const double* F0,
                                  int f0_ncomp, double tol_rel, double tol_abs, agb_solve_report* rep, int* used,
                                  int where) {
    TRY(check_guess_args(h, net, b, u, F0, f0_ncomp));
    auto t0 = std::chrono::steady_clock::now();
    const int64_t N = nodes(h);
    const size_t bytes = sizeof(double) * 3 * N;
    const void *db = nullptr, *dF = nullptr;
    void* du = nullptr;
    TRY(dev_in(h, 1, b, bytes, where, &db));
    if (f0_ncomp) TRY(dev_in(h, 3, F0, sizeof(double) * f0_ncomp * N, where, &dF));
    TRY(dev_out(h, 0, u, bytes, where, &du));
    double* rhs0 = nullptr;
    int ok = 0;
    TRY(learned_guess_dev(h, net, db, dF, f0_ncomp, nullptr, &ok, &rhs0));
    if (used) *used = ok;
    CK(cudaMemcpyAsync(du, h->L64[0].cor, bytes, cudaMemcpyDeviceToDevice, h->stream));
    // a kept guess's FP32 residual (the fallback test's) starts the mixed
    // refinement; the FP64 residuals after each inner solve decide
    const float* r32 = (ok && h->opts.precision == AGB_PRECISION_MIXED) ? h->L32[0].rescor : nullptr;
    const agb_status st = solve_dev(h, (double*)du, rhs0, tol_rel, tol_abs, rep, ok == 0, r32, true);
    if (st != AGB_OK && st != AGB_NOT_CONVERGED) return st;
    TRY(finish_out(h, u, du, bytes, where));
    if (rep) rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return st;
}

agb_status agb_elastic_stress_strain(agb_elastic* h, const double* u, const double* F0, int f0_ncomp, double* stress,
                                     double* strain, double* energy, int where) {
    if (!h || !u) return fail(AGB_BAD_ARG, "null argument");
    if (!(f0_ncomp == 0 || f0_ncomp == 1 || f0_ncomp == 9) || (f0_ncomp && !F0))
        return fail(AGB_BAD_ARG, "f0_ncomp must be 0, 1 or 9 (with F0 given)");
    if (!h->model_set) return fail(AGB_NOT_READY, "model not set");
    const int64_t N = nodes(h);
    const void *du = nullptr, *dF = nullptr;
    TRY(dev_in(h, 0, u, sizeof(double) * 3 * N, where, &du));
    if (f0_ncomp) TRY(dev_in(h, 3, F0, sizeof(double) * f0_ncomp * N, where, &dF));
    double *ds = nullptr, *de = nullptr, *den = nullptr;
    if (where == AGB_MEM_DEVICE) {
        ds = stress; de = strain; den = energy;
    } else {
        if (!h->dw) CK(cudaMalloc(&h->dw, sizeof(double) * 9 * N));
        TRY(ensure_io(h, 1, sizeof(double) * 10 * N));
        ds = stress ? h->dw : nullptr;
        de = strain ? h->io[1] : nullptr;
        den = energy ? h->io[1] + 9 * N : nullptr;
    }
    CK(launch_stress_strain(h->sym, (const double*)du, (const double*)dF, f0_ncomp, h->L64[0].C, h->L64[0].G, ds, de,
                            den, h->stream));
    h->launches++;
    if (where == AGB_MEM_HOST) {
        if (stress) CK(cudaMemcpyAsync(stress, ds, sizeof(double) * 9 * N, cudaMemcpyDeviceToHost, h->stream));
        if (strain) CK(cudaMemcpyAsync(strain, de, sizeof(double) * 9 * N, cudaMemcpyDeviceToHost, h->stream));
        if (energy) CK(cudaMemcpyAsync(energy, den, sizeof(double) * N, cudaMemcpyDeviceToHost, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    return AGB_OK;
}

agb_status agb_newton_solve_neohookean(agb_elastic* h, const double* model, double* u, const double* b,
                                       double tol_rel, double tol_abs, int nriters, double nrtolerance,
                                       agb_solve_report* rep, double* relnorm, int where) {
    if (!h || !model || !u || !b) return fail(AGB_BAD_ARG, "null argument");
    if (h->sym != SYM_MAJ) return fail(AGB_BAD_ARG, "the NeoHookean tangent needs a handle of AGB_SYM_MAJOR");
    if (nriters < 1) return fail(AGB_BAD_ARG, "nriters must be >= 1");
    auto t0 = std::chrono::steady_clock::now();
    const int64_t N = nodes(h);
    const size_t bytes = sizeof(double) * 3 * N;
    const void *dm = nullptr, *db = nullptr;
    void* du = nullptr;
    // the model as (mu, kappa) SoA, kept on the handle
    TRY(dev_in(h, 3, model, sizeof(double) * 2 * N, where, &dm));
    if (!h->nh_model) CK(cudaMalloc(&h->nh_model, sizeof(double) * 2 * N));
    CK(launch_aos_to_soa((const double*)dm, h->nh_model, N, 2, h->stream));
    TRY(dev_in(h, 1, b, bytes, where, &db));
    TRY(dev_out(h, 0, u, bytes, where, &du));
    if (where == AGB_MEM_HOST) CK(cudaMemcpyAsync(du, u, bytes, cudaMemcpyHostToDevice, h->stream));
    if (!h->dw) CK(cudaMalloc(&h->dw, sizeof(double) * 9 * N));
    TRY(ensure_io(h, 2, 2 * bytes));
    double* rhs = h->io[2];
    double* dsol = h->io[2] + 3 * N;
    agb_status st = AGB_OK;
    double rn = 0.0;
    for (int it = 0; it < nriters; it++) {
        // DW and DDW at F = I + grad u; DDW is the operator's stiffness
        // (Newton.H:193, Elastic::SetModel) and every level is rebuilt
        CK(launch_neohookean(h->nh_model, (const double*)du, h->L64[0].G, h->dw, h->L64[0].C, h->stream));
        h->model_set = true;
        h->prepared = false;
        h->have_f32 = false;
        h->have_df = false;
        h->bot_src = 0;
        CK(launch_rhs_from_dw((const double*)du, (const double*)db, h->dw, h->L64[0].G, h->bc, rhs, h->stream));
        h->launches += 2;
        CK(cudaMemsetAsync(dsol, 0, bytes, h->stream));
        st = solve_dev(h, dsol, rhs, tol_rel, tol_abs, rep, true);
        if (st != AGB_OK && st != AGB_NOT_CONVERGED) return st;
        double n2[2];
        TRY(vec_norms(h, dsol, 3 * N, n2));
        rn = n2[0];
        CK(launch_axpy(1.0, dsol, (double*)du, 3 * N, h->stream));
        h->launches++;
        if (rn < nrtolerance) break;
    }
    if (relnorm) *relnorm = rn;
    TRY(finish_out(h, u, du, bytes, where));
    if (rep) rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return st;
}

agb_status agb_elastic_tensor(agb_elastic* h, const double* u, int which, int voigt, double* out, int where) {
    if (!h || !u || !out) return fail(AGB_BAD_ARG, "null argument");
    if (which != 0 && which != 1) return fail(AGB_BAD_ARG, "which must be 0 (stress) or 1 (strain)");
    if (!h->model_set) return fail(AGB_NOT_READY, "model not set");
    const int64_t N = nodes(h);
    const size_t ob = sizeof(double) * (voigt ? 6 : 9) * N;
    const void* du = nullptr;
    void* dout = nullptr;
    TRY(dev_in(h, 0, u, sizeof(double) * 3 * N, where, &du));
    TRY(dev_out(h, 1, out, ob, where, &dout));
    CK(launch_op_tensor(h->sym, (const double*)du, h->L64[0].C, h->L64[0].G, which, voigt ? 1 : 0, (double*)dout,
                        h->stream));
    h->launches++;
    return finish_out(h, out, dout, ob, where);
}

agb_status agb_profile_enable(agb_elastic* h, int on) {
    if (!h) return fail(AGB_BAD_ARG, "null handle");
    h->prof = on != 0;
    return AGB_OK;
}

agb_status agb_profile_reset(agb_elastic* h) {
    if (!h) return fail(AGB_BAD_ARG, "null handle");
    prof_collect(h);
    for (int f = 0; f < AGB_K_NFAMILIES; f++) { h->prof_count[f] = 0; h->prof_ms[f] = 0.0; h->prof_bytes[f] = 0.0; }
    return AGB_OK;
}

agb_status agb_profile_bytes(agb_elastic* h, int family, double* bytes) {
    if (!h || !bytes || family < 0 || family >= AGB_K_NFAMILIES) return fail(AGB_BAD_ARG, "bad argument");
    *bytes = h->prof_bytes[family];
    return AGB_OK;
}

agb_status agb_profile_get(agb_elastic* h, int family, int64_t* launches, double* ms) {
    if (!h || family < 0 || family >= AGB_K_NFAMILIES) return fail(AGB_BAD_ARG, "bad argument");
    prof_collect(h);
    if (launches) *launches = h->prof_count[family];
    if (ms) *ms = h->prof_ms[family];
    return AGB_OK;
}

agb_status agb_launch_count(agb_elastic* h, int64_t* n) {
    if (!h || !n) return fail(AGB_BAD_ARG, "null argument");
    *n = h->launches;
    return AGB_OK;
}

const char* agb_status_string(int s) {
    switch (s) {
        case AGB_OK: return "AGB_OK";
        case AGB_NOT_CONVERGED: return "AGB_NOT_CONVERGED";
        case AGB_NAN: return "AGB_NAN";
        case AGB_BAD_ARG: return "AGB_BAD_ARG";
        case AGB_CUDA_ERROR: return "AGB_CUDA_ERROR";
        case AGB_NOT_READY: return "AGB_NOT_READY";
        case AGB_OUT_OF_MEMORY: return "AGB_OUT_OF_MEMORY";
        case AGB_LIMIT: return "AGB_LIMIT";
        default: return "AGB_UNKNOWN";
    }
}

const char* agb_last_error(void) { return g_last_error.c_str(); }

const char* agb_version(void) { return "alamo_gb300 0.1 (sm_103a)"; }

}  // extern "C"

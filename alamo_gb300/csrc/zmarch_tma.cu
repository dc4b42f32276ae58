// FP32 stencil kernels of the multigrid levels with the stiffness staged by
// TMA.
//
// A 32 x 8 thread block marches its tile of interior columns (nodes 1..n-2 in
// x and y, so the 255 interior columns of a 257-node axis fill 8 tiles of 32
// exactly) through a chunk of z-planes.  Per plane it needs
//   * the displacement of planes k-1, k, k+1 with a one-node x/y halo
//     (3 x 10 x 34 values): a 4-slot ring filled by 4-byte cp.async, plane
//     k+2 issued at the top of step k;
//   * the stiffness of plane k with the x/y halo (for the in-plane
//     derivatives of C) and of plane k+1 at the block's own columns (for
//     the z-derivative): a 3-slot ring of TMA boxes (36 x 10 nodes x NC
//     entries), plane k+2 issued at the top of step k into the slot plane
//     k-1 has left.
// In the major-minor kernel, what a column needs again one plane later
// stays in its registers: the own-column stiffness of planes k-1 and k, and
// the displacement of planes k-1 and k at the column and its four in-plane
// axis neighbours.  A step then reads from shared memory the stiffness of
// plane k at the four in-plane neighbours and of plane k+1 at the column,
// plane k+1's five displacement points and plane k's four in-plane
// diagonals: 108 values per node instead of 153, at offsets that are
// compile-time constants.  The isotropic kernel carries only the own-column
// stiffness of plane k-1.  Each array is read from HBM about once per sweep.
// The six boundary faces (2.3% of the nodes at 257^3) run in a second, thin
// kernel: inside the marching blocks their branchy rows held
// every step of the edge tiles back at the block barrier.  The TMA box
// starts at x = x0 - 1 = 32 * blockIdx.x, a multiple of 4 floats (16 bytes);
// the stiffness copy it reads has its x pitch padded to a multiple of 4
// floats so every global stride is a multiple of 16 bytes.
//
// Every wait on an mbarrier is bounded: after the limit the block records
// the failure in *err, stops marching (uniformly, through a shared flag),
// waits (bounded) for its TMA copies still in flight and returns.
//
// Epilogues: FAPPLY out = A x; JACOBI one damped-Jacobi sweep, written as
// x + omega (b - A x) / diag with the inverse diagonal (the reference's
// (1 - omega) x + omega (b - (A x - x diag)) / diag rearranged: one multiply
// instead of a division per component in this FP32 preconditioner); RESIDUAL
// out = b - A x.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>

#include "agb_launch.h"
#include "operator.cuh"
#include "zmarch_tma.h"

namespace agb {

namespace {

constexpr int TX = 32, TY = 8, NT = TX * TY;
constexpr int UHX = TX + 2, UHY = TY + 2;
constexpr int UPL = 3 * UHY * UHX;                // displacement values per staged plane
constexpr int U_PER_T = (UPL + NT - 1) / NT;      // cp.async per thread per plane
constexpr int CBX = 36, CBY = 10;                 // TMA box (x, y) of a stiffness plane
constexpr int CEL = CBX * CBY;                    // floats per stiffness entry in a slot
constexpr uint64_t WAIT_NS = 1000000000ull;       // 1 s: a TMA load takes microseconds

// Prefetch distance and ring sizes.  Step k reads planes k and k+1 (plane
// k-1 is in registers), and issues plane k+1+DIST; plane k+DIST must have landed before step k+1.  The isotropic
// planes are small (2 stiffness entries), so one plane of work does not
// cover a load's latency: they look two planes ahead.  The major-minor
// planes (21 entries) cover it with one, and two would not fit two blocks
// per SM in shared memory.
template <int NC>
struct ZtSmem {
    static constexpr int DIST = NC <= 2 ? 2 : 1;
    static constexpr int CS = 2 + DIST;   // stiffness ring slots
    static constexpr int US = 3 + DIST;   // displacement ring slots
    static constexpr int slot_bytes = ((NC * CEL * 4 + 127) / 128) * 128;
    static constexpr int c_bytes = CS * slot_bytes;
    static constexpr int u_bytes = US * UPL * 4;
    static constexpr int bar_off = c_bytes + u_bytes;
    static constexpr int total = bar_off + CS * 8 + 128;  // + alignment slack
    static constexpr uint32_t box_bytes = NC * CEL * 4;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
// true once the phase of the given parity has completed; false when it has
// not completed within WAIT_NS (each try_wait returns after at most a short
// hardware time limit, so the loop ends)
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    uint64_t t0 = 0;
    for (int it = 0;; it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (it == 0) t0 = global_ns();
        else if (global_ns() - t0 > WAIT_NS) return false;
    }
}
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int x, int y, int z, int e,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(e), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void cp_async4(uint32_t dst, const float* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
// wait until at most N of this thread's most recent cp.async groups are pending
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// isotropic: three blocks per SM (at most 85 registers), major-minor: two
template <int SYM, int MODE>
__global__ void __launch_bounds__(NT, SYM == SYM_ISO ? 3 : 2)
    k_zmarch_tma(const __grid_constant__ CUtensorMap cmap, const float* __restrict__ x, LevelGeom<float> G,
                 const float* __restrict__ b, const float* __restrict__ dg, float omega, float* __restrict__ out,
                 int kchunk, int* __restrict__ err) {
    constexpr int NC = SYM == SYM_ISO ? 2 : 21;
    using SM = ZtSmem<NC>;
    constexpr int CS = SM::CS, US = SM::US, DIST = SM::DIST;
    extern __shared__ unsigned char zt_raw[];
    __shared__ int abort_flag;
    const uint32_t raw = smem_u32(zt_raw);
    const uint32_t pad = ((raw + 127u) & ~127u) - raw;
    unsigned char* sm = zt_raw + pad;
    float* Cs = reinterpret_cast<float*>(sm);
    float* Us = reinterpret_cast<float*>(sm + SM::c_bytes);
    const uint32_t cs_u32 = raw + pad;
    const uint32_t us_u32 = cs_u32 + SM::c_bytes;
    const uint32_t bar_u32 = cs_u32 + SM::bar_off;

    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    const int x0 = 1 + blockIdx.x * TX, y0 = 1 + blockIdx.y * TY;
    const int k0 = 1 + blockIdx.z * kchunk;
    const int k1 = min(k0 + kchunk, G.nz - 1);
    const int i = x0 + tx, j = y0 + ty;
    const bool col = (i <= G.nx - 2) & (j <= G.ny - 2);
    const int64_t N = G.N, sy = G.sy, sz = G.sz;

    // this thread's share of a staged displacement plane
    int soff[U_PER_T];
    int64_t goff[U_PER_T];
    bool gval[U_PER_T];
#pragma unroll
    for (int r = 0; r < U_PER_T; r++) {
        const int q = tid + r * NT;
        const int p = q / (UHY * UHX), rem = q - p * (UHY * UHX), yy = rem / UHX, xx = rem - yy * UHX;
        const int gx = x0 - 1 + xx, gy = y0 - 1 + yy;
        soff[r] = q;
        gval[r] = (q < UPL) & (gx < G.nx) & (gy < G.ny);
        goff[r] = p * N + gx + sy * gy;
    }
    // one commit group per call (planes past the chunk commit an empty
    // group, so "the DIST-1 most recent groups" always means the planes
    // issued after the one waited for)
    // plane kk into ring slot su (displacement) / s (stiffness)
    auto issue_u_at = [&](int kk, int su, bool real) {
        const uint32_t dst = us_u32 + (uint32_t)(su * UPL) * 4u;
        if (real) {
            const float* xk = x + sz * (int64_t)kk;
#pragma unroll
            for (int r = 0; r < U_PER_T; r++)
                if (gval[r]) cp_async4(dst + soff[r] * 4u, xk + goff[r]);
        }
        cp_async_commit();
    };
    auto issue_u = [&](int kk, bool real) { issue_u_at(kk, kk % US, real); };
    auto issue_c_at = [&](int kk, int s) {  // one thread
        mbar_expect_tx(bar_u32 + 8u * s, SM::box_bytes);
        tma_load_4d(cs_u32 + (uint32_t)(s * SM::slot_bytes), &cmap, TX * blockIdx.x, TY * blockIdx.y, kk, 0,
                    bar_u32 + 8u * s);
    };
    auto issue_c = [&](int kk) { issue_c_at(kk, kk % CS); };
    // plane kk is the n-th load into its slot, n = (kk - (k0 - 1)) / CS
    auto parity = [&](int kk) { return (uint32_t)(((kk - (k0 - 1)) / CS) & 1); };
    auto cslot = [&](int kk) { return Cs + (kk % CS) * (SM::slot_bytes / 4) + (ty + 1) * CBX + (tx + 1); };

    if (tid == 0) {
        abort_flag = 0;
        for (int s = 0; s < CS; s++) mbar_init(bar_u32 + 8u * s, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    // planes k0-1 .. k0+DIST (plane k0+DIST only if the chunk reaches it)
    int issued = k0 + 1;  // last plane issued (thread 0 uses it on abort)
    if (tid == 0) {
        issue_c(k0 - 1);
        issue_c(k0);
        issue_c(k0 + 1);
    }
    issue_u(k0 - 1, true);
    issue_u(k0, true);
    issue_u(k0 + 1, true);
#pragma unroll
    for (int d = 2; d <= DIST; d++) {
        const bool real = k0 + d <= k1;
        if (real) {
            if (tid == 0) issue_c(k0 + d);
            issued = k0 + d;
        }
        issue_u(k0 + d, real);
    }

    // one thread waits for the stiffness planes (the block barrier then
    // orders everyone's reads after the completed copies); no thread polls
    // while others compute
    if (tid == 0) {
        const bool ok = mbar_wait(bar_u32 + 8u * ((k0 - 1) % CS), parity(k0 - 1)) &&
                        mbar_wait(bar_u32 + 8u * (k0 % CS), parity(k0)) &&
                        mbar_wait(bar_u32 + 8u * ((k0 + 1) % CS), parity(k0 + 1));
        if (!ok) {
            abort_flag = 1;
            if (err) atomicExch(err, 1);
        }
    }
    cp_async_wait_group<DIST - 1>();
    __syncthreads();
    // carried from step to step in registers: the own column's stiffness of
    // plane k-1 and, in the major-minor kernel (ZC), of plane k and the
    // displacement of planes k-1 and k at the column and its four in-plane
    // axis neighbours (each step then reads plane k+1's five points and
    // plane k's four in-plane diagonals).  Measured at 257^3: +1.3 % on the
    // major-minor sweep, whose 21 stiffness entries dominate the shared
    // loads; -1.3 % on the isotropic one, which is issue bound and pays
    // more for the register copies than it saves in loads.
    constexpr bool ZC = SYM == SYM_MM;
    constexpr int PL = UHY * UHX;
    float Cp[NC], Cc[NC], Um[3][5], Uc[3][5];
    auto load5 = [&](const float* s, float v[3][5]) {
#pragma unroll
        for (int p = 0; p < 3; p++) {
            v[p][0] = s[p * PL];
            v[p][1] = s[p * PL + 1];
            v[p][2] = s[p * PL - 1];
            v[p][3] = s[p * PL + UHX];
            v[p][4] = s[p * PL - UHX];
        }
    };
    {
        const float* c = cslot(k0 - 1);
        const float* cz = cslot(k0);
#pragma unroll
        for (int e = 0; e < NC; e++) {
            Cp[e] = c[e * CEL];
            Cc[e] = cz[e * CEL];
        }
        if (ZC) {
            const int o = (ty + 1) * UHX + (tx + 1);
            load5(Us + ((k0 - 1) % US) * UPL + o, Um);
            load5(Us + (k0 % US) * UPL + o, Uc);
        }
    }
    // the first step reloads the slot of plane k0 - 1: everyone has read it
    __syncthreads();

    // right-hand side and diagonal of the own column, loaded one plane ahead
    // so their latency hides behind a whole step
    float bq[3] = {0.f, 0.f, 0.f}, dq[3] = {1.f, 1.f, 1.f};
    auto load_bd = [&](int kk, float bb[3], float dd[3]) {
        if (col && kk < k1) {
            const int64_t idk = i + sy * j + sz * (int64_t)kk;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                if (MODE >= 1) bb[c] = b[c * N + idk];
                if (MODE == 1) dd[c] = dg[c * N + idk];
            }
        }
    };
    load_bd(k0, bq, dq);

    // ring slots advance by one per step.  The major-minor kernel keeps them
    // as counters (plane k's slots su (displacement) and sc (stiffness), the
    // slot and mbarrier parity of plane k+2, the plane waited for) -- 1 %
    // faster; the isotropic kernel measured faster with the modulo
    // expressions (fewer live registers), so it recomputes them per step.
    constexpr bool RC = SYM == SYM_MM;
    auto wrap = [](int v, int n) { return v >= n ? v - n : v; };
    int su = k0 % US, sc = k0 % CS;
    int sw = (k0 + 2) % CS;
    uint32_t pw = parity(k0 + 2);
    const int sbase = (k0 - 1) % CS;  // a slot's load count grows when the plane index passes it
    const int o = (ty + 1) * UHX + (tx + 1);
    const int oc = (ty + 1) * CBX + (tx + 1);
    for (int k = k0; k < k1 && !abort_flag; k++) {
        if (!RC) {
            su = k % US;
            sc = k % CS;
            sw = (k + 2) % CS;
            pw = parity(k + 2);
        }
        {
            const int kn = k + 1 + DIST;
            const bool real = kn <= k1;
            if (real) {
                if (tid == 0) {
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    issue_c_at(kn, wrap(sc + 1 + DIST, CS));
                }
                issued = kn;
            }
            issue_u_at(kn, wrap(su + 1 + DIST, US), real);
        }
        const int64_t id = i + sy * j + sz * (int64_t)k;
        float bn[3] = {0.f, 0.f, 0.f}, dn[3] = {1.f, 1.f, 1.f};
        load_bd(k + 1, bn, dn);
        const float* cc = Cs + sc * (SM::slot_bytes / 4) + oc;
        if (col) {
            const float* cn = Cs + wrap(sc + 1, CS) * (SM::slot_bytes / 4) + oc;
            const float* u0 = Us + su * UPL + o;
            const float* um = Us + wrap(su + US - 1, US) * UPL + o;
            const float* up = Us + wrap(su + 1, US) * UPL + o;
            // ZC: plane k+1's five points (kept for the next step), every
            // stiffness entry of its own column (the next step's centre) and
            // plane k's in-plane diagonals; otherwise the own column of plane
            // k, and the displacement is read where the stencil needs it
            float Up[3][5], Cn[NC], Ud[3][4];
            if (ZC) {
                load5(up, Up);
#pragma unroll
                for (int e = 0; e < NC; e++) Cn[e] = cn[e * CEL];
#pragma unroll
                for (int p = 0; p < 3; p++) {
                    Ud[p][0] = u0[p * PL + UHX + 1];
                    Ud[p][1] = u0[p * PL - UHX - 1];
                    Ud[p][2] = u0[p * PL - UHX + 1];
                    Ud[p][3] = u0[p * PL + UHX - 1];
                }
            } else {
#pragma unroll
                for (int e = 0; e < NC; e++) Cc[e] = cc[e * CEL];
            }
            // (a, bb) with at most one non-zero: 0 centre, 1 +x, 2 -x, 3 +y, 4 -y;
            // both non-zero: the diagonals (1,1), (-1,-1), (1,-1), (-1,1)
            auto U = [&](int p, int a, int bb, int c) -> float {
                if (!ZC) {
                    const float* s = c == 0 ? u0 : (c < 0 ? um : up);
                    return s[p * PL + bb * UHX + a];
                }
                const int q5 = a == 1 ? 1 : (a == -1 ? 2 : (bb == 1 ? 3 : (bb == -1 ? 4 : 0)));
                if (c < 0) return Um[p][q5];
                if (c > 0) return Up[p][q5];
                if (a != 0 && bb != 0) return Ud[p][a == bb ? (a > 0 ? 0 : 1) : (a > 0 ? 2 : 3)];
                return Uc[p][q5];
            };
            auto Cf = [&](int e, int a, int bb, int c) -> float {
                if (c > 0) return ZC ? Cn[e] : cn[e * CEL];
                if (c < 0) return Cp[e];
                if (a == 0 && bb == 0) return Cc[e];
                return cc[e * CEL + bb * CBX + a];
            };
            float r[3];
            interior_rows<float, SYM>(U, Cf, G, r);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const int64_t q = c * N + id;
                if (MODE == 0) {
                    out[q] = r[c];
                } else if (MODE == 1) {
                    const float xv = ZC ? Uc[c][0] : u0[c * PL];
                    out[q] = xv + omega * (bq[c] - r[c]) * dq[c];
                } else {
                    out[q] = bq[c] - r[c];
                }
            }
#pragma unroll
            for (int e = 0; e < NC; e++) {
                Cp[e] = Cc[e];
                if (ZC) Cc[e] = Cn[e];
            }
            if (ZC) {
#pragma unroll
                for (int p = 0; p < 3; p++)
#pragma unroll
                    for (int q = 0; q < 5; q++) {
                        Um[p][q] = Uc[p][q];
                        Uc[p][q] = Up[p][q];
                    }
            }
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
            bq[c] = bn[c];
            dq[c] = dn[c];
        }
        // plane k+2 (read by step k+1) must have landed; the DIST-1 newer
        // planes may still be in flight
        cp_async_wait_group<DIST - 1>();
        if (tid == 0 && k + 2 <= k1 && !mbar_wait(bar_u32 + 8u * sw, pw)) {
            abort_flag = 1;
            if (err) atomicExch(err, 1);
        }
        __syncthreads();
        if (RC) {
            su = wrap(su + 1, US);
            sc = wrap(sc + 1, CS);
            sw = wrap(sw + 1, CS);
            if (sw == sbase) pw ^= 1u;
        }
    }
    cp_async_wait_all();
    if (abort_flag && tid == 0) {
        // bounded wait for the TMA loads still in flight (at most the
        // latest load of each slot) before the block gives its shared
        // memory back
        for (int kk = max(issued - (CS - 1), k0 - 1); kk <= issued; kk++)
            mbar_wait(bar_u32 + 8u * (kk % CS), parity(kk));
    }
}

// Boundary faces: blockIdx.z picks the face (z = 0, z = nz-1, y = 0,
// y = ny-1, x = 0, x = nx-1) and a 32 x 8 thread tile covers its two free
// coordinates, the contiguous one across the warp where the face has one
// (the x faces are strided in memory whatever the mapping).  Edges and
// corners belong to the z faces, then to the y faces.  32-bit index
// arithmetic; the boundary-type table is copied to shared memory with
// constant offsets so no thread keeps a local copy of the parameter.
template <int SYM, int MODE>
__global__ void __launch_bounds__(256) k_zt_faces(const float* __restrict__ x, const float* __restrict__ C,
                                                  LevelGeom<float> G, BcTable bc, const float* __restrict__ b,
                                                  const float* __restrict__ dg, float omega,
                                                  float* __restrict__ out) {
    __shared__ unsigned char sbt[80];
    if (threadIdx.x == 0 && threadIdx.y == 0) {
#pragma unroll
        for (int q = 0; q < 78; q++) sbt[q] = bc.t[q];
    }
    __syncthreads();
    const int f = blockIdx.z;
    const int a = blockIdx.x * TX + threadIdx.x, c2 = blockIdx.y * TY + threadIdx.y;
    int i, j, k;
    if (f < 2) {
        i = a; j = c2; k = f == 0 ? 0 : G.nz - 1;
        if (i >= G.nx || j >= G.ny) return;
    } else if (f < 4) {
        i = a; k = 1 + c2; j = f == 2 ? 0 : G.ny - 1;
        if (i >= G.nx || k > G.nz - 2) return;
    } else {
        j = 1 + a; k = 1 + c2; i = f == 4 ? 0 : G.nx - 1;
        if (j > G.ny - 2 || k > G.nz - 2) return;
    }
    const int64_t N = G.N, sy = G.sy, sz = G.sz;
    const int64_t id = i + sy * j + sz * (int64_t)k;
    auto U = [&](int p, int da, int db, int dc) { return x[p * N + id + da + sy * db + sz * dc]; };
    auto cf = [&](int e) { return C[e * N + id]; };
    float r[3];
    boundary_rows<float, SYM>(U, cf, G, sbt, i, j, k, r);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const int64_t q = c * N + id;
        if (MODE == 0) {
            out[q] = r[c];
        } else if (MODE == 1) {
            const float xv = x[q];
            out[q] = xv + omega * (b[q] - r[c]) * dg[q];
        } else {
            out[q] = b[q] - r[c];
        }
    }
}

// FP32 stiffness, SoA (nc, nz, ny, nx) -> padded (nc, nz, ny, px), zero pad
__global__ void k_pad_planes(const float* __restrict__ src, float* __restrict__ dst, int nx, int px, int64_t rows) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < rows * px;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = t / px;
        const int xx = (int)(t - row * px);
        dst[t] = xx < nx ? src[row * nx + xx] : 0.f;
    }
}

// planes per block (the z-chunk): the chunk that minimises
//   ceil(W) / W * (kc + 2) / kc,   W = blocks / (152 * blocks per SM),
// the idle share of a last, partial wave of blocks times the two extra
// planes every chunk stages; chunks of 4 to 64 planes.  (257^3 major-minor:
// 37 planes, 7 chunks, 5.9 waves; 129^3: 15 planes, 9 chunks, 1.9 waves.)
int zt_kchunk(int ni, int nj, int nk, int per_sm) {
    const int64_t tiles = (int64_t)((ni + TX - 1) / TX) * ((nj + TY - 1) / TY);
    const double slots = 152.0 * per_sm;
    int best = 4;
    double best_cost = 1e300;
    for (int kc = 4; kc <= 64; kc++) {
        const int chunks = (nk + kc - 1) / kc;
        if (kc > 4 && (nk + kc - 2) / (kc - 1) == chunks) continue;  // same chunks, more planes each
        const double w = (double)(tiles * chunks) / slots;
        const double cost = std::ceil(w) / w * (kc + 2.0) / kc;
        if (cost < best_cost - 1e-12) {
            best_cost = cost;
            best = kc;
        }
    }
    return best;
}

}  // namespace

bool zmarch_tma_supported(int nx, int ny, int nz) {
    // an interior on every axis; 32-bit TMA coordinates
    return nx >= 3 && ny >= 3 && nz >= 3 && nx < (1 << 30) && ny < (1 << 30) && nz < (1 << 30);
}

int64_t zmarch_tma_pitch(int nx) { return (nx + 3) / 4 * 4; }

cudaError_t make_stiffness_map(const float* Cpad, int nx, int ny, int nz, int nc, CUtensorMap* map) {
    using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static EncodeFn encode = nullptr;
    if (!encode) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess) return e;
        if (q != cudaDriverEntryPointSuccess || !fn) return cudaErrorSymbolNotFound;
        encode = reinterpret_cast<EncodeFn>(fn);
    }
    const int64_t px = zmarch_tma_pitch(nx);
    const cuuint64_t dims[4] = {(cuuint64_t)px, (cuuint64_t)ny, (cuuint64_t)nz, (cuuint64_t)nc};
    const cuuint64_t strides[3] = {(cuuint64_t)px * 4, (cuuint64_t)px * ny * 4, (cuuint64_t)px * ny * nz * 4};
    const cuuint32_t box[4] = {(cuuint32_t)CBX, (cuuint32_t)CBY, 1u, (cuuint32_t)nc};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(Cpad), dims, strides, box,
                              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t launch_pad_stiffness(const float* C, float* Cpad, int nx, int ny, int nz, int nc, cudaStream_t s) {
    const int64_t px = zmarch_tma_pitch(nx);
    const int64_t rows = (int64_t)nc * nz * ny;
    int64_t blocks = (rows * px + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_pad_planes<<<(int)blocks, 256, 0, s>>>(C, Cpad, nx, (int)px, rows);
    return cudaGetLastError();
}

template <int SYM, int MODE>
static cudaError_t zt_launch(const CUtensorMap& map, const float* x, const float* C, const LevelGeom<float>& G,
                             const BcTable& bc, const float* b, const float* dg, float omega, float* out, int* err,
                             cudaStream_t s, cudaStream_t s_faces) {
    constexpr int NC = SYM == SYM_ISO ? 2 : 21;
    constexpr int bytes = ZtSmem<NC>::total;
    static bool configured[64] = {};  // the attribute is set once per device
    int dev = 0;
    cudaError_t e0 = cudaGetDevice(&dev);
    if (e0 != cudaSuccess) return e0;
    if (dev < 0 || dev >= 64 || !configured[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k_zmarch_tma<SYM, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             bytes);
        if (e != cudaSuccess) return e;
        if (dev >= 0 && dev < 64) configured[dev] = true;
    }
    const int ni = G.nx - 2, nj = G.ny - 2, nk = G.nz - 2;
    const int kc = zt_kchunk(ni, nj, nk, NC <= 2 ? 3 : 2);
    dim3 blk(TX, TY, 1), grd((ni + TX - 1) / TX, (nj + TY - 1) / TY, (nk + kc - 1) / kc);
    const int fa = G.nx > G.ny ? G.nx : G.ny, fb = G.ny > G.nz ? G.ny : G.nz;
    dim3 fgrd((fa + TX - 1) / TX, (fb + TY - 1) / TY, 6);
    // faces first: on a separate stream they then overlap the interior sweep
    k_zt_faces<SYM, MODE><<<fgrd, blk, 0, s_faces ? s_faces : s>>>(x, C, G, bc, b, dg, omega, out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_zmarch_tma<SYM, MODE><<<grd, blk, bytes, s>>>(map, x, G, b, dg, omega, out, kc, err);
    return cudaGetLastError();
}

cudaError_t launch_zmarch_tma(int mode, int sym, const CUtensorMap& map, const float* x, const float* C,
                              const LevelGeom<float>& G, const BcTable& bc, const float* b, const float* dg,
                              float omega, float* out, int* err, cudaStream_t s, cudaStream_t s_faces) {
    if (!zmarch_tma_supported(G.nx, G.ny, G.nz) || sym == SYM_MAJ) return cudaErrorInvalidValue;
    if (sym == SYM_ISO) {
        if (mode == 0) return zt_launch<SYM_ISO, 0>(map, x, C, G, bc, b, dg, omega, out, err, s, s_faces);
        if (mode == 1) return zt_launch<SYM_ISO, 1>(map, x, C, G, bc, b, dg, omega, out, err, s, s_faces);
        return zt_launch<SYM_ISO, 2>(map, x, C, G, bc, b, dg, omega, out, err, s, s_faces);
    }
    if (mode == 0) return zt_launch<SYM_MM, 0>(map, x, C, G, bc, b, dg, omega, out, err, s, s_faces);
    if (mode == 1) return zt_launch<SYM_MM, 1>(map, x, C, G, bc, b, dg, omega, out, err, s, s_faces);
    return zt_launch<SYM_MM, 2>(map, x, C, G, bc, b, dg, omega, out, err, s, s_faces);
}

}  // namespace agb

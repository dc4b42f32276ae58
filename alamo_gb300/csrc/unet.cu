// Kernels of the learned initial guess: a 3D U-Net on the node grid,
// BF16 activations and weights, FP32 accumulation.
//
// 3x3x3 convolutions run on the 5th-generation tensor cores: tcgen05.mma
// (kind::f16, BF16 A and B, FP32 accumulator in tensor memory) issued by one
// thread of the CTA, operands in shared memory in the K-major no-swizzle
// canonical layout.  A CTA owns an output tile of 8 x 16 x 1 nodes (M = 128
// rows) and all N output channels.  Per 16-channel slice of the input it
// stages the 10 x 18 x 3 input patch once, as two 8-channel planes of 16-byte
// node records; for tap (dz, dy, dx) the A operand of the MMA is then simply
// the descriptor of the patch shifted by (dz, dy, dx) -- rows are 8
// x-consecutive nodes (one 128-byte core matrix), the 16 row groups are the
// tile's y rows (stride 160 bytes), and the second 8 channels are one patch
// plane further (no im2col buffer).  The weights of the slice (27 taps x N x
// 16) are staged beside it.  27 MMAs per slice, one commit to an mbarrier,
// a bounded wait, then the next slice; the epilogue reads the accumulator
// rows with tcgen05.ld and applies bias, ReLU and an optional ReLU mask.
//
// Activations are channels-last ([node][channel], channel count a multiple of
// 16, zero padded), so one node's 8 channels are one 16-byte record.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "unet.h"

namespace agb {
namespace {

constexpr int CX = 8, CY = 16;                 // output tile (x, y), one z plane
constexpr int PX = CX + 2, PY = CY + 2, PZ = 3;  // input patch
constexpr int PATCH_PLANE = PZ * PY * PX * 16;   // bytes of one 8-channel plane of the patch (8640)
constexpr int PATCH_BYTES = 2 * PATCH_PLANE;     // 16 channels
constexpr uint64_t WAIT_NS = 1000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
// shared-memory matrix descriptor: K-major, no swizzle; lbo = byte distance
// of the two 8-element K halves, sbo = byte distance of 8-row groups
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}
// instruction descriptor of kind::f16: D F32, A and B BF16, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    uint64_t t0 = 0;
    for (int it = 0;; it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (it == 0) t0 = global_ns();
        else if (global_ns() - t0 > WAIT_NS) return false;
    }
}

template <int N>
struct ConvCfg {
    static constexpr int TMEM_COLS = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;
    static constexpr int W_BYTES = 27 * N * 32;  // 27 taps x N rows x 16 BF16
    static constexpr int SMEM = PATCH_BYTES + W_BYTES + 128;
};

// X [V][Cin] BF16, Wt [Cin/16][27][N][16] BF16, bias [N] or null,
// Y [V][N] (BF16, or FP32 when yf), mask [V][N] BF16 or null (Y *= mask > 0).
// relu: max(0, .) after the bias.  Cin % 16 == 0.
template <int N>
__global__ void __launch_bounds__(128) k_conv3_tc(const __nv_bfloat16* __restrict__ X, int Cin,
                                                  const __nv_bfloat16* __restrict__ Wt,
                                                  const float* __restrict__ bias, int nx, int ny, int nz, int relu,
                                                  const __nv_bfloat16* __restrict__ mask,
                                                  __nv_bfloat16* __restrict__ Y, float* __restrict__ Yf,
                                                  int* __restrict__ err) {
    using CFG = ConvCfg<N>;
    extern __shared__ unsigned char cv_raw[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    const uint32_t raw = smem_u32(cv_raw);
    const uint32_t pad = ((raw + 127u) & ~127u) - raw;
    unsigned char* patch = cv_raw + pad;
    unsigned char* wsm = patch + PATCH_BYTES;
    const uint32_t patch_u32 = raw + pad, w_u32 = patch_u32 + PATCH_BYTES, bar_u32 = smem_u32(&bar);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int x0 = blockIdx.x * CX, y0 = blockIdx.y * CY, z0 = blockIdx.z;

    if (tid == 0) {
        abort_flag = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_u32) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(CFG::TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;
    constexpr uint32_t IDESC = idesc_bf16(128, N);
    const int nslice = Cin / 16;

    for (int sl = 0; sl < nslice; sl++) {
        // input patch of this 16-channel slice: plane h (channels 8h..8h+7),
        // record (pz, py, px) at ((h*PZ + pz)*PY + py)*PX + px, zero outside
        for (int q = tid; q < 2 * PZ * PY * PX; q += 128) {
            const int h = q / (PZ * PY * PX), r = q - h * (PZ * PY * PX);
            const int pz = r / (PY * PX), r2 = r - pz * (PY * PX), py = r2 / PX, px = r2 - py * PX;
            const int gx = x0 - 1 + px, gy = y0 - 1 + py, gz = z0 - 1 + pz;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (gx >= 0 && gx < nx && gy >= 0 && gy < ny && gz >= 0 && gz < nz) {
                const int64_t node = gx + (int64_t)nx * (gy + (int64_t)ny * gz);
                v = *reinterpret_cast<const uint4*>(X + node * Cin + sl * 16 + h * 8);
            }
            *reinterpret_cast<uint4*>(patch + q * 16) = v;
        }
        // weights of the slice: (tap, K half kc, row n) at ((tap*2 + kc)*N/8 + n/8)*128 + (n%8)*16
        const __nv_bfloat16* wsrc = Wt + (int64_t)sl * 27 * N * 16;
        for (int q = tid; q < 27 * N * 2; q += 128) {
            const int tap = q / (2 * N), r = q - tap * 2 * N, n = r >> 1, kc = r & 1;
            const uint4 v = *reinterpret_cast<const uint4*>(wsrc + ((int64_t)tap * N + n) * 16 + kc * 8);
            *reinterpret_cast<uint4*>(wsm + ((tap * 2 + kc) * (N / 8) + (n >> 3)) * 128 + (n & 7) * 16) = v;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int tap = 0; tap < 27; tap++) {
                const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;  // 0..2 = offset + 1
                const uint32_t a = patch_u32 + ((dz * PY + dy) * PX + dx) * 16;
                const uint64_t ad = sdesc(a, PATCH_PLANE, PX * 16);
                const uint64_t bd = sdesc(w_u32 + tap * 2 * (N / 8) * 128, (N / 8) * 128, 128);
                const uint32_t acc = (sl > 0 || tap > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar_u32)
                         : "memory");
        }
        // the slice's MMAs must finish before its smem is overwritten
        if (!mbar_wait(bar_u32, (uint32_t)(sl & 1))) {
            abort_flag = 1;
            if (err) atomicExch(err, 1);
        }
        __syncthreads();
        if (abort_flag) break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!abort_flag) {
        // row m = 32 warp + lane -> node (x0 + m % 8, y0 + m / 8, z0)
        const int m = warp * 32 + lane;
        const int gx = x0 + (m & 7), gy = y0 + (m >> 3);
        const bool live = gx < nx && gy < ny;
        const int64_t node = gx + (int64_t)nx * (gy + (int64_t)ny * z0);
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += 16) {
            uint32_t r[16];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (live) {
                float v[16];
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    float a = __uint_as_float(r[j]);
                    if (bias) a += bias[c0 + j];
                    if (relu) a = fmaxf(a, 0.f);
                    v[j] = a;
                }
                if (mask) {
                    const uint4* mp = reinterpret_cast<const uint4*>(mask + node * N + c0);
                    const uint4 m0 = mp[0], m1 = mp[1];
                    const __nv_bfloat16* mb0 = reinterpret_cast<const __nv_bfloat16*>(&m0);
                    const __nv_bfloat16* mb1 = reinterpret_cast<const __nv_bfloat16*>(&m1);
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        if (!(__bfloat162float(mb0[j]) > 0.f)) v[j] = 0.f;
                        if (!(__bfloat162float(mb1[j]) > 0.f)) v[8 + j] = 0.f;
                    }
                }
                if (Yf) {
                    float4* dst = reinterpret_cast<float4*>(Yf + node * N + c0);
#pragma unroll
                    for (int j = 0; j < 4; j++) dst[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
                } else {
                    __align__(16) __nv_bfloat16 o[16];
#pragma unroll
                    for (int j = 0; j < 16; j++) o[j] = __float2bfloat16(v[j]);
                    uint4* dst = reinterpret_cast<uint4*>(Y + node * N + c0);
                    dst[0] = reinterpret_cast<const uint4*>(o)[0];
                    dst[1] = reinterpret_cast<const uint4*>(o)[1];
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(CFG::TMEM_COLS)
                     : "memory");
}

template <int N>
cudaError_t conv_launch(const __nv_bfloat16* X, int Cin, const __nv_bfloat16* Wt, const float* bias, int nx, int ny,
                        int nz, int relu, const __nv_bfloat16* mask, __nv_bfloat16* Y, float* Yf, int* err,
                        cudaStream_t s) {
    constexpr int bytes = ConvCfg<N>::SMEM;
    static bool configured[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64 || !configured[dev]) {
        e = cudaFuncSetAttribute(k_conv3_tc<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        if (dev >= 0 && dev < 64) configured[dev] = true;
    }
    dim3 grd((nx + CX - 1) / CX, (ny + CY - 1) / CY, nz);
    k_conv3_tc<N><<<grd, 128, bytes, s>>>(X, Cin, Wt, bias, nx, ny, nz, relu, mask, Y, Yf, err);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Weight gradient of the 3x3x3 convolution on the tensor cores:
//   dW[o][c][t] += sum_v dY[v][o] X[v + t][c],  db[o] += sum_v dY[v][o].
// As a GEMM per CTA: D[m][o] = sum_k A[m][k] B[o][k] with the reduction over
// the nodes k of the CTA's run of nodes; row m = (tap, channel) of one
// 8-tap x 16-channel tile (M = 128), column o = output channel (N = Cout).
// A[m][k] = X[node k shifted by tap][channel] (zero outside the grid),
// B[o][k] = dY[node k][o] rounded to BF16.  Per stage of 64 nodes the CTA
// gathers both operands into shared memory in the K-major no-swizzle layout
// of the forward kernel (core matrices of 8 rows x 8 nodes; K halves LBO
// apart, 8-row groups 128 bytes apart), one thread issues the stage's four
// tcgen05.mma (K = 16 each) and commits to the stage buffer's mbarrier; two
// buffers let the next gather overlap the MMAs.  The FP32 accumulator rows
// are read back with tcgen05.ld and added into dW with atomics (the node runs
// of different CTAs add up); the bias gradient is summed by the CTAs of the
// first tile.
constexpr int WT_STAGE_NODES = 64;  // nodes per stage (4 MMAs of K = 16)
constexpr int WT_STAGES = 16;       // stages per CTA: 1024 nodes

template <int N>
struct WgCfg {
    static constexpr int TMEM_COLS = ConvCfg<N>::TMEM_COLS;
    static constexpr int A_KS = 128 * 16 * 2;  // bytes of A per 16-node K step
    static constexpr int B_KS = N * 16 * 2;
    static constexpr int A_ST = 4 * A_KS, B_ST = 4 * B_KS;
    static constexpr int BUF = A_ST + B_ST;   // one stage buffer
    static constexpr int SMEM = 2 * BUF + 128;
};

template <int N>
__global__ void __launch_bounds__(128) k_wgrad_tc(const __nv_bfloat16* __restrict__ X, int Cin, int CinW,
                                                  const float* __restrict__ dY, int nx, int ny, int nz,
                                                  float* __restrict__ dW, float* __restrict__ db,
                                                  int* __restrict__ err) {
    using CFG = WgCfg<N>;
    extern __shared__ unsigned char wg_raw[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    __shared__ float sdb[N];
    const uint32_t raw = smem_u32(wg_raw);
    const uint32_t pad = ((raw + 127u) & ~127u) - raw;
    unsigned char* buf = wg_raw + pad;
    const uint32_t buf_u32 = raw + pad;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t V = (int64_t)nx * ny * nz;
    const int64_t v0 = (int64_t)blockIdx.x * (WT_STAGE_NODES * WT_STAGES);
    const int tg = blockIdx.y & 3, cs = blockIdx.y >> 2;  // tap group (8 taps), 16-channel slice
    const bool first_tile = blockIdx.y == 0;

    if (tid == 0) {
        abort_flag = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[1])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int q = tid; q < N; q += 128) sdb[q] = 0.f;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(CFG::TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;
    constexpr uint32_t IDESC = idesc_bf16(128, N);

    // gather one stage (nodes vs .. vs + 63) into buffer b
    auto gather = [&](int st, int b) {
        unsigned char* A = buf + b * CFG::BUF;
        unsigned char* B = A + CFG::A_ST;
        const int64_t vs = v0 + (int64_t)st * WT_STAGE_NODES;
        // A: (local tap tl, node j) pairs, 16 channels each
        for (int q = tid; q < 8 * WT_STAGE_NODES; q += 128) {
            const int tl = q / WT_STAGE_NODES, j = q - tl * WT_STAGE_NODES;
            const int t = tg * 8 + tl;
            const int64_t v = vs + j;
            uint4 lo4 = make_uint4(0, 0, 0, 0), hi4 = make_uint4(0, 0, 0, 0);
            if (t < 27 && v < V) {
                const int x = (int)(v % nx), y = (int)((v / nx) % ny), z = (int)(v / ((int64_t)nx * ny));
                const int xx = x + t % 3 - 1, yy = y + (t / 3) % 3 - 1, zz = z + t / 9 - 1;
                if (xx >= 0 && xx < nx && yy >= 0 && yy < ny && zz >= 0 && zz < nz) {
                    const uint4* src = reinterpret_cast<const uint4*>(
                        X + (xx + (int64_t)nx * (yy + (int64_t)ny * zz)) * Cin + cs * 16);
                    lo4 = src[0];
                    hi4 = src[1];
                }
            }
            const __nv_bfloat16* e0 = reinterpret_cast<const __nv_bfloat16*>(&lo4);
            const __nv_bfloat16* e1 = reinterpret_cast<const __nv_bfloat16*>(&hi4);
            const int ks = j >> 4, kh = (j >> 3) & 1, e = j & 7;
            unsigned char* base = A + ks * CFG::A_KS + e * 2;
#pragma unroll
            for (int c = 0; c < 16; c++) {
                const int m = tl * 16 + c;
                *reinterpret_cast<__nv_bfloat16*>(base + (kh * 16 + (m >> 3)) * 128 + (m & 7) * 16) =
                    c < 8 ? e0[c] : e1[c - 8];
            }
        }
        // B: (node j, group of 8 output channels)
        for (int q = tid; q < WT_STAGE_NODES * (N / 8); q += 128) {
            const int j = q / (N / 8), g = q - j * (N / 8);
            const int64_t v = vs + j;
            float f[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            if (v < V) {
                const float4* src = reinterpret_cast<const float4*>(dY + v * N + g * 8);
                const float4 a = src[0], bb = src[1];
                f[0] = a.x; f[1] = a.y; f[2] = a.z; f[3] = a.w;
                f[4] = bb.x; f[5] = bb.y; f[6] = bb.z; f[7] = bb.w;
                if (first_tile) {
#pragma unroll
                    for (int i = 0; i < 8; i++) atomicAdd(&sdb[g * 8 + i], f[i]);
                }
            }
            const int ks = j >> 4, kh = (j >> 3) & 1, e = j & 7;
            unsigned char* base = B + ks * CFG::B_KS + (kh * (N / 8) + g) * 128 + e * 2;
#pragma unroll
            for (int i = 0; i < 8; i++) *reinterpret_cast<__nv_bfloat16*>(base + i * 16) = __float2bfloat16(f[i]);
        }
    };
    auto issue = [&](int st, int b) {  // one thread
        const uint32_t a_u32 = buf_u32 + b * CFG::BUF;
        const uint32_t b_u32 = a_u32 + CFG::A_ST;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        for (int ks = 0; ks < 4; ks++) {
            const uint64_t ad = sdesc(a_u32 + ks * CFG::A_KS, 16 * 128, 128);
            const uint64_t bd = sdesc(b_u32 + ks * CFG::B_KS, (N / 8) * 128, 128);
            const uint32_t acc = (st > 0 || ks > 0) ? 1u : 0u;
            asm volatile(
                "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
                : "memory");
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(&bars[b]))
                     : "memory");
    };

    int nst = 0;
    for (int st = 0; st < WT_STAGES; st++) {
        if (v0 + (int64_t)st * WT_STAGE_NODES >= V) break;
        const int b = st & 1;
        if (st >= 2) {
            // the MMAs of stage st - 2 read this buffer
            if (tid == 0 && !mbar_wait(smem_u32(&bars[b]), (uint32_t)(((st - 2) >> 1) & 1))) {
                abort_flag = 1;
                if (err) atomicExch(err, 1);
            }
            __syncthreads();
            if (abort_flag) break;
        }
        gather(st, b);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) issue(st, b);
        nst = st + 1;
    }
    // the last stage's commit covers every MMA issued before it; waited for
    // (bounded) after an abort too, before the accumulator is freed
    if (nst > 0 && tid == 0) {
        const int last = nst - 1;
        if (!mbar_wait(smem_u32(&bars[last & 1]), (uint32_t)((last >> 1) & 1))) {
            abort_flag = 1;
            if (err) atomicExch(err, 1);
        }
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (nst > 0 && !abort_flag) {
        const int m = warp * 32 + lane;
        const int tl = m >> 4, c = cs * 16 + (m & 15), t = tg * 8 + tl;
        const bool live = t < 27 && c < CinW;
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += 16) {
            uint32_t r[16];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (live) {
#pragma unroll
                for (int jj = 0; jj < 16; jj++)
                    atomicAdd(&dW[((int64_t)(c0 + jj) * CinW + c) * 27 + t], __uint_as_float(r[jj]));
            }
        }
        if (first_tile)
            for (int q = tid; q < N; q += 128) atomicAdd(&db[q], sdb[q]);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(CFG::TMEM_COLS)
                     : "memory");
}

template <int N>
cudaError_t wgrad_launch(const __nv_bfloat16* X, int Cin, int CinW, const float* dY, int nx, int ny, int nz,
                         float* dW, float* db, int* err, cudaStream_t s) {
    constexpr int bytes = WgCfg<N>::SMEM;
    static bool configured[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64 || !configured[dev]) {
        e = cudaFuncSetAttribute(k_wgrad_tc<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        if (dev >= 0 && dev < 64) configured[dev] = true;
    }
    const int64_t V = (int64_t)nx * ny * nz;
    const int64_t per = (int64_t)WT_STAGE_NODES * WT_STAGES;
    dim3 grd((unsigned)((V + per - 1) / per), 4 * (Cin / 16), 1);
    k_wgrad_tc<N><<<grd, 128, bytes, s>>>(X, Cin, CinW, dY, nx, ny, nz, dW, db, err);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_conv3(const __nv_bfloat16* X, int Cin, const __nv_bfloat16* Wt, const float* bias, int Cout,
                         int nx, int ny, int nz, int relu, const __nv_bfloat16* mask, __nv_bfloat16* Y, float* Yf,
                         int* err, cudaStream_t s) {
    if (Cin <= 0 || Cin % 16 || nx < 1 || ny < 1 || nz < 1) return cudaErrorInvalidValue;
    switch (Cout) {
        case 16: return conv_launch<16>(X, Cin, Wt, bias, nx, ny, nz, relu, mask, Y, Yf, err, s);
        case 32: return conv_launch<32>(X, Cin, Wt, bias, nx, ny, nz, relu, mask, Y, Yf, err, s);
        case 48: return conv_launch<48>(X, Cin, Wt, bias, nx, ny, nz, relu, mask, Y, Yf, err, s);
        case 64: return conv_launch<64>(X, Cin, Wt, bias, nx, ny, nz, relu, mask, Y, Yf, err, s);
        case 96: return conv_launch<96>(X, Cin, Wt, bias, nx, ny, nz, relu, mask, Y, Yf, err, s);
        case 128: return conv_launch<128>(X, Cin, Wt, bias, nx, ny, nz, relu, mask, Y, Yf, err, s);
        case 192: return conv_launch<192>(X, Cin, Wt, bias, nx, ny, nz, relu, mask, Y, Yf, err, s);
        default: return cudaErrorInvalidValue;
    }
}


// ---------------------------------------------------------------------------
// Non-tensor-core layers (FP32 arithmetic on the CUDA cores): weight
// packing, weight gradients, nodal down/up sampling, concatenation, the
// 1x1x1 head, the loss, the optimiser and the feature/output conversions.
// ---------------------------------------------------------------------------
namespace {

__global__ void k_pack_fwd(const float* __restrict__ W, int Cout, int Cin_real, int Cin,
                           __nv_bfloat16* __restrict__ Wt) {
    // W [Cout][Cin_real][27] -> Wt [Cin/16][27][Cout][16], zero for c >= Cin_real
    const int64_t tot = (int64_t)Cin * 27 * Cout;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < tot; q += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(q % 16);
        int64_t r = q / 16;
        const int o = (int)(r % Cout);
        r /= Cout;
        const int tap = (int)(r % 27);
        const int sl = (int)(r / 27);
        const int c = sl * 16 + k;
        Wt[q] = __float2bfloat16(c < Cin_real ? W[((int64_t)o * Cin_real + c) * 27 + tap] : 0.f);
    }
}

__global__ void k_pack_dgrad(const float* __restrict__ W, int Cout, int Cin, __nv_bfloat16* __restrict__ Wd) {
    // transpose + tap flip: Wd [Cout/16][27][Cin][16], Wd[s][t][c][k] = W[16 s + k][c][26 - t]
    const int64_t tot = (int64_t)Cout * 27 * Cin;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < tot; q += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(q % 16);
        int64_t r = q / 16;
        const int c = (int)(r % Cin);
        r /= Cin;
        const int tap = (int)(r % 27);
        const int sl = (int)(r / 27);
        const int o = sl * 16 + k;
        Wd[q] = __float2bfloat16(W[((int64_t)o * Cin + c) * 27 + (26 - tap)]);
    }
}

// dW[o][c][tap] += sum_v dY[v][o] X[v + tap][c] for c < CinW (the weight
// tensor's input channels; X has Cin >= CinW, the rest zero padding);
// db[o] += sum_v dY[v][o].  Block (16 o x 16 c threads) over a run of nodes;
// 27 accumulators per thread.
constexpr int WG_NODES = 512;
__global__ void __launch_bounds__(256) k_wgrad(const __nv_bfloat16* __restrict__ X, int Cin, int CinW,
                                               const float* __restrict__ dY, int Cout, int nx, int ny, int nz,
                                               float* __restrict__ dW, float* __restrict__ db) {
    const int c = blockIdx.y * 16 + (threadIdx.x & 15);
    const int o = blockIdx.z * 16 + (threadIdx.x >> 4);
    const int64_t V = (int64_t)nx * ny * nz;
    const int64_t v0 = (int64_t)blockIdx.x * WG_NODES;
    const int64_t v1 = v0 + WG_NODES < V ? v0 + WG_NODES : V;
    float acc[27];
#pragma unroll
    for (int t = 0; t < 27; t++) acc[t] = 0.f;
    float bacc = 0.f;
    for (int64_t v = v0; v < v1; v++) {
        const float g = dY[v * Cout + o];
        bacc += g;
        const int x = (int)(v % nx), y = (int)((v / nx) % ny), z = (int)(v / ((int64_t)nx * ny));
#pragma unroll
        for (int t = 0; t < 27; t++) {
            const int dz = t / 9 - 1, dy = (t / 3) % 3 - 1, dx = t % 3 - 1;
            const int xx = x + dx, yy = y + dy, zz = z + dz;
            if (xx >= 0 && xx < nx && yy >= 0 && yy < ny && zz >= 0 && zz < nz) {
                const int64_t u = xx + (int64_t)nx * (yy + (int64_t)ny * zz);
                acc[t] += g * __bfloat162float(X[u * Cin + c]);
            }
        }
    }
    if (c < CinW) {
#pragma unroll
        for (int t = 0; t < 27; t++) atomicAdd(&dW[((int64_t)o * CinW + c) * 27 + t], acc[t]);
    }
    if (blockIdx.y == 0 && (threadIdx.x & 15) == 0) atomicAdd(&db[o], bacc);
}

// nodal full-weighting down-sampling (weights 1/2, 1/4 per axis, zero
// outside): Yc[I][c] = s * sum w(a) w(b) w(d) X[2I + (a, b, d)][c]
template <typename TI, typename TO>
__global__ void k_down(const TI* __restrict__ X, int nx, int ny, int nz, int C, TO* __restrict__ Y, int mx, int my,
                       int mz, float s) {
    const int64_t tot = (int64_t)mx * my * mz * C;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < tot; q += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(q % C);
        const int64_t node = q / C;
        const int I = (int)(node % mx), J = (int)((node / mx) % my), K = (int)(node / ((int64_t)mx * my));
        float acc = 0.f;
        for (int d = -1; d <= 1; d++) {
            const int z = 2 * K + d;
            if (z < 0 || z >= nz) continue;
            const float wz = d == 0 ? 0.5f : 0.25f;
            for (int b = -1; b <= 1; b++) {
                const int y = 2 * J + b;
                if (y < 0 || y >= ny) continue;
                const float wy = b == 0 ? 0.5f : 0.25f;
                for (int a = -1; a <= 1; a++) {
                    const int x = 2 * I + a;
                    if (x < 0 || x >= nx) continue;
                    const float wx = a == 0 ? 0.5f : 0.25f;
                    acc += wz * wy * wx * (float)X[(x + (int64_t)nx * (y + (int64_t)ny * z)) * C + c];
                }
            }
        }
        Y[q] = (TO)(s * acc);
    }
}

// nodal trilinear up-sampling: Yf[i][c] = s * sum over the coarse nodes I
// with |i - 2I| <= 1 per axis of p(i - 2I) Yc[I][c], p(0) = 1, p(+-1) = 1/2
template <typename TI, typename TO>
__global__ void k_up(const TI* __restrict__ Yc, int mx, int my, int mz, int C, TO* __restrict__ Y, int nx, int ny,
                     int nz, float s) {
    const int64_t tot = (int64_t)nx * ny * nz * C;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < tot; q += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(q % C);
        const int64_t node = q / C;
        const int x = (int)(node % nx), y = (int)((node / nx) % ny), z = (int)(node / ((int64_t)nx * ny));
        float acc = 0.f;
        const int Ix0 = x >> 1, Iy0 = y >> 1, Iz0 = z >> 1;
        for (int K = Iz0; K <= Iz0 + (z & 1); K++) {
            if (K >= mz) continue;
            const float pz = (z & 1) ? 0.5f : 1.f;
            for (int J = Iy0; J <= Iy0 + (y & 1); J++) {
                if (J >= my) continue;
                const float py = (y & 1) ? 0.5f : 1.f;
                for (int I = Ix0; I <= Ix0 + (x & 1); I++) {
                    if (I >= mx) continue;
                    const float px = (x & 1) ? 0.5f : 1.f;
                    acc += pz * py * px * (float)Yc[(I + (int64_t)mx * (J + (int64_t)my * K)) * C + c];
                }
            }
        }
        Y[q] = (TO)(s * acc);
    }
}

// out[v] = [a[v] (Ca channels) | b[v] (Cb channels)]
__global__ void k_concat(const __nv_bfloat16* __restrict__ a, int Ca, const __nv_bfloat16* __restrict__ b, int Cb,
                         __nv_bfloat16* __restrict__ out, int64_t V) {
    const int C = Ca + Cb;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < V * C; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = q / C;
        const int c = (int)(q - v * C);
        out[q] = c < Ca ? a[v * Ca + c] : b[v * Cb + (c - Ca)];
    }
}

// g (FP32, [V][C] with row stride ldg, channel offset off) -> BF16 [V][C],
// zeroed where mask <= 0 (mask may be null); acc: add into an FP32 buffer
// instead (out_f += g)
__global__ void k_grad_cast(const float* __restrict__ g, int ldg, int off, int C, const __nv_bfloat16* __restrict__ mask,
                            __nv_bfloat16* __restrict__ out, float* __restrict__ out_f, int64_t V) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < V * C; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = q / C;
        const int c = (int)(q - v * C);
        float x = g[v * ldg + off + c];
        if (mask && !(__bfloat162float(mask[q]) > 0.f)) x = 0.f;
        if (out_f) out_f[q] += x;
        else out[q] = __float2bfloat16(x);
    }
}

// 1x1x1 head: u[v][o] = bh[o] + sum_c Wh[o][c] X[v][c], C = 16, 3 outputs
__global__ void k_head_fwd(const __nv_bfloat16* __restrict__ X, const float* __restrict__ Wh,
                           const float* __restrict__ bh, float* __restrict__ u, int64_t V) {
    __shared__ float w[48], b[3];
    if (threadIdx.x < 48) w[threadIdx.x] = Wh[threadIdx.x];
    if (threadIdx.x < 3) b[threadIdx.x] = bh[threadIdx.x];
    __syncthreads();
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
        float x[16];
#pragma unroll
        for (int c = 0; c < 16; c++) x[c] = __bfloat162float(X[v * 16 + c]);
#pragma unroll
        for (int o = 0; o < 3; o++) {
            float a = b[o];
#pragma unroll
            for (int c = 0; c < 16; c++) a += w[o * 16 + c] * x[c];
            u[v * 3 + o] = a;
        }
    }
}

// loss = sum (u - t)^2 / (3 V); du = 2 (u - t) / (3 V);
// dX[v][c] = sum_o Wh[o][c] du[v][o], zeroed where X <= 0 (ReLU input);
// dWh += du^T X, dbh += sum du; loss accumulated in FP64
__global__ void __launch_bounds__(256) k_head_bwd(const __nv_bfloat16* __restrict__ X, const float* __restrict__ Wh,
                                                  const float* __restrict__ u, const float* __restrict__ t,
                                                  float* __restrict__ dX, float* __restrict__ dWh,
                                                  float* __restrict__ dbh, double* __restrict__ loss, int64_t V) {
    __shared__ float w[48];
    __shared__ float red[52][8];
    if (threadIdx.x < 48) w[threadIdx.x] = Wh[threadIdx.x];
    __syncthreads();
    float gw[48], gb[3];
#pragma unroll
    for (int q = 0; q < 48; q++) gw[q] = 0.f;
    gb[0] = gb[1] = gb[2] = 0.f;
    double l = 0.0;
    const float sc = 2.f / (3.f * (float)V);
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
        float du[3];
#pragma unroll
        for (int o = 0; o < 3; o++) {
            const float e = u[v * 3 + o] - t[v * 3 + o];
            l += (double)e * e;
            du[o] = sc * e;
            gb[o] += du[o];
        }
#pragma unroll
        for (int c = 0; c < 16; c++) {
            const float x = __bfloat162float(X[v * 16 + c]);
            const float g = w[c] * du[0] + w[16 + c] * du[1] + w[32 + c] * du[2];
            dX[v * 16 + c] = x > 0.f ? g : 0.f;
#pragma unroll
            for (int o = 0; o < 3; o++) gw[o * 16 + c] += du[o] * x;
        }
    }
    // block reduction of the 51 parameter gradients and the loss
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int q = 0; q < 51; q++) {
        float v = q < 48 ? gw[q] : gb[q - 48];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[q][wid] = v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    __shared__ double lred[8];
    if (lane == 0) lred[wid] = l;
    __syncthreads();
    if (threadIdx.x < 51) {
        float v = 0.f;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) v += red[threadIdx.x][q];
        if (threadIdx.x < 48) atomicAdd(&dWh[threadIdx.x], v);
        else atomicAdd(&dbh[threadIdx.x - 48], v);
    }
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) s += lred[q];
        atomicAdd(loss, s / (3.0 * (double)V));
    }
}

// Adam (Kingma & Ba 2015) on FP32 parameters
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float c1,
                       float c2) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const float gq = g[q];
        const float mq = b1 * m[q] + (1.f - b1) * gq;
        const float vq = b2 * v[q] + (1.f - b2) * gq * gq;
        m[q] = mq;
        v[q] = vq;
        p[q] -= lr * (mq / c1) / (sqrtf(vq / c2) + eps);
    }
}

// network input: channels (log(lambda)/log 20, log(mu)/log 20, F0/0.02, 0...)
// from SoA FP64 fields (3 components: lambda, mu, F0), [V][16] BF16
__global__ void k_features(const double* __restrict__ f3, int64_t V, __nv_bfloat16* __restrict__ X) {
    const float il = 1.f / logf(20.f);
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < V * 16; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = q >> 4;
        const int c = (int)(q & 15);
        float x = 0.f;
        if (c == 0) x = logf(fmaxf((float)f3[v], 1e-6f)) * il;
        else if (c == 1) x = logf(fmaxf((float)f3[V + v], 1e-6f)) * il;
        else if (c == 2) x = (float)f3[2 * V + v] * 50.f;
        X[q] = __float2bfloat16(x);
    }
}

// SoA FP64 [3][V] * s -> channels-last FP32 [V][3], and back
__global__ void k_soa_to_cl(const double* __restrict__ u, int64_t V, double s, float* __restrict__ o) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < 3 * V; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = q / 3;
        const int c = (int)(q - v * 3);
        o[q] = (float)(u[c * V + v] * s);
    }
}
__global__ void k_cl_to_soa(const float* __restrict__ o, int64_t V, double s, double* __restrict__ u) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < 3 * V; q += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(q / V);
        const int64_t v = q - c * V;
        u[q] = (double)o[v * 3 + c] * s;
    }
}

int flat_grid(int64_t n) {
    const int64_t b = (n + 255) / 256;
    return (int)(b < 152 * 16 ? (b < 1 ? 1 : b) : 152 * 16);
}

}  // namespace

cudaError_t launch_pack_conv_fwd(const float* W, int Cout, int Cin_real, int Cin, __nv_bfloat16* Wt, cudaStream_t s) {
    k_pack_fwd<<<flat_grid((int64_t)Cin * 27 * Cout), 256, 0, s>>>(W, Cout, Cin_real, Cin, Wt);
    return cudaGetLastError();
}
cudaError_t launch_pack_conv_dgrad(const float* W, int Cout, int Cin, __nv_bfloat16* Wd, cudaStream_t s) {
    k_pack_dgrad<<<flat_grid((int64_t)Cout * 27 * Cin), 256, 0, s>>>(W, Cout, Cin, Wd);
    return cudaGetLastError();
}
cudaError_t launch_conv_wgrad(const __nv_bfloat16* X, int Cin, int CinW, const float* dY, int Cout, int nx, int ny,
                              int nz, float* dW, float* db, cudaStream_t s) {
    if (Cin % 16 || Cout % 16 || CinW > Cin) return cudaErrorInvalidValue;
    const int64_t V = (int64_t)nx * ny * nz;
    dim3 grd((unsigned)((V + WG_NODES - 1) / WG_NODES), (CinW + 15) / 16, Cout / 16);
    k_wgrad<<<grd, 256, 0, s>>>(X, Cin, CinW, dY, Cout, nx, ny, nz, dW, db);
    return cudaGetLastError();
}
cudaError_t launch_conv_wgrad_tc(const __nv_bfloat16* X, int Cin, int CinW, const float* dY, int Cout, int nx, int ny,
                                 int nz, float* dW, float* db, int* err, cudaStream_t s) {
    if (Cin <= 0 || Cin % 16 || CinW > Cin || nx < 1 || ny < 1 || nz < 1) return cudaErrorInvalidValue;
    switch (Cout) {
        case 16: return wgrad_launch<16>(X, Cin, CinW, dY, nx, ny, nz, dW, db, err, s);
        case 32: return wgrad_launch<32>(X, Cin, CinW, dY, nx, ny, nz, dW, db, err, s);
        case 48: return wgrad_launch<48>(X, Cin, CinW, dY, nx, ny, nz, dW, db, err, s);
        case 64: return wgrad_launch<64>(X, Cin, CinW, dY, nx, ny, nz, dW, db, err, s);
        case 96: return wgrad_launch<96>(X, Cin, CinW, dY, nx, ny, nz, dW, db, err, s);
        case 128: return wgrad_launch<128>(X, Cin, CinW, dY, nx, ny, nz, dW, db, err, s);
        case 192: return wgrad_launch<192>(X, Cin, CinW, dY, nx, ny, nz, dW, db, err, s);
        default: return cudaErrorInvalidValue;
    }
}
cudaError_t launch_down_bf16(const __nv_bfloat16* X, int nx, int ny, int nz, int C, __nv_bfloat16* Y, int mx, int my,
                             int mz, float s, cudaStream_t st) {
    k_down<__nv_bfloat16, __nv_bfloat16><<<flat_grid((int64_t)mx * my * mz * C), 256, 0, st>>>(X, nx, ny, nz, C, Y, mx,
                                                                                               my, mz, s);
    return cudaGetLastError();
}
cudaError_t launch_down_f32(const float* X, int nx, int ny, int nz, int C, float* Y, int mx, int my, int mz, float s,
                            cudaStream_t st) {
    k_down<float, float><<<flat_grid((int64_t)mx * my * mz * C), 256, 0, st>>>(X, nx, ny, nz, C, Y, mx, my, mz, s);
    return cudaGetLastError();
}
cudaError_t launch_up_bf16(const __nv_bfloat16* Yc, int mx, int my, int mz, int C, __nv_bfloat16* Y, int nx, int ny,
                           int nz, float s, cudaStream_t st) {
    k_up<__nv_bfloat16, __nv_bfloat16><<<flat_grid((int64_t)nx * ny * nz * C), 256, 0, st>>>(Yc, mx, my, mz, C, Y, nx,
                                                                                             ny, nz, s);
    return cudaGetLastError();
}
cudaError_t launch_up_f32(const float* Yc, int mx, int my, int mz, int C, float* Y, int nx, int ny, int nz, float s,
                          cudaStream_t st) {
    k_up<float, float><<<flat_grid((int64_t)nx * ny * nz * C), 256, 0, st>>>(Yc, mx, my, mz, C, Y, nx, ny, nz, s);
    return cudaGetLastError();
}
cudaError_t launch_concat(const __nv_bfloat16* a, int Ca, const __nv_bfloat16* b, int Cb, __nv_bfloat16* out,
                          int64_t V, cudaStream_t s) {
    k_concat<<<flat_grid(V * (Ca + Cb)), 256, 0, s>>>(a, Ca, b, Cb, out, V);
    return cudaGetLastError();
}
cudaError_t launch_grad_cast(const float* g, int ldg, int off, int C, const __nv_bfloat16* mask, __nv_bfloat16* out,
                             float* out_f, int64_t V, cudaStream_t s) {
    k_grad_cast<<<flat_grid(V * C), 256, 0, s>>>(g, ldg, off, C, mask, out, out_f, V);
    return cudaGetLastError();
}
cudaError_t launch_head_fwd(const __nv_bfloat16* X, const float* Wh, const float* bh, float* u, int64_t V,
                            cudaStream_t s) {
    k_head_fwd<<<flat_grid(V), 256, 0, s>>>(X, Wh, bh, u, V);
    return cudaGetLastError();
}
cudaError_t launch_head_bwd(const __nv_bfloat16* X, const float* Wh, const float* u, const float* t, float* dX,
                            float* dWh, float* dbh, double* loss, int64_t V, cudaStream_t s) {
    const int64_t b = (V + 255) / 256;
    k_head_bwd<<<(int)(b < 152 * 4 ? b : 152 * 4), 256, 0, s>>>(X, Wh, u, t, dX, dWh, dbh, loss, V);
    return cudaGetLastError();
}
cudaError_t launch_adam(float* p, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2,
                        float eps, int step, cudaStream_t s) {
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_adam<<<flat_grid(n), 256, 0, s>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}
cudaError_t launch_soa_to_channels_last(const double* u, int64_t V, double scale, float* out, cudaStream_t s) {
    k_soa_to_cl<<<flat_grid(3 * V), 256, 0, s>>>(u, V, scale, out);
    return cudaGetLastError();
}
cudaError_t launch_channels_last_to_soa(const float* in, int64_t V, double scale, double* u, cudaStream_t s) {
    k_cl_to_soa<<<flat_grid(3 * V), 256, 0, s>>>(in, V, scale, u);
    return cudaGetLastError();
}
cudaError_t launch_features(const double* f3, int64_t V, __nv_bfloat16* X, cudaStream_t s) {
    k_features<<<flat_grid(V * 16), 256, 0, s>>>(f3, V, X);
    return cudaGetLastError();
}

}  // namespace agb

// Allocation-free residual with norms.
//
// For callers that cannot call cudaMalloc.  Examples: a host code whose
// memory arena reserved the whole device at start-up (nothing is left to
// allocate), a plugin that lives inside such a code, and a time-stepping
// loop that must not call cudaMalloc/cudaFree between steps because those
// calls can synchronise the whole device and stall its other streams.  They
// pass their own inputs and outputs; the per-block partial norms this kernel
// needs live in a fixed array in the library's device image instead of in
// allocated memory.
//
// The scratch array is file-scope device memory of AGB_NOALLOC_MAX_BLOCKS
// pairs of doubles plus the two final norms (2 MiB); every GPU that loads
// the library holds it until the process exits.  In host code the array's
// name is only a host-side stand-in, so its device address is looked up
// with cudaGetSymbolAddress, once per device, by the first call made with
// that device current, and cached.  A device reset (cudaDeviceReset) after
// that first call is not supported: the cached address would be stale.
// Every call uses the same array and leaves its contents behind: the
// kernels overwrite every entry they later read, and two calls that overlap
// on the GPU (different streams, no ordering) race on it and produce wrong
// norms.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/agb.h"
#include "agb_launch.h"
#include "operator.cuh"

namespace agb {

static constexpr int NA_MAX_DEVICES = 64;

// partial (max, sum of squares) per block, then the two final norms
__device__ __align__(256) double g_noalloc_scratch[2 * AGB_NOALLOC_MAX_BLOCKS + 2];

static double* g_scratch_ptr[NA_MAX_DEVICES] = {nullptr};
static std::mutex g_scratch_mutex;

static cudaError_t scratch_address(int dev, double** out) {
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

}  // namespace agb

extern "C" agb_status agb_residual_norms_noalloc(int nx, int ny, int nz, const double dx[3], int sym,
                                                 const double* C_soa, const int* bc_type, const double* x,
                                                 const double* b, double* r, double norms[2], void* stream) {
    using namespace agb;
    if (nx < 3 || ny < 3 || nz < 3 || !dx || !(dx[0] > 0) || !(dx[1] > 0) || !(dx[2] > 0)) return AGB_BAD_ARG;
    if (sym != AGB_SYM_ISOTROPIC && sym != AGB_SYM_MAJORMINOR) return AGB_BAD_ARG;
    if (!C_soa || !bc_type || !x || !b || !r || !norms) return AGB_BAD_ARG;
    // the residual kernel's own block count (one partial pair per block)
    const int64_t nblocks = residual_blocks(nx, ny, nz);
    if (nblocks > AGB_NOALLOC_MAX_BLOCKS) {
        char msg[160];
        std::snprintf(msg, sizeof msg,
                      "agb_residual_norms_noalloc: the grid needs %lld residual blocks; the fixed scratch "
                      "holds %d (AGB_NOALLOC_MAX_BLOCKS)",
                      (long long)nblocks, AGB_NOALLOC_MAX_BLOCKS);
        set_last_error(msg);
        return AGB_LIMIT;
    }
    BcTable bc;
    for (int q = 0; q < 78; q++) {
        if (bc_type[q] < AGB_BC_DISPLACEMENT || bc_type[q] > AGB_BC_NONE) return AGB_BAD_ARG;
        bc.t[q] = (unsigned char)bc_type[q];
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) return AGB_CUDA_ERROR;
    double* scratch = nullptr;
    if (scratch_address(dev, &scratch) != cudaSuccess) return AGB_CUDA_ERROR;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const LevelGeom<double> G = make_geom<double>(nx, ny, nz, dx);
    int nb = 0;
    if (launch_residual<double>(sym, x, b, C_soa, G, bc, r, scratch, &nb, s) != cudaSuccess) return AGB_CUDA_ERROR;
    if (nb < 1 || nb > AGB_NOALLOC_MAX_BLOCKS) {
        // unreachable while residual_blocks() describes the launch; the
        // partials would have run past the fixed array
        set_last_error("agb_residual_norms_noalloc: residual launch used more blocks than the fixed scratch holds");
        return AGB_LIMIT;
    }
    double* fin = scratch + 2 * AGB_NOALLOC_MAX_BLOCKS;
    if (launch_reduce_norms(scratch, nb, fin, s) != cudaSuccess) return AGB_CUDA_ERROR;
    if (cudaMemcpyAsync(norms, fin, 2 * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return AGB_CUDA_ERROR;
    if (cudaStreamSynchronize(s) != cudaSuccess) return AGB_CUDA_ERROR;
    return AGB_OK;
}

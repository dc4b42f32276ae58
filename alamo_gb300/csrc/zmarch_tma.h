// Launchers of the TMA-staged FP32 fine-level stencil kernels
// (zmarch_tma.cu).  Host code includes this with g++: only declarations.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>

#include "agb_types.h"

namespace agb {

// grids the kernels cover (an interior on every axis)
bool zmarch_tma_supported(int nx, int ny, int nz);
// x pitch (floats) of the padded stiffness copy: nx rounded up to 4
int64_t zmarch_tma_pitch(int nx);
// FP32 stiffness SoA (nc, nz, ny, nx) -> padded copy of nc * nz * ny * pitch
// floats: isotropic (2, nz, ny, pitch); major-minor five float4 groups
// (5, nz, ny, pitch, 4) of entries 0..19, then entry 20 (nz, ny, pitch)
cudaError_t launch_pad_stiffness(const float* C, float* Cpad, int nx, int ny, int nz, int nc, cudaStream_t s);
// tensor maps over the padded copy: isotropic main = 4-D (x, y, z, entry),
// box 36 x 10 x 1 x 2 (tail unused); major-minor main = 5-D (4, x, y, z,
// group), box 4 x 36 x 10 x 1 x 5, tail = 4-D over entry 20, box 36 x 10 x 1 x 1
struct ZtMaps {
    CUtensorMap main;
    CUtensorMap tail;
};
cudaError_t make_stiffness_maps(const float* Cpad, int nx, int ny, int nz, int nc, ZtMaps* maps);
// mode 0: out = A x; 1: one damped-Jacobi sweep (b, dg = the INVERSE diagonal,
// omega) in the form x + omega (b - A x) / diag; 2: out = b - A x.
// C is the unpadded FP32 stiffness (boundary faces), map the padded copy's
// tensor map (interior).  *err is set to 1 when a TMA wait gave up.  The
// interior kernel goes to s; the boundary-face kernel to s_faces when it is
// not null (the caller orders s_faces after s's earlier work and s after
// the faces), else to s before the interior.
cudaError_t launch_zmarch_tma(int mode, int sym, const ZtMaps& map, const float* x, const float* C,
                              const LevelGeom<float>& G, const BcTable& bc, const float* b, const float* dg,
                              float omega, float* out, int* err, cudaStream_t s, cudaStream_t s_faces);

}  // namespace agb

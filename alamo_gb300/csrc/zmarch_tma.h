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
// FP32 stiffness SoA (nc, nz, ny, nx) -> padded copy (nc, nz, ny, pitch)
cudaError_t launch_pad_stiffness(const float* C, float* Cpad, int nx, int ny, int nz, int nc, cudaStream_t s);
// 4-D tensor map (x, y, z, entry) over the padded copy, box 36 x 10 x 1 x nc
cudaError_t make_stiffness_map(const float* Cpad, int nx, int ny, int nz, int nc, CUtensorMap* map);
// mode 0: out = A x; 1: one damped-Jacobi sweep (b, dg = the INVERSE diagonal,
// omega) in the form x + omega (b - A x) / diag; 2: out = b - A x.
// C is the unpadded FP32 stiffness (boundary faces), map the padded copy's
// tensor map (interior).  *err is set to 1 when a TMA wait gave up.  The
// interior kernel goes to s; the boundary-face kernel to s_faces when it is
// not null (the caller orders s_faces after s's earlier work and s after
// the faces), else to s before the interior.
cudaError_t launch_zmarch_tma(int mode, int sym, const CUtensorMap& map, const float* x, const float* C,
                              const LevelGeom<float>& G, const BcTable& bc, const float* b, const float* dg,
                              float omega, float* out, int* err, cudaStream_t s, cudaStream_t s_faces);

}  // namespace agb

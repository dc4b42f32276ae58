// Launchers of the composite solve's level transfers (composite.cu).  Host
// code includes this with g++: only declarations.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace agb {

// fine (n fn, level-index offset foff) from the coarse field (cn, coff),
// trilinear nodal interpolation, ncomp SoA components; mode 0 assign, 1 add,
// 2 assign the fine array's outer ring (its ghost nodes) only
cudaError_t launch_interp(const double* c, const int cn[3], const int coff[3], double* f, const int fn[3],
                          const int foff[3], int ncomp, int mode, cudaStream_t s);
// coarse nodes c0 .. c0 + cnt - 1 (device int[3] each; ncov = their count)
// = full weighting (inject 0) or injection (inject 1) of the fine array whose
// node 1 + 2 a lies on covered node c0 + a; component stride / element
// stride fcs, fes (fine) and ccs, ces (coarse): SoA vectors (N, 1), AoS
// stiffness (1, nc)
cudaError_t launch_restrict_box(const double* f, const int fn[3], int64_t fcs, int64_t fes, double* c, const int cn[3],
                                int64_t ccs, int64_t ces, const int* c0_dev, const int* cnt_dev, int64_t ncov,
                                int ncomp, int inject, cudaStream_t s);
// the outer ring of an array set to zero
cudaError_t launch_zero_ring(double* v, const int n[3], int ncomp, cudaStream_t s);
// *out = max(*out, bits of max |v|) over the array without its ring (ring
// != 0) and without the covered block (c0_dev non-null); *out starts at 0
cudaError_t launch_masked_max(const double* v, const int n[3], int ring, const int* c0_dev, const int* cnt_dev,
                              int ncomp, unsigned long long* out, cudaStream_t s);

}  // namespace agb

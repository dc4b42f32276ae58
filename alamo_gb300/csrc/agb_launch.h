// Host-side launchers of the CUDA kernels (implemented in kernels.cu and
// bottom.cu).  Every launcher enqueues on `stream` and returns the launch's
// cudaError_t; none of them synchronises.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "agb_types.h"

namespace agb {

template <typename T>
LevelGeom<T> make_geom(int nx, int ny, int nz, const double dx[3]);

// f = A u (Operator::Elastic::Fapply)
template <typename T>
cudaError_t launch_fapply(int sym, const T* u, const T* C, const LevelGeom<T>& G, const BcTable& bc, T* f,
                          cudaStream_t s);
// diag of A (Operator::Elastic::Diagonal)
template <typename T>
cudaError_t launch_diagonal(int sym, const T* C, const LevelGeom<T>& G, const BcTable& bc, T* diag, cudaStream_t s);
// one colour (0..7) of the multicolour Gauss-Seidel sweep, in place on x
template <typename T>
cudaError_t launch_gs_colour(int sym, T* x, const T* b, const T* diag, const T* C, const LevelGeom<T>& G,
                             const BcTable& bc, T omega_b, int colour, cudaStream_t s);
// One damped-Jacobi sweep fused with the operator:
//   xout = (1-w) x + w (b - (A x - diag x)) / diag     (x == nullptr: x = 0)
template <typename T>
cudaError_t launch_jacobi(int sym, const T* x, const T* b, const T* diag, const T* C, const LevelGeom<T>& G,
                          const BcTable& bc, T omega, T* xout, cudaStream_t s);
// r = b - A x; when `partials` is non-null each block also writes its
// max |r| and sum r^2 (as doubles) to partials[2*block], partials[2*block+1]
template <typename T>
cudaError_t launch_residual(int sym, const T* x, const T* b, const T* C, const LevelGeom<T>& G, const BcTable& bc,
                            T* r, double* partials, int* nblocks_out, cudaStream_t s);
// block count the residual kernel uses for a level (sizes the partials buffer)
int residual_blocks(int nx, int ny, int nz);
// norms[0] = max over blocks, norms[1] = sqrt(sum) over blocks
cudaError_t launch_reduce_norms(const double* partials, int nblocks, double* norms, cudaStream_t s);
// max |v| and sum v^2 of a plain vector, same partials convention
cudaError_t launch_vec_norms(const double* v, int64_t n, double* partials, int nblocks, double* norms,
                             cudaStream_t s);

// nodal full weighting of a 3-component field, fine level -> coarse level
template <typename T>
cudaError_t launch_restrict(const T* fine, const LevelGeom<T>& Gf, T* crse, const LevelGeom<T>& Gc, cudaStream_t s);
// the restriction fused with the coarse level's first Jacobi sweep from a
// zero correction: xout = omega crse / diag
template <typename T>
cudaError_t launch_restrict_jacobi(const T* fine, const LevelGeom<T>& Gf, T* crse, const LevelGeom<T>& Gc,
                                   const T* diag, T omega, T* xout, cudaStream_t s);
// same weights on nc stiffness components (SoA)
cudaError_t launch_restrict_C(const double* Cf, const LevelGeom<double>& Gf, double* Cc, const LevelGeom<double>& Gc,
                              int nc, cudaStream_t s);
cudaError_t launch_restrict_C(const float* Cf, const LevelGeom<float>& Gf, float* Cc, const LevelGeom<float>& Gc,
                              int nc, cudaStream_t s);
// fine += P crse (trilinear nodal prolongation)
template <typename T>
cudaError_t launch_prolong_add(const T* crse, const LevelGeom<T>& Gc, T* fine, const LevelGeom<T>& Gf,
                               cudaStream_t s);

// NeoHookean (Newton.H:144-196, NeoHookean.H:21-121): dw = DW(F) (SoA 9),
// C = DDW(F) (SoA 45) at F = I + grad u for the model (mu, kappa) SoA
cudaError_t launch_neohookean(const double* model, const double* u, const LevelGeom<double>& G, double* dw,
                              double* C, cudaStream_t s);
// rhs = b - div dw / b - BC(u, grad u, dw) for a given stress field dw (SoA 9)
cudaError_t launch_rhs_from_dw(const double* u, const double* b, const double* dw, const LevelGeom<double>& G,
                               const BcTable& bc, double* rhs, cudaStream_t s);

// psi (Elastic::SetPsi / averageDownCoeffs, src/Operator/Elastic.cpp:118-137,
// 839-905) in the ghosted layout of LevelGeom::psi: the fine level from the
// caller's cells, and one coarsening
cudaError_t launch_psi_embed(const double* cells, const LevelGeom<double>& G, double* psi, cudaStream_t s);
cudaError_t launch_coarsen_psi(const double* pf, const LevelGeom<double>& Gf, double* pc, const LevelGeom<double>& Gc,
                               cudaStream_t s);

// layout and precision helpers
cudaError_t launch_aos_to_soa(const double* aos, double* soa, int64_t N, int nc, cudaStream_t s);
// (lambda, mu, F0) per node, SoA 3 x N: the isotropic entries or the Voigt
// average of a major-minor tensor; F0 scalar (f0n 1) or trace / 3 (f0n 9)
cudaError_t launch_guess_features(int sym, const double* C, int64_t N, const double* F0, int f0n, double* out,
                                  cudaStream_t s);
cudaError_t launch_soa_to_aos(const double* soa, double* aos, int64_t N, int nc, cudaStream_t s);
cudaError_t launch_to_float(const double* in, float* out, int64_t n, double scale, cudaStream_t s);
// out = 1 / in (FP32)
cudaError_t launch_recip(const float* in, float* out, int64_t n, cudaStream_t s);
// out(double) += scale * in(float)
cudaError_t launch_add_float(const float* in, double* out, int64_t n, double scale, cudaStream_t s);
cudaError_t launch_axpy(double a, const double* x, double* y, int64_t n, cudaStream_t s);
cudaError_t launch_axpy(float a, const float* x, float* y, int64_t n, cudaStream_t s);

// BC::Operator::Elastic::Constant::Init: boundary values into b
cudaError_t launch_bc_init(double* b, const LevelGeom<double>& G, const BcTable& bc, const double* bcval_dev,
                           int homogeneous, cudaStream_t s);
// Newton RHS (src/Solver/Nonlocal/Newton.H:144-231): dw = C (grad u - F0),
// rhs = b - div dw (interior) or b - BC(u, grad u, dw) (boundary); u = nullptr
// stands for u = 0 (nothing is read; without F0, rhs = b)
cudaError_t launch_build_rhs(int sym, const double* u, const double* b, const double* F0, int f0_ncomp,
                             const double* C, const LevelGeom<double>& G, const BcTable& bc, double* dw, double* rhs,
                             cudaStream_t s);
// stress = C (grad u - F0), strain = sym grad u (9 values per node, AoS
// row-major), energy = 0.5 sigma:eps; any output may be null
cudaError_t launch_stress_strain(int sym, const double* u, const double* F0, int f0_ncomp, const double* C,
                                 const LevelGeom<double>& G, double* stress, double* strain, double* energy,
                                 cudaStream_t s);
// Elastic::Stress (which 0: C grad u times psi_avg) / Elastic::Strain (which 1:
// sym grad u), SoA per component, 6 Voigt (00, 11, 22, 12, 20, 01) or 9
// row-major components
cudaError_t launch_op_tensor(int sym, const double* u, const double* C, const LevelGeom<double>& G, int which,
                             int voigt, double* out, cudaStream_t s);

// Bottom solve on the coarsest level in one thread block: BiCGStab on the
// diagonally normalised system (the reference's normalize), FP64, followed by
// `nsmooth_ok` Fsmooth calls after success or, after a breakdown, a zeroed
// correction and `nsmooth_fail` calls.  work: 7 * 3N doubles;
// info[0] = BiCGStab return code, info[1] = iterations.
cudaError_t launch_bottom_bicgstab_ex(int sym, const double* C, const double* diag, const LevelGeom<double>& G,
                                      const BcTable& bc, const double* rhs, double* sol, double* work, int max_iter,
                                      double tol_rel, double tol_abs, int nsmooth_ok, int nsmooth_fail, double omega,
                                      int* info, cudaStream_t s);
cudaError_t launch_bottom_bicgstab(int sym, const double* C, const double* diag, const LevelGeom<double>& G,
                                   const BcTable& bc, const double* rhs, double* sol, double* work, int max_iter,
                                   double tol_rel, double tol_abs, int* info, cudaStream_t s);

}  // namespace agb

namespace agb {
// Krylov helpers (FP64 block and grid reductions; FP32 vectors summed in
// compensated FP32 within a thread)
int multidot_blocks();
// out[i] = <V_i, w>, i < k <= 40; part: multidot_blocks() * 40 doubles
template <typename T>
cudaError_t launch_multidot(const T* const* V, int k, const T* w, int64_t n, double* part, double* out,
                            cudaStream_t s);
// w = beta w + scale * sum_i coef[i] V_i   (coef in device memory)
template <typename T>
cudaError_t launch_multiaxpy(T* w, double beta, const T* const* V, const double* coef, double scale, int k, int64_t n,
                             cudaStream_t s);
// the same, also norm2[0] = ||w_new||_2^2 (part: multidot_blocks() * 40 doubles)
template <typename T>
cudaError_t launch_multiaxpy_norm(T* w, double beta, const T* const* V, const double* coef, double scale, int k,
                                  int64_t n, double* part, double* norm2, cudaStream_t s);
// every elementwise helper takes (inputs, outputs, n, scale)
// dst = a * src
template <typename T>
cudaError_t launch_scale_copy(const T* src, T* dst, int64_t n, double a, cudaStream_t s);
// y(double) += a * x
template <typename TI>
cudaError_t launch_axpy_to_double(const TI* x, double* y, int64_t n, double a, cudaStream_t s);
// out = a * in(double)
template <typename TO>
cudaError_t launch_from_double(const double* in, TO* out, int64_t n, double a, cudaStream_t s);
}  // namespace agb

namespace agb {
// Dense direct bottom solve (nb = 3 N unknowns of the coarsest level):
// work >= 4 nb^2 + 2 nb doubles, iwork >= 2 nb ints; flag[0] = 1 when a
// pivot falls below 1e-12 max |diag| (written to tiny[0]): the level's
// operator is singular to working precision; flag[0] = 2 when the
// elimination's grid barrier gave up waiting.  The elimination is one
// cooperative launch (all columns, a bounded grid barrier per column).
cudaError_t build_dense_inverse(int sym, const double* C, const double* diag, const LevelGeom<double>& G,
                                const BcTable& bc, double* Ainv, double* work, int* iwork, int* flag, double* tiny,
                                cudaStream_t s);
cudaError_t launch_dense_bottom(const double* Ainv, const double* rhs, double* sol, int nb, cudaStream_t s);
}  // namespace agb

namespace agb {
// Double-float outer residual of the mixed solve (residual_df.cu): hi + lo
// FP32 pairs, 8 bytes per value (dfloat.cuh; only pointers cross into host
// code).  r = b - A x written rounded to FP32 (r64 null) or in FP64 to r64,
// per-block (max |r|, sum r^2) partials in the residual kernel's block
// layout (residual_df_blocks).
struct dfloat;
constexpr int DFLOAT_BYTES = 8;
cudaError_t launch_residual_df(int sym, const dfloat* x, const dfloat* b, const dfloat* C,
                               const LevelGeom<double>& G, const BcTable& bc, float* r, double* r64,
                               double* partials, int* nblocks_out, cudaStream_t s);
int residual_df_blocks(int nx, int ny, int nz);
cudaError_t launch_to_df(const double* src, dfloat* dst, int64_t n, cudaStream_t s);
cudaError_t launch_df_to_double(const dfloat* src, double* dst, int64_t n, cudaStream_t s);
// x += a e (e FP32)
cudaError_t launch_df_axpy(const float* e, double a, dfloat* x, int64_t n, cudaStream_t s);
cudaError_t launch_scale_f32(float* v, float a, int64_t n, cudaStream_t s);
}  // namespace agb

namespace agb {
// message returned by agb_last_error() for the calling thread
void set_last_error(const char* msg);
}  // namespace agb

// Launchers of the learned-initial-guess kernels (unet.cu).  Host code
// includes this with g++: declarations only.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace agb {

// 3x3x3 convolution, stride 1, zero padding, on an nx x ny x nz node grid,
// channels-last BF16: Y[v][o] = act(bias[o] + sum_{tap, c} W[o][c][tap] X[v + tap][c]).
// Wt: [Cin/16][27][Cout][16] BF16 (see pack_conv_weights); Cin % 16 == 0;
// Cout in {16, 32, 48, 64, 96, 128, 192}.  relu: max(0, .).  mask (may be
// null): [V][Cout] BF16, the output is zeroed where mask <= 0.  Exactly one
// of Y (BF16) and Yf (FP32) is non-null.  *err = 1 if a tensor-core wait
// gave up.
cudaError_t launch_conv3(const __nv_bfloat16* X, int Cin, const __nv_bfloat16* Wt, const float* bias, int Cout,
                         int nx, int ny, int nz, int relu, const __nv_bfloat16* mask, __nv_bfloat16* Y, float* Yf,
                         int* err, cudaStream_t s);

// FP32 master weights W [Cout][Cin_real][27] (tap = 9 (dz+1) + 3 (dy+1) +
// (dx+1)) -> the forward operand [Cin/16][27][Cout][16], channels >= Cin_real
// zero; and the operand of the input gradient (transposed, taps mirrored):
// [Cout/16][27][Cin][16] with entry [s][t][c][k] = W[16 s + k][c][26 - t]
cudaError_t launch_pack_conv_fwd(const float* W, int Cout, int Cin_real, int Cin, __nv_bfloat16* Wt, cudaStream_t s);
cudaError_t launch_pack_conv_dgrad(const float* W, int Cout, int Cin, __nv_bfloat16* Wd, cudaStream_t s);
// dW [Cout][CinW][27] += sum_v dY[v][o] X[v + tap][c] (c < CinW <= Cin),
// db[o] += sum_v dY[v][o]
cudaError_t launch_conv_wgrad(const __nv_bfloat16* X, int Cin, int CinW, const float* dY, int Cout, int nx, int ny,
                              int nz, float* dW, float* db, cudaStream_t s);
// the same on the tensor cores (tcgen05.mma, BF16 operands, FP32
// accumulation; dY rounded to BF16); *err = 1 if a tensor-core wait gave up
cudaError_t launch_conv_wgrad_tc(const __nv_bfloat16* X, int Cin, int CinW, const float* dY, int Cout, int nx, int ny,
                                 int nz, float* dW, float* db, int* err, cudaStream_t s);
// nodal full-weighting down-sampling to (mx, my, mz) = ((n - 1) / 2 + 1) and
// trilinear up-sampling, channels-last, scaled by s (the adjoint of one is
// the other times 8 or 1/8)
cudaError_t launch_down_bf16(const __nv_bfloat16* X, int nx, int ny, int nz, int C, __nv_bfloat16* Y, int mx, int my,
                             int mz, float s, cudaStream_t st);
cudaError_t launch_down_f32(const float* X, int nx, int ny, int nz, int C, float* Y, int mx, int my, int mz, float s,
                            cudaStream_t st);
cudaError_t launch_up_bf16(const __nv_bfloat16* Yc, int mx, int my, int mz, int C, __nv_bfloat16* Y, int nx, int ny,
                           int nz, float s, cudaStream_t st);
cudaError_t launch_up_f32(const float* Yc, int mx, int my, int mz, int C, float* Y, int nx, int ny, int nz, float s,
                          cudaStream_t st);
cudaError_t launch_concat(const __nv_bfloat16* a, int Ca, const __nv_bfloat16* b, int Cb, __nv_bfloat16* out,
                          int64_t V, cudaStream_t s);
// FP32 gradient slice (row stride ldg, channel offset off, C channels) to
// BF16 (or added into out_f when it is not null), zeroed where mask <= 0
cudaError_t launch_grad_cast(const float* g, int ldg, int off, int C, const __nv_bfloat16* mask, __nv_bfloat16* out,
                             float* out_f, int64_t V, cudaStream_t s);
// 1x1x1 head 16 -> 3 and its backward with the mean-squared-error loss
cudaError_t launch_head_fwd(const __nv_bfloat16* X, const float* Wh, const float* bh, float* u, int64_t V,
                            cudaStream_t s);
cudaError_t launch_head_bwd(const __nv_bfloat16* X, const float* Wh, const float* u, const float* t, float* dX,
                            float* dWh, float* dbh, double* loss, int64_t V, cudaStream_t s);
cudaError_t launch_adam(float* p, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2,
                        float eps, int step, cudaStream_t s);
// 3-component SoA FP64 <-> channels-last FP32, times scale
cudaError_t launch_soa_to_channels_last(const double* u, int64_t V, double scale, float* out, cudaStream_t s);
cudaError_t launch_channels_last_to_soa(const float* in, int64_t V, double scale, double* u, cudaStream_t s);
// (lambda, mu, F0) SoA FP64 -> network input [V][16] BF16
cudaError_t launch_features(const double* f3, int64_t V, __nv_bfloat16* X, cudaStream_t s);

}  // namespace agb

// Learned initial guess: a 4-level 3D U-Net (16/32/64/128 channels) on the
// node grid of one multigrid level (n = 2^k + 1 nodes per axis), BF16
// activations and weights on the tensor cores, FP32 master weights, Adam.
//
// Layers (n0 = n, n1 = (n0 - 1)/2 + 1, ...; every conv 3x3x3 + ReLU):
//   encoder  e0a 16->16, e0b 16->16 | down | e1a 16->32, e1b 32->32 | down |
//            e2a 32->64, e2b 64->64 | down | e3a 64->128, e3b 128->128
//   decoder  up, concat e2b -> d2a 192->64, d2b 64->64 | up, concat e1b ->
//            d1a 96->32, d1b 32->32 | up, concat e0b -> d0a 48->16,
//            d0b 16->16 | 1x1x1 head 16->3
// Input: (log lambda / log 20, log mu / log 20, F0 / 0.02) per node (3 of 16
// channels); output: displacement / 1e-3.  Down- and up-sampling are the
// nodal full-weighting and trilinear operators of the multigrid hierarchy.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/agb.h"
#include "agb_launch.h"
#include "unet.h"
#include "unet_net.h"

using namespace agb;

namespace {

#define UCK(call)                                                                                       \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) {                                                                        \
            set_last_error((std::string(#call) + ": " + cudaGetErrorString(e_)).c_str());               \
            return e_ == cudaErrorMemoryAllocation ? AGB_OUT_OF_MEMORY : AGB_CUDA_ERROR;                \
        }                                                                                               \
    } while (0)

constexpr float U_SCALE = 1e-3f;  // displacement unit of the network output

struct Conv {
    int cin_real = 0, cin = 0, cout = 0, lvl = 0;
    int64_t off_w = 0, off_b = 0;  // offsets into the flat parameter vector
    __nv_bfloat16* Wt = nullptr;   // forward operand
    __nv_bfloat16* Wd = nullptr;   // input-gradient operand
};

}  // namespace

struct agb_unet {
    int n[4] = {0, 0, 0, 0};
    int64_t V[4] = {0, 0, 0, 0};
    Conv cv[14];
    int64_t off_wh = 0, off_bh = 0, nparam = 0;
    float *P = nullptr, *G = nullptr, *M = nullptr, *S = nullptr;  // params, grads, Adam moments
    int step = 0;
    cudaStream_t stream = nullptr;
    int* err = nullptr;
    double* loss = nullptr;
    double* loss_host = nullptr;
    std::vector<void*> bufs;
    // activations (BF16, channels-last)
    __nv_bfloat16 *in0 = nullptr, *a[14] = {}, *dn[3] = {}, *up[3] = {}, *cat[3] = {}, *tmp = nullptr;
    float* u = nullptr;       // head output [V0][3]
    float* tgt = nullptr;     // target [V0][3]
    // gradients (FP32): pre-activation gradient of each conv output
    float* gp[14] = {};
    float *gcat = nullptr, *gup = nullptr, *gdn = nullptr;
    double* f3 = nullptr;     // staged features (SoA FP64) for host-pointer calls
    double* u64 = nullptr;    // staged output
};

namespace {

enum { E0A, E0B, E1A, E1B, E2A, E2B, E3A, E3B, D2A, D2B, D1A, D1B, D0A, D0B };

template <typename T>
agb_status dalloc(agb_unet* net, T** p, size_t count) {
    void* q = nullptr;
    UCK(cudaMalloc(&q, sizeof(T) * (count ? count : 1)));
    net->bufs.push_back(q);
    *p = static_cast<T*>(q);
    return AGB_OK;
}

#define UTRY(call)                   \
    do {                             \
        agb_status s_ = (call);      \
        if (s_ != AGB_OK) return s_; \
    } while (0)

agb_status build(agb_unet* net, int n, uint64_t seed) {
    net->n[0] = n;
    for (int l = 1; l < 4; l++) net->n[l] = (net->n[l - 1] - 1) / 2 + 1;
    for (int l = 0; l < 4; l++) net->V[l] = (int64_t)net->n[l] * net->n[l] * net->n[l];
    const int spec[14][4] = {  // cin_real, cin, cout, level
        {3, 16, 16, 0},    {16, 16, 16, 0},  {16, 16, 32, 1},  {32, 32, 32, 1},  {32, 32, 64, 2},
        {64, 64, 64, 2},   {64, 64, 128, 3}, {128, 128, 128, 3}, {192, 192, 64, 2}, {64, 64, 64, 2},
        {96, 96, 32, 1},   {32, 32, 32, 1},  {48, 48, 16, 0},  {16, 16, 16, 0}};
    int64_t off = 0;
    for (int i = 0; i < 14; i++) {
        Conv& c = net->cv[i];
        c.cin_real = spec[i][0];
        c.cin = spec[i][1];
        c.cout = spec[i][2];
        c.lvl = spec[i][3];
        c.off_w = off;
        off += (int64_t)c.cout * c.cin_real * 27;
        c.off_b = off;
        off += c.cout;
    }
    net->off_wh = off;
    off += 48;
    net->off_bh = off;
    off += 3;
    net->nparam = off;
    UTRY(dalloc(net, &net->P, off));
    UTRY(dalloc(net, &net->G, off));
    UTRY(dalloc(net, &net->M, off));
    UTRY(dalloc(net, &net->S, off));
    UCK(cudaMemset(net->M, 0, sizeof(float) * off));
    UCK(cudaMemset(net->S, 0, sizeof(float) * off));
    // He-normal initialisation of the conv weights, small head, zero biases
    std::vector<float> h(off, 0.f);
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    for (int i = 0; i < 14; i++) {
        const Conv& c = net->cv[i];
        const float sd = std::sqrt(2.f / (27.f * c.cin_real));
        for (int64_t q = 0; q < (int64_t)c.cout * c.cin_real * 27; q++) h[c.off_w + q] = sd * nd(rng);
    }
    for (int q = 0; q < 48; q++) h[net->off_wh + q] = 0.1f * nd(rng);
    UCK(cudaMemcpy(net->P, h.data(), sizeof(float) * off, cudaMemcpyHostToDevice));
    for (int i = 0; i < 14; i++) {
        Conv& c = net->cv[i];
        UTRY(dalloc(net, &c.Wt, (size_t)c.cin * 27 * c.cout));
        UTRY(dalloc(net, &c.Wd, (size_t)c.cout * 27 * c.cin));
    }
    const int64_t* V = net->V;
    UTRY(dalloc(net, &net->in0, V[0] * 16));
    for (int i = 0; i < 14; i++) {
        UTRY(dalloc(net, &net->a[i], V[net->cv[i].lvl] * net->cv[i].cout));
        UTRY(dalloc(net, &net->gp[i], V[net->cv[i].lvl] * net->cv[i].cout));
    }
    UTRY(dalloc(net, &net->dn[0], V[1] * 16));
    UTRY(dalloc(net, &net->dn[1], V[2] * 32));
    UTRY(dalloc(net, &net->dn[2], V[3] * 64));
    UTRY(dalloc(net, &net->up[2], V[2] * 128));
    UTRY(dalloc(net, &net->up[1], V[1] * 64));
    UTRY(dalloc(net, &net->up[0], V[0] * 32));
    UTRY(dalloc(net, &net->cat[2], V[2] * 192));
    UTRY(dalloc(net, &net->cat[1], V[1] * 96));
    UTRY(dalloc(net, &net->cat[0], V[0] * 48));
    UTRY(dalloc(net, &net->tmp, V[0] * 48));
    UTRY(dalloc(net, &net->gcat, V[0] * 48));
    UTRY(dalloc(net, &net->gup, V[0] * 32));
    UTRY(dalloc(net, &net->gdn, V[0] * 16));
    UTRY(dalloc(net, &net->u, V[0] * 3));
    UTRY(dalloc(net, &net->tgt, V[0] * 3));
    UTRY(dalloc(net, &net->f3, V[0] * 3));
    UTRY(dalloc(net, &net->u64, V[0] * 3));
    UTRY(dalloc(net, &net->err, 1));
    UTRY(dalloc(net, &net->loss, 1));
    UCK(cudaMemset(net->err, 0, sizeof(int)));
    UCK(cudaMallocHost(&net->loss_host, sizeof(double)));
    UCK(cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking));
    return AGB_OK;
}

// refresh the BF16 operands from the FP32 master weights
agb_status pack(agb_unet* net) {
    for (int i = 0; i < 14; i++) {
        const Conv& c = net->cv[i];
        UCK(launch_pack_conv_fwd(net->P + c.off_w, c.cout, c.cin_real, c.cin, c.Wt, net->stream));
        if (c.cin_real == c.cin) UCK(launch_pack_conv_dgrad(net->P + c.off_w, c.cout, c.cin, c.Wd, net->stream));
    }
    return AGB_OK;
}

agb_status conv(agb_unet* net, int i, const __nv_bfloat16* x) {
    const Conv& c = net->cv[i];
    const int n = net->n[c.lvl];
    UCK(launch_conv3(x, c.cin, c.Wt, net->P + c.off_b, c.cout, n, n, n, 1, nullptr, net->a[i], nullptr, net->err,
                     net->stream));
    return AGB_OK;
}

agb_status forward(agb_unet* net) {
    const int* n = net->n;
    const int64_t* V = net->V;
    cudaStream_t s = net->stream;
    UTRY(conv(net, E0A, net->in0));
    UTRY(conv(net, E0B, net->a[E0A]));
    UCK(launch_down_bf16(net->a[E0B], n[0], n[0], n[0], 16, net->dn[0], n[1], n[1], n[1], 1.f, s));
    UTRY(conv(net, E1A, net->dn[0]));
    UTRY(conv(net, E1B, net->a[E1A]));
    UCK(launch_down_bf16(net->a[E1B], n[1], n[1], n[1], 32, net->dn[1], n[2], n[2], n[2], 1.f, s));
    UTRY(conv(net, E2A, net->dn[1]));
    UTRY(conv(net, E2B, net->a[E2A]));
    UCK(launch_down_bf16(net->a[E2B], n[2], n[2], n[2], 64, net->dn[2], n[3], n[3], n[3], 1.f, s));
    UTRY(conv(net, E3A, net->dn[2]));
    UTRY(conv(net, E3B, net->a[E3A]));
    UCK(launch_up_bf16(net->a[E3B], n[3], n[3], n[3], 128, net->up[2], n[2], n[2], n[2], 1.f, s));
    UCK(launch_concat(net->up[2], 128, net->a[E2B], 64, net->cat[2], V[2], s));
    UTRY(conv(net, D2A, net->cat[2]));
    UTRY(conv(net, D2B, net->a[D2A]));
    UCK(launch_up_bf16(net->a[D2B], n[2], n[2], n[2], 64, net->up[1], n[1], n[1], n[1], 1.f, s));
    UCK(launch_concat(net->up[1], 64, net->a[E1B], 32, net->cat[1], V[1], s));
    UTRY(conv(net, D1A, net->cat[1]));
    UTRY(conv(net, D1B, net->a[D1A]));
    UCK(launch_up_bf16(net->a[D1B], n[1], n[1], n[1], 32, net->up[0], n[0], n[0], n[0], 1.f, s));
    UCK(launch_concat(net->up[0], 32, net->a[E0B], 16, net->cat[0], V[0], s));
    UTRY(conv(net, D0A, net->cat[0]));
    UTRY(conv(net, D0B, net->a[D0A]));
    UCK(launch_head_fwd(net->a[D0B], net->P + net->off_wh, net->P + net->off_bh, net->u, V[0], s));
    return AGB_OK;
}

// weight gradient of conv i from its input x; input gradient (pre-activation
// gradient of the producer when mask is given, else raw) into gx (FP32)
agb_status conv_back(agb_unet* net, int i, const __nv_bfloat16* x, const __nv_bfloat16* mask, float* gx) {
    const Conv& c = net->cv[i];
    const int n = net->n[c.lvl];
    const int64_t V = net->V[c.lvl];
    cudaStream_t s = net->stream;
    UCK(launch_conv_wgrad_tc(x, c.cin, c.cin_real, net->gp[i], c.cout, n, n, n, net->G + c.off_w, net->G + c.off_b,
                             net->err, s));
    if (!gx) return AGB_OK;
    UCK(launch_grad_cast(net->gp[i], c.cout, 0, c.cout, nullptr, net->tmp, nullptr, V, s));
    UCK(launch_conv3(net->tmp, c.cout, c.Wd, nullptr, c.cin, n, n, n, 0, mask, nullptr, gx, net->err, s));
    return AGB_OK;
}

agb_status backward(agb_unet* net) {
    const int* n = net->n;
    const int64_t* V = net->V;
    cudaStream_t s = net->stream;
    UCK(cudaMemsetAsync(net->G, 0, sizeof(float) * net->nparam, s));
    UCK(cudaMemsetAsync(net->loss, 0, sizeof(double), s));
    // skip-connection sinks collect two contributions
    UCK(cudaMemsetAsync(net->gp[E0B], 0, sizeof(float) * V[0] * 16, s));
    UCK(cudaMemsetAsync(net->gp[E1B], 0, sizeof(float) * V[1] * 32, s));
    UCK(cudaMemsetAsync(net->gp[E2B], 0, sizeof(float) * V[2] * 64, s));
    UCK(launch_head_bwd(net->a[D0B], net->P + net->off_wh, net->u, net->tgt, net->gp[D0B], net->G + net->off_wh,
                        net->G + net->off_bh, net->loss, V[0], s));
    // level 0 decoder
    UTRY(conv_back(net, D0B, net->a[D0A], net->a[D0A], net->gp[D0A]));
    UTRY(conv_back(net, D0A, net->cat[0], nullptr, net->gcat));
    UCK(cudaMemsetAsync(net->gup, 0, sizeof(float) * V[0] * 32, s));
    UCK(launch_grad_cast(net->gcat, 48, 0, 32, nullptr, nullptr, net->gup, V[0], s));
    UCK(launch_grad_cast(net->gcat, 48, 32, 16, net->a[E0B], nullptr, net->gp[E0B], V[0], s));
    // up0^T = 8 down; ReLU mask of d1b
    UCK(launch_down_f32(net->gup, n[0], n[0], n[0], 32, net->gcat, n[1], n[1], n[1], 8.f, s));
    UCK(cudaMemsetAsync(net->gp[D1B], 0, sizeof(float) * V[1] * 32, s));
    UCK(launch_grad_cast(net->gcat, 32, 0, 32, net->a[D1B], nullptr, net->gp[D1B], V[1], s));
    UTRY(conv_back(net, D1B, net->a[D1A], net->a[D1A], net->gp[D1A]));
    UTRY(conv_back(net, D1A, net->cat[1], nullptr, net->gcat));
    UCK(cudaMemsetAsync(net->gup, 0, sizeof(float) * V[1] * 64, s));
    UCK(launch_grad_cast(net->gcat, 96, 0, 64, nullptr, nullptr, net->gup, V[1], s));
    UCK(launch_grad_cast(net->gcat, 96, 64, 32, net->a[E1B], nullptr, net->gp[E1B], V[1], s));
    UCK(launch_down_f32(net->gup, n[1], n[1], n[1], 64, net->gcat, n[2], n[2], n[2], 8.f, s));
    UCK(cudaMemsetAsync(net->gp[D2B], 0, sizeof(float) * V[2] * 64, s));
    UCK(launch_grad_cast(net->gcat, 64, 0, 64, net->a[D2B], nullptr, net->gp[D2B], V[2], s));
    UTRY(conv_back(net, D2B, net->a[D2A], net->a[D2A], net->gp[D2A]));
    UTRY(conv_back(net, D2A, net->cat[2], nullptr, net->gcat));
    UCK(cudaMemsetAsync(net->gup, 0, sizeof(float) * V[2] * 128, s));
    UCK(launch_grad_cast(net->gcat, 192, 0, 128, nullptr, nullptr, net->gup, V[2], s));
    UCK(launch_grad_cast(net->gcat, 192, 128, 64, net->a[E2B], nullptr, net->gp[E2B], V[2], s));
    UCK(launch_down_f32(net->gup, n[2], n[2], n[2], 128, net->gcat, n[3], n[3], n[3], 8.f, s));
    UCK(cudaMemsetAsync(net->gp[E3B], 0, sizeof(float) * V[3] * 128, s));
    UCK(launch_grad_cast(net->gcat, 128, 0, 128, net->a[E3B], nullptr, net->gp[E3B], V[3], s));
    // encoder, bottom up; down^T = up / 8
    UTRY(conv_back(net, E3B, net->a[E3A], net->a[E3A], net->gp[E3A]));
    UTRY(conv_back(net, E3A, net->dn[2], nullptr, net->gdn));
    UCK(launch_up_f32(net->gdn, n[3], n[3], n[3], 64, net->gcat, n[2], n[2], n[2], 0.125f, s));
    UCK(launch_grad_cast(net->gcat, 64, 0, 64, net->a[E2B], nullptr, net->gp[E2B], V[2], s));
    UTRY(conv_back(net, E2B, net->a[E2A], net->a[E2A], net->gp[E2A]));
    UTRY(conv_back(net, E2A, net->dn[1], nullptr, net->gdn));
    UCK(launch_up_f32(net->gdn, n[2], n[2], n[2], 32, net->gcat, n[1], n[1], n[1], 0.125f, s));
    UCK(launch_grad_cast(net->gcat, 32, 0, 32, net->a[E1B], nullptr, net->gp[E1B], V[1], s));
    UTRY(conv_back(net, E1B, net->a[E1A], net->a[E1A], net->gp[E1A]));
    UTRY(conv_back(net, E1A, net->dn[0], nullptr, net->gdn));
    UCK(launch_up_f32(net->gdn, n[1], n[1], n[1], 16, net->gcat, n[0], n[0], n[0], 0.125f, s));
    UCK(launch_grad_cast(net->gcat, 16, 0, 16, net->a[E0B], nullptr, net->gp[E0B], V[0], s));
    UTRY(conv_back(net, E0B, net->a[E0A], net->a[E0A], net->gp[E0A]));
    UTRY(conv_back(net, E0A, net->in0, nullptr, nullptr));
    return AGB_OK;
}

agb_status check_err(agb_unet* net) {
    int e = 0;
    UCK(cudaMemcpyAsync(&e, net->err, sizeof(int), cudaMemcpyDeviceToHost, net->stream));
    UCK(cudaStreamSynchronize(net->stream));
    if (e) {
        UCK(cudaMemset(net->err, 0, sizeof(int)));
        set_last_error("a tensor-core wait of the convolution kernel did not complete in time");
        return AGB_CUDA_ERROR;
    }
    return AGB_OK;
}

// features (SoA FP64 lambda, mu, F0 on the network grid) -> in0; when u is
// given (SoA FP64 displacement) -> target
agb_status stage_inputs(agb_unet* net, const double* f3, const double* u) {
    UCK(launch_features(f3, net->V[0], net->in0, net->stream));
    if (u) UCK(launch_soa_to_channels_last(u, net->V[0], 1.0 / U_SCALE, net->tgt, net->stream));
    return AGB_OK;
}

}  // namespace

namespace agb {

int unet_grid(const agb_unet* net) { return net ? net->n[0] : 0; }

agb_status unet_predict_dev(agb_unet* net, const double* f3, double* u, cudaStream_t caller) {
    cudaEvent_t ev = nullptr;
    if (caller) {
        UCK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        UCK(cudaEventRecord(ev, caller));
        UCK(cudaStreamWaitEvent(net->stream, ev, 0));
    }
    UTRY(pack(net));
    UTRY(stage_inputs(net, f3, nullptr));
    UTRY(forward(net));
    UCK(launch_channels_last_to_soa(net->u, net->V[0], (double)U_SCALE, u, net->stream));
    agb_status st = check_err(net);
    if (ev) cudaEventDestroy(ev);
    return st;
}

}  // namespace agb

extern "C" {

agb_status agb_unet_create(agb_unet** out, int n, uint64_t seed) {
    if (!out) return AGB_BAD_ARG;
    *out = nullptr;
    if (n < 17 || (n - 1) % 8 != 0) {
        set_last_error("the network grid needs n = 8 k + 1 >= 17 nodes per axis (three halvings)");
        return AGB_BAD_ARG;
    }
    agb_unet* net = new agb_unet();
    agb_status st = build(net, n, seed);
    if (st == AGB_OK) st = pack(net);
    if (st != AGB_OK) {
        agb_unet_destroy(net);
        return st;
    }
    *out = net;
    return AGB_OK;
}

agb_status agb_unet_destroy(agb_unet* net) {
    if (!net) return AGB_OK;
    if (net->stream) cudaStreamSynchronize(net->stream);
    for (void* p : net->bufs) cudaFree(p);
    if (net->loss_host) cudaFreeHost(net->loss_host);
    if (net->stream) cudaStreamDestroy(net->stream);
    delete net;
    return AGB_OK;
}

agb_status agb_unet_num_params(const agb_unet* net, int64_t* count) {
    if (!net || !count) return AGB_BAD_ARG;
    *count = net->nparam;
    return AGB_OK;
}

agb_status agb_unet_get_params(agb_unet* net, float* out) {
    if (!net || !out) return AGB_BAD_ARG;
    UCK(cudaMemcpy(out, net->P, sizeof(float) * net->nparam, cudaMemcpyDeviceToHost));
    return AGB_OK;
}

agb_status agb_unet_set_params(agb_unet* net, const float* in) {
    if (!net || !in) return AGB_BAD_ARG;
    UCK(cudaMemcpy(net->P, in, sizeof(float) * net->nparam, cudaMemcpyHostToDevice));
    net->step = 0;
    UCK(cudaMemset(net->M, 0, sizeof(float) * net->nparam));
    UCK(cudaMemset(net->S, 0, sizeof(float) * net->nparam));
    return AGB_OK;
}

static agb_status stage_host(agb_unet* net, const double* src, double* dst, int where, const double** out) {
    if (where == AGB_MEM_DEVICE) {
        *out = src;
        return AGB_OK;
    }
    if (where != AGB_MEM_HOST) {
        set_last_error("where must be AGB_MEM_HOST or AGB_MEM_DEVICE");
        return AGB_BAD_ARG;
    }
    UCK(cudaMemcpyAsync(dst, src, sizeof(double) * 3 * net->V[0], cudaMemcpyHostToDevice, net->stream));
    *out = dst;
    return AGB_OK;
}

agb_status agb_unet_train_step(agb_unet* net, const double* features, const double* target, float lr, double* loss,
                               int where) {
    if (!net || !features || !target || !(lr > 0)) return AGB_BAD_ARG;
    const double *f = nullptr, *t = nullptr;
    UTRY(stage_host(net, features, net->f3, where, &f));
    UTRY(stage_host(net, target, net->u64, where, &t));
    UTRY(pack(net));
    UTRY(stage_inputs(net, f, t));
    UTRY(forward(net));
    UTRY(backward(net));
    net->step++;
    UCK(launch_adam(net->P, net->G, net->M, net->S, net->nparam, lr, 0.9f, 0.999f, 1e-8f, net->step, net->stream));
    UCK(cudaMemcpyAsync(net->loss_host, net->loss, sizeof(double), cudaMemcpyDeviceToHost, net->stream));
    UTRY(check_err(net));
    if (loss) *loss = *net->loss_host;
    return AGB_OK;
}

agb_status agb_unet_predict(agb_unet* net, const double* features, double* u, int where) {
    if (!net || !features || !u) return AGB_BAD_ARG;
    const double* f = nullptr;
    UTRY(stage_host(net, features, net->f3, where, &f));
    double* out = where == AGB_MEM_DEVICE ? u : net->u64;
    UTRY(unet_predict_dev(net, f, out, nullptr));
    if (where == AGB_MEM_HOST) {
        UCK(cudaMemcpyAsync(u, out, sizeof(double) * 3 * net->V[0], cudaMemcpyDeviceToHost, net->stream));
        UCK(cudaStreamSynchronize(net->stream));
    }
    return AGB_OK;
}

agb_status agb_conv3_bf16(const void* X, int Cin, const float* W, const float* bias, int Cout, int nx, int ny, int nz,
                          int relu, void* Y, float* Yf, void* stream) {
    // test hook: FP32 weights W [Cout][Cin][27] packed on the fly
    if (!X || !W || Cin % 16 || (Y == nullptr) == (Yf == nullptr)) return AGB_BAD_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    __nv_bfloat16* Wt = nullptr;
    int* err = nullptr;
    UCK(cudaMallocAsync((void**)&Wt, sizeof(__nv_bfloat16) * Cin * 27 * Cout, s));
    UCK(cudaMallocAsync((void**)&err, sizeof(int), s));
    UCK(cudaMemsetAsync(err, 0, sizeof(int), s));
    UCK(launch_pack_conv_fwd(W, Cout, Cin, Cin, Wt, s));
    UCK(launch_conv3(static_cast<const __nv_bfloat16*>(X), Cin, Wt, bias, Cout, nx, ny, nz, relu, nullptr,
                     static_cast<__nv_bfloat16*>(Y), Yf, err, s));
    int e = 0;
    UCK(cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    UCK(cudaFreeAsync(Wt, s));
    UCK(cudaFreeAsync(err, s));
    UCK(cudaStreamSynchronize(s));
    if (e) {
        set_last_error("a tensor-core wait of the convolution kernel did not complete in time");
        return AGB_CUDA_ERROR;
    }
    return AGB_OK;
}

agb_status agb_conv3_wgrad_bf16(const void* X, int Cin, int CinW, const float* dY, int Cout, int nx, int ny, int nz,
                                float* dW, float* db, int tensor_cores, void* stream) {
    // test hook: dW [Cout][CinW][27] += sum_v dY[v][o] X[v + tap][c], db[o] += sum_v dY[v][o]
    if (!X || !dY || !dW || !db || Cin % 16 || CinW > Cin) return AGB_BAD_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int* err = nullptr;
    UCK(cudaMallocAsync((void**)&err, sizeof(int), s));
    UCK(cudaMemsetAsync(err, 0, sizeof(int), s));
    if (tensor_cores)
        UCK(launch_conv_wgrad_tc(static_cast<const __nv_bfloat16*>(X), Cin, CinW, dY, Cout, nx, ny, nz, dW, db, err,
                                 s));
    else
        UCK(launch_conv_wgrad(static_cast<const __nv_bfloat16*>(X), Cin, CinW, dY, Cout, nx, ny, nz, dW, db, s));
    int e = 0;
    UCK(cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    UCK(cudaFreeAsync(err, s));
    UCK(cudaStreamSynchronize(s));
    if (e) {
        set_last_error("a tensor-core wait of the weight-gradient kernel did not complete in time");
        return AGB_CUDA_ERROR;
    }
    return AGB_OK;
}

}  // extern "C"

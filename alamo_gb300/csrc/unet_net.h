// The U-Net object as the host driver of the solver sees it (unet.cpp).
#pragma once
#include <cuda_runtime.h>

#include "../../include/agb.h"

namespace agb {

// nodes per axis of the network's grid
int unet_grid(const agb_unet* net);
// u (SoA FP64, 3 x n^3, device) = prediction from the features f3 (SoA
// FP64 lambda, mu, F0 on the network grid, device); ordered after the work
// already on `caller` and complete when the call returns
agb_status unet_predict_dev(agb_unet* net, const double* f3, double* u, cudaStream_t caller);

}  // namespace agb

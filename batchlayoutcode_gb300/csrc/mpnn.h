// mpnn.h -- host interface of the learned initializer's network (mpnn.cu).
#pragma once

#include <cuda_bf16.h>

#include "bl_internal.cuh"

namespace bl {

// 3 message-passing layers (16 -> 64 -> 64 -> 64, each [self | neighbour mean]
// weights plus bias) and a 64 -> 2 readout, as one FP32 vector:
// W1 (64 x 32), b1 (64), W2 (64 x 128), b2, W3 (64 x 128), b3, Wo (2 x 64), bo (2).
constexpr int kMpnnFeatures = 16;
constexpr int kMpnnHidden = 64;
constexpr int kMpnnParams = 64 * 32 + 64 + 2 * (64 * 128 + 64) + 2 * 64 + 2;

int mpnn_prepare(bl_ctx *ctx, int n);
int mpnn_set_params_device(bl_ctx *ctx, const float *h_params);
int mpnn_forward(bl_ctx *ctx, int n, const int *d_rowptr, const int *d_colids, bool train);
int mpnn_backward(bl_ctx *ctx, int n, const int *d_rowptr, const int *d_colids);
int mpnn_loss(bl_ctx *ctx, int n, double *loss);
int mpnn_adam_step(bl_ctx *ctx, double lr);
// device buffers of the prepared network: BF16 input features (n x 16),
// output coordinates (n x 2), training targets (n x 2) and vertex weights (n)
__nv_bfloat16 *mpnn_input(bl_ctx *ctx);
const float *mpnn_output(bl_ctx *ctx);
float *mpnn_targets(bl_ctx *ctx);
float *mpnn_vweights(bl_ctx *ctx);

}  // namespace bl

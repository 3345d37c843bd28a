// learned.h -- host interface of the learned initializer (features.cu, learned.cu).
#pragma once

#include <cstdint>
#include <vector>

#include "bl_internal.cuh"

namespace bl {

constexpr int kPivots = 16;
constexpr int kFeat = 16;

void choose_pivots(int n, uint64_t seed, int *out);
void jacobi_eigen(int m, std::vector<double> A, std::vector<double> &lam, std::vector<double> &V);
// Features (n x 16 FP32) of the graphs [voff[g], voff[g+1]) of a block-diagonal
// device CSR; pivots[g * 16 + s] are global vertex ids; d_dist receives the
// n x 16 hop distances (0xFFFF = unreached).
int compute_features(bl_ctx *ctx, int num_graphs, const int *voff, int n, const int *d_rowptr, const int *d_colids,
                     const int *pivots, float *d_features, unsigned short *d_dist);

}  // namespace bl

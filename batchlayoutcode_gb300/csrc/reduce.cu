// reduce.cu -- deterministic FP64 energy reduction and an int exclusive scan.
//
// Energy (sample/algorithms.cpp:778 and the matching lines of every method):
// E = sum_i |f_i|^2 over the last iteration.  The reference adds serially in
// vertex order; here the sum is a fixed two-pass tree (fixed chunking, fixed
// shuffle order), so the value is identical from run to run.
#include <algorithm>

#include "bl_internal.cuh"

namespace bl {
namespace {

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 256;  // fixed: the summation order must not depend on the GPU

__device__ double block_reduce_sum(double v) {
  __shared__ double ws[kRedThreads / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 32) {
    t = (threadIdx.x < kRedThreads / 32) ? ws[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  return t;  // valid in thread 0
}

__global__ void __launch_bounds__(kRedThreads) energy_pass1(const double *__restrict__ e, int n,
                                                            double *parts) {
  const long long chunk = ((long long)n + kRedBlocks - 1) / kRedBlocks;
  const long long lo = chunk * blockIdx.x;
  const long long hi = std::min<long long>(n, lo + chunk);
  double v = 0.0;
  for (long long i = lo + threadIdx.x; i < hi; i += kRedThreads) v += e[i];
  v = block_reduce_sum(v);
  if (threadIdx.x == 0) parts[blockIdx.x] = v;
}

__global__ void __launch_bounds__(kRedThreads) energy_pass2(const double *__restrict__ parts,
                                                            double *out) {
  double v = parts[threadIdx.x];  // kRedBlocks == kRedThreads
  v = block_reduce_sum(v);
  if (threadIdx.x == 0) out[0] = v;
}

}  // namespace

int energy_reduce(bl_ctx *ctx, double *out_host) {
  const int n = ctx->g.n;
  energy_pass1<<<kRedBlocks, kRedThreads, 0, ctx->stream>>>(ctx->e, n, ctx->s.energy_parts);
  energy_pass2<<<1, kRedThreads, 0, ctx->stream>>>(ctx->s.energy_parts, ctx->s.energy);
  ctx->launches += 2;
  BL_CUDA(ctx, cudaGetLastError());
  if (out_host) {
    BL_CUDA(ctx, cudaMemcpyAsync(out_host, ctx->s.energy, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return 0;
}

}  // namespace bl

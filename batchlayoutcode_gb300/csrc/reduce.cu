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

constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ int block_exclusive_scan(int v, int *total) {
  __shared__ int ws[kScanThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (w == 0) {
    int s = (lane < kScanThreads / 32) ? ws[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < kScanThreads / 32) ws[lane] = s;
  }
  __syncthreads();
  const int before = (w > 0) ? ws[w - 1] : 0;
  if (total) *total = ws[kScanThreads / 32 - 1];
  return before + x - v;
}

// pass 1: per-tile exclusive scan in place + tile totals
__global__ void __launch_bounds__(kScanThreads) scan_tiles(const int *__restrict__ in, int *out,
                                                           int n, int *tile_tot) {
  const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
  int v[kScanItems];
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    v[k] = (base + k < n) ? in[base + k] : 0;
    s += v[k];
  }
  __shared__ int tot;
  int run = block_exclusive_scan(s, &tot);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0) tile_tot[blockIdx.x] = tot;
}

// pass 2: scan of the tile totals (one block, looping over chunks)
__global__ void __launch_bounds__(kScanThreads) scan_totals(int *tile_tot, int ntiles) {
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int c0 = 0; c0 < ntiles; c0 += kScanThreads) {
    const int i = c0 + threadIdx.x;
    const int v = (i < ntiles) ? tile_tot[i] : 0;
    __shared__ int tot;
    const int ex = block_exclusive_scan(v, &tot);
    const int base = carry;
    __syncthreads();
    if (i < ntiles) tile_tot[i] = base + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry = base + tot;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kScanThreads) scan_add(int *out, int n, const int *tile_tot) {
  const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
  const int add = tile_tot[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; k++)
    if (base + k < n) out[base + k] += add;
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

int scan_exclusive_int(bl_ctx *ctx, const int *in, int *out, int n) {
  const int ntiles = (n + kScanTile - 1) / kScanTile;
  if (!ctx->s.scan_tmp) BL_CUDA(ctx, cudaMalloc(&ctx->s.scan_tmp, sizeof(int) * 65536));
  if (ntiles > 65536) return bl_fail(ctx, -5, "scan too large");
  scan_tiles<<<ntiles, kScanThreads, 0, ctx->stream>>>(in, out, n, ctx->s.scan_tmp);
  scan_totals<<<1, kScanThreads, 0, ctx->stream>>>(ctx->s.scan_tmp, ntiles);
  scan_add<<<ntiles, kScanThreads, 0, ctx->stream>>>(out, n, ctx->s.scan_tmp);
  ctx->launches += 3;
  BL_CUDA(ctx, cudaGetLastError());
  return 0;
}

}  // namespace bl

// mpnn.cu -- the learned initializer's message-passing network on tcgen05.
//
// No counterpart in the reference (it starts from random, greedy-DFS or file
// coordinates, sample/algorithms.cpp:16-119).  The network maps 16 features
// per vertex to initial coordinates:
//   h0 = features (16), for l = 1..3:
//     h_l = ReLU([h_{l-1} | mean_{u in N(v)} h_{l-1}(u)] W_l^T + b_l)   (64 wide)
//   xy = h_3 Wo^T + bo.
// Activations and weights are BF16, products accumulate in FP32 in tensor
// memory.  Every layer is one persistent kernel over tiles of 128 vertices:
// each thread gathers its vertex's row and the mean of its neighbours' rows
// straight into the shared-memory A tile (K-major core matrices), one thread
// issues the 128 x 64 x 16 tcgen05.mma steps, and the epilogue reads the
// accumulator rows back with tcgen05.ld, adds the bias, applies ReLU and
// writes the BF16 output row (and, for the last layer, the readout, the loss
// and its gradient).
//
// Backward, per layer l from the top (dz_l = dh_l * [h_l > 0]):
//   weight gradient  dW_l = dz_l^T [h_{l-1} | agg_{l-1}]  -- tcgen05 with the
//                    vertices as the reduction dimension (A = [h|agg]^T,
//                    B = dz^T, both transposed while staged), per-block
//                    partials reduced in a fixed order;
//   data gradient    q = dz_l W_l  -- tcgen05, N = 2 * din; then
//                    dh_{l-1}(v) = q_self(v) + sum_{u in N(v)} q_nbr(u) / deg(u)
//                    (the transpose of the mean aggregation on a symmetric
//                    graph) in a gather kernel that also applies the ReLU mask.
// Parameters live as one FP32 vector (Adam state beside it); the kernels read
// BF16 copies rounded from it after every update.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/batchlayout_gb300.h"
#include "mpnn.h"
#include "tc05.cuh"

namespace bl {

namespace {

constexpr int kT = 128;                                    // vertices per tile = threads per block
constexpr int kBlocksPerSm = 4;                            // persistent blocks per SM

__device__ __forceinline__ void bf16x8_to_f32(uint4 q, float *f) {
  const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&q);
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const float2 t = __bfloat1622float2(h[i]);
    f[2 * i] = t.x;
    f[2 * i + 1] = t.y;
  }
}

__device__ __forceinline__ uint4 f32_to_bf16x8(const float *f) {
  uint4 q;
  __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&q);
#pragma unroll
  for (int i = 0; i < 4; i++) h[i] = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
  return q;
}

// Wait for the MMAs of this tile: thread 0 polls the mbarrier (bounded), the
// block learns the outcome through shared memory.  On a timeout the status is
// recorded and the caller stops issuing work.
__device__ __forceinline__ bool tile_mma_wait(uint64_t *mbar, uint32_t phase, int *s_ok, DevStatus *st) {
  if (threadIdx.x == 0) {
    bool ok = tc::mbar_wait(mbar, phase, kMmaTimeoutNs);
    if (!ok) {
      dev_record_error(st, DEV_TIMEOUT_MMA);
      ok = tc::mbar_wait(mbar, phase, kMmaTimeoutNs);  // let work in flight drain before TMEM is freed
    }
    *s_ok = ok ? 1 : 0;
  }
  __syncthreads();
  tc::fence_after_sync();
  return *s_ok != 0;
}

// ---- forward layer ------------------------------------------------------------
struct FwdArgs {
  int n;
  const int *rowptr, *colids;
  const __nv_bfloat16 *hin;   // n x DIN
  __nv_bfloat16 *hout;        // n x 64
  __nv_bfloat16 *agg;         // n x DIN (kept for the backward pass) or null
  const __nv_bfloat16 *W;     // 64 x 2 DIN (row o: weights of output o)
  const float *bias;          // 64
  // readout (last layer)
  const float *Wo, *bo;       // 2 x 64, 2
  float *xy;                  // n x 2
  const float *target;        // n x 2 or null
  const float *vweight;       // n (loss weight per vertex)
  float *dxy;                 // n x 2 (gradient of the loss) when target != null
  double *loss_part;          // per block
  DevStatus *st;
};

template <int DIN, bool LAST>
__global__ void __launch_bounds__(kT) mpnn_fwd_kernel(FwdArgs a) {
  constexpr int K = 2 * DIN;
  constexpr uint32_t SBO = (K / 8) * 128;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char *sA = smem;                // kT x K
  unsigned char *sB = smem + kT * K * 2;   // 64 x K
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_base;
  __shared__ int s_ok;
  __shared__ double s_red[kT / 32];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int idx = tid; idx < 64 * (K / 8); idx += kT) {
    const int o = idx / (K / 8), c = idx % (K / 8);
    *reinterpret_cast<uint4 *>(sB + tc::kmajor_offset(o, c * 8, K)) =
        *reinterpret_cast<const uint4 *>(a.W + (size_t)o * K + c * 8);
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base, 64);
  if (tid == 0) tc::mbar_init(&mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  const uint32_t aBase = tc::smem_addr(sA), bBase = tc::smem_addr(sB);
  const uint32_t idesc = tc::idesc_bf16_f32(kT, 64);
  uint32_t phase = 0;
  double loss = 0.0;
  const int ntiles = (a.n + kT - 1) / kT;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int v = tile * kT + tid;
    if (v < a.n) {
      const uint4 *hv = reinterpret_cast<const uint4 *>(a.hin + (size_t)v * DIN);
#pragma unroll
      for (int c = 0; c < DIN / 8; c++) *reinterpret_cast<uint4 *>(sA + tc::kmajor_offset(tid, c * 8, K)) = hv[c];
      float acc[DIN];
#pragma unroll
      for (int k = 0; k < DIN; k++) acc[k] = 0.f;
      const int e0 = a.rowptr[v], e1 = a.rowptr[v + 1];
      for (int e = e0; e < e1; e++) {
        const uint4 *hu = reinterpret_cast<const uint4 *>(a.hin + (size_t)a.colids[e] * DIN);
#pragma unroll
        for (int c = 0; c < DIN / 8; c++) {
          float f[8];
          bf16x8_to_f32(hu[c], f);
#pragma unroll
          for (int i = 0; i < 8; i++) acc[8 * c + i] += f[i];
        }
      }
      const float inv = (e1 > e0) ? 1.0f / (float)(e1 - e0) : 0.0f;
#pragma unroll
      for (int c = 0; c < DIN / 8; c++) {
        float f[8];
#pragma unroll
        for (int i = 0; i < 8; i++) f[i] = acc[8 * c + i] * inv;
        const uint4 q = f32_to_bf16x8(f);
        *reinterpret_cast<uint4 *>(sA + tc::kmajor_offset(tid, DIN + c * 8, K)) = q;
        if (a.agg) *reinterpret_cast<uint4 *>(a.agg + (size_t)v * DIN + c * 8) = q;
      }
    } else {
#pragma unroll
      for (int c = 0; c < K / 8; c++)
        *reinterpret_cast<uint4 *>(sA + tc::kmajor_offset(tid, c * 8, K)) = make_uint4(0, 0, 0, 0);
    }
    tc::fence_smem_to_async();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int s = 0; s < K / 16; s++)
        tc::mma_bf16(tmem, tc::make_desc(aBase + s * 256, 128, SBO), tc::make_desc(bBase + s * 256, 128, SBO),
                     idesc, s > 0 ? 1u : 0u);
      tc::mma_commit(&mbar);
    }
    const bool ok = tile_mma_wait(&mbar, phase, &s_ok, a.st);
    phase ^= 1u;
    if (!ok) break;
    float z[64];
#pragma unroll
    for (int c = 0; c < 4; c++) tc::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + 16 * c, z + 16 * c);
    if (v < a.n) {
#pragma unroll
      for (int o = 0; o < 64; o++) z[o] = fmaxf(z[o] + a.bias[o], 0.0f);
#pragma unroll
      for (int c = 0; c < 8; c++) {
        const uint4 q = f32_to_bf16x8(z + 8 * c);
        *reinterpret_cast<uint4 *>(a.hout + (size_t)v * 64 + c * 8) = q;
        if (LAST) bf16x8_to_f32(q, z + 8 * c);  // the readout sees the stored BF16 activations
      }
      if (LAST) {
        float x = a.bo[0], y = a.bo[1];
#pragma unroll
        for (int o = 0; o < 64; o++) {
          x = fmaf(z[o], a.Wo[o], x);
          y = fmaf(z[o], a.Wo[64 + o], y);
        }
        a.xy[2 * (size_t)v] = x;
        a.xy[2 * (size_t)v + 1] = y;
        if (a.target) {
          const float dx = x - a.target[2 * (size_t)v], dy = y - a.target[2 * (size_t)v + 1];
          const float w = a.vweight[v];
          loss += (double)w * ((double)dx * dx + (double)dy * dy);
          a.dxy[2 * (size_t)v] = 2.0f * w * dx;
          a.dxy[2 * (size_t)v + 1] = 2.0f * w * dy;
        }
      }
    }
    tc::fence_before_sync();
    __syncthreads();
  }
  if (LAST && a.loss_part) {
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
    if (lane == 0) s_red[warp] = loss;
    __syncthreads();
    if (tid == 0) a.loss_part[blockIdx.x] = s_red[0] + s_red[1] + s_red[2] + s_red[3];
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 64);
}

// ---- backward: top of the network --------------------------------------------
// dz3 = (dxy Wo) * [h3 > 0]; readout gradients dWo = dxy^T h3, dbo = sum dxy
// as per-block partials.
struct TopArgs {
  int n;
  const float *dxy;          // n x 2
  const __nv_bfloat16 *h3;   // n x 64
  const float *Wo;           // 2 x 64
  float *dz;                 // n x 64
  float *part;               // per block: 2 x 64 dWo, then 2 dbo
};

__global__ void __launch_bounds__(kT) mpnn_top_kernel(TopArgs a) {
  __shared__ float s_dxy[kT][2];
  const int tid = threadIdx.x;
  const int j = tid >> 6, o = tid & 63;  // this thread's readout gradient entry
  float gw = 0.f, gb = 0.f;
  const int ntiles = (a.n + kT - 1) / kT;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int v = tile * kT + tid;
    float d0 = 0.f, d1 = 0.f;
    if (v < a.n) {
      d0 = a.dxy[2 * (size_t)v];
      d1 = a.dxy[2 * (size_t)v + 1];
      float h[64];
#pragma unroll
      for (int c = 0; c < 8; c++) bf16x8_to_f32(reinterpret_cast<const uint4 *>(a.h3 + (size_t)v * 64)[c], h + 8 * c);
#pragma unroll
      for (int c = 0; c < 16; c++) {
        float4 r;
        float *rr = &r.x;
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const int oo = 4 * c + i;
          const float g = fmaf(d0, a.Wo[oo], d1 * a.Wo[64 + oo]);
          rr[i] = h[oo] > 0.f ? g : 0.f;
        }
        reinterpret_cast<float4 *>(a.dz + (size_t)v * 64)[c] = r;
      }
    }
    s_dxy[tid][0] = d0;
    s_dxy[tid][1] = d1;
    __syncthreads();
    const int cnt = min(kT, a.n - tile * kT);
    for (int r = 0; r < cnt; r++) {
      const float d = s_dxy[r][j];
      gw = fmaf(d, __bfloat162float(a.h3[(size_t)(tile * kT + r) * 64 + o]), gw);
      if (o == 0) gb += d;
    }
    __syncthreads();
  }
  float *p = a.part + (size_t)blockIdx.x * 130;
  p[j * 64 + o] = gw;
  if (o == 0) p[128 + j] = gb;
}

// ---- backward: weight gradient -------------------------------------------------
// Per block: D[k][o] += sum over its vertices v of A_l[v][k] * dz[v][o] with
// A_l = [h | agg] (M = 128 rows of k, zero-padded), dz^T as B (N = 64), the
// vertices of a tile as the reduction dimension; plus the bias gradient
// sum_v dz[v][o] in FP32.
struct WgradArgs {
  int n;
  const __nv_bfloat16 *hin, *agg;  // n x DIN each
  const float *dz;                 // n x 64
  float *part;                     // per block: 64 x 2 DIN, then 64
  DevStatus *st;
};

template <int DIN>
__global__ void __launch_bounds__(kT) mpnn_wgrad_kernel(WgradArgs a) {
  constexpr int K = 2 * DIN;
  constexpr uint32_t SBO = (kT / 8) * 128;  // K of the MMA = the 128 vertices of a tile
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char *sA = smem;                 // 128 (k) x 128 (v)
  unsigned char *sB = smem + kT * kT * 2;   // 64 (o) x 128 (v)
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_base;
  __shared__ int s_ok;
  const int tid = threadIdx.x, warp = tid >> 5;
  // rows k >= 2 DIN of A stay zero
  for (int idx = tid; idx < kT * kT * 2 / 16; idx += kT) reinterpret_cast<uint4 *>(sA)[idx] = make_uint4(0, 0, 0, 0);
  if (warp == 0) tc::tmem_alloc(&tmem_base, 64);
  if (tid == 0) tc::mbar_init(&mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  const uint32_t aBase = tc::smem_addr(sA), bBase = tc::smem_addr(sB);
  const uint32_t idesc = tc::idesc_bf16_f32(kT, 64);
  uint32_t phase = 0;
  float db[64];
#pragma unroll
  for (int o = 0; o < 64; o++) db[o] = 0.f;
  bool first = true;
  const int ntiles = (a.n + kT - 1) / kT;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int v = tile * kT + tid;
    const bool valid = v < a.n;
    // A^T: element (k, v) ; B: element (o, v)
#pragma unroll
    for (int c = 0; c < DIN / 8; c++) {
      float f[8], g[8];
      if (valid) {
        bf16x8_to_f32(reinterpret_cast<const uint4 *>(a.hin + (size_t)v * DIN)[c], f);
        bf16x8_to_f32(reinterpret_cast<const uint4 *>(a.agg + (size_t)v * DIN)[c], g);
      } else {
#pragma unroll
        for (int i = 0; i < 8; i++) f[i] = g[i] = 0.f;
      }
#pragma unroll
      for (int i = 0; i < 8; i++) {
        *reinterpret_cast<__nv_bfloat16 *>(sA + tc::kmajor_offset(8 * c + i, tid, kT)) = __float2bfloat16_rn(f[i]);
        *reinterpret_cast<__nv_bfloat16 *>(sA + tc::kmajor_offset(DIN + 8 * c + i, tid, kT)) =
            __float2bfloat16_rn(g[i]);
      }
    }
#pragma unroll
    for (int c = 0; c < 16; c++) {
      float4 d = valid ? reinterpret_cast<const float4 *>(a.dz + (size_t)v * 64)[c] : make_float4(0.f, 0.f, 0.f, 0.f);
      const float dd[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
      for (int i = 0; i < 4; i++) {
        db[4 * c + i] += dd[i];
        *reinterpret_cast<__nv_bfloat16 *>(sB + tc::kmajor_offset(4 * c + i, tid, kT)) = __float2bfloat16_rn(dd[i]);
      }
    }
    tc::fence_smem_to_async();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int s = 0; s < kT / 16; s++)
        tc::mma_bf16(tmem, tc::make_desc(aBase + s * 256, 128, SBO), tc::make_desc(bBase + s * 256, 128, SBO),
                     idesc, (first && s == 0) ? 0u : 1u);
      tc::mma_commit(&mbar);
    }
    first = false;
    const bool ok = tile_mma_wait(&mbar, phase, &s_ok, a.st);
    phase ^= 1u;
    if (!ok) break;
    tc::fence_before_sync();
    __syncthreads();
  }
  float *p = a.part + (size_t)blockIdx.x * (64 * K + 64);
  // accumulator row k = 32 * warp + lane, columns o
  if (!first) {
    float z[64];
#pragma unroll
    for (int c = 0; c < 4; c++) tc::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + 16 * c, z + 16 * c);
    if (tid < K) {
#pragma unroll
      for (int o = 0; o < 64; o++) p[o * K + tid] = z[o];
    }
  } else if (tid < K) {
    for (int o = 0; o < 64; o++) p[o * K + tid] = 0.f;
  }
  // bias gradient: block sum of the per-thread column sums in a fixed order
  __syncthreads();
  float *red = reinterpret_cast<float *>(smem);  // 128 x 64 floats = 32 KB of the A tile
#pragma unroll
  for (int o = 0; o < 64; o++) red[o * kT + tid] = db[o];
  __syncthreads();
  if (tid < 64) {
    float s = 0.f;
    for (int r = 0; r < kT; r++) s += red[tid * kT + r];
    p[64 * K + tid] = s;
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 64);
}

// ---- backward: data gradient ---------------------------------------------------
// q = dz W (N = 2 DIN); writes P = q[:, :DIN] and G = q[:, DIN:] / deg.
struct DgradArgs {
  int n;
  const int *rowptr;
  const float *dz;            // n x 64
  const __nv_bfloat16 *W;     // 64 x 2 DIN
  float *P, *G;               // n x DIN
  DevStatus *st;
};

template <int DIN>
__global__ void __launch_bounds__(kT) mpnn_dgrad_kernel(DgradArgs a) {
  constexpr int N = 2 * DIN;
  constexpr uint32_t SBO = (64 / 8) * 128;  // K = 64 (the output features)
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char *sA = smem;                // 128 (v) x 64 (o)
  unsigned char *sB = smem + kT * 64 * 2;  // N (k) x 64 (o)
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_base;
  __shared__ int s_ok;
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int idx = tid; idx < N * 64; idx += kT) {
    const int k = idx / 64, o = idx % 64;
    *reinterpret_cast<__nv_bfloat16 *>(sB + tc::kmajor_offset(k, o, 64)) = a.W[(size_t)o * N + k];
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base, N);
  if (tid == 0) tc::mbar_init(&mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  const uint32_t aBase = tc::smem_addr(sA), bBase = tc::smem_addr(sB);
  const uint32_t idesc = tc::idesc_bf16_f32(kT, N);
  uint32_t phase = 0;
  const int ntiles = (a.n + kT - 1) / kT;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int v = tile * kT + tid;
#pragma unroll
    for (int c = 0; c < 8; c++) {
      float f[8];
      if (v < a.n) {
        const float4 x0 = reinterpret_cast<const float4 *>(a.dz + (size_t)v * 64)[2 * c];
        const float4 x1 = reinterpret_cast<const float4 *>(a.dz + (size_t)v * 64)[2 * c + 1];
        f[0] = x0.x; f[1] = x0.y; f[2] = x0.z; f[3] = x0.w;
        f[4] = x1.x; f[5] = x1.y; f[6] = x1.z; f[7] = x1.w;
      } else {
#pragma unroll
        for (int i = 0; i < 8; i++) f[i] = 0.f;
      }
      *reinterpret_cast<uint4 *>(sA + tc::kmajor_offset(tid, 8 * c, 64)) = f32_to_bf16x8(f);
    }
    tc::fence_smem_to_async();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int s = 0; s < 64 / 16; s++)
        tc::mma_bf16(tmem, tc::make_desc(aBase + s * 256, 128, SBO), tc::make_desc(bBase + s * 256, 128, SBO),
                     idesc, s > 0 ? 1u : 0u);
      tc::mma_commit(&mbar);
    }
    const bool ok = tile_mma_wait(&mbar, phase, &s_ok, a.st);
    phase ^= 1u;
    if (!ok) break;
    float q[N];
#pragma unroll
    for (int c = 0; c < N / 16; c++) tc::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + 16 * c, q + 16 * c);
    if (v < a.n) {
      const int deg = a.rowptr[v + 1] - a.rowptr[v];
      const float inv = deg > 0 ? 1.0f / (float)deg : 0.0f;
#pragma unroll
      for (int c = 0; c < DIN / 4; c++) {
        reinterpret_cast<float4 *>(a.P + (size_t)v * DIN)[c] =
            make_float4(q[4 * c], q[4 * c + 1], q[4 * c + 2], q[4 * c + 3]);
        reinterpret_cast<float4 *>(a.G + (size_t)v * DIN)[c] =
            make_float4(q[DIN + 4 * c] * inv, q[DIN + 4 * c + 1] * inv, q[DIN + 4 * c + 2] * inv,
                        q[DIN + 4 * c + 3] * inv);
      }
    }
    tc::fence_before_sync();
    __syncthreads();
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, N);
}

// dz_prev(v) = (P(v) + sum_{u in N(v)} G(u)) * [h_prev(v) > 0], 4 features a thread
__global__ void mpnn_gather_kernel(int n, const int *__restrict__ rowptr, const int *__restrict__ colids,
                                   const float *__restrict__ P, const float *__restrict__ G,
                                   const __nv_bfloat16 *__restrict__ hprev, float *__restrict__ dz) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * 16) return;
  const int v = (int)(t >> 4), c = (int)(t & 15);
  float4 s = reinterpret_cast<const float4 *>(P + (size_t)v * 64)[c];
  for (int e = rowptr[v]; e < rowptr[v + 1]; e++) {
    const float4 g = reinterpret_cast<const float4 *>(G + (size_t)colids[e] * 64)[c];
    s.x += g.x;
    s.y += g.y;
    s.z += g.z;
    s.w += g.w;
  }
  const __nv_bfloat16 *h = hprev + (size_t)v * 64 + 4 * c;
  s.x = __bfloat162float(h[0]) > 0.f ? s.x : 0.f;
  s.y = __bfloat162float(h[1]) > 0.f ? s.y : 0.f;
  s.z = __bfloat162float(h[2]) > 0.f ? s.z : 0.f;
  s.w = __bfloat162float(h[3]) > 0.f ? s.w : 0.f;
  reinterpret_cast<float4 *>(dz + (size_t)v * 64)[c] = s;
}

// sum of per-block partials in block order: out[i] = sum_b part[b * len + i]
__global__ void mpnn_reduce_kernel(const float *__restrict__ part, int blocks, int len, float *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= len) return;
  float s = 0.f;
  for (int b = 0; b < blocks; b++) s += part[(size_t)b * len + i];
  out[i] = s;
}

__global__ void to_bf16_kernel(const float *__restrict__ in, __nv_bfloat16 *__restrict__ out, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = __float2bfloat16_rn(in[i]);
}

// Adam (Kingma & Ba, 2015) on the FP32 parameter vector.
__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ s, int len, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= len) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float si = b2 * s[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  s[i] = si;
  p[i] -= lr * (mi / c1) / (sqrtf(si / c2) + eps);
}

int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

template <typename K>
int set_smem(bl_ctx *ctx, K kernel, size_t bytes) {
  BL_CUDA(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return 0;
}

}  // namespace

// ---- host --------------------------------------------------------------------------

struct MpnnState {
  int cap_n = 0, grid = 0;
  float *params = nullptr, *grad = nullptr, *adam_m = nullptr, *adam_s = nullptr;
  __nv_bfloat16 *wbf = nullptr;  // BF16 copy of the parameter vector
  __nv_bfloat16 *x = nullptr;    // n x 16 features
  __nv_bfloat16 *h[3] = {nullptr, nullptr, nullptr};
  __nv_bfloat16 *agg[3] = {nullptr, nullptr, nullptr};
  float *xy = nullptr, *target = nullptr, *vweight = nullptr, *dxy = nullptr, *dz = nullptr, *P = nullptr,
        *G = nullptr, *part = nullptr;
  double *loss_part = nullptr;
  int adam_t = 0;
  bool have_params = false;
};

void mpnn_free(MpnnState *m) {
  if (!m) return;
  cudaFree(m->params); cudaFree(m->grad); cudaFree(m->adam_m); cudaFree(m->adam_s); cudaFree(m->wbf);
  cudaFree(m->x);
  for (int l = 0; l < 3; l++) {
    cudaFree(m->h[l]);
    cudaFree(m->agg[l]);
  }
  cudaFree(m->xy); cudaFree(m->target); cudaFree(m->vweight); cudaFree(m->dxy); cudaFree(m->dz); cudaFree(m->P);
  cudaFree(m->G); cudaFree(m->part); cudaFree(m->loss_part);
  delete m;
}

namespace {

int ensure_mpnn(bl_ctx *ctx, int n) {
  if (!ctx->mpnn) {
    ctx->mpnn = new MpnnState();
    MpnnState &m = *ctx->mpnn;
    BL_CUDA(ctx, cudaMalloc(&m.params, sizeof(float) * kMpnnParams));
    BL_CUDA(ctx, cudaMalloc(&m.grad, sizeof(float) * kMpnnParams));
    BL_CUDA(ctx, cudaMalloc(&m.adam_m, sizeof(float) * kMpnnParams));
    BL_CUDA(ctx, cudaMalloc(&m.adam_s, sizeof(float) * kMpnnParams));
    BL_CUDA(ctx, cudaMalloc(&m.wbf, sizeof(__nv_bfloat16) * kMpnnParams));
    // four resident 128-thread blocks per SM (48 KB of shared memory and 64
    // tensor-memory columns each): the layers' neighbour gathers are
    // latency-bound, and two blocks per SM left 88 % of the warp slots empty
    m.grid = ctx->num_sms * kBlocksPerSm;
    BL_CUDA(ctx, cudaMalloc(&m.part, sizeof(float) * (size_t)m.grid * (64 * 128 + 64)));
    BL_CUDA(ctx, cudaMalloc(&m.loss_part, sizeof(double) * m.grid));
    if (!ctx->s.status) {
      BL_CUDA(ctx, cudaMalloc(&ctx->s.status, sizeof(DevStatus)));
      BL_CUDA(ctx, cudaMemset(ctx->s.status, 0, sizeof(DevStatus)));
    }
    if (int rc = set_smem(ctx, mpnn_fwd_kernel<16, false>, kT * 32 * 2 + 64 * 32 * 2)) return rc;
    if (int rc = set_smem(ctx, mpnn_fwd_kernel<64, false>, kT * 128 * 2 + 64 * 128 * 2)) return rc;
    if (int rc = set_smem(ctx, mpnn_fwd_kernel<64, true>, kT * 128 * 2 + 64 * 128 * 2)) return rc;
    if (int rc = set_smem(ctx, mpnn_wgrad_kernel<16>, kT * kT * 2 + 64 * kT * 2)) return rc;
    if (int rc = set_smem(ctx, mpnn_wgrad_kernel<64>, kT * kT * 2 + 64 * kT * 2)) return rc;
    if (int rc = set_smem(ctx, mpnn_dgrad_kernel<64>, kT * 64 * 2 + 128 * 64 * 2)) return rc;
  }
  MpnnState &m = *ctx->mpnn;
  if (n > m.cap_n) {
    cudaFree(m.x);
    for (int l = 0; l < 3; l++) {
      cudaFree(m.h[l]);
      cudaFree(m.agg[l]);
    }
    cudaFree(m.xy); cudaFree(m.target); cudaFree(m.vweight); cudaFree(m.dxy); cudaFree(m.dz); cudaFree(m.P);
    cudaFree(m.G);
    const size_t N = (size_t)std::max(n, 1);
    BL_CUDA(ctx, cudaMalloc(&m.x, N * 16 * 2));
    for (int l = 0; l < 3; l++) {
      BL_CUDA(ctx, cudaMalloc(&m.h[l], N * 64 * 2));
      BL_CUDA(ctx, cudaMalloc(&m.agg[l], N * 64 * 2));
    }
    BL_CUDA(ctx, cudaMalloc(&m.xy, N * 2 * 4));
    BL_CUDA(ctx, cudaMalloc(&m.target, N * 2 * 4));
    BL_CUDA(ctx, cudaMalloc(&m.vweight, N * 4));
    BL_CUDA(ctx, cudaMalloc(&m.dxy, N * 2 * 4));
    BL_CUDA(ctx, cudaMalloc(&m.dz, N * 64 * 4));
    BL_CUDA(ctx, cudaMalloc(&m.P, N * 64 * 4));
    BL_CUDA(ctx, cudaMalloc(&m.G, N * 64 * 4));
    m.cap_n = n;
  }
  return 0;
}

// offsets of the parameter blocks in the flat vector
constexpr int kOffW[3] = {0, 64 * 32 + 64, 64 * 32 + 64 + 64 * 128 + 64};
constexpr int kOffWo = 64 * 32 + 64 + 2 * (64 * 128 + 64);
constexpr int kOffBo = kOffWo + 128;

int sync_weights(bl_ctx *ctx) {
  MpnnState &m = *ctx->mpnn;
  to_bf16_kernel<<<nblk(kMpnnParams, 256), 256, 0, ctx->stream>>>(m.params, m.wbf, kMpnnParams);
  ctx->launches++;
  BL_CUDA(ctx, cudaGetLastError());
  return 0;
}

}  // namespace

// Forward over a graph already on the device (n vertices, CSR rowptr/colids,
// features in m.x).  With `train`, keeps the aggregates, computes the loss
// against m.target/m.vweight and its gradient dxy.
int mpnn_forward(bl_ctx *ctx, int n, const int *d_rowptr, const int *d_colids, bool train) {
  MpnnState &m = *ctx->mpnn;
  cudaStream_t st = ctx->stream;
  const int grid = std::min(m.grid, std::max(1, nblk(n, kT)));
  FwdArgs a{};
  a.n = n;
  a.rowptr = d_rowptr;
  a.colids = d_colids;
  a.st = ctx->s.status;
  bl_time_begin(ctx, "mpnn_forward");
  for (int l = 0; l < 3; l++) {
    a.hin = l == 0 ? m.x : m.h[l - 1];
    a.hout = m.h[l];
    a.agg = train ? m.agg[l] : nullptr;
    a.W = m.wbf + kOffW[l];
    a.bias = m.params + kOffW[l] + (l == 0 ? 64 * 32 : 64 * 128);
    if (l == 0) {
      mpnn_fwd_kernel<16, false><<<grid, kT, kT * 32 * 2 + 64 * 32 * 2, st>>>(a);
    } else if (l == 1) {
      mpnn_fwd_kernel<64, false><<<grid, kT, kT * 128 * 2 + 64 * 128 * 2, st>>>(a);
    } else {
      a.Wo = m.params + kOffWo;
      a.bo = m.params + kOffBo;
      a.xy = m.xy;
      a.target = train ? m.target : nullptr;
      a.vweight = m.vweight;
      a.dxy = m.dxy;
      a.loss_part = m.loss_part;
      mpnn_fwd_kernel<64, true><<<grid, kT, kT * 128 * 2 + 64 * 128 * 2, st>>>(a);
    }
    ctx->launches++;
    BL_CUDA(ctx, cudaGetLastError());
  }
  bl_time_end(ctx, "mpnn_forward");
  return 0;
}

// Backward after a training forward: gradient of the loss into m.grad.
int mpnn_backward(bl_ctx *ctx, int n, const int *d_rowptr, const int *d_colids) {
  MpnnState &m = *ctx->mpnn;
  cudaStream_t st = ctx->stream;
  const int grid = std::min(m.grid, std::max(1, nblk(n, kT)));
  TopArgs t{n, m.dxy, m.h[2], m.params + kOffWo, m.dz, m.part};
  mpnn_top_kernel<<<grid, kT, 0, st>>>(t);
  mpnn_reduce_kernel<<<1, 256, 0, st>>>(m.part, grid, 130, m.grad + kOffWo);
  ctx->launches += 2;
  for (int l = 2; l >= 0; l--) {
    const int din = l == 0 ? 16 : 64;
    const int len = 64 * 2 * din + 64;
    WgradArgs w{n, l == 0 ? m.x : m.h[l - 1], m.agg[l], m.dz, m.part, ctx->s.status};
    if (l == 0) mpnn_wgrad_kernel<16><<<grid, kT, kT * kT * 2 + 64 * kT * 2, st>>>(w);
    else mpnn_wgrad_kernel<64><<<grid, kT, kT * kT * 2 + 64 * kT * 2, st>>>(w);
    mpnn_reduce_kernel<<<nblk(len, 256), 256, 0, st>>>(m.part, grid, len, m.grad + kOffW[l]);
    ctx->launches += 2;
    BL_CUDA(ctx, cudaGetLastError());
    if (l > 0) {
      DgradArgs d{n, d_rowptr, m.dz, m.wbf + kOffW[l], m.P, m.G, ctx->s.status};
      mpnn_dgrad_kernel<64><<<grid, kT, kT * 64 * 2 + 128 * 64 * 2, st>>>(d);
      mpnn_gather_kernel<<<nblk((long long)n * 16, 256), 256, 0, st>>>(n, d_rowptr, d_colids, m.P, m.G, m.h[l - 1],
                                                                      m.dz);
      ctx->launches += 2;
      BL_CUDA(ctx, cudaGetLastError());
    }
  }
  return 0;
}

int mpnn_loss(bl_ctx *ctx, int n, double *loss) {
  MpnnState &m = *ctx->mpnn;
  const int grid = std::min(m.grid, std::max(1, nblk(n, kT)));
  std::vector<double> lp(grid);
  BL_CUDA(ctx, cudaMemcpyAsync(lp.data(), m.loss_part, sizeof(double) * grid, cudaMemcpyDeviceToHost, ctx->stream));
  BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  double s = 0.0;
  for (double v : lp) s += v;
  *loss = s;
  return 0;
}

int mpnn_adam_step(bl_ctx *ctx, double lr) {
  MpnnState &m = *ctx->mpnn;
  m.adam_t++;
  const double b1 = 0.9, b2 = 0.999;
  adam_kernel<<<nblk(kMpnnParams, 256), 256, 0, ctx->stream>>>(
      m.params, m.grad, m.adam_m, m.adam_s, kMpnnParams, (float)lr, (float)b1, (float)b2, 1e-8f,
      (float)(1.0 - std::pow(b1, m.adam_t)), (float)(1.0 - std::pow(b2, m.adam_t)));
  ctx->launches++;
  BL_CUDA(ctx, cudaGetLastError());
  return sync_weights(ctx);
}

int mpnn_prepare(bl_ctx *ctx, int n) { return ensure_mpnn(ctx, n); }

__nv_bfloat16 *mpnn_input(bl_ctx *ctx) { return ctx->mpnn->x; }
const float *mpnn_output(bl_ctx *ctx) { return ctx->mpnn->xy; }
float *mpnn_targets(bl_ctx *ctx) { return ctx->mpnn->target; }
float *mpnn_vweights(bl_ctx *ctx) { return ctx->mpnn->vweight; }

int mpnn_set_params_device(bl_ctx *ctx, const float *h_params) {
  if (int rc = ensure_mpnn(ctx, 1)) return rc;
  MpnnState &m = *ctx->mpnn;
  BL_CUDA(ctx, cudaMemcpyAsync(m.params, h_params, sizeof(float) * kMpnnParams, cudaMemcpyHostToDevice, ctx->stream));
  BL_CUDA(ctx, cudaMemsetAsync(m.adam_m, 0, sizeof(float) * kMpnnParams, ctx->stream));
  BL_CUDA(ctx, cudaMemsetAsync(m.adam_s, 0, sizeof(float) * kMpnnParams, ctx->stream));
  m.adam_t = 0;
  m.have_params = true;
  return sync_weights(ctx);
}

}  // namespace bl

// ---- C ABI -------------------------------------------------------------------------
extern "C" {

int bl_mpnn_set_params(bl_ctx *ctx, const float *params) try {
  if (!ctx || !params) return BL_ERR_ARG;
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  if (int rc = bl::mpnn_set_params_device(ctx, params)) return rc;
  BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_mpnn_get_params(bl_ctx *ctx, float *params) try {
  if (!ctx || !params) return BL_ERR_ARG;
  if (!ctx->mpnn || !ctx->mpnn->have_params) return bl_fail(ctx, BL_ERR_STATE, "no network parameters set");
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  BL_CUDA(ctx, cudaMemcpyAsync(params, ctx->mpnn->params, sizeof(float) * bl::kMpnnParams, cudaMemcpyDeviceToHost,
                               ctx->stream));
  BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

// Forward (and, with target != NULL, loss and gradient) on a graph given as
// host arrays.  Outputs: xy (n x 2), optionally h (3 x n x 64 BF16 as
// uint16), loss and grad (kMpnnParams floats).
int bl_mpnn_run(bl_ctx *ctx, int n, const int *rowptr, const int *colids, const float *features,
                const float *target, const float *vweight, float *xy, unsigned short *h, double *loss,
                float *grad) try {
  using namespace bl;
  if (!ctx || n < 1 || !rowptr || !features || !xy) return BL_ERR_ARG;
  if (target && (!vweight || !loss || !grad)) return bl_fail(ctx, BL_ERR_ARG, "training run needs vweight, loss, grad");
  if (!ctx->mpnn || !ctx->mpnn->have_params) return bl_fail(ctx, BL_ERR_STATE, "no network parameters set");
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  const long long nnz = rowptr[n];
  for (int v = 0; v < n; v++)
    if (rowptr[v + 1] < rowptr[v]) return bl_fail(ctx, BL_ERR_ARG, "rowptr decreases");
  for (long long e = 0; e < nnz; e++)
    if (colids[e] < 0 || colids[e] >= n) return bl_fail(ctx, BL_ERR_ARG, "colid out of range");
  if (int rc = ensure_mpnn(ctx, n)) return rc;
  MpnnState &m = *ctx->mpnn;
  cudaStream_t st = ctx->stream;
  int *d_rp = nullptr, *d_ci = nullptr;
  float *d_f = nullptr;
  int rc = 0;
  auto fail = [&](cudaError_t e, const char *w) {
    if (rc == 0) rc = bl_cuda_fail(ctx, e, w);
  };
  cudaError_t e;
  if ((e = cudaMalloc(&d_rp, sizeof(int) * (n + 1))) != cudaSuccess) fail(e, "cudaMalloc");
  if (!rc && (e = cudaMalloc(&d_ci, sizeof(int) * std::max<long long>(nnz, 1))) != cudaSuccess) fail(e, "cudaMalloc");
  if (!rc && (e = cudaMalloc(&d_f, sizeof(float) * 16 * (size_t)n)) != cudaSuccess) fail(e, "cudaMalloc");
  if (!rc) {
    cudaMemcpyAsync(d_rp, rowptr, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st);
    if (nnz) cudaMemcpyAsync(d_ci, colids, sizeof(int) * nnz, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_f, features, sizeof(float) * 16 * (size_t)n, cudaMemcpyHostToDevice, st);
    to_bf16_kernel<<<nblk(16LL * n, 256), 256, 0, st>>>(d_f, m.x, 16LL * n);
    ctx->launches++;
    if (target) {
      cudaMemcpyAsync(m.target, target, sizeof(float) * 2 * (size_t)n, cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(m.vweight, vweight, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, st);
    }
    rc = mpnn_forward(ctx, n, d_rp, d_ci, target != nullptr);
    if (!rc && target) rc = mpnn_backward(ctx, n, d_rp, d_ci);
    if (!rc && (e = cudaStreamSynchronize(st)) != cudaSuccess) fail(e, "mpnn kernels");
    if (!rc) rc = bl_check_status(ctx);
    if (!rc) {
      cudaMemcpy(xy, m.xy, sizeof(float) * 2 * (size_t)n, cudaMemcpyDeviceToHost);
      if (h)
        for (int l = 0; l < 3; l++)
          cudaMemcpy(h + (size_t)l * n * 64, m.h[l], sizeof(unsigned short) * 64 * (size_t)n, cudaMemcpyDeviceToHost);
      if (target) {
        cudaMemcpy(grad, m.grad, sizeof(float) * kMpnnParams, cudaMemcpyDeviceToHost);
        rc = mpnn_loss(ctx, n, loss);
      }
    }
  }
  cudaFree(d_rp);
  cudaFree(d_ci);
  cudaFree(d_f);
  return rc;
} catch (...) {
  return bl_host_exception(ctx);
}

}  // extern "C"

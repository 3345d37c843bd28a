// greedy.cu -- algo 5, greedy approximation, first phase
// (approxForceDirectedAlgorithm, sample/algorithms.cpp:1085-1190).
//
// For the first (int)(0.8 * ITERATIONS) + 1 iterations the reference gives
// every vertex i the attraction W|d|d of its CSR neighbours and the
// repulsion -d/|d|^2 of the vertices a bounded depth-first walk reaches
// (:1126-1170): the stack starts with i's neighbours in CSR order; popping u
// scans u's row and every entry v outside {i} u N(i) repels, is pushed and
// spends one unit of a budget of 200; the walk ends after the row that spends
// the budget, or when the stack is empty.  Reached vertices are not marked,
// so a walk visits few distinct vertices many times (about 22 distinct among
// ~200 on the benchmark graphs).
//
// GB300 design.  The walk depends on the graph only, so it runs once per
// graph instead of once per vertex and iteration: walk_kernel (a warp per
// vertex, the stack in HBM, each popped row scanned 32 entries at a time,
// pushes kept in CSR order by a ballot) merges repeated sources in shared
// memory and stores each vertex's walk as (source, count) pairs, in a count
// pass and a fill pass around a prefix sum.  An iteration is then a sparse
// gather: greedy_iteration_kernel runs all first-phase iterations in one
// launch of a single thread-block cluster.  For each minibatch, 16 lanes per
// target sum the attraction over its CSR row and count x repulsion over its
// pairs (FP32, fixed shuffle tree), a cluster barrier closes the force phase
// (Jacobi inside the batch), the targets move, and a second cluster barrier
// publishes the moved positions to the next batch (Gauss-Seidel across
// batches).  Batches are sequential, so one cluster of 8 or 16 SMs connected
// by hardware barriers (no spin-waits) does the whole phase; positions
// (8 B per vertex) stay in L2.
//
// Summation order differs from the reference's (pairs instead of walk
// order, FP32 instead of FP64): results agree within FP32 rounding.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "../../include/batchlayout_gb300.h"
#include "bl_device.cuh"

namespace bl {
namespace {

constexpr int kGreedyBudget = 200;  // countNodes (algorithms.cpp:1147)

// ---- walk construction ---------------------------------------------------------

constexpr int kWalkThreads = 256;
constexpr int kWalkWarps = kWalkThreads / 32;
constexpr int kUniq = 128;  // distinct sources merged per walk in shared memory

struct WalkArgs {
  int n;
  const int *rowptr, *colids;          // the CSR (push order)
  const int *srt_rowptr, *srt_colids;  // rows sorted (membership test)
  int *stack;
  long long stack_cap;                 // ints per warp
  long long *count;                    // count pass: pairs per vertex
  const long long *off;                // fill pass: first pair of each vertex
  int2 *pairs;
  DevStatus *st;
};

// v in N(i): binary search of the sorted row [m0, m1)
__device__ __forceinline__ bool row_contains(const int *srt, int m0, int m1, int v) {
  while (m0 < m1) {
    const int mid = (m0 + m1) >> 1;
    const int c = __ldg(&srt[mid]);
    if (c == v) return true;
    if (c < v) m0 = mid + 1;
    else m1 = mid;
  }
  return false;
}

template <bool kFill>
__global__ void __launch_bounds__(kWalkThreads) walk_kernel(WalkArgs a) {
  __shared__ int uv[kWalkWarps][kUniq];
  __shared__ int um[kWalkWarps][kUniq];
  if (!block_status_ok(a.st)) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long gw = (long long)blockIdx.x * kWalkWarps + warp;
  const long long nw = (long long)gridDim.x * kWalkWarps;
  int *stack = a.stack + gw * a.stack_cap;
  int *myv = uv[warp], *mym = um[warp];
  const unsigned lt = (1u << lane) - 1u;
  for (long long ii = gw; ii < a.n; ii += nw) {
    const int i = (int)ii;
    const int r0 = __ldg(&a.rowptr[i]), r1 = __ldg(&a.rowptr[i + 1]);
    const int m0 = __ldg(&a.srt_rowptr[i]), m1 = __ldg(&a.srt_rowptr[i + 1]);
    // the stack starts with N(i) in CSR order (:1130-1144); the capacity
    // covers deg(i) + 199 + max degree entries
    for (int k = lane; k < r1 - r0; k += 32) stack[k] = __ldg(&a.colids[r0 + k]);
    long long sp = r1 - r0;
    int nu = 0, budget = kGreedyBudget;
    long long nover = 0;  // pairs stored directly once the table is full
    const long long obase = kFill ? a.off[i] : 0;
    long long pops = 0;
    bool bad = false;
    __syncwarp();
    while (sp > 0) {
      // every pop either pushes (spending budget) or shrinks the stack, so
      // the walk ends after at most stack_cap pops; the check is a guard
      if (++pops > a.stack_cap + 1) {
        bad = true;
        break;
      }
      const int u = stack[sp - 1];
      sp--;
      const int u0 = __ldg(&a.rowptr[u]), u1 = __ldg(&a.rowptr[u + 1]);
      int pushed = 0;
      for (int e0 = u0; e0 < u1; e0 += 32) {
        const int e = e0 + lane;
        int v = -1;
        bool push = false;
        if (e < u1) {
          v = __ldg(&a.colids[e]);
          push = v != i && !row_contains(a.srt_colids, m0, m1, v);
        }
        unsigned mask = __ballot_sync(0xffffffffu, push);
        const long long at = sp + __popc(mask & lt);
        if (push) {
          if (at < a.stack_cap) stack[at] = v;
          else bad = true;
        }
        sp += __popc(mask);
        pushed += __popc(mask);
        // merge the pushed sources, in push order
        while (mask) {
          const int src = __ffs(mask) - 1;
          mask &= mask - 1u;
          const int cv = __shfl_sync(0xffffffffu, v, src);
          int found = -1;
          for (int q = lane; q < nu; q += 32)
            if (myv[q] == cv) found = q;
          const unsigned fm = __ballot_sync(0xffffffffu, found >= 0);
          if (fm) {
            if (lane == __ffs(fm) - 1) mym[found]++;
          } else if (nu < kUniq) {
            if (lane == 0) {
              myv[nu] = cv;
              mym[nu] = 1;
            }
            nu++;
          } else {
            if (kFill && lane == 0) a.pairs[obase + nover] = make_int2(cv, 1);
            nover++;
          }
          __syncwarp();
        }
      }
      if (__any_sync(0xffffffffu, bad)) break;
      __syncwarp();
      budget -= pushed;
      if (budget <= 0) break;  // :1167
    }
    if (__any_sync(0xffffffffu, bad)) {
      if (lane == 0) dev_record_error(a.st, DEV_BAD_INDEX);
      return;
    }
    if (!kFill) {
      if (lane == 0) a.count[i] = nover + nu;
    } else {
      for (int q = lane; q < nu; q += 32) a.pairs[obase + nover + q] = make_int2(myv[q], mym[q]);
    }
    __syncwarp();
  }
}

// ---- first-phase iterations ----------------------------------------------------

constexpr int kIterThreads = 512;
constexpr int kLanes = 16;  // lanes per target
constexpr int kTargetsPerCta = kIterThreads / kLanes;

struct IterArgs {
  int n, batch, nbatches, iterations, energy_last;
  float W;
  double step0, decay;
  const int *rowptr, *colids;
  const long long *off;
  const int2 *pairs;
  float2 *pos;
  double2 *force;
  double *e;
};

__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ unsigned int cluster_rank() {
  unsigned int r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ unsigned int cluster_count() {
  unsigned int r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}

// One launch = one cluster; every thread of every CTA runs the same loop
// trip counts, so every cluster barrier is reached by all of them.
__global__ void __launch_bounds__(kIterThreads, 1) greedy_iteration_kernel(IterArgs a) {
  const unsigned int rank = cluster_rank(), csize = cluster_count();
  const int grp = threadIdx.x / kLanes, gl = threadIdx.x % kLanes;
  const int gt = (int)rank * kTargetsPerCta + grp, ngt = (int)csize * kTargetsPerCta;
  const int tid = (int)rank * kIterThreads + threadIdx.x, nthr = (int)csize * kIterThreads;
  double step = a.step0;
  for (int it = 0; it < a.iterations; it++) {
    const bool energy_it = a.energy_last && it == a.iterations - 1;
    const float stepf = (float)step;
    for (int c = 0; c < a.nbatches; c++) {
      const int base = c * a.batch;
      const int cnt = min(a.batch, a.n - base);
      // forces of the batch from its start positions
      for (int t0 = 0; t0 < cnt; t0 += ngt) {  // same trip count in every lane group
        const int t = t0 + gt;
        float fx = 0.f, fy = 0.f;
        if (t < cnt) {
          const int i = base + t;
          const float2 pi = __ldcg(&a.pos[i]);
          const int r0 = __ldg(&a.rowptr[i]), r1 = __ldg(&a.rowptr[i + 1]);
          for (int k = r0 + gl; k < r1; k += kLanes) {
            const float2 pj = __ldcg(&a.pos[__ldg(&a.colids[k])]);
            attract_pair(MODEL_FR, a.W, pj.x, pj.y, pi.x, pi.y, fx, fy);
          }
          const long long w0 = __ldg(&a.off[i]), w1 = __ldg(&a.off[i + 1]);
          for (long long k = w0 + gl; k < w1; k += kLanes) {
            const int2 p = __ldg(&a.pairs[k]);
            const float2 pj = __ldcg(&a.pos[p.x]);
            float rx = 0.f, ry = 0.f;
            rep_pair(pj.x, pj.y, pi.x, pi.y, rx, ry);
            fx = fmaf((float)p.y, rx, fx);
            fy = fmaf((float)p.y, ry, fy);
          }
        }
#pragma unroll
        for (int o = kLanes / 2; o > 0; o >>= 1) {
          fx += __shfl_xor_sync(0xffffffffu, fx, o);
          fy += __shfl_xor_sync(0xffffffffu, fy, o);
        }
        if (t < cnt && gl == 0) a.force[base + t] = make_double2((double)fx, (double)fy);
      }
      cluster_barrier();
      // move the batch (:1171-1177)
      for (int t = tid; t < cnt; t += nthr) {
        const int i = base + t;
        const double2 f = __ldcg(&a.force[i]);
        a.pos[i] = unit_step(__ldcg(&a.pos[i]), f.x, f.y, stepf);
        if (energy_it) a.e[i] = f.x * f.x + f.y * f.y;
      }
      cluster_barrier();
    }
    step = step * a.decay;
  }
}

// Largest cluster (16, else 8, 4, 2, 1 CTAs) that can be scheduled.
int iteration_cluster(bl_ctx *ctx) {
  static int cached[64] = {0};
  if (ctx->device >= 0 && ctx->device < 64 && cached[ctx->device]) return cached[ctx->device];
  cudaFuncSetAttribute(greedy_iteration_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  int best = 1;
  for (int c : {16, 8, 4, 2}) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(c);
    cfg.blockDim = dim3(kIterThreads);
    cfg.dynamicSmemBytes = 0;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = c;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, greedy_iteration_kernel, &cfg) == cudaSuccess && clusters >= 1) {
      best = c;
      break;
    }
    cudaGetLastError();  // clear a refused size
  }
  if (ctx->device >= 0 && ctx->device < 64) cached[ctx->device] = best;
  return best;
}

}  // namespace

int ensure_sorted_csr(bl_ctx *ctx) {
  if (ctx->g.max_degree >= 0) return 0;
  const int n = ctx->g.n;
  const std::vector<int> &rp = ctx->h_rowptr, &ci = ctx->h_colids;
  bool sorted = true;
  int maxd = 0;
  for (int i = 0; i < n; i++) {
    maxd = std::max(maxd, rp[i + 1] - rp[i]);
    for (int k = rp[i] + 1; k < rp[i + 1] && sorted; k++)
      if (ci[k] < ci[k - 1]) sorted = false;
  }
  if (sorted) {
    ctx->g.srt_rowptr = ctx->g.rowptr;
    ctx->g.srt_colids = ctx->g.colids;
  } else {
    std::vector<int> sc(ci);
    for (int i = 0; i < n; i++) std::sort(sc.begin() + rp[i], sc.begin() + rp[i + 1]);
    BL_CUDA(ctx, cudaMalloc(&ctx->g.srt_rowptr, (size_t)(n + 1) * sizeof(int)));
    BL_CUDA(ctx, cudaMalloc(&ctx->g.srt_colids, std::max<size_t>(sc.size(), 1) * sizeof(int)));
    BL_CUDA(ctx, cudaMemcpy(ctx->g.srt_rowptr, rp.data(), (size_t)(n + 1) * sizeof(int), cudaMemcpyHostToDevice));
    if (!sc.empty())
      BL_CUDA(ctx, cudaMemcpy(ctx->g.srt_colids, sc.data(), sc.size() * sizeof(int), cudaMemcpyHostToDevice));
  }
  ctx->g.max_degree = maxd;
  return 0;
}

int greedy_walks_build(bl_ctx *ctx) {
  if (ctx->s.walk_total >= 0) return 0;
  if (int rc = ensure_sorted_csr(ctx)) return rc;
  const int n = ctx->g.n;
  // stack bound: deg(i) + (199 + the degree of the row that spends the budget)
  const long long cap = 2LL * ctx->g.max_degree + 256;
  long long blocks = std::min<long long>((n + kWalkWarps - 1) / kWalkWarps, (long long)ctx->num_sms * 8);
  const long long max_warps = std::max<long long>(kWalkWarps, (512LL << 20) / (cap * (long long)sizeof(int)));
  blocks = std::max<long long>(1, std::min(blocks, max_warps / kWalkWarps));
  int *stack = nullptr;
  long long *count = nullptr;
  BL_CUDA(ctx, cudaMalloc(&stack, (size_t)(blocks * kWalkWarps * cap) * sizeof(int)));
  cudaError_t e = cudaMalloc(&count, (size_t)n * sizeof(long long));
  if (e != cudaSuccess) {
    cudaFree(stack);
    return bl_cuda_fail(ctx, e, "cudaMalloc");
  }
  auto cleanup = [&]() {
    cudaFree(stack);
    cudaFree(count);
  };
  WalkArgs a;
  a.n = n;
  a.rowptr = ctx->g.rowptr;
  a.colids = ctx->g.colids;
  a.srt_rowptr = ctx->g.srt_rowptr;
  a.srt_colids = ctx->g.srt_colids;
  a.stack = stack;
  a.stack_cap = cap;
  a.count = count;
  a.off = nullptr;
  a.pairs = nullptr;
  a.st = ctx->s.status;
  bl_time_begin(ctx, "walk_kernel");
  walk_kernel<false><<<(unsigned)blocks, kWalkThreads, 0, ctx->stream>>>(a);
  bl_time_end(ctx, "walk_kernel");
  ctx->launches++;
  std::vector<long long> off(n + 1, 0);
  e = cudaMemcpyAsync(off.data() + 1, count, (size_t)n * sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cleanup();
    return bl_cuda_fail(ctx, e, "walk count");
  }
  if (int rc = bl_check_status(ctx)) {
    cleanup();
    return rc;
  }
  std::partial_sum(off.begin(), off.end(), off.begin());
  const long long total = off[n];
  if (!ctx->s.walk_off) {
    e = cudaMalloc(&ctx->s.walk_off, (size_t)(n + 1) * sizeof(long long));
    if (e != cudaSuccess) {
      cleanup();
      return bl_cuda_fail(ctx, e, "cudaMalloc");
    }
  }
  if (ctx->s.walk_pairs) cudaFree(ctx->s.walk_pairs);  // left by a failed build
  ctx->s.walk_pairs = nullptr;
  e = cudaMalloc(&ctx->s.walk_pairs, (size_t)std::max<long long>(total, 1) * sizeof(int2));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ctx->s.walk_off, off.data(), (size_t)(n + 1) * sizeof(long long), cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e != cudaSuccess) {
    cleanup();
    return bl_cuda_fail(ctx, e, "walk pairs");
  }
  a.count = nullptr;
  a.off = ctx->s.walk_off;
  a.pairs = ctx->s.walk_pairs;
  bl_time_begin(ctx, "walk_kernel");
  walk_kernel<true><<<(unsigned)blocks, kWalkThreads, 0, ctx->stream>>>(a);
  bl_time_end(ctx, "walk_kernel");
  ctx->launches++;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cleanup();
  if (e != cudaSuccess) return bl_cuda_fail(ctx, e, "walk fill");
  if (int rc = bl_check_status(ctx)) return rc;
  ctx->s.walk_total = total;
  return 0;
}

int greedy_walk_run(bl_ctx *ctx, int batch, int iterations, double step0, double decay, bool want_energy,
                    double *energy_out) {
  const int n = ctx->g.n;
  if (batch < 1) return bl_fail(ctx, BL_ERR_ARG, "batch must be >= 1");
  if (iterations <= 0) return 0;
  if (int rc = greedy_walks_build(ctx)) return rc;
  if (int rc = bl_check_status(ctx)) return rc;
  batch = std::min(batch, n);
  const int csize = iteration_cluster(ctx);
  IterArgs a;
  a.n = n;
  a.batch = batch;
  a.nbatches = (n + batch - 1) / batch;
  a.iterations = iterations;
  a.energy_last = want_energy ? 1 : 0;
  a.W = (float)ctx->weight;
  a.step0 = step0;
  a.decay = decay;
  a.rowptr = ctx->g.rowptr;
  a.colids = ctx->g.colids;
  a.off = ctx->s.walk_off;
  a.pairs = ctx->s.walk_pairs;
  a.pos = ctx->pos;
  a.force = ctx->force;
  a.e = ctx->e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(csize);
  cfg.blockDim = dim3(kIterThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  bl_time_begin(ctx, "greedy_iteration_kernel");
  BL_CUDA(ctx, cudaLaunchKernelEx(&cfg, greedy_iteration_kernel, a));
  bl_time_end(ctx, "greedy_iteration_kernel");
  ctx->launches++;
  if (want_energy) {
    if (int rc = energy_reduce(ctx, energy_out)) return rc;
  } else {
    BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return bl_check_status(ctx);
}

}  // namespace bl

extern "C" int bl_greedy_walks(bl_ctx *ctx, long long *offsets, int *sources, int *counts, long long cap,
                               long long *total) {
  if (!ctx || !offsets || !total || cap < 0 || (cap > 0 && (!sources || !counts))) return BL_ERR_ARG;
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  if (int rc = bl::greedy_walks_build(ctx)) return rc;
  const int n = ctx->g.n;
  *total = ctx->s.walk_total;
  BL_CUDA(ctx, cudaMemcpy(offsets, ctx->s.walk_off, (size_t)(n + 1) * sizeof(long long), cudaMemcpyDeviceToHost));
  const long long m = std::min(cap, ctx->s.walk_total);
  if (m > 0) {
    std::vector<int2> p((size_t)m);
    BL_CUDA(ctx, cudaMemcpy(p.data(), ctx->s.walk_pairs, (size_t)m * sizeof(int2), cudaMemcpyDeviceToHost));
    for (long long k = 0; k < m; k++) {
      sources[k] = p[k].x;
      counts[k] = p[k].y;
    }
  }
  return BL_OK;
}

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
// gather over a per-vertex term list (CSR entries, then walk pairs):
// greedy_iteration_kernel runs all first-phase iterations in one launch of a
// single thread-block cluster (batches are sequential, so one cluster of up
// to 16 SMs joined by hardware barriers -- no spin-waits -- does the whole
// phase).  Each CTA takes a share of every batch with about the same number
// of terms, sums its targets' terms through warp segmented scans into
// fixed-point shared-memory accumulators (deterministic), and moves its
// targets; positions alternate between two arrays by the parity of the
// number of moves, which keeps the batch's start positions readable while
// it moves (Jacobi inside the batch) and leaves one cluster barrier per
// batch to publish the moves (Gauss-Seidel across batches).  The next
// batch's target positions and first terms are loaded during the batch
// before.  Positions (8 B per vertex) stay in L2.
//
// Summation order differs from the reference's (pairs instead of walk
// order, FP32 terms summed in warp order and 2^-28 fixed point instead of
// FP64): results agree within FP32 rounding.
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

// Term list of a vertex i, at term_off[i] = rowptr[i] + walk_off[i]: its CSR
// entries as (neighbour, 0) -- attraction -- then its walk pairs as
// (source, count) -- count x repulsion -- each with its target i.
__global__ void term_list_kernel(int n, const int *__restrict__ rowptr, const int *__restrict__ colids,
                                 const long long *__restrict__ walk_off, const int2 *__restrict__ walk_pairs,
                                 int2 *__restrict__ terms, int *__restrict__ term_tgt) {
  const int warp = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (warp >= n) return;
  const int i = warp;
  const int r0 = rowptr[i], r1 = rowptr[i + 1];
  const long long w0 = walk_off[i], w1 = walk_off[i + 1];
  const long long q0 = (long long)r0 + w0;
  for (int k = r0 + lane; k < r1; k += 32) {
    terms[q0 + (k - r0)] = make_int2(colids[k], 0);
    term_tgt[q0 + (k - r0)] = i;
  }
  const long long qa = q0 + (r1 - r0);
  for (long long k = w0 + lane; k < w1; k += 32) {
    terms[qa + (k - w0)] = walk_pairs[k];
    term_tgt[qa + (k - w0)] = i;
  }
}

constexpr int kIterThreads = 512;
constexpr int kPre = 2;  // terms per thread loaded ahead of each batch

// Fixed-point force accumulators (units of 2^-28, the minibatch sweep's
// format): integer atomics are exact and order-free, so the per-target sums
// do not depend on which warp adds first.  A partial beyond +-2^34 is
// reported instead of wrapping.
constexpr float kFix = 268435456.0f;
constexpr double kFixInv = 1.0 / 268435456.0;
constexpr float kFixLimit = 17179869184.0f;

struct IterArgs {
  int n, batch, nbatches, iterations, energy_last;
  float W;
  double step0, decay;
  const long long *term_off;  // per vertex
  const int2 *terms;
  const int *term_tgt;
  const int *share;  // [nbatches][CTAs + 1]: first target (batch-relative) of each CTA's share
  float2 *pos0, *pos1;  // positions after an even / odd number of moves
  double2 *force;
  double *e;
  DevStatus *st;
};

__device__ __forceinline__ void cluster_arrive() {
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}

__device__ __forceinline__ void cluster_wait() {
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
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

__device__ __forceinline__ void fix_add_shared(long long *dst, float v, DevStatus *st) {
  if (!(fabsf(v) < kFixLimit)) {
    dev_record_error(st, DEV_FORCE_RANGE);
    return;
  }
  atomicAdd(reinterpret_cast<unsigned long long *>(dst), (unsigned long long)__float2ll_rn(v * kFix));
}

// One launch = one cluster running every batch of every first-phase
// iteration.
//
// Each CTA owns a share of every batch: a range of consecutive targets whose
// terms (consecutive in the term list) add up to about 1/CTAs of the batch's
// terms, so a target's partial sums meet in one CTA's shared memory
// (warp segmented scans, then fixed-point shared atomics) and the CTA moves
// its own targets after a CTA barrier.  Jacobi inside the batch without a
// second cluster barrier: a vertex's position lives in pos0 or pos1 by the
// parity of the number of times it has moved, so the moves of batch c go to
// the other array while other CTAs still read the batch's start positions;
// a reader picks the array from the vertex id (moved once more in this
// iteration iff it lies before the current batch).  One cluster barrier per
// batch publishes the moves.  The next batch's share, target positions
// (staged in shared memory) and first terms are loaded during the batch
// before (they do not move in it).
__global__ void __launch_bounds__(kIterThreads, 1) greedy_iteration_kernel(IterArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  long long *acc = reinterpret_cast<long long *>(smem_raw);                // [batch][2]
  float2 *tpos = reinterpret_cast<float2 *>(acc + 2 * (size_t)a.batch);  // [2][batch]
  const unsigned int rank = cluster_rank(), csize = cluster_count();
  const int tid = threadIdx.x, lane = tid & 31;
  const bool single = a.nbatches == 1;  // the batch moves its own next targets
  auto P = [&](int moves) { return (moves & 1) ? a.pos1 : a.pos0; };
  auto share_of = [&](int c, int &lo, int &hi) {
    lo = __ldg(&a.share[(size_t)c * (csize + 1) + rank]);
    hi = __ldg(&a.share[(size_t)c * (csize + 1) + rank + 1]);
  };
  for (int t = tid; t < 2 * a.batch; t += kIterThreads) acc[t] = 0;
  // batch 0: share, staged targets, first terms
  int t_lo, t_hi;
  share_of(0, t_lo, t_hi);
  for (int t = t_lo + tid; t < t_hi; t += kIterThreads) tpos[t] = __ldcg(&a.pos0[t]);
  int2 pt[kPre];
  int pg[kPre];
  long long q0, q1;  // this CTA's terms of the batch
  auto load_terms = [&](int base, int lo, int hi) {
    q0 = __ldg(&a.term_off[base + lo]);
    q1 = __ldg(&a.term_off[base + hi]);
#pragma unroll
    for (int j = 0; j < kPre; j++) {
      const long long q = q0 + (long long)j * kIterThreads + tid;
      pg[j] = -1;
      if (q < q1) {
        pt[j] = __ldg(&a.terms[q]);
        pg[j] = __ldg(&a.term_tgt[q]);
      }
    }
  };
  load_terms(0, t_lo, t_hi);
  cluster_arrive();
  cluster_wait();
  double step = a.step0;
  unsigned int seq = 0;  // batches processed, for the staging buffer parity
  for (int it = 0; it < a.iterations; it++) {
    const bool last_it = it == a.iterations - 1;
    const bool energy_it = a.energy_last && last_it;
    const float stepf = (float)step;
    float2 *const pnew = P(it + 1);
    for (int c = 0; c < a.nbatches; c++, seq++) {
      const int base = c * a.batch;
      const int buf = (int)(seq & 1u) * a.batch, nbuf = a.batch - buf;
      // the next batch: its share now, its target positions (unmoved in this
      // batch unless there is only one batch) staged at the end
      const int cn = (c + 1 < a.nbatches) ? c + 1 : 0;
      const int nbase = cn * a.batch;
      const int nmoves = (cn > c) ? it : it + 1;  // moves of the next targets by then
      int n_lo, n_hi;
      share_of(cn, n_lo, n_hi);
      float2 stage = make_float2(0.f, 0.f);
      if (!single && n_lo + tid < n_hi) stage = __ldcg(&P(nmoves)[nbase + n_lo + tid]);
      // ---- partial forces of this CTA's targets from the batch's start ----
      // a term's contribution, summed per target over the warp's run of
      // equal targets (segmented inclusive scan), added by the run's last lane
      auto add_term = [&](int tg, int2 term, float2 pj) {
        float fx = 0.f, fy = 0.f;
        if (tg >= 0) {
          const float2 pi = tpos[buf + (tg - base)];
          if (term.y == 0) {
            attract_pair(MODEL_FR, a.W, pj.x, pj.y, pi.x, pi.y, fx, fy);
          } else {
            float rx = 0.f, ry = 0.f;
            rep_pair(pj.x, pj.y, pi.x, pi.y, rx, ry);
            fx = (float)term.y * rx;
            fy = (float)term.y * ry;
          }
        }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const float ux = __shfl_up_sync(0xffffffffu, fx, o);
          const float uy = __shfl_up_sync(0xffffffffu, fy, o);
          const int ut = __shfl_up_sync(0xffffffffu, tg, o);
          if (lane >= o && ut == tg) {
            fx += ux;
            fy += uy;
          }
        }
        const int nt = __shfl_down_sync(0xffffffffu, tg, 1);
        if (tg >= 0 && (lane == 31 || nt != tg)) {
          fix_add_shared(&acc[2 * (tg - base)], fx, a.st);
          fix_add_shared(&acc[2 * (tg - base) + 1], fy, a.st);
        }
      };
      auto gather = [&](int tg, int j) {
        return tg >= 0 ? __ldcg(&P(it + (j < base ? 1 : 0))[j]) : make_float2(0.f, 0.f);
      };
      // the loaded-ahead terms: every gather issued before the first use
      float2 pj[kPre];
#pragma unroll
      for (int j = 0; j < kPre; j++) pj[j] = gather(pg[j], pt[j].x);
#pragma unroll
      for (int j = 0; j < kPre; j++) add_term(pg[j], pt[j], pj[j]);
      // the rest of the share (CTA-uniform trip count)
      for (long long q = q0 + (long long)kPre * kIterThreads; q < q1; q += kIterThreads) {
        int tg = -1;
        int2 term = make_int2(0, 0);
        if (q + tid < q1) {
          term = __ldg(&a.terms[q + tid]);
          tg = __ldg(&a.term_tgt[q + tid]);
        }
        add_term(tg, term, gather(tg, term.x));
      }
      __syncthreads();
      // ---- this CTA's targets move (:1171-1177) into the other array ----
      for (int t = t_lo + tid; t < t_hi; t += kIterThreads) {
        const int i = base + t;
        const long long vx = acc[2 * t], vy = acc[2 * t + 1];
        acc[2 * t] = 0;
        acc[2 * t + 1] = 0;
        const double dfx = (double)vx * kFixInv, dfy = (double)vy * kFixInv;
        const float2 np = unit_step(tpos[buf + t], dfx, dfy, stepf);
        pnew[i] = np;
        if (single) tpos[nbuf + t] = np;  // this CTA's next targets are the same
        if (last_it) a.force[i] = make_double2(dfx, dfy);
        if (energy_it) a.e[i] = dfx * dfx + dfy * dfy;
      }
      if (!single) {
        if (n_lo + tid < n_hi) tpos[nbuf + n_lo + tid] = stage;
        for (int t = n_lo + tid + kIterThreads; t < n_hi; t += kIterThreads)
          tpos[nbuf + t] = __ldcg(&P(nmoves)[nbase + t]);
      }
      cluster_arrive();
      load_terms(nbase, n_lo, n_hi);  // registers only
      t_lo = n_lo;
      t_hi = n_hi;
      cluster_wait();
    }
    step = step * a.decay;
  }
}

// Largest cluster (16, else 8, 4, 2, 1 CTAs) of `kernel` with `smem` bytes
// of dynamic shared memory per CTA that can be scheduled (0: none).
template <typename Kernel>
int largest_cluster(Kernel kernel, size_t smem) {
  cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (smem) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  for (int c : {16, 8, 4, 2, 1}) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(c);
    cfg.blockDim = dim3(kIterThreads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = c;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, kernel, &cfg) == cudaSuccess && clusters >= 1) return c;
    cudaGetLastError();  // clear a refused size
  }
  return 0;
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

int greedy_terms_build(bl_ctx *ctx) {
  if (ctx->s.terms) return 0;
  if (int rc = greedy_walks_build(ctx)) return rc;
  const int n = ctx->g.n;
  const long long total = ctx->g.nnz + ctx->s.walk_total;
  // term offsets = CSR offsets + walk offsets
  std::vector<long long> woff(n + 1);
  BL_CUDA(ctx, cudaMemcpy(woff.data(), ctx->s.walk_off, (size_t)(n + 1) * sizeof(long long), cudaMemcpyDeviceToHost));
  for (int i = 0; i <= n; i++) woff[i] += ctx->h_rowptr[i];
  ctx->s.h_term_off = woff;
  BL_CUDA(ctx, cudaMalloc(&ctx->s.term_off, (size_t)(n + 1) * sizeof(long long)));
  BL_CUDA(ctx, cudaMemcpy(ctx->s.term_off, woff.data(), (size_t)(n + 1) * sizeof(long long), cudaMemcpyHostToDevice));
  BL_CUDA(ctx, cudaMalloc(&ctx->s.term_tgt, (size_t)std::max<long long>(total, 1) * sizeof(int)));
  BL_CUDA(ctx, cudaMalloc(&ctx->s.terms, (size_t)std::max<long long>(total, 1) * sizeof(int2)));
  const long long threads = 32LL * n;
  term_list_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, ctx->stream>>>(
      n, ctx->g.rowptr, ctx->g.colids, ctx->s.walk_off, ctx->s.walk_pairs, ctx->s.terms, ctx->s.term_tgt);
  ctx->launches++;
  BL_CUDA(ctx, cudaGetLastError());
  return 0;
}

int greedy_walk_run(bl_ctx *ctx, int batch, int iterations, double step0, double decay, bool want_energy,
                    double *energy_out) {
  const int n = ctx->g.n;
  if (batch < 1) return bl_fail(ctx, BL_ERR_ARG, "batch must be >= 1");
  if (iterations <= 0) return 0;
  if (int rc = greedy_terms_build(ctx)) return rc;
  if (int rc = bl_check_status(ctx)) return rc;
  batch = std::min(batch, n);
  const size_t smem = (size_t)batch * 2 * sizeof(long long) + (size_t)2 * batch * sizeof(float2);
  int smem_optin = 0;
  cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
  if (smem + 1024 > (size_t)smem_optin)
    return bl_fail(ctx, BL_ERR_TOO_LARGE, "algo 5: batch too large for the shared-memory accumulators");
  const int csize = largest_cluster(greedy_iteration_kernel, smem);
  if (csize < 1) return bl_fail(ctx, BL_ERR_TOO_LARGE, "algo 5: no thread-block cluster fits");
  const int nbatches = (n + batch - 1) / batch;
  // each CTA's share of every batch: consecutive targets with about
  // 1/csize of the batch's terms (graph-only; kept for this batch size)
  if (ctx->s.greedy_share_key != (long long)batch * 64 + csize) {
    std::vector<int> share((size_t)nbatches * (csize + 1));
    const std::vector<long long> &to = ctx->s.h_term_off;
    for (int c = 0; c < nbatches; c++) {
      const int base = c * batch, cnt = std::min(batch, n - base);
      const long long q0 = to[base], T = to[base + cnt] - q0;
      int t = 0;
      for (int r = 0; r <= csize; r++) {
        const long long want = (r == csize) ? T : (T * r + csize - 1) / csize;
        while (t < cnt && to[base + t] - q0 < want) t++;
        share[(size_t)c * (csize + 1) + r] = (r == csize) ? cnt : t;
      }
    }
    if (ctx->s.greedy_share) cudaFree(ctx->s.greedy_share);
    ctx->s.greedy_share = nullptr;
    ctx->s.greedy_share_key = -1;
    BL_CUDA(ctx, cudaMalloc(&ctx->s.greedy_share, share.size() * sizeof(int)));
    BL_CUDA(ctx, cudaMemcpy(ctx->s.greedy_share, share.data(), share.size() * sizeof(int), cudaMemcpyHostToDevice));
    ctx->s.greedy_share_key = (long long)batch * 64 + csize;
  }
  if (!ctx->s.greedy_pos) BL_CUDA(ctx, cudaMalloc(&ctx->s.greedy_pos, (size_t)std::max(n, 2) * sizeof(float2)));
  IterArgs a;
  a.n = n;
  a.batch = batch;
  a.nbatches = nbatches;
  a.iterations = iterations;
  a.energy_last = want_energy ? 1 : 0;
  a.W = (float)ctx->weight;
  a.step0 = step0;
  a.decay = decay;
  a.term_off = ctx->s.term_off;
  a.terms = ctx->s.terms;
  a.term_tgt = ctx->s.term_tgt;
  a.share = ctx->s.greedy_share;
  a.pos0 = ctx->pos;
  a.pos1 = ctx->s.greedy_pos;
  a.force = ctx->force;
  a.e = ctx->e;
  a.st = ctx->s.status;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(csize);
  cfg.blockDim = dim3(kIterThreads);
  cfg.dynamicSmemBytes = smem;
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
  // every vertex moved `iterations` times: an odd count leaves them in pos1
  if (iterations & 1)
    BL_CUDA(ctx, cudaMemcpyAsync(ctx->pos, ctx->s.greedy_pos, (size_t)n * sizeof(float2), cudaMemcpyDeviceToDevice,
                                 ctx->stream));
  if (want_energy) {
    if (int rc = energy_reduce(ctx, energy_out)) return rc;
  } else {
    BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return bl_check_status(ctx);
}

}  // namespace bl

extern "C" int bl_greedy_walks(bl_ctx *ctx, long long *offsets, int *sources, int *counts, long long cap,
                               long long *total) try {
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
} catch (...) {
  return bl_host_exception(ctx);
}

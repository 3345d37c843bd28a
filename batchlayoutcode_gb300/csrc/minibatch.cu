// minibatch.cu -- all-pairs stochastic minibatch update (algo 2 / 3 / 8, and
// algo 7 and the second phase of algo 5).
//
// Reference: sample/algorithms.cpp:739-783 (FR), :894-936 (LinLog),
// :967-1009 (FA), :536-590 (algo 7: attraction over every CSR neighbour, the
// neighbours' repulsion removed), :1112-1125 (algo 5 after 80 % of the
// iterations: repulsion -d/|d| instead of -d/|d|^2).  Vertices are processed in consecutive batches of `batch`
// ids; every force of a batch uses the positions at the start of that batch
// (Jacobi inside a batch) and the batch then moves by STEP * f/|f| before the
// next batch starts (Gauss-Seidel across batches).  f_i is attraction over
// the neighbours matched by the sorted-CSR cursor (kindex, :758-762) plus
// repulsion -d/|d|^2 over every other vertex with |d| > 0.
//
// GB300 design: one persistent cooperative kernel runs every iteration and
// batch.  Each block owns a contiguous slice of source vertices kept in shared
// memory for the whole run (8 B per vertex, float2).  For batch c every block
// sweeps its slice against the batch's targets with a branch-free inner loop
// (repulsion for all pairs; 7 FP32 instructions per pair, one MUFU rcp), and
// writes one FP32 partial force per target.  After a grid barrier the block(s)
// whose slice holds batch c sum the partials in FP64 in a fixed order, correct
// the neighbour pairs (remove their repulsion, add the model's attraction --
// the decomposition the reference's own algo 7 uses, :553-579), move the
// vertices and refresh their shared-memory copy.  Blocks that do not own
// batch c go straight on to batch c+1: the only values that changed are batch
// c's own positions, which live in the owners' slices.
//
// Algorithmic work: 10 flops per ordered pair (2 sub, 3 for |d|^2, 1 rcp,
// 2 FMA x 2 components counted as 4), n*n pairs per iteration.
#include <cooperative_groups.h>

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <mutex>

#include "../../include/batchlayout_gb300.h"
#include "bl_device.cuh"

namespace bl {
namespace {

constexpr int kThreads = 512;
constexpr int kGroups = 4;                     // source sub-slices per block
constexpr int kGroup = kThreads / kGroups;     // 128 threads per group
constexpr int kChunk = 2 * kGroup;             // 256 targets per sweep pass
constexpr int kWarps = kThreads / 32;
constexpr int kMaxBatch = 4096;

// Block partial forces are summed across blocks as 64-bit fixed-point
// integers (units of 2^-28): integer addition is exact and associative, so
// the total does not depend on the order of the atomics and stays
// deterministic.  A partial beyond +-2^34 (forces of ~1e10, coincident
// vertices) is reported as an error instead of wrapping.
// Every buffer of accumulators has kAccCopies copies; block s adds into copy
// s % kAccCopies, so fewer blocks queue on one address at the same time, and
// the owners add the copies up (integer sums: exact in any order).
constexpr int kAccCopies = 8;
constexpr float kFixScale = 268435456.0f;        // 2^28
constexpr double kFixInv = 1.0 / 268435456.0;    // 2^-28
constexpr float kFixLimit = 17179869184.0f;      // 2^34

__device__ __forceinline__ void acc_add(long long *dst, float v, DevStatus *st) {
  if (!(fabsf(v) < kFixLimit)) {
    dev_record_error(st, DEV_FORCE_RANGE);
    return;
  }
  atomicAdd(reinterpret_cast<unsigned long long *>(dst), (unsigned long long)__float2ll_rn(v * kFixScale));
}

struct MinibatchArgs {
  int n, batch, nbatches, model, grid;
  double W;
  const int *eff_rowptr, *eff_colids;
  // cursor[s * n + i]: neighbours of i below the first vertex of block s's
  // slice (null: found by binary search)
  const int *cursor;
  float2 *pos;
  double2 *force;
  double *e;
  long long *acc;         // [2][kAccCopies][batch][2] fixed-point force sums (2^-28 units)
  double *energy;         // energy per iteration (device)
  double *energy_parts;   // [grid]
  long long *loops;       // iterations run (device, 1 value)
  DevStatus *st;
  int iterations;
  double step0, decay;
  int converged;
  double engt;
  long long max_loops;
};

// The reference's kindex cursor (algorithms.cpp:746,758-762) restricted to
// this block's slice: the target's matched neighbours inside [slo, shi) are
// staged in shared memory (up to kNbCap, slice-local indices) with the
// batch's targets, so stepping the cursor reads shared memory; a target with
// more neighbours in the slice continues from global memory.
constexpr int kNbCap = 16;

struct NbList {
  int *ids;    // [kChunk][kNbCap] slice-local ids
  int *meta;   // [kChunk][2]: number of neighbours in the slice, first CSR index
};

// Stage the neighbours of targets [base, base + cnt) (cnt <= kChunk) that lie
// in [slo, shi).  One thread per target.
__device__ __forceinline__ void stage_neighbours(const MinibatchArgs &a, NbList L, int s, int base, int cnt,
                                                 int slo, int shi, int sbase) {
  for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
    const int i = base + t;
    const int r0 = a.eff_rowptr[i], r1 = a.eff_rowptr[i + 1];
    int k0, k1;
    if (a.cursor) {
      k0 = r0 + a.cursor[(size_t)s * a.n + i];
      k1 = (s + 1 < a.grid) ? r0 + a.cursor[(size_t)(s + 1) * a.n + i] : r1;
    } else {  // lower bounds of slo and shi in the sorted neighbour list
      int lo = r0, hi = r1;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&a.eff_colids[mid]) < slo) lo = mid + 1;
        else hi = mid;
      }
      k0 = lo;
      hi = r1;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&a.eff_colids[mid]) < shi) lo = mid + 1;
        else hi = mid;
      }
      k1 = lo;
    }
    const int m = min(k1 - k0, kNbCap);
    for (int q = 0; q < m; q++) L.ids[t * kNbCap + q] = __ldg(&a.eff_colids[k0 + q]) - sbase;
    L.meta[2 * t] = k1 - k0;
    L.meta[2 * t + 1] = k0;
  }
}

struct Cursor {
  int ptr, cnt, k0, next;
  const int *ids;
};

__device__ __forceinline__ int cursor_at(const MinibatchArgs &a, const Cursor &c, int sbase) {
  if (c.ptr >= c.cnt) return INT_MAX;
  if (c.ptr < kNbCap) return c.ids[c.ptr];
  return __ldg(&a.eff_colids[c.k0 + c.ptr]) - sbase;  // beyond the staged ones
}

// Cursor of target t positioned at the group's first source `from` (slice-local).
__device__ __forceinline__ void cursor_init(Cursor &c, const MinibatchArgs &a, NbList L, int t, int from,
                                            int sbase) {
  c.ids = L.ids + t * kNbCap;
  c.cnt = L.meta[2 * t];
  c.k0 = L.meta[2 * t + 1];
  c.ptr = 0;
  c.next = cursor_at(a, c, sbase);
  // bounded by the neighbours inside the slice
  while (c.next < from) {
    c.ptr++;
    c.next = cursor_at(a, c, sbase);
  }
}

// For each matched neighbour q of the target with ga <= q < gb: remove the
// repulsion the sweep added (identical FP32 operations) and add the model's
// attraction -- the reference applies attraction instead of repulsion to
// these pairs (algorithms.cpp:758-768).
template <int kRep>
__device__ __noinline__ void correct_neighbours(const MinibatchArgs &a, Cursor c, int ga, int gb,
                                                const float2 *slice, float2 pi, int sbase, float &fx, float &fy) {
  // bounded by the target's neighbours inside the slice
  for (int q = c.next; q < gb; q = c.next) {
    if (q >= ga) {
      const float2 pj = slice[q];
      const float dx = pj.x - pi.x, dy = pj.y - pi.y;
      const float d2 = fmaf(dx, dx, fmaf(dy, dy, kTinyD2));
      const float r = (kRep == REP_UNIT) ? rsqrt_approx(d2) : rcp_approx(d2);
      fx = fmaf(dx, r, fx);
      fy = fmaf(dy, r, fy);
      attract_pair(a.model, (float)a.W, pj.x, pj.y, pi.x, pi.y, fx, fy);
    }
    c.ptr++;
    c.next = cursor_at(a, c, sbase);
  }
}

// Slice of sources owned by block s: [lo, hi).
__device__ __forceinline__ void slice_of(int n, int grid, int s, int &lo, int &hi) {
  lo = (int)(((long long)n * s) / grid);
  hi = (int)(((long long)n * (s + 1)) / grid);
}

__device__ double block_sum(double v, double *red) {
  // fixed-order tree: warp xor-shuffle, then warp 0 over the warp sums
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  if (w == 0) {
    t = (l < kWarps) ? red[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  const double r = red[0];
  __syncthreads();
  return r;
}

template <int kRep>
__global__ void __launch_bounds__(kThreads, 1) minibatch_kernel(MinibatchArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int s = blockIdx.x;
  int slo, shi;
  slice_of(a.n, a.grid, s, slo, shi);
  const int sbase = slo & ~1;  // even so that pairs of sources load as float4
  const int slen = shi - sbase;
  float2 *slice = reinterpret_cast<float2 *>(smem_raw);
  const int slen_pad = (slen + 3) & ~3;
  float2 *gsum = slice + slen_pad;              // [kGroups-1][kChunk]
  float2 *tbuf = gsum + (kGroups - 1) * kChunk;  // [2][batch]: targets of this and the next batch
  int *nbmem = reinterpret_cast<int *>(tbuf + 2 * a.batch);  // [2][kChunk * (kNbCap + 2)]
  auto nblist = [&](unsigned int b) {
    NbList L;
    L.ids = nbmem + b * (kChunk * (kNbCap + 2));
    L.meta = L.ids + kChunk * kNbCap;
    return L;
  };
  __shared__ double red[kWarps];

  const int tid = threadIdx.x;
  const int grp = tid / kGroup, gl = tid % kGroup;

  for (int k = tid; k < slen; k += kThreads) slice[k] = __ldcg(&a.pos[sbase + k]);
  // group sub-ranges of [slo, shi) in slice-local indices
  const int la = slo - sbase, lb = shi - sbase;
  const int ga = la + (int)((long long)(lb - la) * grp / kGroups);
  const int gb = la + (int)((long long)(lb - la) * (grp + 1) / kGroups);
  __syncthreads();

  unsigned int epoch = 0;
  double step = a.step0;
  double e_prev = DBL_MAX, e_cur = 0.0;
  long long loop = 0;
  bool ok = true;
  bool prefetched = false;
  unsigned int seq = 0;  // batches processed in this launch

  while (ok) {
    if (a.converged) {
      if (!(fabs(e_prev - e_cur) / e_prev > a.engt) || loop >= a.max_loops) break;
    } else if (loop >= a.iterations) {
      break;
    }
    const bool need_energy = a.converged || (loop == a.iterations - 1);
    for (int c = 0; c < a.nbatches && ok; c++, seq++) {
      const int base = c * a.batch;
      const int cnt = min(a.batch, a.n - base);
      // buffers alternate by the batch's position in the whole run, so the
      // last batch of an iteration and the first of the next never share one
      const int buf = (int)(seq & 1u);
      float2 *tpos = tbuf + buf * a.batch;
      // the targets of batch c are normally prefetched during batch c-1;
      // the first batch of the run, and every batch when there is only one,
      // loads them here
      if (!prefetched) {
        for (int t = tid; t < cnt; t += kThreads) tpos[t] = __ldcg(&a.pos[base + t]);
        if (cnt <= kChunk) stage_neighbours(a, nblist(buf), s, base, cnt, slo, shi, sbase);
      }
      __syncthreads();
      // ---- sweep: partial force of this block's slice on every target ----
      // repulsion for every source, attraction instead for the target's
      // matched neighbours (found by a sorted cursor, rare), as in the
      // reference's j loop
      for (int c0 = 0; c0 < cnt; c0 += kChunk) {
        const int t0 = c0 + gl, t1 = t0 + kGroup;
        const bool v0 = t0 < cnt, v1 = t1 < cnt;
        const float2 p0 = v0 ? tpos[t0] : make_float2(0.f, 0.f);
        const float2 p1 = v1 ? tpos[t1] : make_float2(0.f, 0.f);
        NbList L = nblist(buf);
        if (cnt > kChunk) {  // several chunks: stage this chunk's neighbours now
          __syncthreads();
          stage_neighbours(a, L, s, base + c0, min(kChunk, cnt - c0), slo, shi, sbase);
          __syncthreads();
        }
        Cursor c0r, c1r;
        c0r.next = c1r.next = INT_MAX;
        c0r.ptr = c0r.cnt = c1r.ptr = c1r.cnt = 0;
        if (v0) cursor_init(c0r, a, L, gl, ga, sbase);
        if (v1) cursor_init(c1r, a, L, gl + kGroup, ga, sbase);
        float fx0a = 0.f, fy0a = 0.f, fx0b = 0.f, fy0b = 0.f;
        float fx1a = 0.f, fy1a = 0.f, fx1b = 0.f, fy1b = 0.f;
        // branch-free repulsion over the group's sources ...
        int k = ga;
        if ((k & 1) && k < gb) {
          const float2 q = slice[k];
          rep_law_pair<kRep>(q.x, q.y, p0.x, p0.y, fx0a, fy0a);
          rep_law_pair<kRep>(q.x, q.y, p1.x, p1.y, fx1a, fy1a);
          k++;
        }
#pragma unroll 4
        for (; k + 1 < gb; k += 2) {
          const float4 q = *reinterpret_cast<const float4 *>(&slice[k]);
          rep_law_pair<kRep>(q.x, q.y, p0.x, p0.y, fx0a, fy0a);
          rep_law_pair<kRep>(q.z, q.w, p0.x, p0.y, fx0b, fy0b);
          rep_law_pair<kRep>(q.x, q.y, p1.x, p1.y, fx1a, fy1a);
          rep_law_pair<kRep>(q.z, q.w, p1.x, p1.y, fx1b, fy1b);
        }
        if (k < gb) {
          const float2 q = slice[k];
          rep_law_pair<kRep>(q.x, q.y, p0.x, p0.y, fx0b, fy0b);
          rep_law_pair<kRep>(q.x, q.y, p1.x, p1.y, fx1b, fy1b);
        }
        // ... then the matched neighbours in [ga, gb): take their repulsion
        // back (same FP32 formula) and add the model's attraction instead
        if (v0) correct_neighbours<kRep>(a, c0r, ga, gb, slice, p0, sbase, fx0b, fy0b);
        if (v1) correct_neighbours<kRep>(a, c1r, ga, gb, slice, p1, sbase, fx1b, fy1b);
        const float2 r0 = make_float2(fx0a + fx0b, fy0a + fy0b);
        const float2 r1 = make_float2(fx1a + fx1b, fy1a + fy1b);
        if (grp > 0) {
          gsum[(grp - 1) * kChunk + gl] = r0;
          gsum[(grp - 1) * kChunk + gl + kGroup] = r1;
        }
        __syncthreads();
        if (grp == 0) {
          float2 o0 = r0, o1 = r1;
#pragma unroll
          for (int g = 0; g < kGroups - 1; g++) {
            const float2 u0 = gsum[g * kChunk + gl], u1 = gsum[g * kChunk + gl + kGroup];
            o0.x += u0.x; o0.y += u0.y;
            o1.x += u1.x; o1.y += u1.y;
          }
          long long *A = a.acc + ((size_t)buf * kAccCopies + s % kAccCopies) * a.batch * 2;
          if (t0 < cnt) {
            acc_add(&A[2 * t0], o0.x, a.st);
            acc_add(&A[2 * t0 + 1], o0.y, a.st);
          }
          if (t1 < cnt) {
            acc_add(&A[2 * t1], o1.x, a.st);
            acc_add(&A[2 * t1 + 1], o1.y, a.st);
          }
        }
        __syncthreads();
      }
      // announce this block's partials, then prefetch the next batch's targets
      // and cursors while the other blocks arrive: its vertices do not move
      // before it, and the cursors depend on the graph only.  Positions are
      // read through L2: other blocks moved them.
      grid_arrive(a.st, epoch);
      {
        const int cn = (c + 1 < a.nbatches) ? c + 1 : 0;
        prefetched = (cn != c);  // a single batch moves itself: reload after the update
        if (prefetched) {
          const int nbase = cn * a.batch;
          const int ncnt = min(a.batch, a.n - nbase);
          float2 *ntpos = tbuf + (int)((seq + 1u) & 1u) * a.batch;
          for (int t = tid; t < ncnt; t += kThreads) ntpos[t] = __ldcg(&a.pos[nbase + t]);
          if (ncnt <= kChunk) stage_neighbours(a, nblist((seq + 1u) & 1u), s, nbase, ncnt, slo, shi, sbase);
        }
      }
      ok = grid_wait(a.st, epoch);
      if (!ok) break;
      // ---- owners: read the summed force, update, clear the accumulator -----
      const int olo = max(slo, base), ohi = min(shi, base + cnt);
      if (olo < ohi) {
        long long *A = a.acc + (size_t)buf * kAccCopies * a.batch * 2;
        const float stepf = (float)step;
        for (int i = olo + tid; i < ohi; i += kThreads) {
          const int t = i - base;
          longlong2 v = make_longlong2(0, 0);
#pragma unroll
          for (int k = 0; k < kAccCopies; k++) {
            long long *Ak = A + (size_t)k * a.batch * 2;
            const longlong2 u = __ldcg(reinterpret_cast<const longlong2 *>(&Ak[2 * t]));
            // cleared for the batch after next, which reuses this buffer
            *reinterpret_cast<longlong2 *>(&Ak[2 * t]) = make_longlong2(0, 0);
            v.x += u.x;
            v.y += u.y;
          }
          const double dfx = (double)v.x * kFixInv, dfy = (double)v.y * kFixInv;
          const float2 pi = tpos[t];
          const float fx = (float)dfx, fy = (float)dfy;
          float2 np = pi;
          const float m2 = fmaf(fx, fx, fy * fy);
          if (m2 >= 1.17549435e-38f && m2 <= 3.0e38f) {
            const float rm = rsqrt_approx(m2);
            np.x = fmaf(stepf, fx * rm, pi.x);
            np.y = fmaf(stepf, fy * rm, pi.y);
          } else if (fx != 0.f || fy != 0.f) {  // |f|^2 outside the FP32 range
            const double mag = sqrt(dfx * dfx + dfy * dfy);
            np.x = (float)((double)pi.x + (dfx / mag) * step);
            np.y = (float)((double)pi.y + (dfy / mag) * step);
          }
          a.pos[i] = np;
          slice[i - sbase] = np;
          a.force[i] = make_double2(dfx, dfy);
          a.e[i] = dfx * dfx + dfy * dfy;
        }
      }
      // owner warps still read tpos and write the slice: finish before the
      // next batch reloads tpos and sweeps the slice
      __syncthreads();
    }
    if (!ok) break;
    if (need_energy) {
      ok = grid_barrier(a.st, epoch);
      if (!ok) break;
      double v = 0.0;
      for (int i = slo + tid; i < shi; i += kThreads) v += __ldcg(&a.e[i]);
      v = block_sum(v, red);
      if (tid == 0) a.energy_parts[s] = v;
      ok = grid_barrier(a.st, epoch);
      if (!ok) break;
      double tot = 0.0;
      if (tid == 0)
        for (int q = 0; q < a.grid; q++) tot += __ldcg(&a.energy_parts[q]);
      if (tid == 0) red[0] = tot;
      __syncthreads();
      tot = red[0];
      __syncthreads();
      e_prev = e_cur;
      e_cur = tot;
      if (s == 0 && tid == 0) a.energy[0] = tot;
    }
    step = step * a.decay;
    loop++;
  }
  if (s == 0 && tid == 0) *a.loops = loop;
}

// cursor[s * n + i] = number of matched neighbours of i below slice_lo(s)
__global__ void cursor_table_kernel(const int *__restrict__ rowptr, const int *__restrict__ colids, int n,
                                    int grid, int *cursor) {
  const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= (long long)n * grid) return;
  const int s = (int)(gid / n), i = (int)(gid % n);
  int slo, shi;
  slice_of(n, grid, s, slo, shi);
  int lo = rowptr[i], hi = rowptr[i + 1];
  const int k0 = lo;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (colids[mid] < slo) lo = mid + 1;
    else hi = mid;
  }
  cursor[gid] = lo - k0;
}

}  // namespace

int ensure_minibatch_scratch(bl_ctx *ctx, int batch, int grid) {
  (void)grid;
  const size_t need = (size_t)2 * kAccCopies * batch * 2 * sizeof(long long);
  if (ctx->s.partials_bytes < need) {
    if (ctx->s.partials) cudaFree(ctx->s.partials);
    ctx->s.partials = nullptr;
    ctx->s.partials_bytes = 0;
    BL_CUDA(ctx, cudaMalloc(&ctx->s.partials, need));
    ctx->s.partials_bytes = need;
  }
  return 0;
}

int minibatch_run(bl_ctx *ctx, int model, int batch, int iterations, double step0,
                  double decay, bool converged, double engt, long long max_loops,
                  double *energy_out, long long *loops_out) {
  const int n = ctx->g.n;
  if (batch < 1) return bl_fail(ctx, -1, "batch must be >= 1");
  if (n < 1) return bl_fail(ctx, -7, "no graph loaded");
  batch = std::min(batch, n);  // a batch larger than n is one Jacobi batch
  if (batch > kMaxBatch)
    return bl_fail(ctx, -5, "minibatch path supports batch <= 4096 (got " + std::to_string(batch) + ")");
  if (!converged && iterations <= 0) {
    if (energy_out) *energy_out = 0.0;
    if (loops_out) *loops_out = 0;
    return 0;
  }
  // model 2 / 3 / 8: the cursor-matched neighbours, inverse-distance
  // repulsion; 7 (algo 7): FR over every CSR neighbour; 5 (algo 5, second
  // phase): FR over the cursor-matched neighbours, unit-vector repulsion
  const int attract = (model == MODEL_SD || model == MODEL_GREEDY_EXACT) ? (int)MODEL_FR : model;
  const bool unit_rep = model == MODEL_GREEDY_EXACT;
  const bool full_rows = model == MODEL_SD;
  if (full_rows)
    if (int rc = ensure_sorted_csr(ctx)) return rc;
  const int *nb_rowptr = full_rows ? ctx->g.srt_rowptr : ctx->g.eff_rowptr;
  const int *nb_colids = full_rows ? ctx->g.srt_colids : ctx->g.eff_colids;
  // the cursor table belongs to one neighbour set; the full rows share the
  // cursor-matched set's table when the two sets are the same arrays
  const bool own_table = full_rows && nb_colids != ctx->g.eff_colids;
  int *&cursor = own_table ? ctx->s.cursor_full : ctx->s.cursor;
  int &cursor_grid = own_table ? ctx->s.cursor_full_grid : ctx->s.cursor_grid;
  void (*kernel)(MinibatchArgs) = unit_rep ? minibatch_kernel<REP_UNIT> : minibatch_kernel<REP_INV>;
  int grid = std::min(ctx->num_sms, std::max(1, (n + 127) / 128));
  int dev_smem_optin = 0;
  cudaDeviceGetAttribute(&dev_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
  auto smem_for = [&](int g) {
    const int slice_max = (n + g - 1) / g + 2;
    return (size_t)(((slice_max + 3) & ~3) + (kGroups - 1) * kChunk + 2 * batch) * sizeof(float2) +
           (size_t)2 * kChunk * (kNbCap + 2) * sizeof(int);
  };
  while (smem_for(grid) + 1024 > (size_t)dev_smem_optin && grid < ctx->num_sms) grid++;
  const size_t smem = smem_for(grid);
  if (smem + 1024 > (size_t)dev_smem_optin)
    return bl_fail(ctx, -5, "graph too large for the shared-memory source slices of the minibatch path");
  BL_CUDA(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 0;
  BL_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kThreads, smem));
  if (occ < 1 || grid > occ * ctx->num_sms)
    return bl_fail(ctx, -5, "minibatch kernel cannot be co-resident");
  if (int rc = ensure_minibatch_scratch(ctx, batch, grid)) return rc;
  if (cursor_grid != grid) {
    if (cursor) cudaFree(cursor);
    cursor = nullptr;
    cursor_grid = 0;
    BL_CUDA(ctx, cudaMalloc(&cursor, (size_t)n * grid * sizeof(int)));
    const long long total = (long long)n * grid;
    cursor_table_kernel<<<(unsigned)((total + 255) / 256), 256, 0, ctx->stream>>>(nb_rowptr, nb_colids, n, grid,
                                                                                cursor);
    BL_CUDA(ctx, cudaGetLastError());
    ctx->launches++;
    cursor_grid = grid;
  }
  BL_CUDA(ctx, cudaMemsetAsync(ctx->s.status, 0, sizeof(DevStatus), ctx->stream));
  BL_CUDA(ctx, cudaMemsetAsync(ctx->s.partials, 0, (size_t)2 * kAccCopies * batch * 2 * sizeof(long long),
                               ctx->stream));

  MinibatchArgs a;
  a.n = n;
  a.batch = batch;
  a.nbatches = (n + batch - 1) / batch;
  a.model = attract;
  a.grid = grid;
  a.W = ctx->weight;
  a.eff_rowptr = nb_rowptr;
  a.eff_colids = nb_colids;
  a.cursor = cursor;
  a.pos = ctx->pos;
  a.force = ctx->force;
  a.e = ctx->e;
  a.acc = reinterpret_cast<long long *>(ctx->s.partials);
  a.energy = ctx->s.energy;
  a.energy_parts = ctx->s.energy_parts;
  a.loops = reinterpret_cast<long long *>(ctx->s.energy + 1);
  a.st = ctx->s.status;
  a.iterations = iterations;
  a.step0 = step0;
  a.decay = decay;
  a.converged = converged ? 1 : 0;
  a.engt = engt;
  a.max_loops = max_loops;
  void *args[] = {&a};
  bl_time_begin(ctx, "minibatch_kernel");
  BL_CUDA(ctx, cudaLaunchCooperativeKernel((const void *)kernel, dim3(grid), dim3(kThreads), args, smem,
                                           ctx->stream));
  bl_time_end(ctx, "minibatch_kernel");
  ctx->launches++;
  double host[2];
  BL_CUDA(ctx, cudaMemcpyAsync(host, ctx->s.energy, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (int rc = bl_check_status(ctx)) return rc;
  long long loops;
  memcpy(&loops, &host[1], sizeof(loops));
  if (energy_out) *energy_out = host[0];
  if (loops_out) *loops_out = loops;
  return 0;
}

}  // namespace bl

// ---------------------------------------------------------------------------
// Allocation-free entry point.
//
// Some callers cannot allocate device memory once they are running: services
// that reserve all GPU memory up front in their own pool, real-time loops
// that forbid allocation after start-up, or code that enqueues work on a
// stream another component owns.  bl_minibatch_iteration_noalloc runs the
// same minibatch kernel as bl_minibatch_iteration, but every scratch buffer
// it needs (partial forces, energy partials, the device status word) lives
// in the fixed array below, so the call allocates nothing.  The caller passes
// its inputs and outputs as device pointers.
//
// Limits: batch <= 256 and at most 160 blocks (one per SM); the scratch is a
// fixed 768 KiB (force accumulators, energy partials, status word).
// The array exists once per device for the lifetime of the process and every
// call on that device shares it: calls that overlap on the GPU (different
// streams, or host threads that do not serialise) race and give wrong
// results.  The first call on a device looks up the array's device address
// (cudaGetSymbolAddress) with that device current; make that first call
// before any stream capture.
// ---------------------------------------------------------------------------
namespace bl {
namespace {

constexpr int kNoAllocMaxBatch = 256;
constexpr int kNoAllocMaxGrid = 160;
constexpr size_t kNoAllocPartialBytes = (size_t)2 * kNoAllocMaxBatch * kNoAllocMaxGrid * sizeof(float2);
constexpr size_t kNoAllocBytes = 768 * 1024;
static_assert((size_t)2 * kAccCopies * kNoAllocMaxBatch * 2 * sizeof(long long) <= kNoAllocPartialBytes,
              "no-alloc accumulators too small");
static_assert(kNoAllocPartialBytes + kNoAllocMaxGrid * sizeof(double) + 4 * sizeof(double) +
                      sizeof(DevStatus) <= kNoAllocBytes,
              "no-alloc scratch too small");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
unsigned char *g_noalloc_ptr[kMaxDevices] = {nullptr};

}  // namespace
}  // namespace bl

extern "C" int bl_minibatch_iteration_noalloc(int n, const int *d_rowptr, const int *d_colids,
                                              float *d_xy, double *d_force, double *d_vertex_energy,
                                              int model, int batch, double weight, double step,
                                              double *energy_out, void *stream) try {
  using namespace bl;
  if (n < 1 || !d_rowptr || !d_colids || !d_xy || !d_force || !d_vertex_energy)
    return BL_ERR_ARG;
  if (model != MODEL_FR && model != MODEL_LINLOG && model != MODEL_FA) return BL_ERR_ARG;
  if (batch < 1) return BL_ERR_ARG;
  batch = std::min(batch, n);
  if (batch > kNoAllocMaxBatch) return BL_ERR_TOO_LARGE;  // scratch holds batch <= 256
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) return BL_ERR_CUDA;
  unsigned char *base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return BL_ERR_CUDA;
      g_noalloc_ptr[device] = static_cast<unsigned char *>(p);
    }
    base = g_noalloc_ptr[device];
  }
  int num_sms = 0, smem_optin = 0;
  cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device);
  cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  // same block count and shared-memory sizing as the context path
  int grid = std::min(num_sms, std::max(1, (n + 127) / 128));
  auto smem_for = [&](int g) {
    const int slice_max = (n + g - 1) / g + 2;
    return (size_t)(((slice_max + 3) & ~3) + (kGroups - 1) * kChunk + 2 * batch) * sizeof(float2) +
           (size_t)2 * kChunk * (kNbCap + 2) * sizeof(int);
  };
  while (smem_for(grid) + 1024 > (size_t)smem_optin && grid < num_sms) grid++;
  if (grid > kNoAllocMaxGrid) return BL_ERR_TOO_LARGE;  // scratch holds 160 blocks of partials
  const size_t smem = smem_for(grid);
  if (smem + 1024 > (size_t)smem_optin) return BL_ERR_TOO_LARGE;
  if (cudaFuncSetAttribute(minibatch_kernel<REP_INV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return BL_ERR_CUDA;
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, minibatch_kernel<REP_INV>, kThreads, smem) != cudaSuccess ||
      occ < 1 || grid > occ * num_sms)
    return BL_ERR_TOO_LARGE;
  // carve the scratch: force accumulators | energy parts | energy + loops | status
  float2 *partials = reinterpret_cast<float2 *>(base);
  double *energy_parts = reinterpret_cast<double *>(base + kNoAllocPartialBytes);
  double *energy = energy_parts + kNoAllocMaxGrid;
  DevStatus *status = reinterpret_cast<DevStatus *>(energy + 4);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the status word (barrier counter, error code) and the force accumulators
  // must start at zero; every other scratch value is written before it is read
  if (cudaMemsetAsync(status, 0, sizeof(DevStatus), st) != cudaSuccess) return BL_ERR_CUDA;
  if (cudaMemsetAsync(partials, 0, (size_t)2 * kAccCopies * batch * 2 * sizeof(long long), st) != cudaSuccess)
    return BL_ERR_CUDA;
  MinibatchArgs a;
  a.n = n;
  a.batch = batch;
  a.nbatches = (n + batch - 1) / batch;
  a.model = model;
  a.grid = grid;
  a.W = weight;
  a.eff_rowptr = d_rowptr;
  a.eff_colids = d_colids;
  a.cursor = nullptr;
  a.pos = reinterpret_cast<float2 *>(d_xy);
  a.force = reinterpret_cast<double2 *>(d_force);
  a.e = d_vertex_energy;
  a.acc = reinterpret_cast<long long *>(partials);
  a.energy = energy;
  a.energy_parts = energy_parts;
  a.loops = reinterpret_cast<long long *>(energy + 1);
  a.st = status;
  a.iterations = 1;
  a.step0 = step;
  a.decay = 1.0;
  a.converged = 0;
  a.engt = 0.0;
  a.max_loops = 0;
  void *args[] = {&a};
  if (cudaLaunchCooperativeKernel((const void *)minibatch_kernel<REP_INV>, dim3(grid), dim3(kThreads), args, smem,
                                  st) !=
      cudaSuccess)
    return BL_ERR_CUDA;
  double host_energy = 0.0;
  DevStatus host_status;
  if (cudaMemcpyAsync(&host_energy, energy, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(&host_status, status, sizeof(DevStatus), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return BL_ERR_CUDA;
  if (host_status.code != DEV_OK) return BL_ERR_DEVICE_TIMEOUT;
  if (energy_out) *energy_out = host_energy;
  return BL_OK;
} catch (...) {
  return bl_host_exception(nullptr);
}

// barnes_hut.cu -- Barnes-Hut minibatch layout (algo 4) on the device.
//
// Reference: sample/algorithms.cpp:1038-1072 (iteration), sample/MortonCode.h
// (frame, quantisation, order), sample/BarnesHut.h:114-225 (sort, quadtree
// build, opening test, unit-vector repulsion).
//
// Per iteration:
//   1. bbox of the positions; Morton frame {minX, minY, MAXMIN} and 64-bit keys
//      (y-major interleave of the two 32-bit quantised coordinates, quantised
//      in FP64 exactly as the reference: (uint32)(4294967295.0*(x-minX)/MAXMIN)).
//   2. stable LSD radix sort of (key, vertex) pairs on the high 32 bits (4
//      passes of 8 bits), then each run of equal high halves sorted on its
//      own (they are rare).
//   3. binary radix tree over the sorted keys (Karras 2012), then a bottom-up
//      pass that merges the x-bit level into the y-bit level of the same
//      digit, giving exactly the reference quadtree without its single-child
//      chain nodes; centroids are the unweighted means of the children summed
//      in quadrant order, in FP64, bit-identical to the reference, computed
//      bottom-up by the last-arriving child of every node (no barriers).
//   4. pre-order layout with skip links: 16-byte records {x, y, D^2, skip}
//      walked without a stack.
//   5. repulsion of every vertex in Morton order (coherent warps).  A vertex
//      is only moved by its own batch, so its query position and the tree
//      snapshot are both the iteration-start positions: all n traversals are
//      independent.  The opening test D/dist < theta is evaluated in FP32 and
//      re-evaluated in FP64 when the FP32 margin is within its error bound,
//      so every decision equals the reference's FP64 decision.
//   6. attraction + update.  Vertex i reads the new position of a neighbour j
//      from an earlier batch and the iteration-start position otherwise, so
//      the batch order only constrains i after its earlier-batch neighbours:
//      vertices are grouped into dependency levels (computed once per graph
//      and batch size) and each level is one parallel launch.  This produces
//      the same values as the reference's sequential batch loop.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>

#include "bh_device.cuh"

namespace bl {
namespace {

constexpr int kQuadLevels = 33;  // quad levels 0..31, 32 for runs of identical keys


// ---- stable LSD radix sort, 8-bit digits ------------------------------------
//
// Each digit pass is three kernels without any inter-block waiting: the tile
// digit counts (hist[d * ntiles + tile]), one block that turns every digit
// row into exclusive offsets across tiles and scans the digit totals, and the
// scatter, which ranks its tile's keys stably and writes them to
// digit offset + row offset + rank.  Tiles are 2,048 keys (one wave of four
// 256-thread blocks per SM for a million keys; 1,024-key tiles took 1.3
// waves and 6 % longer); warp w of a block owns keys [w*256, (w+1)*256) of
// its tile and ranks them with warp-private counters, so no block barrier
// sits inside the ranking loop.
constexpr int kRsThreads = 256;
constexpr int kRsItems = 8;
constexpr int kRsTile = kRsThreads * kRsItems;
constexpr int kRsWarps = kRsThreads / 32;

__global__ void __launch_bounds__(kRsThreads) rs_count_kernel(const u64 *__restrict__ keys, int n, int shift,
                                                              int ntiles, unsigned int *hist) {
  __shared__ unsigned int cnt[kRsWarps][256];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
#pragma unroll
  for (int w = 0; w < kRsWarps; w++) cnt[w][tid] = 0;
  __syncthreads();
  const int wbase = blockIdx.x * kRsTile + warp * (kRsItems * 32);
#pragma unroll 4
  for (int r = 0; r < kRsItems; r++) {
    const int idx = wbase + r * 32 + lane;
    if (idx < n) atomicAdd(&cnt[warp][(unsigned int)(keys[idx] >> shift) & 255u], 1u);
  }
  __syncthreads();
  unsigned int tot = 0;
#pragma unroll
  for (int w = 0; w < kRsWarps; w++) tot += cnt[w][tid];
  hist[(size_t)tid * ntiles + blockIdx.x] = tot;
}

// Block d turns digit row d (ntiles contiguous counts) into exclusive
// offsets across tiles, 256 tiles at a time, and stores the row total.
__global__ void __launch_bounds__(256) rs_rowscan_kernel(unsigned int *hist, int ntiles,
                                                         unsigned int *row_total) {
  __shared__ unsigned int ws[8];
  __shared__ unsigned int carry;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  unsigned int *row = hist + (size_t)blockIdx.x * ntiles;
  if (tid == 0) carry = 0;
  __syncthreads();
  for (int c0 = 0; c0 < ntiles; c0 += 256) {
    const int b = c0 + tid;
    const unsigned int v = (b < ntiles) ? row[b] : 0u;
    unsigned int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    unsigned int wpre = 0, total = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const unsigned int t = ws[k];
      if (k < w) wpre += t;
      total += t;
    }
    const unsigned int base = carry;
    if (b < ntiles) row[b] = base + wpre + x - v;
    __syncthreads();
    if (tid == 0) carry = base + total;
    __syncthreads();
  }
  if (tid == 0) row_total[blockIdx.x] = carry;
}

// Exclusive scan of one value per thread over a 256-thread block (ws: 8
// words of shared scratch); every thread calls it.
__device__ __forceinline__ unsigned int rs_block_scan256(unsigned int v, unsigned int *ws) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  unsigned int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[warp] = x;
  __syncthreads();
  unsigned int wpre = 0;
#pragma unroll
  for (int k = 0; k < kRsWarps; k++)
    if (k < warp) wpre += ws[k];
  __syncthreads();
  return wpre + x - v;
}

// The tile's keys are ranked (stably: warp order, then lane order within a
// warp's 32-key rows), placed in shared memory grouped by digit, and written
// out from there: consecutive threads write consecutive keys of a digit's
// run, so each run of the tile reaches L2 as whole sectors rather than as one
// partial sector per key.
__global__ void __launch_bounds__(kRsThreads) rs_scatter_kernel(
    const u64 *__restrict__ kin, const int *__restrict__ vin, u64 *__restrict__ kout, int *__restrict__ vout,
    int n, int shift, int ntiles, const unsigned int *__restrict__ hist, const unsigned int *__restrict__ row_total) {
  __shared__ unsigned int s_cnt[kRsWarps][256];  // per-warp counts, then per-warp offsets within the digit
  __shared__ unsigned int s_base[256];            // global position of the tile's first key of each digit
  __shared__ unsigned int s_loc[256];             // position of the tile's first key of each digit in the tile
  __shared__ unsigned int s_ws[kRsWarps];
  __shared__ u64 s_key[kRsTile];
  __shared__ int s_val[kRsTile];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
#pragma unroll
  for (int w = 0; w < kRsWarps; w++) s_cnt[w][tid] = 0;
  // digit offset = exclusive scan of the 256 row totals (every block does it)
  s_base[tid] = rs_block_scan256(row_total[tid], s_ws) + hist[(size_t)tid * ntiles + blockIdx.x];
  const int wbase = blockIdx.x * kRsTile + warp * (kRsItems * 32);
  const unsigned int lt = (1u << lane) - 1u;
  u64 key[kRsItems];
  int val[kRsItems];
  unsigned int rd[kRsItems];  // rank within the warp's keys (low 16 bits) | digit << 16, digit 256 = none
#pragma unroll
  for (int r = 0; r < kRsItems; r++) {
    const int idx = wbase + r * 32 + lane;
    const bool valid = idx < n;
    key[r] = valid ? kin[idx] : 0ull;
    val[r] = valid ? vin[idx] : 0;
    const unsigned int d = valid ? ((unsigned int)(key[r] >> shift) & 255u) : 256u;
    const unsigned int peers = __match_any_sync(0xffffffffu, d);
    const unsigned int leader = __ffs(peers) - 1;
    unsigned int old = 0;
    if (d < 256u) old = s_cnt[warp][d];
    __syncwarp();
    if (d < 256u && lane == leader) s_cnt[warp][d] = old + __popc(peers);
    __syncwarp();
    rd[r] = (old + __popc(peers & lt)) | (d << 16);
  }
  __syncthreads();
  unsigned int run = 0;
#pragma unroll
  for (int w = 0; w < kRsWarps; w++) {
    const unsigned int c = s_cnt[w][tid];
    s_cnt[w][tid] = run;
    run += c;
  }
  s_loc[tid] = rs_block_scan256(run, s_ws);  // its barriers also publish s_cnt
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kRsItems; r++) {
    const unsigned int d = rd[r] >> 16;
    if (d < 256u) {
      const unsigned int p = s_loc[d] + s_cnt[warp][d] + (rd[r] & 0xffffu);
      s_key[p] = key[r];
      s_val[p] = val[r];
    }
  }
  __syncthreads();
  const int cnt = min(kRsTile, n - (int)blockIdx.x * kRsTile);
  for (int p = tid; p < cnt; p += kRsThreads) {
    const u64 k = s_key[p];
    const unsigned int d = (unsigned int)(k >> shift) & 255u;
    const unsigned int g = s_base[d] + ((unsigned int)p - s_loc[d]);
    if (g < (unsigned int)n) {
      kout[g] = k;
      vout[g] = s_val[p];
    }
  }
}

// ---- frame and keys: one cooperative launch ---------------------------------
//
// Bounding box of the positions (MortonCode.h:42-58), the FP64 frame
// {minX, minY, MAXMIN, 1/MAXMIN} and the 64-bit Morton key of every point,
// together with the tile digit counts of the first sort pass (bits
// shift..shift+7), so that pass starts at its row scan.  Block b handles
// sort tiles b, b + grid, ...; one grid barrier separates the box from the
// keys.  box[0..3] = {min x, ~max x, min y, ~max y} in the order-preserving
// integer form of the floats and box[4] the arrivals, all reset to
// 0xffffffff before the launch: every slot only decreases.
__global__ void __launch_bounds__(kRsThreads, 8) frame_keys_kernel(const float2 *__restrict__ pos, int n, int ntiles,
                                                                unsigned int *box, double *frame, u64 *keys,
                                                                int *vals, int shift, unsigned int *hist,
                                                                double inv_theta2, float *ztab, DevStatus *st) {
  __shared__ unsigned int s_box[kRsWarps][4];
  __shared__ unsigned int cnt[kRsWarps][256];
  __shared__ double s_frame[4];
  __shared__ unsigned int s_ok;
  if (!block_status_ok(st)) return;  // every block sees the same value: no barrier is left waiting
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  unsigned int mnx = 0xffffffffu, mxx = 0u, mny = 0xffffffffu, mxy = 0u;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
#pragma unroll
    for (int r = 0; r < kRsItems; r++) {
      const int idx = tile * kRsTile + r * kRsThreads + tid;
      if (idx < n) {
        const float2 p = pos[idx];
        const unsigned int ux = f2ord(p.x), uy = f2ord(p.y);
        mnx = min(mnx, ux); mxx = max(mxx, ux);
        mny = min(mny, uy); mxy = max(mxy, uy);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    mnx = min(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
    mxx = max(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
    mny = min(mny, __shfl_xor_sync(0xffffffffu, mny, o));
    mxy = max(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
  }
  if (lane == 0) {
    s_box[warp][0] = mnx;
    s_box[warp][1] = ~mxx;
    s_box[warp][2] = mny;
    s_box[warp][3] = ~mxy;
  }
  __syncthreads();
  if (tid < 4) {
    unsigned int v = 0xffffffffu;
#pragma unroll
    for (int w = 0; w < kRsWarps; w++) v = min(v, s_box[w][tid]);
    atomicMin(&box[tid], v);
  }
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    atomicSub(&box[4], 1u);
    const unsigned int target = 0xffffffffu - gridDim.x;  // every block arrived
    const unsigned long long t0 = dev_globaltimer();
    unsigned int ok = 1, polls = 0;
    while (ld_acquire_gpu(&box[4]) > target) {
      if ((++polls & 127u) == 0u && dev_globaltimer() - t0 > kBarrierTimeoutNs) {
        dev_record_error(st, DEV_TIMEOUT_GRID_BARRIER);
        ok = 0;
        break;
      }
    }
    if (ok) {
      unsigned int bb[4];
      bb[0] = ld_volatile_u32(&box[0]);
      bb[1] = ~ld_volatile_u32(&box[1]);
      bb[2] = ld_volatile_u32(&box[2]);
      bb[3] = ~ld_volatile_u32(&box[3]);
      double minX, minY, maxmin;
      frame_from_bbox(bb, minX, minY, maxmin);
      s_frame[0] = minX;
      s_frame[1] = minY;
      s_frame[2] = maxmin;
      s_frame[3] = (maxmin > 0.0) ? 1.0 / maxmin : 0.0;
      if (blockIdx.x == 0) {
        for (int k = 0; k < 4; k++) frame[k] = s_frame[k];
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  if (!s_ok) return;
  const double minX = s_frame[0], minY = s_frame[1], maxmin = s_frame[2], inv = s_frame[3];
  // the records' z by quad level: D^2 / theta^2 with D = MAXMIN / 2^level
  if (blockIdx.x == 0 && tid < kQuadLevels) ztab[tid] = bh_record_z(ldexp(maxmin, -tid), inv_theta2);
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
#pragma unroll
    for (int w = 0; w < kRsWarps; w++) cnt[w][tid] = 0;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRsItems; r++) {
      const int idx = tile * kRsTile + r * kRsThreads + tid;
      if (idx < n) {
        const u64 key = morton_key(pos[idx], minX, minY, maxmin, inv);
        keys[idx] = key;
        vals[idx] = idx;
        atomicAdd(&cnt[warp][(unsigned int)(key >> shift) & 255u], 1u);
      }
    }
    __syncthreads();
    unsigned int tot = 0;
#pragma unroll
    for (int w = 0; w < kRsWarps; w++) tot += cnt[w][tid];
    hist[(size_t)tid * ntiles + tile] = tot;
    __syncthreads();
  }
}

// ---- the low 32 bits: only inside runs of equal high halves ---------------------
//
// The four LSD passes on bits 32..63 leave the keys ordered by their high
// halves and, within a run of equal high halves, by vertex id (the passes are
// stable and the keys started in vertex order).  A run means two points in
// the same cell of a 65,536 x 65,536 grid over the frame: rare (a uniform
// million points give ~100 runs of two).  So each run is finished on its own,
// by (key, vertex id): runs of up to 32 keys by one thread (insertion sort),
// longer ones by one block each (bitonic network in shared memory up to
// kRunCap keys, beyond that stable 8-bit LSD passes through global memory).
// The result is the stable order of the full 64-bit keys.
constexpr int kRunShort = 32;
constexpr int kRunCap = 2048;
constexpr int kRunThreads = 512;

__device__ __forceinline__ unsigned int hi32(u64 k) { return (unsigned int)(k >> 32); }

// One thread per position; a run's first position sorts a short run or
// queues a long one (runs[0] = count, then start, length pairs; runs_cap
// exceeds n / (kRunShort + 1), the most long runs there can be).
__global__ void run_fix_kernel(u64 *__restrict__ keys, int *__restrict__ vals, int n, int *runs, int runs_cap,
                               DevStatus *st) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const unsigned int h = hi32(keys[k]);
  if (k > 0 && hi32(keys[k - 1]) == h) return;        // not a run start
  if (k + 1 >= n || hi32(keys[k + 1]) != h) return;   // a run of one
  int len = 2;
  while (k + len < n && hi32(keys[k + len]) == h && len <= kRunShort) len++;  // bounded scan
  if (len <= kRunShort) {
    // insertion sort by (key, vertex id); already in vertex-id order
    for (int a = k + 1; a < k + len; a++) {
      const u64 ka = keys[a];
      const int va = vals[a];
      int b = a - 1;
      while (b >= k && (keys[b] > ka || (keys[b] == ka && vals[b] > va))) {
        keys[b + 1] = keys[b];
        vals[b + 1] = vals[b];
        b--;
      }
      keys[b + 1] = ka;
      vals[b + 1] = va;
    }
    return;
  }
  while (k + len < n && hi32(keys[k + len]) == h) len++;  // the whole run
  const int slot = atomicAdd(&runs[0], 1);
  if (slot < runs_cap) {
    runs[1 + 2 * slot] = k;
    runs[2 + 2 * slot] = len;
  } else {
    dev_record_error(st, DEV_BAD_INDEX);  // cannot happen (see runs_cap)
  }
}

struct RunSmem {
  union {
    struct {
      u64 k[kRunCap];
      int v[kRunCap];
    } b;
    struct {
      unsigned int cnt[kRunThreads / 32][256];
      unsigned int base[256];
      unsigned int carry[256];
      unsigned int tot[256];
    } c;
  } u;
  unsigned int ws[kRunThreads / 32];
};

// Exclusive scan of x over the first 256 threads; all threads call.
__device__ __forceinline__ unsigned int run_scan256(unsigned int x, RunSmem &S) {
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  unsigned int inc = x;
  if (tid < 256) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned int y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    if (lane == 31) S.ws[w] = inc;
  }
  __syncthreads();
  unsigned int pre = 0;
  if (tid < 256)
    for (int q = 0; q < w; q++) pre += S.ws[q];
  __syncthreads();
  return pre + inc - x;
}

// One block per queued run (grid-stride over the queue).
__global__ void __launch_bounds__(kRunThreads) run_sort_kernel(u64 *__restrict__ keys, int *__restrict__ vals,
                                                               u64 *__restrict__ kalt, int *__restrict__ valt,
                                                               const int *runs, int runs_cap) {
  __shared__ RunSmem S;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int count = min(runs[0], runs_cap);
  for (int r = blockIdx.x; r < count; r += gridDim.x) {
    const int start = runs[1 + 2 * r], len = runs[2 + 2 * r];
    if (len <= kRunCap) {
      int m = 2;
      while (m < len) m <<= 1;
      for (int q = tid; q < m; q += kRunThreads) {
        S.u.b.k[q] = q < len ? keys[start + q] : ~0ull;
        S.u.b.v[q] = q < len ? vals[start + q] : INT_MAX;
      }
      __syncthreads();
      for (int size = 2; size <= m; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
          for (int i = tid; i < (m >> 1); i += kRunThreads) {
            const int lo = ((i & ~(stride - 1)) << 1) | (i & (stride - 1));
            const int hi = lo + stride;
            const bool up = (lo & size) == 0;
            const u64 ka = S.u.b.k[lo], kb = S.u.b.k[hi];
            const int va = S.u.b.v[lo], vb = S.u.b.v[hi];
            if ((ka > kb || (ka == kb && va > vb)) == up) {
              S.u.b.k[lo] = kb;
              S.u.b.k[hi] = ka;
              S.u.b.v[lo] = vb;
              S.u.b.v[hi] = va;
            }
          }
          __syncthreads();
        }
      }
      for (int q = tid; q < len; q += kRunThreads) {
        keys[start + q] = S.u.b.k[q];
        vals[start + q] = S.u.b.v[q];
      }
      __syncthreads();
      continue;
    }
    // a long run: four stable 8-bit passes on the low 32 bits through
    // global memory (keys <-> the same range of kalt), chunk by chunk
    const unsigned int lt = (1u << lane) - 1u;
    for (int pass = 0; pass < 4; pass++) {
      const u64 *ks = (pass & 1) ? kalt + start : keys + start;
      const int *vs = (pass & 1) ? valt + start : vals + start;
      u64 *kd = (pass & 1) ? keys + start : kalt + start;
      int *vd = (pass & 1) ? vals + start : valt + start;
      const int shift = 8 * pass;
      if (tid < 256) S.u.c.carry[tid] = 0;
      __syncthreads();
      for (int q = tid; q < len; q += kRunThreads) atomicAdd(&S.u.c.carry[(unsigned int)(ks[q] >> shift) & 255u], 1u);
      __syncthreads();
      const unsigned int pre = run_scan256(tid < 256 ? S.u.c.carry[tid] : 0u, S);
      if (tid < 256) {
        S.u.c.base[tid] = pre;
        S.u.c.carry[tid] = 0;
      }
      __syncthreads();
      for (int c0 = 0; c0 < len; c0 += kRunThreads) {  // one key per thread and chunk
        for (int q = tid; q < (kRunThreads / 32) * 256; q += kRunThreads) (&S.u.c.cnt[0][0])[q] = 0;
        __syncthreads();
        const int q = c0 + tid;
        const bool valid = q < len;
        const u64 key = valid ? ks[q] : 0ull;
        const int val = valid ? vs[q] : 0;
        const unsigned int d = valid ? ((unsigned int)(key >> shift) & 255u) : 256u;
        const unsigned int peers = __match_any_sync(0xffffffffu, d);
        const unsigned int rank = __popc(peers & lt);
        if (d < 256u && lane == __ffs(peers) - 1) S.u.c.cnt[warp][d] = __popc(peers);
        __syncthreads();
        if (tid < 256) {
          unsigned int run = 0;
          for (int w = 0; w < kRunThreads / 32; w++) {
            const unsigned int c = S.u.c.cnt[w][tid];
            S.u.c.cnt[w][tid] = run;
            run += c;
          }
          S.u.c.tot[tid] = run;
        }
        __syncthreads();
        if (d < 256u) {
          const unsigned int p = S.u.c.base[d] + S.u.c.carry[d] + S.u.c.cnt[warp][d] + rank;
          kd[p] = key;
          vd[p] = val;
        }
        __syncthreads();
        if (tid < 256) S.u.c.carry[tid] += S.u.c.tot[tid];
        __syncthreads();
      }
    }
    // four passes end where they started (keys/vals)
  }
}

__global__ void gather_kernel(const float2 *__restrict__ pos, const int *__restrict__ perm, int n,
                              float2 *__restrict__ spos) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) spos[k] = pos[perm[k]];
}

// ---- binary radix tree (Karras 2012) ----------------------------------------
__device__ __forceinline__ int kdelta(const u64 *__restrict__ K, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  const u64 x = K[i] ^ K[j];
  return x ? __clzll((long long)x) : 64 + __clz(i ^ j);
}

// internal node i in [0, n-2]; leaf k encoded as ~k in child links;
// parent[] holds internal parents of internal nodes (index i) and of leaves
// (index n-1+k); the root is internal node 0.
// bnode: the same per internal node packed in 32 bytes for the chain walk,
// ints {first, last, prefix length, parent, left, right, -, -} (the parent
// word is written by the parent's thread).
__global__ void radix_tree_kernel(const u64 *__restrict__ K, int n, int2 *child, int2 *range,
                                  int *dlt, int *parent, int *bnode) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (kdelta(K, n, i, i + 1) - kdelta(K, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = kdelta(K, n, i, i - d);
  int lmax = 2;
  while (kdelta(K, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (kdelta(K, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = kdelta(K, n, i, j);
  int s = 0;
  for (int div = 2;; div <<= 1) {
    const int t = (l + div - 1) / div;
    if (kdelta(K, n, i, i + (s + t) * d) > dnode) s += t;
    if (t <= 1) break;
  }
  const int gamma = i + s * d + min(d, 0);
  const int first = min(i, j), last = max(i, j);
  const int left = (first == gamma) ? ~gamma : gamma;
  const int right = (last == gamma + 1) ? ~(gamma + 1) : gamma + 1;
  child[i] = make_int2(left, right);
  range[i] = make_int2(first, last);
  dlt[i] = dnode;
  parent[left >= 0 ? left : (n - 1 + ~left)] = i;
  parent[right >= 0 ? right : (n - 1 + ~right)] = i;
  if (i == 0) parent[0] = -1;
  int *b = bnode + 8 * (size_t)i;
  b[0] = first;
  b[1] = last;
  b[2] = dnode;
  b[4] = left;
  b[5] = right;
  if (left >= 0) bnode[8 * (size_t)left + 3] = i;
  if (right >= 0) bnode[8 * (size_t)right + 3] = i;
  if (i == 0) b[3] = -1;
}

struct TreeArgs {
  int n;
  const float2 *spos;
  const int2 *range;
  const int *dlt;
  const int *parent;
  int4 *qkids;          // quad children of a quad node, kNoChild-padded
  double2 *qcen;
  int *qbelow;
  int *startcnt;
  int *qpar;     // quad parent of internal node i (index i) and of leaf k (index n-1+k); -1 for the root
  int *qnchild;  // children of a quad node
  // quad nodes whose range spans centroid blocks, by level (0..32):
  // span_cnt[level] (zero before the pass), span_list[level * span_cap + slot]
  int *span_cnt;
  int *span_list;
  int span_cap;
  int *span_pos;  // position of a listed node (span_stage_kernel)
  double2 *stage_val;  // staged listed nodes (span_stage_kernel -> centroid_top_kernel)
  int4 *stage_pend;
  int4 *stage_meta;
  // pre-order records: quad nodes starting before each centroid block
  // (chain_kernel adds them up, block_base_kernel turns them into offsets),
  // startbase[k] = quad nodes starting before sorted position k
  int *blocktot;
  int *startbase;
  // quad nodes that span exactly one block boundary, by boundary b (between
  // blocks b and b+1): their levels (bit mask) and ids (chain_node[b * 33 +
  // level])
  unsigned long long *chain_mask;
  int *chain_node;
  const float *ztab;  // the records' z = D^2 / theta^2 by quad level (frame_keys_kernel)
  float4 *nodes;
  double2 *nodes_c64;
  unsigned char *nodes_lvl;
  const int4 *bnode;  // packed internal nodes, two int4 each (radix_tree_kernel)
  DevStatus *st;
};

constexpr int kNoChild = INT_MIN;
constexpr int kCenSpanC = 1024;  // sorted points per centroid block

__device__ __forceinline__ int quad_level(int p) { return p >= 64 ? 32 : (p >> 1); }


// Structure of the quadtree, one thread per sorted position k.  The binary
// nodes whose range starts at k form the left-child chain above leaf k; the
// chains of different k are disjoint, so each thread owns its nodes and no
// synchronisation is needed.  For every quad node on the chain it records the
// number of quad nodes below it on the chain (qbelow), its quad children, their
// count, and itself as their quad parent; startcnt[k] counts the quad nodes
// starting at k.
__device__ __forceinline__ int chain_walk(const TreeArgs &t, int k);

__global__ void __launch_bounds__(256) chain_kernel(TreeArgs t) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int cnt = k < t.n ? chain_walk(t, k) : 0;
  // quad nodes starting in this warp's 32 positions (one centroid block)
  const int sum = __reduce_add_sync(0xffffffffu, cnt);
  if ((threadIdx.x & 31) == 0 && sum) atomicAdd(&t.blocktot[(k & ~31) / kCenSpanC], sum);
}

__device__ __forceinline__ int chain_walk(const TreeArgs &t, int k) {
  int cnt = 0;
  int cur = t.parent[t.n - 1 + k];
  if (k == 0) t.qpar[0] = -1;  // the root
  const int4 none = make_int4(-1, -1, -1, -1);
  int4 ra = none, rb = none;  // cur's packed record
  if (cur >= 0) {
    ra = __ldg(&t.bnode[2 * cur]);
    rb = __ldg(&t.bnode[2 * cur + 1]);
  }
  // bounded by the tree height: every step moves to a parent.  The parent's
  // record and the children's are loaded together, one round trip a step.
  while (cur >= 0 && ra.x == k) {
    const int par = ra.w;
    int4 pa = none, pb = none;
    if (par >= 0) {
      pa = __ldg(&t.bnode[2 * par]);
      pb = __ldg(&t.bnode[2 * par + 1]);
    }
    const int p = ra.z;
    const int sides[2] = {rb.x, rb.y};
    int4 ca[2] = {none, none}, cb[2] = {none, none};
#pragma unroll
    for (int h = 0; h < 2; h++)
      if (p < 64 && sides[h] >= 0) {
        ca[h] = __ldg(&t.bnode[2 * sides[h]]);
        cb[h] = __ldg(&t.bnode[2 * sides[h] + 1]);
      }
    // cur is merged into its parent's quad node: the x-bit split of the digit
    // whose y-bit split is the parent, or any split inside a run below its top
    const bool sub = cur > 0 && (p >= 64 ? pa.z >= 64 : ((p & 1) && pa.z == p - 1));
    if (!sub) {
      t.qbelow[cur] = cnt++;
      int kids[4] = {kNoChild, kNoChild, kNoChild, kNoChild};
      int m = 0;
      if (p < 64) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int c = sides[h];
          const int pc = ca[h].z;  // the child's prefix length; its parent is cur
          const bool csub = c > 0 && (pc >= 64 ? p >= 64 : ((pc & 1) && p == pc - 1));
          if (c >= 0 && csub) {
            kids[m++] = cb[h].x;
            kids[m++] = cb[h].y;
          } else {
            kids[m++] = c;
          }
        }
        for (int c = 0; c < m; c++) t.qpar[kids[c] >= 0 ? kids[c] : t.n - 1 + ~kids[c]] = cur;
      } else {
        // run of identical keys: every point of the range is a child
        for (int q = ra.x; q <= ra.y; q++) t.qpar[t.n - 1 + q] = cur;
        m = ra.y - ra.x + 1;
      }
      t.qkids[cur] = make_int4(kids[0], kids[1], kids[2], kids[3]);
      t.qnchild[cur] = m;
    } else {
      t.qnchild[cur] = 0;  // merged into its parent: not a quad node
    }
    cur = (cur == 0) ? -1 : par;
    ra = pa;
    rb = pb;
  }
  t.startcnt[k] = cnt;
  return cnt;
}

// Exclusive offsets of the centroid blocks' quad-node counts, in place
// (tot[nb] = the number of quad nodes), and startbase[n] = the same.  One
// block of 1024 threads.
__global__ void __launch_bounds__(1024) block_base_kernel(int *tot, int nb, int *startbase_n) {
  __shared__ int ws[32];
  __shared__ int carry;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  if (tid == 0) carry = 0;
  __syncthreads();
  for (int c0 = 0; c0 < nb; c0 += 1024) {
    const int b = c0 + tid;
    const int v = b < nb ? tot[b] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    int wpre = 0, total = 0;
    for (int q = 0; q < 32; q++) {
      const int u = ws[q];
      if (q < w) wpre += u;
      total += u;
    }
    const int base = carry;
    if (b < nb) tot[b] = base + wpre + x - v;
    __syncthreads();
    if (tid == 0) carry = base + total;
    __syncthreads();
  }
  if (tid == 0) {
    tot[nb] = carry;
    *startbase_n = carry;
  }
}

// Pre-order record of quad node `node` (BarnesHut.h:114-225 as a flat walk):
// the record after the quad nodes starting before position lo = range.x and
// the deeper quad nodes starting at lo; its skip link is the first record
// after its range.  sc_lo = quad nodes starting at lo, sb_lo / sb_hi =
// startbase at lo and at hi = range.y + 1, qb = quad nodes below it starting
// at lo.  False (and DEV_BAD_INDEX) for offsets that cannot be.
__device__ __forceinline__ bool node_record_slot(const TreeArgs &t, int lo, int hi, int qb, int sc_lo, int sb_lo,
                                                 int sb_hi, int &idx, int &skip) {
  const int cap = 2 * t.n - 1;  // records: n leaves + at most n-1 quad nodes
  const int rank = sc_lo - 1 - qb;
  idx = lo + sb_lo + rank;
  skip = hi + sb_hi;
  if (rank < 0 || idx < 0 || idx >= cap || skip <= idx || skip > cap) {
    dev_record_error(t.st, DEV_BAD_INDEX);
    return false;
  }
  return true;
}

// {x, y, D^2 / theta^2, skip} with the FP64 centroid and the level beside it
// (the walk's FP64 re-test reads those two).
__device__ __forceinline__ void write_node_record(const TreeArgs &t, int idx, int skip, int lvl, double2 c) {
  t.nodes[idx] = make_float4(d2f_int(c.x), d2f_int(c.y), t.ztab[lvl], __int_as_float(skip));
  t.nodes_c64[idx] = c;
  t.nodes_lvl[idx] = (unsigned char)lvl;
}

// The same from global memory (startbase of the whole range written).
__device__ __forceinline__ void write_node_record_global(const TreeArgs &t, int node, double2 c) {
  const int2 rg = t.range[node];
  int idx, skip;
  if (node_record_slot(t, rg.x, rg.y + 1, t.qbelow[node], t.startcnt[rg.x], t.startbase[rg.x],
                       t.startbase[rg.y + 1], idx, skip))
    write_node_record(t, idx, skip, quad_level(t.dlt[node]), c);
}

// Centroids bottom-up.  The centroid of a quad node is the unweighted mean of
// its children summed in quadrant order in FP64 (BarnesHut.h:197-217),
// bit-identical to the reference; it can be computed once every child is
// done.  Three passes by how many block boundaries a node's range contains:
// * none — centroid_kernel: a block owns kCenSpan consecutive sorted points;
//   a binary node whose range lies inside them has its index there too (a
//   Karras node's index is one of its range ends), so the block loads those
//   nodes' structure and its points into shared memory with coalesced reads,
//   and processes the nodes in rounds: the nodes whose children are all done
//   form a queue, handled one node per thread so that the FP64 work (a small
//   fraction of the FP32 rate on this part, charged per warp instruction)
//   runs in full warps, and a node's last arriving child appends it to the
//   next round's queue.  The block also lists the spanning nodes whose index
//   it holds.
// * one — boundary_chain_kernel: the nodes containing boundary b and no other
//   are nested, one per level; one warp computes them from the deepest up.
// * more — span_stage_kernel gathers their children over the whole device;
//   centroid_top_kernel, one thread-block cluster, computes them level by
//   level from the deepest, a cluster barrier between levels (a node's
//   children are one level deeper at least).  At one level the quad nodes'
//   ranges are disjoint and each of these contains a block boundary, so a
//   level lists fewer nodes than there are blocks.
// On a uniform 1M-point tree ~5,200 nodes span blocks (15 levels), 341 of
// them (5 levels) more than one boundary.  (A climb by the last arriving child
// through device-scope counters did the spanning nodes before: one serial
// chain of L2 round trips per level, 58 us of the pass.)
constexpr int kCenThreads = 512;
constexpr int kCenSpan = kCenSpanC;

struct CenSmem {
  double2 cen[kCenSpan];
  int4 kids[kCenSpan];
  float2 pts[kCenSpan];
  int dlt[kCenSpan];
  int par[kCenSpan];       // quad parent of the local node at this index
  int leafpar[kCenSpan];   // quad parent of the point at this index
  int arrive[kCenSpan];
  int queue[2][kCenSpan];
  unsigned short need[kCenSpan];  // children of the local quad node here (<= kCenSpan), 0 if none
  int qn[2];
};

// Centroid of quad node `node` from global memory: its children's centroids
// were written by an earlier launch or before the last cluster barrier (read
// through L2).
__device__ double2 quad_centroid_global(const TreeArgs &t, int node) {
  double cx = 0.0, cy = 0.0;
  int cnt = 0;
  if (t.dlt[node] >= 64) {
    const int2 rg = t.range[node];
    for (int q = rg.x; q <= rg.y; q++) {
      const float2 v = t.spos[q];
      cx = cnt ? __dadd_rn(cx, f2d_int(v.x)) : zero_plus(f2d_int(v.x));
      cy = cnt ? __dadd_rn(cy, f2d_int(v.y)) : zero_plus(f2d_int(v.y));
      cnt++;
    }
  } else {
    const int4 kk = t.qkids[node];
    const int kids[4] = {kk.x, kk.y, kk.z, kk.w};
    double vx[4], vy[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {  // the loads first, then the ordered sum
      const int ch = kids[c];
      vx[c] = vy[c] = 0.0;
      if (ch == kNoChild) continue;
      if (ch < 0) {
        const float2 v = t.spos[~ch];
        vx[c] = f2d_int(v.x);
        vy[c] = f2d_int(v.y);
      } else {
        const double2 v = __ldcg(&t.qcen[ch]);
        vx[c] = v.x;
        vy[c] = v.y;
      }
    }
#pragma unroll
    for (int c = 0; c < 4; c++) {
      if (kids[c] == kNoChild) break;
      cx = c ? __dadd_rn(cx, vx[c]) : zero_plus(vx[c]);
      cy = c ? __dadd_rn(cy, vy[c]) : zero_plus(vy[c]);
      cnt++;
    }
  }
  return make_double2(div_count_int(cx, cnt), div_count_int(cy, cnt));
}

// Centroids of the quad nodes that contain boundary b and no other (one
// warp).  They are nested, one per level, each the parent of the
// next deeper one; their other children lie inside block b or b+1 (done) or
// are points.  Lane i takes the i-th deepest node: its structure and its done
// children are loaded in parallel, then the nodes are summed from the deepest
// up, each taking the one below from the lane before it.
__device__ __forceinline__ void chain_centroids(const TreeArgs &t, int b) {
  const int lane = threadIdx.x & 31;
  const unsigned long long mask = __ldcg(&t.chain_mask[b]);
  const int cnt = __popcll(mask);
  if (cnt == 0) return;
  if (cnt > 32) {  // every level: one lane, in order (the others wait at the shuffle-free path)
    if (lane == 0)
      for (int lvl = kQuadLevels - 1; lvl >= 0; lvl--)
        if ((mask >> lvl) & 1ull) {
          const int node = __ldcg(&t.chain_node[b * kQuadLevels + lvl]);
          t.qcen[node] = quad_centroid_global(t, node);
        }
    __syncwarp();
    return;
  }
  // lane i: the level of the (i+1)-th highest set bit
  int lvl = -1;
  {
    int seen = 0;
    for (int l = kQuadLevels - 1; l >= 0; l--)
      if ((mask >> l) & 1ull) {
        if (seen == lane) lvl = l;
        seen++;
      }
  }
  const bool mine = lane < cnt;
  const int node = mine ? __ldcg(&t.chain_node[b * kQuadLevels + lvl]) : -1;
  const int below = __shfl_up_sync(0xffffffffu, node, 1);  // the next deeper chain node
  double2 v[4] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
  int nc = 0, from_below = -1;
  double2 run = make_double2(0.0, 0.0);
  bool is_run = false;
  if (mine) {
    const int p = t.dlt[node];
    if (p >= 64) {  // a run: points only
      is_run = true;
      run = quad_centroid_global(t, node);
    } else {
      const int4 kk = t.qkids[node];
      const int kids[4] = {kk.x, kk.y, kk.z, kk.w};
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const int ch = kids[c];
        if (ch == kNoChild) continue;
        nc = c + 1;
        if (lane > 0 && ch == below) {
          from_below = c;
        } else if (ch < 0) {
          const float2 pt = t.spos[~ch];
          v[c] = make_double2(f2d_int(pt.x), f2d_int(pt.y));
        } else {
          v[c] = __ldcg(&t.qcen[ch]);
        }
      }
    }
  }
  double2 prev = make_double2(0.0, 0.0), mine_c = make_double2(0.0, 0.0);
  for (int i = 0; i < cnt; i++) {
    if (lane == i) {
      if (is_run) {
        mine_c = run;
      } else {
        double cx = 0.0, cy = 0.0;
#pragma unroll
        for (int c = 0; c < 4; c++) {
          if (c >= nc) break;
          const double2 u = c == from_below ? prev : v[c];
          cx = c ? __dadd_rn(cx, u.x) : zero_plus(u.x);
          cy = c ? __dadd_rn(cy, u.y) : zero_plus(u.y);
        }
        mine_c = make_double2(div_count_int(cx, nc), div_count_int(cy, nc));
      }
    }
    prev.x = __shfl_sync(0xffffffffu, mine_c.x, i);
    prev.y = __shfl_sync(0xffffffffu, mine_c.y, i);
  }
  if (mine) t.qcen[node] = mine_c;
}

// One warp per block boundary (boundaries 0 .. nb-2).
constexpr int kChainThreads = 128;
__global__ void __launch_bounds__(kChainThreads) boundary_chain_kernel(TreeArgs t, int nbound) {
  if (!block_status_ok(t.st)) return;
  const int b = blockIdx.x * (kChainThreads / 32) + (threadIdx.x >> 5);
  if (b < nbound) chain_centroids(t, b);
}

__global__ void __launch_bounds__(kCenThreads) centroid_kernel(TreeArgs t) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CenSmem &S = *reinterpret_cast<CenSmem *>(smem_raw);
  if (!block_status_ok(t.st)) return;
  const int tid = threadIdx.x;
  const int lo = blockIdx.x * kCenSpan, hi = min(t.n, lo + kCenSpan);
  // the block's points and local quad nodes, coalesced
  for (int j = lo + tid; j < hi; j += kCenThreads) {
    const int q = j - lo;
    S.pts[q] = t.spos[j];
    S.leafpar[q] = t.qpar[t.n - 1 + j];
    S.arrive[q] = 0;
    int need = 0;
    if (j < t.n - 1) {
      const int m = t.qnchild[j];
      const int2 rg = t.range[j];
      if (m > 0 && rg.x >= lo && rg.y < hi) {
        need = m;
        S.kids[q] = t.qkids[j];
        S.dlt[q] = t.dlt[j];
        S.par[q] = t.qpar[j];
      } else if (m > 0) {  // spans blocks
        const int lvl = quad_level(t.dlt[j]);
        const int bl = rg.x / kCenSpan;
        if (rg.y / kCenSpan == bl + 1) {  // one boundary: boundary_chain_kernel
          t.chain_node[bl * kQuadLevels + lvl] = j;
          atomicOr(&t.chain_mask[bl], 1ull << lvl);
        } else {  // more: centroid_top_kernel
          const int slot = atomicAdd(&t.span_cnt[lvl], 1);
          if (slot < t.span_cap) t.span_list[lvl * t.span_cap + slot] = j;
          else dev_record_error(t.st, DEV_BAD_INDEX);  // cannot happen (see above)
        }
      }
    }
    S.need[q] = (unsigned short)need;
  }
  if (tid < 2) S.qn[tid] = 0;
  __syncthreads();
  auto is_local = [&](int node) { return node >= lo && node < hi && S.need[node - lo] != 0; };
  // round 0: every point arrives at its quad parent
  for (int k = lo + tid; k < hi; k += kCenThreads) {
    const int par = S.leafpar[k - lo];
    if (par < 0 || !is_local(par)) continue;  // a spanning parent is listed by its own block
    if (atomicAdd(&S.arrive[par - lo], 1) == (int)S.need[par - lo] - 1) S.queue[0][atomicAdd(&S.qn[0], 1)] = par;
  }
  __syncthreads();
  // rounds: the ready local nodes, one per thread (bounded by the depth of
  // the block's subtrees: every round moves up one node)
  for (int cur = 0;; cur ^= 1) {
    const int cnt = S.qn[cur];
    if (cnt == 0) break;
    if (tid == 0) S.qn[cur ^ 1] = 0;
    __syncthreads();
    for (int q = tid; q < cnt; q += kCenThreads) {
      const int node = S.queue[cur][q];
      const int ln = node - lo;
      double cx = 0.0, cy = 0.0;
      int nc = 0;
      if (S.dlt[ln] >= 64) {
        // run of identical keys: every point is a child (the reference
        // recurses without end here; see the oracle's note)
        const int2 rg = t.range[node];
        for (int k = rg.x; k <= rg.y; k++) {
          const float2 v = S.pts[k - lo];
          cx = nc ? __dadd_rn(cx, f2d_int(v.x)) : zero_plus(f2d_int(v.x));
          cy = nc ? __dadd_rn(cy, f2d_int(v.y)) : zero_plus(f2d_int(v.y));
          nc++;
        }
      } else {
        const int4 kk = S.kids[ln];
        const int kids[4] = {kk.x, kk.y, kk.z, kk.w};
#pragma unroll
        for (int c = 0; c < 4; c++) {
          const int ch = kids[c];
          if (ch == kNoChild) break;
          double vx, vy;
          if (ch < 0) {  // a point of this block
            const float2 v = S.pts[~ch - lo];
            vx = f2d_int(v.x);
            vy = f2d_int(v.y);
          } else {  // a local node, done in an earlier round
            const double2 v = S.cen[ch - lo];
            vx = v.x;
            vy = v.y;
          }
          cx = c ? __dadd_rn(cx, vx) : zero_plus(vx);
          cy = c ? __dadd_rn(cy, vy) : zero_plus(vy);
          nc++;
        }
      }
      const double2 c2 = make_double2(div_count_int(cx, nc), div_count_int(cy, nc));
      S.cen[ln] = c2;
      t.qcen[node] = c2;
      const int up = S.par[ln];
      if (up < 0 || !is_local(up)) continue;
      if (atomicAdd(&S.arrive[up - lo], 1) == (int)S.need[up - lo] - 1)
        S.queue[cur ^ 1][atomicAdd(&S.qn[cur ^ 1], 1)] = up;
    }
    __syncthreads();
  }
  // startbase over the block (the round queues are free now): the blocks
  // before it plus an exclusive scan of startcnt inside it
  __syncthreads();
  const int span = hi - lo;
  const int q0 = 2 * tid, q1 = 2 * tid + 1;  // kCenSpan == 2 * kCenThreads
  const int c0 = q0 < span ? t.startcnt[lo + q0] : 0, c1 = q1 < span ? t.startcnt[lo + q1] : 0;
  const int bbase = t.blocktot[blockIdx.x];
  int x = c0 + c1;
  const int lane = tid & 31, w = tid >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  int *wsum = S.queue[0];
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  int wpre = 0;
  for (int q = 0; q < w; q++) wpre += wsum[q];
  const int excl = bbase + wpre + x - (c0 + c1);
  if (q0 < span) t.startbase[lo + q0] = excl;
  if (q1 < span) t.startbase[lo + q1] = excl + c0;
}

// Pre-order records of the points and of the quad nodes inside one centroid
// block, one thread per sorted position (the nodes that span blocks are
// written by boundary_chain_kernel and centroid_top_kernel, beside which this
// kernel runs).
__global__ void __launch_bounds__(256) layout_local_kernel(TreeArgs t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (!block_status_ok(t.st)) return;
  const int cap = 2 * t.n - 1;  // records: n leaves + at most n-1 quad nodes
  // every load that depends only on i first, then the range ends' offsets
  const bool leaf = i < t.n, inner = i < t.n - 1;
  const int sb = leaf ? t.startbase[i] : 0, sc = leaf ? t.startcnt[i] : 0;
  const float2 pt = leaf ? t.spos[i] : make_float2(0.f, 0.f);
  const int m = inner ? t.qnchild[i] : 0;
  const int2 rg = inner ? t.range[i] : make_int2(0, 0);
  const int qb = inner ? t.qbelow[i] : 0;
  const int p = inner ? t.dlt[i] : 0;
  const double2 c = inner ? t.qcen[i] : make_double2(0.0, 0.0);
  // a quad node (binary internal node i) inside one block or spanning one
  // boundary; the nodes spanning more are written by centroid_top_kernel
  const bool node = m > 0 && rg.y / kCenSpan - rg.x / kCenSpan <= 1;
  int sc_lo = 0, sb_lo = 0, sb_hi = 0;
  if (node) {
    sc_lo = t.startcnt[rg.x];
    sb_lo = t.startbase[rg.x];
    sb_hi = t.startbase[rg.y + 1];
  }
  if (leaf) {  // leaf (sorted point) i, after the quad nodes starting at i
    const int idx = i + sb + sc;
    if (idx < 0 || idx >= cap) {
      dev_record_error(t.st, DEV_BAD_INDEX);
      return;
    }
    // a leaf's z = -inf is never in doubt: no FP64 centroid or level needed
    t.nodes[idx] = make_float4(pt.x, pt.y, kLeafZ, __int_as_float(idx + 1));
  }
  int idx, skip;
  if (node && node_record_slot(t, rg.x, rg.y + 1, qb, sc_lo, sb_lo, sb_hi, idx, skip))
    write_node_record(t, idx, skip, quad_level(p), c);
}

constexpr int kTopCtas = 8;  // one cluster (the portable maximum size)
constexpr int kTopThreads = 1024;
constexpr int kTopCap = 1024;  // listed nodes per block held in shared memory (104 KB)
constexpr int kStageThreads = 128;

__device__ __forceinline__ void top_cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ unsigned int top_cluster_rank() {
  unsigned int r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// v = the double2 at `p` in the shared memory of block `rank` of the cluster.
__device__ __forceinline__ double2 ld_cluster_double2(const double2 *p, unsigned int rank) {
  const unsigned int a = (unsigned int)__cvta_generic_to_shared(p);
  unsigned int ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
  double x, y;
  asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(x), "=d"(y) : "r"(ra));
  return make_double2(x, y);
}

// Position g of a listed node: level lvl's nodes follow the deeper levels'
// (off[lvl] = the deeper levels' count), node q of a level at g = off + q.
// In the cluster, block g % kTopCtas holds it in slot g / kTopCtas; its staged
// record sits at (g % kTopCtas) * kTopCap + g / kTopCtas.
struct SpanLevels {
  int cnt[kQuadLevels], off[kQuadLevels], total;
};

// Every thread of the block calls it.
__device__ __forceinline__ void span_levels(const TreeArgs &t, SpanLevels &L) {
  if (threadIdx.x < kQuadLevels) L.cnt[threadIdx.x] = max(0, min(t.span_cnt[threadIdx.x], t.span_cap));
  __syncthreads();
  if (threadIdx.x == 0) {
    int o = 0;
    for (int lvl = kQuadLevels - 1; lvl >= 0; lvl--) {
      L.off[lvl] = o;
      o += L.cnt[lvl];
    }
    L.total = o;
  }
  __syncthreads();
}

__device__ __forceinline__ int span_level_of(const SpanLevels &L, int g) {
  int lvl = 0;
  while (lvl < kQuadLevels - 1 && g < L.off[lvl]) lvl++;
  return lvl;
}

// Staging of the listed nodes, one thread each, over the whole device (the
// gathers of a node's children are scattered loads; on the cluster's few SMs
// alone they queue): the node's position, its record's place, and per child
// its centroid when it is final (a point, or a node within one block or
// spanning one boundary) or its node id when it is a listed node itself.  A run of identical keys (children: points only) is
// computed here.  Nothing is staged when the cluster cannot hold the nodes.
__global__ void __launch_bounds__(kStageThreads) span_stage_kernel(TreeArgs t) {
  __shared__ SpanLevels L;
  if (!block_status_ok(t.st)) return;
  span_levels(t, L);
  const int total = L.total;
  const int g = blockIdx.x * kStageThreads + threadIdx.x;
  if (total > kTopCtas * kTopCap || g >= total) return;
  const int lvl = span_level_of(L, g);
  const int idx = (g % kTopCtas) * kTopCap + g / kTopCtas;
  const int node = t.span_list[lvl * t.span_cap + (g - L.off[lvl])];
  if (node < 0 || node >= t.n - 1) {
    dev_record_error(t.st, DEV_BAD_INDEX);
    t.stage_meta[idx] = make_int4(-1, 0, -1, 0);
    t.stage_pend[idx] = make_int4(-1, -1, -1, -1);
    t.stage_val[idx] = make_double2(0.0, 0.0);
    return;
  }
  t.span_pos[node] = g;
  const int p = t.dlt[node];
  const int4 kk = t.qkids[node];
  const int2 nr = t.range[node];
  const int qb = t.qbelow[node];
  // its record's place (startbase of the whole range was written by centroid_kernel)
  int ridx, skip;
  if (!node_record_slot(t, nr.x, nr.y + 1, qb, t.startcnt[nr.x], t.startbase[nr.x], t.startbase[nr.y + 1], ridx,
                        skip))
    ridx = -1;
  const int lvl8 = quad_level(p) << 8;
  if (p >= 64) {  // a run
    t.stage_val[idx] = quad_centroid_global(t, node);
    t.stage_meta[idx] = make_int4(node, lvl8, ridx, skip);
    t.stage_pend[idx] = make_int4(-1, -1, -1, -1);
    return;
  }
  const int kids[4] = {kk.x, kk.y, kk.z, kk.w};
  int2 rg[4];
  double2 qc[4];
  float2 pt[4];
#pragma unroll
  for (int c = 0; c < 4; c++) {  // independent loads issued together
    const int ch = kids[c];
    rg[c] = make_int2(0, 0);
    qc[c] = make_double2(0.0, 0.0);
    pt[c] = make_float2(0.f, 0.f);
    if (ch == kNoChild) continue;
    if (ch < 0) {
      pt[c] = t.spos[~ch];
    } else {
      rg[c] = t.range[ch];
      qc[c] = __ldcg(&t.qcen[ch]);  // used only when the child is done (at most one boundary)
    }
  }
  int pend[4] = {-1, -1, -1, -1};
  int nc = 0;
#pragma unroll
  for (int c = 0; c < 4; c++) {
    const int ch = kids[c];
    if (ch == kNoChild) break;
    nc++;
    double2 v = make_double2(0.0, 0.0);
    if (ch < 0) v = make_double2(f2d_int(pt[c].x), f2d_int(pt[c].y));
    else if (rg[c].y / kCenSpan - rg[c].x / kCenSpan >= 2) pend[c] = ch;  // listed
    else v = qc[c];
    t.stage_val[(size_t)c * kTopCtas * kTopCap + idx] = v;
  }
  t.stage_pend[idx] = make_int4(pend[0], pend[1], pend[2], pend[3]);
  t.stage_meta[idx] = make_int4(node, nc | lvl8, ridx, skip);
}

struct TopSmem {
  double2 val[4][kTopCap];  // the children's centroids in quadrant order
  double2 cen[kTopCap];     // the node's centroid (read by the other blocks)
  int4 pend[kTopCap];       // cluster position of a listed child, -1 otherwise
  int node[kTopCap];
  int nc[kTopCap];          // children; 0 for a run (done when staged) or a bad entry
};

// The listed nodes, level by level from the deepest, in one cluster: each
// block loads its staged records and the positions of their listed children,
// then one level per round, a listed child read from the shared memory of the
// block holding it, a cluster barrier after every round.  Every thread reads
// the same level counts, so all take the same cluster barriers; every block
// reads the error record before the first barrier and this kernel records
// errors only after it, so all blocks leave together or none.  Each block
// then writes its nodes' centroids and pre-order records.  More listed nodes
// than the blocks can hold: the same rounds through global memory.
__global__ void __cluster_dims__(kTopCtas, 1, 1) __launch_bounds__(kTopThreads, 1)
    centroid_top_kernel(TreeArgs t) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TopSmem &S = *reinterpret_cast<TopSmem *>(smem_raw);
  __shared__ SpanLevels L;
  __shared__ unsigned int s_code;
  const int tid = threadIdx.x;
  if (tid == 0) s_code = ld_volatile_u32(&t.st->code);
  top_cluster_sync();
  if (s_code != 0u) return;  // the tree of this iteration is not valid
  span_levels(t, L);
  const int total = L.total;
  if (total > kTopCtas * kTopCap) {
    for (int lvl = kQuadLevels - 1; lvl >= 0; lvl--) {
      const int cnt = L.cnt[lvl];
      if (cnt == 0) continue;
      for (int q = blockIdx.x * kTopThreads + tid; q < cnt; q += kTopCtas * kTopThreads) {
        const int node = t.span_list[lvl * t.span_cap + q];
        if (node < 0 || node >= t.n - 1) {
          dev_record_error(t.st, DEV_BAD_INDEX);
          continue;
        }
        const double2 c = quad_centroid_global(t, node);
        t.qcen[node] = c;  // read by the next levels
        write_node_record_global(t, node, c);
      }
      top_cluster_sync();
    }
    return;
  }
  const int crank = (int)top_cluster_rank();
  const int nslots = total > crank ? (total - crank + kTopCtas - 1) / kTopCtas : 0;
  for (int l = tid; l < nslots; l += kTopThreads) {
    const int idx = crank * kTopCap + l;
    const int4 meta = t.stage_meta[idx];
    const int4 pk = t.stage_pend[idx];
    int pend[4] = {pk.x, pk.y, pk.z, pk.w};
    int gc[4];
#pragma unroll
    for (int c = 0; c < 4; c++) gc[c] = pend[c] >= 0 ? __ldcg(&t.span_pos[pend[c]]) : -1;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      if (pend[c] >= 0 && (gc[c] < 0 || gc[c] >= total)) {
        dev_record_error(t.st, DEV_BAD_INDEX);
        gc[c] = -1;
      }
      S.val[c][l] = t.stage_val[(size_t)c * kTopCtas * kTopCap + idx];
    }
    S.pend[l] = make_int4(gc[0], gc[1], gc[2], gc[3]);
    S.node[l] = meta.x;
    S.nc[l] = meta.y & 255;
    if ((meta.y & 255) == 0) S.cen[l] = S.val[0][l];  // a run (or a bad entry: zero)
  }
  top_cluster_sync();  // every block's staged records (and runs) in place
  // this thread's positions of level lvl: g = first + k * kTopCtas * kTopThreads
  auto first_of = [&](int lvl) {
    const int off = L.off[lvl];
    return off + (crank - off % kTopCtas + kTopCtas) % kTopCtas + kTopCtas * tid;
  };
  // the rounds (runs, level 32, were done when staged)
  for (int lvl = kQuadLevels - 2; lvl >= 0; lvl--) {
    if (L.cnt[lvl] == 0) continue;
    const int end = L.off[lvl] + L.cnt[lvl];
    for (int g = first_of(lvl); g < end; g += kTopCtas * kTopThreads) {
      const int l = g / kTopCtas;
      const int nc = S.nc[l];
      if (nc == 0) continue;
      const int4 pk = S.pend[l];
      const int pend[4] = {pk.x, pk.y, pk.z, pk.w};
      double2 v[4];
#pragma unroll
      for (int c = 0; c < 4; c++) {
        v[c] = S.val[c][l];
        if (c < nc && pend[c] >= 0) v[c] = ld_cluster_double2(&S.cen[pend[c] / kTopCtas], pend[c] % kTopCtas);
      }
      double cx = 0.0, cy = 0.0;
#pragma unroll
      for (int c = 0; c < 4; c++) {
        if (c >= nc) break;
        cx = c ? __dadd_rn(cx, v[c].x) : zero_plus(v[c].x);
        cy = c ? __dadd_rn(cy, v[c].y) : zero_plus(v[c].y);
      }
      S.cen[l] = make_double2(div_count_int(cx, nc), div_count_int(cy, nc));
    }
    // no global store is pending here, so the barrier's release has only
    // this round's shared-memory stores to order; it also keeps every
    // block's shared memory alive while the others read it
    top_cluster_sync();
  }
  for (int l = tid; l < nslots; l += kTopThreads) {
    const int4 meta = t.stage_meta[crank * kTopCap + l];
    if (meta.x < 0) continue;
    t.qcen[meta.x] = S.cen[l];  // every quad node's centroid stays readable by node id
    if (meta.z >= 0) write_node_record(t, meta.z, meta.w, meta.y >> 8, S.cen[l]);
  }
}

struct TraverseArgs {
  int n;
  DevStatus *st;
  const float4 *nodes;
  const double2 *nodes_c64;
  const unsigned char *nodes_lvl;
  const double *frame;
  const float2 *spos;
  const int *perm;
  float2 *rep;
  double theta;
  unsigned long long *stats;  // [visits, fp64 decisions] or null
  // the attraction of the neighbours that have not moved yet in this
  // iteration (unmoved_attraction_kernel); the walk adds minus the
  // repulsion; null to skip
  float4 *f0;
};

// FR attraction (algorithms.cpp:1056-1058) of the neighbours of v that have
// not moved before v in the iteration (same or later batch), float-float, by
// vertex id.  It needs no tree, so it runs on the second stream beside the
// tree's spanning passes; the walk then adds minus the repulsion.
__global__ void __launch_bounds__(256) unmoved_attraction_kernel(int n, const int *__restrict__ rowptr,
                                                                 const int *__restrict__ colids,
                                                                 const float2 *pold, int batch, float W,
                                                                 float4 *f0) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n) f0[v] = bh_unmoved_attraction(v, rowptr, colids, pold, batch, W);
}


// 128 threads per block: measured 1.5 % faster than 256 and 512 on the 1M
// graph (finer blocks, smaller tail); 64 is no better.
constexpr int kTravThreads = 128;

template <bool kStats>
__global__ void __launch_bounds__(kTravThreads) traverse_kernel(TraverseArgs a) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (!block_status_ok(a.st)) return;  // the tree of this iteration is not valid
  if (k >= a.n) return;
  const float2 q = a.spos[k];
  // record 0 is the root; its skip link is the number of records
  int total = __float_as_int(__ldg(&a.nodes[0]).w);
  if (total < 0 || total > 2 * a.n - 1) {
    dev_record_error(a.st, DEV_BAD_INDEX);
    total = 0;
  }
  unsigned int visits = 0, exact = 0;
  const float2 rep = bh_repulsion<true, kStats>(a.nodes, a.nodes_c64, a.nodes_lvl, a.frame[2], a.theta,
                                                total, q, visits, exact);
  const int v = a.perm[k];
  a.rep[v] = rep;
  // minus the repulsion into v's sum of unmoved neighbours' attraction
  if (a.f0) a.f0[v] = bh_minus_repulsion(a.f0[v], rep);
  if (kStats) {  // one atomic per group of converged lanes, not per thread
    const unsigned int m = __activemask();
    const unsigned int sv = __reduce_add_sync(m, visits), se = __reduce_add_sync(m, exact);
    if ((threadIdx.x & 31u) == (unsigned int)(__ffs(m) - 1)) {
      atomicAdd(&a.stats[0], (unsigned long long)sv);
      if (se) atomicAdd(&a.stats[1], (unsigned long long)se);
    }
  }
}

struct SweepArgs {
  const int *order;      // vertices grouped by dependency level
  const int *level_off;  // levels + 1 offsets into order
  const int *early_off;  // per level-order slot: earlier-batch neighbours
  const int *early_col;
  int levels;
  const float4 *f0;      // attraction of unmoved neighbours minus repulsion (float-float)
  float4 *f0out;         // the same array: the final float-float force when write_out
  const float2 *pold;
  float2 *pnew;          // every entry kUnmoved before the launch
  int write_out;
  float W;
  float step;
  DevStatus *st;
};

constexpr int kSweepThreads = 1024;

// A new position not yet written: both coordinates NaN, all bits set
// (no layout coordinate is NaN).  pnew is filled with it before the sweep.
constexpr unsigned long long kUnmoved = 0xffffffffffffffffull;

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const float2 *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed_u64(float2 *p, float2 v) {
  const unsigned long long b =
      (unsigned long long)__float_as_uint(v.x) | ((unsigned long long)__float_as_uint(v.y) << 32);
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(b) : "memory");
}

__device__ __forceinline__ float2 unpack_pos(unsigned long long b) {
  return make_float2(__uint_as_float((unsigned int)b), __uint_as_float((unsigned int)(b >> 32)));
}

// The new position of neighbour c, which an earlier dependency level writes:
// the 8-byte word is the position and its own ready flag (a single-copy
// atomic 64-bit access), so one load both tests and reads it.  The wait is
// bounded; false when it ran out or another thread recorded an error.
__device__ __forceinline__ bool wait_moved(const SweepArgs &a, int c, unsigned long long &b) {
  if (b != kUnmoved) return true;
  const unsigned long long t0 = dev_globaltimer();
  for (unsigned int polls = 1;; polls++) {
    __nanosleep(100);  // fewer polls queued at L2 while the writer works
    b = ld_relaxed_u64(&a.pnew[c]);
    if (b != kUnmoved) return true;
    if ((polls & 63u) == 0u) {
      if (ld_volatile_u32(&a.st->code) != 0u) return false;
      if (dev_globaltimer() - t0 > kBarrierTimeoutNs) {
        dev_record_error(a.st, DEV_TIMEOUT_SWEEP);
        return false;
      }
    }
  }
}

// A vertex's data that does not change during the sweep: its slot in the
// level order, id, iteration-start position, f0, earlier-batch neighbour
// range and the first four of those neighbours (most vertices have no more).
struct SweepVertex {
  int t, i;
  float2 pi;
  float4 f;
  int e0, e1;
  int c[4];
};

__device__ __forceinline__ void sweep_load(const SweepArgs &a, int t, SweepVertex &v) {
  v.t = t;
  v.i = a.order[t];
  v.pi = a.pold[v.i];
  v.f = a.f0[v.i];
  v.e0 = a.early_off[t];
  v.e1 = a.early_off[t + 1];
#pragma unroll
  for (int q = 0; q < 4; q++) v.c[q] = (v.e0 + q < v.e1) ? a.early_col[v.e0 + q] : 0;
}

// Adds the attraction of the neighbours that moved earlier in this iteration
// (earlier batches, their new positions, each waited for) to f0, then the
// unit-step update (algorithms.cpp:1056-1066).  FP32 terms, float-float sum,
// FP32 unit vector.  False when a wait gave up.
__device__ __forceinline__ bool sweep_vertex(const SweepArgs &a, const SweepVertex &v) {
  float hx = v.f.x, hy = v.f.y, lx = v.f.z, ly = v.f.w;
  const int m = min(v.e1 - v.e0, 4);
  // the loads of the first (up to) four moved neighbours are issued
  // together; the terms are added in neighbour order
  unsigned long long b[4];
#pragma unroll
  for (int q = 0; q < 4; q++) b[q] = (q < m) ? ld_relaxed_u64(&a.pnew[v.c[q]]) : 0ull;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    if (q < m) {
      if (!wait_moved(a, v.c[q], b[q])) return false;
      bh_attract(unpack_pos(b[q]), v.pi, a.W, hx, lx, hy, ly);
    }
  }
  // more than four (rare): one at a time
  for (int e = v.e0 + 4; e < v.e1; e++) {
    const int c = a.early_col[e];
    unsigned long long bb = ld_relaxed_u64(&a.pnew[c]);
    if (!wait_moved(a, c, bb)) return false;
    bh_attract(unpack_pos(bb), v.pi, a.W, hx, lx, hy, ly);
  }
  const float2 np = bh_step(v.pi, hx, lx, hy, ly, a.step);
  // the force's float-float sums replace f0 (read above, not needed again);
  // bh_forces_kernel turns them into the FP64 force and |f|^2 in full warps
  if (a.write_out) a.f0out[v.i] = make_float4(hx, hy, lx, ly);
  st_relaxed_u64(&a.pnew[v.i], np);  // publishes the position: later levels wait for this word
  return true;
}

// All dependency levels of an iteration in one launch, without barriers: a
// vertex waits only for the new positions of its own earlier-batch
// neighbours (bounded waits on their position words).  The slots of each
// level are cut into 32-slot groups, numbered across the levels in level
// order, and group G goes to warp G mod W (W warps in the grid, numbered so
// that consecutive groups land on different SMs): every warp gets about the
// same number of groups, and takes them in level order.  A warp finishes a
// level (__syncwarp) before it starts the next, so a slot waits only on slots
// of lower levels held by other warps or by this warp's finished groups; with
// every block resident (a cooperative launch) the warp holding the lowest
// unfinished slot can always proceed, so the sweep cannot deadlock.  A thread
// loads its next slot's vertex data before it waits on the current slot's
// neighbours.
__global__ void __launch_bounds__(kSweepThreads, 1) sweep_kernel(SweepArgs a) {
  if (!block_status_ok(a.st)) return;
  const int W = gridDim.x * (blockDim.x >> 5);
  const int lane = threadIdx.x & 31;
  const int w = ((int)threadIdx.x >> 5) * (int)gridDim.x + (int)blockIdx.x;
  // (lv, j): the warp's current group j of level lv; gb: groups of the levels below lv
  int lv = 0, j = 0;
  long long gb = 0;
  auto first_group = [&](int l, long long base) { return (int)((((long long)w - base) % W + W) % W); };
  auto settle = [&](int &l, int &jj, long long &base) {
    while (l < a.levels) {
      const int lo = a.level_off[l], hi = a.level_off[l + 1];
      if (lo + 32 * jj < hi) return;
      base += (hi - lo + 31) / 32;
      l++;
      jj = first_group(l, base);
    }
  };
  j = first_group(0, 0);
  settle(lv, j, gb);
  auto slot = [&](int l, int jj) { return a.level_off[l] + 32 * jj + lane; };
  SweepVertex cur{};
  bool has = lv < a.levels && slot(lv, j) < a.level_off[lv + 1];
  if (has) sweep_load(a, slot(lv, j), cur);
  bool ok = true;
  while (lv < a.levels) {
    int nlv = lv, nj = j + W;
    long long ngb = gb;
    settle(nlv, nj, ngb);
    SweepVertex nxt{};
    const bool nhas = nlv < a.levels && slot(nlv, nj) < a.level_off[nlv + 1];
    if (nhas) sweep_load(a, slot(nlv, nj), nxt);
    if (has && ok) ok = sweep_vertex(a, cur);
    if (nlv != lv) __syncwarp();  // the warp's level is done before its next level starts
    lv = nlv;
    j = nj;
    gb = ngb;
    cur = nxt;
    has = nhas;
  }
}

// The FP64 force f = hi + lo of each vertex (exact conversions, one addition
// per component) and |f|^2, from the float-float sums the sweep left: the
// values the reference's prevCoordinates and energy take, computed in full
// warps by vertex id.
__global__ void bh_forces_kernel(const float4 *__restrict__ ff, int n, double2 *__restrict__ force,
                                 double *__restrict__ e) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 v = ff[i];
  const double fx = __dadd_rn(f2d_int(v.x), f2d_int(v.z)), fy = __dadd_rn(f2d_int(v.y), f2d_int(v.w));
  force[i] = make_double2(fx, fy);
  e[i] = __fma_rn(fx, fx, __dmul_rn(fy, fy));
}

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

int ensure_bh_scratch(bl_ctx *ctx) {
  const size_t n = (size_t)ctx->g.n;
  Scratch &s = ctx->s;
  if (s.bh_n >= n && s.keys) return 0;
  auto fr = [](void *p) { if (p) cudaFree(p); };
  fr(s.keys); fr(s.keys_alt); fr(s.perm); fr(s.perm_alt); fr(s.hist); fr(s.spos);
  fr(s.bparent); fr(s.bchild); fr(s.brange); fr(s.bdelta); fr(s.qkids); fr(s.qpar); fr(s.qnchild);
  fr(s.span); fr(s.span_stage); fr(s.ztab); fr(s.chain); fr(s.qcen);
  fr(s.qbelow); fr(s.startcnt); fr(s.startbase); fr(s.nodes); fr(s.nodes_c64);
  fr(s.nodes_lvl); fr(s.rep); fr(s.f0); fr(s.pos_alt); fr(s.runs); fr(s.bnode);
  const size_t nb = (n + kRsTile - 1) / kRsTile;
  s.hist_entries = 256 * std::max<size_t>(nb, 1) + 256;
  const size_t m = std::max<size_t>(n, 2);
  BL_CUDA(ctx, cudaMalloc(&s.keys, m * 8));
  BL_CUDA(ctx, cudaMalloc(&s.keys_alt, m * 8));
  BL_CUDA(ctx, cudaMalloc(&s.perm, m * 4));
  BL_CUDA(ctx, cudaMalloc(&s.perm_alt, m * 4));
  BL_CUDA(ctx, cudaMalloc(&s.hist, s.hist_entries * 4));
  BL_CUDA(ctx, cudaMalloc(&s.spos, m * sizeof(float2)));
  BL_CUDA(ctx, cudaMalloc(&s.bparent, 2 * m * sizeof(int)));
  BL_CUDA(ctx, cudaMalloc(&s.bchild, m * sizeof(int2)));
  BL_CUDA(ctx, cudaMalloc(&s.brange, m * sizeof(int2)));
  BL_CUDA(ctx, cudaMalloc(&s.bnode, 2 * m * sizeof(int4)));
  BL_CUDA(ctx, cudaMalloc(&s.bdelta, m * sizeof(int)));
  BL_CUDA(ctx, cudaMalloc(&s.qkids, m * sizeof(int4)));
  BL_CUDA(ctx, cudaMalloc(&s.qpar, 2 * m * sizeof(int)));
  BL_CUDA(ctx, cudaMalloc(&s.qnchild, m * sizeof(int)));
  BL_CUDA(ctx, cudaMalloc(&s.ztab, kQuadLevels * sizeof(float)));
  {
    const size_t cap = (size_t)nblk((long long)m, kCenSpan);
    BL_CUDA(ctx, cudaMalloc(&s.chain, cap * (sizeof(unsigned long long) + kQuadLevels * sizeof(int))));
  }
  s.span_cap = nblk((long long)m, kCenSpan);
  BL_CUDA(ctx, cudaMalloc(&s.span, (kQuadLevels + (s.span_cap + 1) + (size_t)kQuadLevels * s.span_cap + m) *
                                        sizeof(int)));
  BL_CUDA(ctx, cudaMalloc(&s.span_stage, (size_t)kTopCtas * kTopCap * (4 * sizeof(double2) + 2 * sizeof(int4))));
  BL_CUDA(ctx, cudaMalloc(&s.qcen, m * sizeof(double2)));
  BL_CUDA(ctx, cudaMalloc(&s.qbelow, m * sizeof(int)));
  BL_CUDA(ctx, cudaMalloc(&s.startcnt, (m + 1) * sizeof(int)));
  BL_CUDA(ctx, cudaMalloc(&s.startbase, (m + 1) * sizeof(int)));
  BL_CUDA(ctx, cudaMalloc(&s.nodes, 2 * m * sizeof(float4)));
  BL_CUDA(ctx, cudaMalloc(&s.nodes_c64, 2 * m * sizeof(double2)));
  BL_CUDA(ctx, cudaMalloc(&s.nodes_lvl, 2 * m));
  BL_CUDA(ctx, cudaMalloc(&s.rep, m * sizeof(float2)));
  BL_CUDA(ctx, cudaMalloc(&s.f0, m * sizeof(float4)));
  BL_CUDA(ctx, cudaMalloc(&s.pos_alt, m * sizeof(float2)));
  s.runs_cap = (int)(m / (kRunShort + 1) + 1);  // runs longer than kRunShort: at most n / (kRunShort + 1)
  BL_CUDA(ctx, cudaMalloc(&s.runs, (2 * (size_t)s.runs_cap + 1) * sizeof(int)));
  int occ = 0;
  BL_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, frame_keys_kernel, kRsThreads, 0));
  if (occ < 1) return bl_fail(ctx, -5, "frame/key kernel cannot be resident");
  s.fk_grid = ctx->num_sms * occ;
  // set here, outside any stream capture of the iteration
  BL_CUDA(ctx, cudaFuncSetAttribute(centroid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)sizeof(CenSmem)));
  BL_CUDA(ctx, cudaFuncSetAttribute(centroid_top_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)sizeof(TopSmem)));
  s.bh_n = n;
  return 0;
}

// Steps 1-4 for the positions `pos`; leaves the pre-order records in
// ctx->s.nodes (total = n + number of quad nodes, read back by callers that
// need it via startbase[n]).
int bh_build(bl_ctx *ctx, const float2 *pos, double theta, int attract_batch) {
  const int n = ctx->g.n;
  Scratch &s = ctx->s;
  cudaStream_t st = ctx->stream;
  if (n < 2) return 0;
  const int nb = nblk(n, kRsTile);
  unsigned long long *kin = s.keys, *kout = s.keys_alt;
  int *vin = s.perm, *vout = s.perm_alt;
  // hist layout: [256 digits x ntiles counts][256 digit-row totals]
  unsigned int *digit_off = s.hist + (size_t)256 * nb;
  bl_time_begin(ctx, "frame_morton");
  // box and barrier slots to 0xffffffff; then the frame, the keys and the
  // digit counts of the first pass (bits 32..39) in one cooperative launch
  BL_CUDA(ctx, cudaMemsetAsync(s.bbox, 0xff, 5 * sizeof(unsigned int), st));
  {
    const int grid = std::min(nb, s.fk_grid);
    int shift = 32;
    int nn = n;
    int ntiles = nb;
    double inv_theta2 = 1.0 / (theta * theta);
    void *args[] = {(void *)&pos, &nn, &ntiles, &s.bbox, &s.frame, &s.keys, &s.perm, &shift, &s.hist,
                    &inv_theta2, &s.ztab, &s.status};
    BL_CUDA(ctx, cudaLaunchCooperativeKernel((const void *)frame_keys_kernel, dim3(grid), dim3(kRsThreads), args, 0,
                                             st));
    ctx->launches++;
  }
  bl_time_end(ctx, "frame_morton");
  // the walk's attraction part (for the iteration that follows) needs no
  // tree: on the second stream (lower priority) beside the single-wave sort
  // passes; before the frame kernel it slowed that cooperative launch
  if (attract_batch > 0) {
    const bool side = ctx->side && ctx->ev_fork && ctx->ev_join;
    if (side) {
      BL_CUDA(ctx, cudaEventRecord(ctx->ev_fork, st));
      BL_CUDA(ctx, cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
    }
    unmoved_attraction_kernel<<<nblk(n, 256), 256, 0, side ? ctx->side : st>>>(
        n, ctx->g.rowptr, ctx->g.colids, pos, attract_batch, (float)ctx->weight, s.f0);
    ctx->launches++;
  }
  bl_time_begin(ctx, "radix_sort");
  bl_time_begin(ctx, "lsd_passes");
  // bits 32..63 by four LSD passes, then the runs of equal high halves
  for (int pass = 4; pass < 8; pass++) {
    if (pass > 4) {  // the first pass's counts come with the keys
      rs_count_kernel<<<nb, kRsThreads, 0, st>>>(kin, n, 8 * pass, nb, s.hist);
      ctx->launches++;
    }
    rs_rowscan_kernel<<<256, 256, 0, st>>>(s.hist, nb, digit_off);
    rs_scatter_kernel<<<nb, kRsThreads, 0, st>>>(kin, vin, kout, vout, n, 8 * pass, nb, s.hist, digit_off);
    std::swap(kin, kout);
    std::swap(vin, vout);
    ctx->launches += 2;
  }
  bl_time_end(ctx, "lsd_passes");
  // 4 passes: the data is back in keys/perm
  BL_CUDA(ctx, cudaMemsetAsync(s.runs, 0, sizeof(int), st));
  run_fix_kernel<<<nblk(n, 256), 256, 0, st>>>(s.keys, s.perm, n, s.runs, s.runs_cap, s.status);
  run_sort_kernel<<<ctx->num_sms, kRunThreads, 0, st>>>(s.keys, s.perm, s.keys_alt, s.perm_alt, s.runs, s.runs_cap);
  ctx->launches += 2;
  bl_time_end(ctx, "radix_sort");
  bl_time_begin(ctx, "gather_tree");
  gather_kernel<<<nblk(n, 256), 256, 0, st>>>(pos, s.perm, n, s.spos);
  radix_tree_kernel<<<nblk(n - 1, 256), 256, 0, st>>>(s.keys, n, s.bchild, s.brange, s.bdelta, s.bparent,
                                                       reinterpret_cast<int *>(s.bnode));
  bl_time_end(ctx, "gather_tree");
  const int ncb = nblk(n, kCenSpan);  // centroid blocks
  // span_cnt, the block totals and the boundary chains' level masks to 0
  BL_CUDA(ctx, cudaMemsetAsync(s.span, 0, (kQuadLevels + ncb + 1) * sizeof(int), st));
  BL_CUDA(ctx, cudaMemsetAsync(s.chain, 0, (size_t)ncb * sizeof(unsigned long long), st));
  TreeArgs t;
  t.n = n;
  t.spos = s.spos;
  t.range = s.brange;
  t.dlt = s.bdelta;
  t.parent = s.bparent;
  t.qkids = s.qkids;
  t.qcen = s.qcen;
  t.qbelow = s.qbelow;
  t.startcnt = s.startcnt;
  t.qpar = s.qpar;
  t.qnchild = s.qnchild;
  t.span_cnt = s.span;
  t.blocktot = s.span + kQuadLevels;
  t.span_list = t.blocktot + s.span_cap + 1;
  t.span_cap = s.span_cap;
  t.span_pos = t.span_list + (size_t)kQuadLevels * s.span_cap;
  t.startbase = s.startbase;
  t.ztab = s.ztab;
  t.chain_mask = reinterpret_cast<unsigned long long *>(s.chain);
  t.chain_node = reinterpret_cast<int *>(t.chain_mask + s.span_cap);
  t.nodes = s.nodes;
  t.nodes_c64 = s.nodes_c64;
  t.nodes_lvl = s.nodes_lvl;
  t.stage_val = reinterpret_cast<double2 *>(s.span_stage);
  t.stage_pend = reinterpret_cast<int4 *>(t.stage_val + 4 * kTopCtas * kTopCap);
  t.stage_meta = reinterpret_cast<int4 *>(t.stage_pend + kTopCtas * kTopCap);
  t.bnode = s.bnode;
  t.st = s.status;
  bl_time_begin(ctx, "chain_kernel");
  chain_kernel<<<nblk(n, 256), 256, 0, st>>>(t);
  block_base_kernel<<<1, 1024, 0, st>>>(t.blocktot, ncb, s.startbase + n);
  ctx->launches++;
  bl_time_end(ctx, "chain_kernel");
  bl_time_begin(ctx, "centroid_kernel");
  centroid_kernel<<<nblk(n, kCenSpan), kCenThreads, sizeof(CenSmem), st>>>(t);
  // the quad nodes spanning one boundary (one warp per boundary); then on the
  // side stream (at the lower priority) the records of the points and of the
  // nodes spanning at most one boundary, beside the nodes spanning more (one
  // cluster, which leaves most SMs free)
  const bool fork = ctx->side && ctx->ev_fork && ctx->ev_join;
  const bool spans = ncb > 1;  // one block has no spanning node
  bl_time_begin(ctx, "centroid_top");
  if (spans) {
    boundary_chain_kernel<<<nblk(ncb - 1, kChainThreads / 32), kChainThreads, 0, st>>>(t, ncb - 1);
    ctx->launches++;
  }
  if (fork) {
    BL_CUDA(ctx, cudaEventRecord(ctx->ev_fork, st));
    BL_CUDA(ctx, cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
  }
  layout_local_kernel<<<nblk(n, 256), 256, 0, fork ? ctx->side : st>>>(t);
  ctx->launches++;
  if (fork) BL_CUDA(ctx, cudaEventRecord(ctx->ev_join, ctx->side));
  if (spans) {
    span_stage_kernel<<<kTopCtas * kTopCap / kStageThreads, kStageThreads, 0, st>>>(t);
    centroid_top_kernel<<<kTopCtas, kTopThreads, sizeof(TopSmem), st>>>(t);
    ctx->launches += 2;
  }
  if (fork) BL_CUDA(ctx, cudaStreamWaitEvent(st, ctx->ev_join, 0));
  bl_time_end(ctx, "centroid_top");
  bl_time_end(ctx, "centroid_kernel");
  ctx->launches += 4;
  BL_CUDA(ctx, cudaGetLastError());
  return 0;
}

int bh_traverse(bl_ctx *ctx, double theta, bool want_stats, int batch) {
  const int n = ctx->g.n;
  Scratch &s = ctx->s;
  if (n < 2) {  // one vertex: no repulsion and no neighbour
    BL_CUDA(ctx, cudaMemsetAsync(s.rep, 0, sizeof(float2) * std::max(n, 1), ctx->stream));
    if (batch > 0) BL_CUDA(ctx, cudaMemsetAsync(s.f0, 0, sizeof(float4) * std::max(n, 1), ctx->stream));
    return 0;
  }
  TraverseArgs a;
  a.n = n;
  a.nodes = s.nodes;
  a.nodes_c64 = s.nodes_c64;
  a.nodes_lvl = s.nodes_lvl;
  a.frame = s.frame;
  a.spos = s.spos;
  a.perm = s.perm;
  a.rep = s.rep;
  a.theta = theta;
  a.stats = want_stats ? s.stats : nullptr;
  a.st = s.status;
  a.f0 = batch > 0 ? s.f0 : nullptr;
  if (want_stats) BL_CUDA(ctx, cudaMemsetAsync(s.stats, 0, 2 * sizeof(unsigned long long), ctx->stream));
  bl_time_begin(ctx, "traverse_kernel");
  if (want_stats) traverse_kernel<true><<<nblk(n, kTravThreads), kTravThreads, 0, ctx->stream>>>(a);
  else traverse_kernel<false><<<nblk(n, kTravThreads), kTravThreads, 0, ctx->stream>>>(a);
  bl_time_end(ctx, "traverse_kernel");
  ctx->launches++;
  BL_CUDA(ctx, cudaGetLastError());
  return 0;
}

int bh_iteration(bl_ctx *ctx, int batch, double theta, double step, bool want_energy,
                 double *energy_out) {
  if (int rc = ensure_bh_scratch(ctx)) return rc;
  const LevelSchedule *ls = level_schedule(ctx, batch);
  if (!ls) return -2;
  float2 *pold = ctx->pos, *pnew = ctx->s.pos_alt;
  if (int rc = bh_build(ctx, pold, theta, batch)) return rc;  // with the unmoved neighbours' attraction
  if (int rc = bh_traverse(ctx, theta, false, batch)) return rc;
  SweepArgs a;
  a.order = ls->order;
  a.level_off = ls->d_offsets;
  a.early_off = ls->early_off;
  a.early_col = ls->early_col;
  a.levels = ls->levels;
  a.f0 = ctx->s.f0;
  a.f0out = ctx->s.f0;
  a.pold = pold;
  a.pnew = pnew;
  a.write_out = want_energy ? 1 : 0;
  a.W = (float)ctx->weight;
  a.step = (float)step;
  a.st = ctx->s.status;
  int occ = 0;
  BL_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, sweep_kernel, kSweepThreads, 0));
  if (occ < 1) return bl_fail(ctx, -5, "sweep kernel cannot be resident");
  const int sweep_grid = ctx->num_sms * std::min(occ, 2);
  // every new position starts as "not written": the sweep's waits read it
  BL_CUDA(ctx, cudaMemsetAsync(pnew, 0xff, (size_t)ctx->g.n * sizeof(float2), ctx->stream));
  void *args[] = {&a};
  bl_time_begin(ctx, "sweep_kernel");
  BL_CUDA(ctx, cudaLaunchCooperativeKernel((const void *)sweep_kernel, dim3(sweep_grid), dim3(kSweepThreads),
                                           args, 0, ctx->stream));
  bl_time_end(ctx, "sweep_kernel");
  ctx->launches++;
  std::swap(ctx->pos, ctx->s.pos_alt);
  if (want_energy) {
    bh_forces_kernel<<<nblk(ctx->g.n, 256), 256, 0, ctx->stream>>>(ctx->s.f0, ctx->g.n, ctx->force, ctx->e);
    ctx->launches++;
    if (int rc = energy_reduce(ctx, energy_out)) return rc;
    // without a destination (a captured iteration) the energy stays in
    // s.energy for the caller to read after the replay
    return energy_out ? bl_check_status(ctx) : 0;
  }
  return 0;
}

// ---- CUDA-graph replay of the iteration ------------------------------------
// One Barnes-Hut iteration without the energy read-back is a fixed sequence
// of about 45 launches and memsets on fixed buffers; only the positions
// alternate between two buffers and STEP changes.  It is captured once per
// parity of the position buffers and replayed, STEP being set on the sweep's
// kernel node before each replay.
// Captured iterations: [variant][parity], variant 1 also writes the forces
// and |f|^2 and reduces the energy into s.energy; parity p reads the
// position buffer that is ctx->pos when (ctx->pos == pos0) == (p == 0).
// Each is captured the first time it is needed.
struct BhGraph {
  int batch = -1;
  double theta = 0.0;
  float2 *pos0 = nullptr;  // ctx->pos of parity 0
  cudaGraph_t graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  cudaGraphExec_t exec[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  cudaGraphNode_t sweep[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  SweepArgs args[2][2];
  cudaKernelNodeParams params[2][2];
  long long kernels[2][2] = {{0, 0}, {0, 0}};
};

void bh_graph_free(BhGraph *g) {
  if (!g) return;
  for (int v = 0; v < 2; v++)
    for (int p = 0; p < 2; p++) {
      if (g->exec[v][p]) cudaGraphExecDestroy(g->exec[v][p]);
      if (g->graph[v][p]) cudaGraphDestroy(g->graph[v][p]);
    }
  delete g;
}

namespace {

// Capture variant v of the iteration that reads ctx->pos (the parity the
// context is at).  Returns 0, or 1 when the iteration cannot be captured
// (nothing has run).
int bh_graph_capture(bl_ctx *ctx, BhGraph &G, int v, int p, int batch, double theta) {
  float2 *save_pos = ctx->pos, *save_alt = ctx->s.pos_alt;
  const std::string save_timed = ctx->timed_kernel;
  const long long save_launches = ctx->launches;
  ctx->timed_kernel.clear();  // no timing events inside the graph
  if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    ctx->timed_kernel = save_timed;
    return 1;
  }
  const int rc = bh_iteration(ctx, batch, theta, 1.0, v == 1, nullptr);
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
  ctx->pos = save_pos;
  ctx->s.pos_alt = save_alt;
  ctx->timed_kernel = save_timed;
  G.kernels[v][p] = ctx->launches - save_launches;
  ctx->launches = save_launches;
  if (rc || e != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return 1;
  }
  size_t count = 0;
  cudaGraphGetNodes(graph, nullptr, &count);
  std::vector<cudaGraphNode_t> nodes(count);
  cudaGraphGetNodes(graph, nodes.data(), &count);
  cudaGraphNode_t sweep = nullptr;
  for (cudaGraphNode_t nd : nodes) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nd, &t) != cudaSuccess || t != cudaGraphNodeTypeKernel) continue;
    cudaKernelNodeParams kp;
    if (cudaGraphKernelNodeGetParams(nd, &kp) != cudaSuccess) continue;
    if (kp.func == (void *)sweep_kernel) {
      sweep = nd;
      G.params[v][p] = kp;
      G.args[v][p] = *static_cast<SweepArgs *>(kp.kernelParams[0]);
    }
  }
  cudaGraphExec_t exec = nullptr;
  if (!sweep || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
    cudaGraphDestroy(graph);
    cudaGetLastError();
    return 1;
  }
  G.graph[v][p] = graph;
  G.exec[v][p] = exec;
  G.sweep[v][p] = sweep;
  return 0;
}

// The context's graphs for (batch, theta), dropped and started afresh when
// they or the position buffers changed.
BhGraph *bh_graph_for(bl_ctx *ctx, int batch, double theta) {
  BhGraph *G = ctx->bh_graph;
  const bool fresh = !G || G->batch != batch || G->theta != theta ||
                     (G->pos0 != ctx->pos && G->pos0 != ctx->s.pos_alt);
  if (fresh) {
    bh_graph_free(G);
    G = ctx->bh_graph = new BhGraph();
    G->batch = batch;
    G->theta = theta;
    G->pos0 = ctx->pos;
  }
  return G;
}

// One replay of variant v with STEP `step`; 1 when it cannot be captured.
int bh_graph_replay(bl_ctx *ctx, BhGraph *G, int v, int batch, double theta, double step) {
  const int p = (ctx->pos == G->pos0) ? 0 : 1;
  if (!G->exec[v][p] && bh_graph_capture(ctx, *G, v, p, batch, theta)) return 1;
  G->args[v][p].step = (float)step;
  void *kargs[] = {&G->args[v][p]};
  cudaKernelNodeParams kp = G->params[v][p];
  kp.kernelParams = kargs;
  BL_CUDA(ctx, cudaGraphExecKernelNodeSetParams(G->exec[v][p], G->sweep[v][p], &kp));
  BL_CUDA(ctx, cudaGraphLaunch(G->exec[v][p], ctx->stream));
  ctx->launches += G->kernels[v][p];
  std::swap(ctx->pos, ctx->s.pos_alt);
  return 0;
}

}  // namespace

// `count` iterations without energy read-back by graph replay, STEP from
// *step (multiplied by 0.999 after each).  Returns 0, an error code, or 1
// when the iteration cannot be captured (nothing has run; launch directly).
int bh_graph_iterations(bl_ctx *ctx, int batch, double theta, double *step, int count) {
  if (count <= 0) return 0;
  if (int rc = ensure_bh_scratch(ctx)) return rc;
  if (!level_schedule(ctx, batch)) return -2;
  BhGraph *G = bh_graph_for(ctx, batch, theta);
  for (int k = 0; k < count; k++) {
    const int r = bh_graph_replay(ctx, G, 0, batch, theta, *step);
    if (r) return k == 0 ? r : -5;  // a parity that cannot be captured after one that could: not expected
    *step *= 0.999;
  }
  return 0;
}

// One iteration with its energy (as bh_iteration with want_energy) by graph
// replay.  Returns 0, an error code, or 1 when it cannot be captured.
int bh_graph_energy_iteration(bl_ctx *ctx, int batch, double theta, double step, double *energy_out) {
  if (int rc = ensure_bh_scratch(ctx)) return rc;
  if (!level_schedule(ctx, batch)) return -2;
  BhGraph *G = bh_graph_for(ctx, batch, theta);
  if (int r = bh_graph_replay(ctx, G, 1, batch, theta, step)) return r;
  // the energy and the device status in one wait
  DevStatus st;
  BL_CUDA(ctx, cudaMemcpyAsync(energy_out, ctx->s.energy, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  BL_CUDA(ctx, cudaMemcpyAsync(&st, ctx->s.status, sizeof(DevStatus), cudaMemcpyDeviceToHost, ctx->stream));
  BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return st.code == 0u ? 0 : bl_check_status(ctx);
}

// `iterations` Barnes-Hut iterations from STEP *step (times 0.999 after
// each); the last one's energy into *energy when it is not null.  In graph
// mode the iterations replay captured graphs (the last one the variant that
// reduces the energy); an iteration that cannot be captured is launched
// directly.
int bh_run(bl_ctx *ctx, int iterations, int batch, double theta, double *step, double *energy) {
  if (batch < 1) return bl_fail(ctx, -1, "batch must be >= 1");  // BL_ERR_ARG
  int it = 0;
  const int replay = energy ? iterations - 1 : iterations;
  if (ctx->graph_mode && replay > 0) {
    const int r = bh_graph_iterations(ctx, batch, theta, step, replay);
    if (r < 0) return r;
    if (r == 0) it = replay;
  }
  for (; it < iterations; it++) {
    const bool last = energy && it == iterations - 1;
    int r = 1;
    if (last && ctx->graph_mode) {
      r = bh_graph_energy_iteration(ctx, batch, theta, *step, energy);
      if (r < 0) return r;
    }
    if (r == 1)
      if (int rc = bh_iteration(ctx, batch, theta, *step, last, last ? energy : nullptr)) return rc;
    *step = *step * 0.999;
  }
  return 0;
}

int bh_canonical_tree(bl_ctx *ctx, int cap, int *lo, int *hi, int *depth, int *nchild,
                      double *centroid) {
  const int n = ctx->g.n;
  if (n < 2) return 0;
  if (int rc = ensure_bh_scratch(ctx)) return rc;
  if (n < 2) return 0;
  if (int rc = bh_build(ctx, ctx->pos, 1.2)) return rc;  // (theta enters only the records)
  // copy the binary tree back and emit quad nodes in pre-order (host walk)
  std::vector<int2> child(n - 1), range(n - 1);
  std::vector<int> dlt(n - 1), parent(2 * n - 1);
  std::vector<double2> qcen(n - 1);
  cudaStream_t st = ctx->stream;
  BL_CUDA(ctx, cudaMemcpyAsync(child.data(), ctx->s.bchild, (n - 1) * sizeof(int2), cudaMemcpyDeviceToHost, st));
  BL_CUDA(ctx, cudaMemcpyAsync(range.data(), ctx->s.brange, (n - 1) * sizeof(int2), cudaMemcpyDeviceToHost, st));
  BL_CUDA(ctx, cudaMemcpyAsync(dlt.data(), ctx->s.bdelta, (n - 1) * sizeof(int), cudaMemcpyDeviceToHost, st));
  BL_CUDA(ctx, cudaMemcpyAsync(parent.data(), ctx->s.bparent, (2 * n - 1) * sizeof(int), cudaMemcpyDeviceToHost, st));
  BL_CUDA(ctx, cudaMemcpyAsync(qcen.data(), ctx->s.qcen, (n - 1) * sizeof(double2), cudaMemcpyDeviceToHost, st));
  BL_CUDA(ctx, cudaStreamSynchronize(st));
  if (int rc = bl_check_status(ctx)) return rc;
  auto sub = [&](int node) {
    if (node <= 0) return false;
    const int p = dlt[node], pp = dlt[parent[node]];
    if (p >= 64) return pp >= 64;
    return (p & 1) && pp == p - 1;
  };
  int count = 0;
  std::vector<int> stack{0};
  while (!stack.empty()) {
    const int v = stack.back();
    stack.pop_back();
    std::vector<int> kids;
    if (dlt[v] >= 64) {
      kids.clear();
    } else {
      const int sides[2] = {child[v].x, child[v].y};
      for (int c : sides) {
        if (c >= 0 && sub(c)) {
          kids.push_back(child[c].x);
          kids.push_back(child[c].y);
        } else {
          kids.push_back(c);
        }
      }
    }
    if (count < cap) {
      lo[count] = range[v].x;
      hi[count] = range[v].y + 1;
      depth[count] = dlt[v] >= 64 ? 32 : dlt[v] / 2;
      nchild[count] = dlt[v] >= 64 ? (range[v].y - range[v].x + 1) : (int)kids.size();
      centroid[2 * count] = qcen[v].x;
      centroid[2 * count + 1] = qcen[v].y;
    }
    count++;
    for (int q = (int)kids.size() - 1; q >= 0; q--)
      if (kids[q] >= 0) stack.push_back(kids[q]);
  }
  return count;
}

// Dependency levels of the attraction sweep for batch size `batch`:
// level(i) = 0 without neighbours in earlier batches, else 1 + the largest
// level among them.  Cached per batch size.
const LevelSchedule *level_schedule(bl_ctx *ctx, int batch) {
  for (auto &ls : ctx->schedules)
    if (ls.batch == batch) return &ls;
  const int n = ctx->g.n;
  const std::vector<int> &rp = ctx->h_rowptr, &ci = ctx->h_colids;
  std::vector<int> lev(n, 0);
  int maxl = 0;
  for (int i = 0; i < n; i++) {
    const int bi = i / batch;
    int l = -1;
    for (int e = rp[i]; e < rp[i + 1]; e++) {
      const int j = ci[e];
      if (j / batch < bi) l = std::max(l, lev[j]);
    }
    lev[i] = l + 1;
    maxl = std::max(maxl, l + 1);
  }
  LevelSchedule ls;
  ls.batch = batch;
  ls.levels = n > 0 ? maxl + 1 : 0;
  ls.offsets.assign(ls.levels + 1, 0);
  for (int i = 0; i < n; i++) ls.offsets[lev[i] + 1]++;
  for (int l = 0; l < ls.levels; l++) ls.offsets[l + 1] += ls.offsets[l];
  std::vector<int> order(std::max(n, 1));
  std::vector<int> fill(ls.offsets.begin(), ls.offsets.end() - 1);
  for (int i = 0; i < n; i++) order[fill[lev[i]]++] = i;
  if (cudaMalloc(&ls.order, order.size() * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&ls.d_offsets, ls.offsets.size() * sizeof(int)) != cudaSuccess) {
    bl_fail(ctx, -2, "cudaMalloc level schedule");
    return nullptr;
  }
  if (cudaMemcpy(ls.d_offsets, ls.offsets.data(), ls.offsets.size() * sizeof(int), cudaMemcpyHostToDevice) !=
      cudaSuccess) {
    bl_fail(ctx, -2, "cudaMemcpy level schedule");
    return nullptr;
  }
  if (cudaMemcpy(ls.order, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
    bl_fail(ctx, -2, "cudaMemcpy level schedule");
    return nullptr;
  }
  // neighbours in earlier batches, per level-order slot, in CSR order
  std::vector<int> eoff(std::max(n, 1) + 1, 0), ecol;
  ecol.reserve(ci.size() / 2 + 1);
  for (int t = 0; t < n; t++) {
    const int i = order[t];
    const int blo = (i / batch) * batch;
    for (int e = rp[i]; e < rp[i + 1]; e++)
      if (ci[e] < blo) ecol.push_back(ci[e]);
    eoff[t + 1] = (int)ecol.size();
  }
  if (ecol.empty()) ecol.push_back(0);
  if (cudaMalloc(&ls.early_off, eoff.size() * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&ls.early_col, ecol.size() * sizeof(int)) != cudaSuccess ||
      cudaMemcpy(ls.early_off, eoff.data(), eoff.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ls.early_col, ecol.data(), ecol.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
    bl_fail(ctx, -2, "level schedule neighbour lists");
    return nullptr;
  }
  ctx->schedules.push_back(std::move(ls));
  return &ctx->schedules.back();
}

}  // namespace bl

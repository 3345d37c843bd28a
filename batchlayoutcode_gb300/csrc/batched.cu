// batched.cu -- many independent graphs in one persistent launch.
//
// The reference lays out one graph per process.  Here a persistent kernel
// takes graphs from a device work queue (largest first) and each block lays
// out one graph by itself, with block barriers only, for all iterations:
//   * minibatch graphs (algo 2/3/8, sample/algorithms.cpp:739-783,
//     :874-945, :947-1018): every coordinate of the graph stays in shared
//     memory for the whole run; a pass handles 512/parts targets, each
//     target's sources split into `parts` contiguous ranges summed separately
//     (parts is picked per graph-size bucket by the autotuner below); the
//     forces of a whole minibatch are computed before any of its vertices
//     moves; matched neighbours (the sorted-CSR cursor's set) swap their
//     repulsion for attraction;
//   * Barnes-Hut graphs (algo 4, :1038-1072): the whole-device pipeline of
//     barnes_hut.cu at block scope, with the same arithmetic (bh_device.cuh),
//     so a graph laid out here gets the same bits as through
//     bl_barnes_hut_iteration: Morton keys, a block LSD radix sort, a
//     top-down breadth-first build of the compressed quadtree (binary
//     searches for the quadrant boundaries), centroids bottom-up, pre-order
//     records with skip links top-down, the stackless traversal, then the
//     batches in order with block barriers.
// The queue reset and the launch are captured once in a CUDA graph and
// replayed; the coordinates are read from xy_in and written to xy_out, so a
// replay repeats the same layout.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/batchlayout_gb300.h"
#include "bh_device.cuh"

namespace bl {

constexpr int kAlgoBH = 4;

struct BatchedGraph {
  int n;           // vertices
  int voff;        // first vertex of the graph in the concatenated coordinates
  int roff;        // first entry of its neighbour rowptr (n + 1 entries, local to eoff)
  int algo;        // MODEL_FR / MODEL_LINLOG / MODEL_FA (minibatch) or kAlgoBH
  long long eoff;  // first entry of its neighbour colids
  int parts;       // minibatch: source ranges per target (1, 2 or 4)
  int pad;
};

struct BatchedArgs {
  int num_graphs, iterations, batch;
  float W;
  double theta, inv_theta2;  // inv_theta2 = 1 / theta^2, folded into the records
  const BatchedGraph *graphs;
  const int *order;            // queue order (largest graph first)
  unsigned int *queue;         // next queue slot
  const int *rowptr;           // concatenated local neighbour CSRs
  const int *colids;
  const double *xy_in;         // concatenated coordinates (x, y pairs)
  double *xy_out;
  double *energy;              // per graph: energy of the last iteration
  unsigned long long *cycles;  // per graph: clock64 cycles (autotuning) or null
  DevStatus *st;
  // Barnes-Hut workspace: one slot of `slot` vertices per block
  int slot;
  u64 *keys;            // 2 slot
  int *perm;            // 2 slot
  float2 *pos;          // slot
  float2 *spos;         // slot
  float4 *f0;           // slot
  int2 *brange;         // slot: breadth-first quad nodes, [lo, hi)
  int *blvl;            // slot: digit level (32 = run of equal keys)
  int4 *bkids;          // slot: children (>= 0 node, ~k leaf, kNoKid none)
  int *bsize;           // slot: records in the subtree
  double2 *bcen;        // slot: FP64 centroid
  int *bidx;            // slot: pre-order record index
  float4 *nodes;        // 2 slot: pre-order records {x, y, D^2, skip}
  double2 *c64;         // 2 slot
  unsigned char *nlvl;  // 2 slot
};

namespace {

constexpr int kBThreads = 512;
constexpr int kBWarps = kBThreads / 32;
constexpr int kSortR = 8;  // keys per thread in a sort tile
constexpr int kSortTile = kBThreads * kSortR;
constexpr int kMaxBfsLevels = 40;  // digit levels 0..32 need at most 34
constexpr int kNoKid = INT_MIN;
constexpr int kMaxBatch = 4096;

// shared memory of the Barnes-Hut path (carved from the dynamic buffer)
struct BhShared {
  unsigned int wcnt[kBWarps][256];
  unsigned int cnt[256];
  unsigned int base[256];
  unsigned int box[4];
  int wsum[kBWarps];
  int lvl_off[kMaxBfsLevels + 2];
  double frame[4];
  int trivial;
};

__device__ double block_sum_d(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  if (w == 0) {
    t = (l < kBWarps) ? red[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  __syncthreads();
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  const double r = red[0];
  __syncthreads();
  return r;
}

// exclusive prefix of v over the block; *total = block sum
__device__ int block_scan_excl(int v, int *wsum, int *total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  __syncthreads();
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  int pre = 0, tot = 0;
#pragma unroll
  for (int k = 0; k < kBWarps; k++) {
    const int t = wsum[k];
    if (k < w) pre += t;
    tot += t;
  }
  *total = tot;
  return pre + x - v;
}

// ---- minibatch graph, entirely inside the block ------------------------------
__device__ void layout_small(const BatchedArgs &a, int g, unsigned char *smem, double *red) {
  const BatchedGraph G = a.graphs[g];
  float2 *fbuf = reinterpret_cast<float2 *>(smem);  // [batch]
  float2 *part = fbuf + a.batch;                    // [kBThreads]
  float2 *pos = part + kBThreads;                   // [n]
  const int tid = threadIdx.x;
  const int n = G.n;
  const int parts = G.parts;
  const int tpp = kBThreads / parts;  // targets per pass
  const int *rp = a.rowptr + G.roff;
  const int *ci = a.colids + G.eoff;
  const double decay = (G.algo == MODEL_FR) ? 0.999 : 0.99;
  for (int k = tid; k < n; k += kBThreads)
    pos[k] = make_float2((float)a.xy_in[2 * (size_t)(G.voff + k)], (float)a.xy_in[2 * (size_t)(G.voff + k) + 1]);
  __syncthreads();
  double step = 1.0, e_part = 0.0;
  const int nb = (n + a.batch - 1) / a.batch;
  for (int it = 0; it < a.iterations; it++) {
    const bool last = it == a.iterations - 1;
    for (int b = 0; b < nb; b++) {
      const int base = b * a.batch;
      const int cnt = min(a.batch, n - base);
      for (int c0 = 0; c0 < cnt; c0 += tpp) {
        const int t = c0 + tid / parts, h = tid % parts;
        if (t < cnt) {
          const int i = base + t;
          const float2 pi = pos[i];
          const int j0 = (int)((long long)n * h / parts), j1 = (int)((long long)n * (h + 1) / parts);
          float fxa = 0.f, fya = 0.f, fxb = 0.f, fyb = 0.f;
          int j = j0;
          for (; j + 1 < j1; j += 2) {
            const float2 q0 = pos[j], q1 = pos[j + 1];
            rep_pair(q0.x, q0.y, pi.x, pi.y, fxa, fya);
            rep_pair(q1.x, q1.y, pi.x, pi.y, fxb, fyb);
          }
          if (j < j1) rep_pair(pos[j].x, pos[j].y, pi.x, pi.y, fxb, fyb);
          // matched neighbours in this range: attraction instead of repulsion
          for (int e = rp[i]; e < rp[i + 1]; e++) {
            const int q = ci[e];
            if (q < j0 || q >= j1) continue;
            const float2 pj = pos[q];
            const float dx = pj.x - pi.x, dy = pj.y - pi.y;
            const float d2 = fmaf(dx, dx, fmaf(dy, dy, kTinyD2));
            const float r = rcp_approx(d2);
            fxb = fmaf(dx, r, fxb);
            fyb = fmaf(dy, r, fyb);
            attract_pair(G.algo, a.W, pj.x, pj.y, pi.x, pi.y, fxb, fyb);
          }
          part[t - c0 + h * tpp] = make_float2(fxa + fxb, fya + fyb);
        }
        __syncthreads();
        if (tid < tpp && c0 + tid < cnt) {
          float hx = 0.f, lx = 0.f, hy = 0.f, ly = 0.f;
          for (int q = 0; q < parts; q++) {
            const float2 v = part[tid + q * tpp];
            ff_add(hx, lx, v.x);
            ff_add(hy, ly, v.y);
          }
          fbuf[c0 + tid] = make_float2(hx + lx, hy + ly);
        }
        __syncthreads();
      }
      // every force of the minibatch is known: move it
      for (int t = tid; t < cnt; t += kBThreads) {
        const float2 f = fbuf[t];
        pos[base + t] = unit_step(pos[base + t], (double)f.x, (double)f.y, (float)step);
        if (last) e_part += (double)f.x * (double)f.x + (double)f.y * (double)f.y;
      }
      __syncthreads();
    }
    step = step * decay;
  }
  for (int k = tid; k < n; k += kBThreads) {
    a.xy_out[2 * (size_t)(G.voff + k)] = (double)pos[k].x;
    a.xy_out[2 * (size_t)(G.voff + k) + 1] = (double)pos[k].y;
  }
  const double e = block_sum_d(e_part, red);
  if (tid == 0) a.energy[g] = e;
}

// ---- Barnes-Hut graph, one block ----------------------------------------------

// digit level of the quad node over sorted keys [lo, hi]: the first digit at
// which they differ, 32 for a run of equal keys
__device__ __forceinline__ int node_level(const u64 *K, int lo, int hi) {
  const u64 x = K[lo] ^ K[hi];
  return x ? (__clzll((long long)x) >> 1) : 32;
}

// first index in [lo, hi) whose digit at `shift` is >= d (digits ascend there)
__device__ __forceinline__ int digit_bound(const u64 *K, int lo, int hi, int shift, unsigned int d) {
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (((unsigned int)(K[mid] >> shift) & 3u) < d) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ void write_leaf(const BatchedArgs &a, float4 *nodes, double2 *c64, unsigned char *nlvl,
                                           const float2 *spos, int k, int idx, int cap) {
  if (idx < 0 || idx >= cap) {
    dev_record_error(a.st, DEV_BAD_INDEX);
    return;
  }
  const float2 p = spos[k];
  nodes[idx] = make_float4(p.x, p.y, kLeafZ, __int_as_float(idx + 1));
  c64[idx] = make_double2((double)p.x, (double)p.y);
  nlvl[idx] = 255;
}

__device__ void layout_bh(const BatchedArgs &a, int g, BhShared &S, double *red) {
  const BatchedGraph G = a.graphs[g];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n = G.n;
  const size_t sb = (size_t)blockIdx.x * a.slot;
  u64 *kin = a.keys + 2 * sb, *kout = kin + a.slot;
  int *vin = a.perm + 2 * sb, *vout = vin + a.slot;
  float2 *pos = a.pos + sb, *spos = a.spos + sb;
  float4 *f0 = a.f0 + sb;
  int2 *brange = a.brange + sb;
  int *blvl = a.blvl + sb, *bsize = a.bsize + sb, *bidx = a.bidx + sb;
  int4 *bkids = a.bkids + sb;
  double2 *bcen = a.bcen + sb;
  float4 *nodes = a.nodes + 2 * sb;
  double2 *c64 = a.c64 + 2 * sb;
  unsigned char *nlvl = a.nlvl + 2 * sb;
  const int *rp = a.rowptr + G.roff;
  const int *ci = a.colids + G.eoff;
  const int cap = 2 * n - 1;  // records: n leaves + at most n - 1 quad nodes
  for (int k = tid; k < n; k += kBThreads)
    pos[k] = make_float2((float)a.xy_in[2 * (size_t)(G.voff + k)], (float)a.xy_in[2 * (size_t)(G.voff + k) + 1]);
  double step = 1.0, e_part = 0.0;
  for (int it = 0; it < a.iterations; it++) {
    const bool last = it == a.iterations - 1;
    // 1. bounding box and Morton frame (MortonCode.h:42-52)
    if (tid == 0) {
      S.box[0] = 0xffffffffu;
      S.box[1] = 0u;
      S.box[2] = 0xffffffffu;
      S.box[3] = 0u;
    }
    __syncthreads();
    {
      unsigned int mnx = 0xffffffffu, mxx = 0u, mny = 0xffffffffu, mxy = 0u;
      for (int k = tid; k < n; k += kBThreads) {
        const float2 p = pos[k];
        const unsigned int ux = f2ord(p.x), uy = f2ord(p.y);
        mnx = min(mnx, ux);
        mxx = max(mxx, ux);
        mny = min(mny, uy);
        mxy = max(mxy, uy);
      }
      for (int o = 16; o > 0; o >>= 1) {
        mnx = min(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
        mxx = max(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mny = min(mny, __shfl_xor_sync(0xffffffffu, mny, o));
        mxy = max(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
      }
      if (lane == 0) {
        atomicMin(&S.box[0], mnx);
        atomicMax(&S.box[1], mxx);
        atomicMin(&S.box[2], mny);
        atomicMax(&S.box[3], mxy);
      }
    }
    __syncthreads();
    if (tid == 0) {
      double minX, minY, maxmin;
      frame_from_bbox(S.box, minX, minY, maxmin);
      S.frame[0] = minX;
      S.frame[1] = minY;
      S.frame[2] = maxmin;
      S.frame[3] = (maxmin > 0.0) ? 1.0 / maxmin : 0.0;
    }
    __syncthreads();
    const double maxmin = S.frame[2];
    // 2. keys
    {
      const double minX = S.frame[0], minY = S.frame[1], inv = S.frame[3];
      for (int k = tid; k < n; k += kBThreads) {
        kin[k] = morton_key(pos[k], minX, minY, maxmin, inv);
        vin[k] = k;
      }
    }
    __syncthreads();
    // 3. stable LSD radix sort of (key, vertex), 8-bit digits: the four
    //    passes on the high 32 bits, then every run of equal high halves (two
    //    points in one cell of a 65,536 x 65,536 grid over the frame: rare)
    //    sorted on its own by (key, vertex) -- the order the whole-device path
    //    produces.  A run longer than 32 keys sends the block through the
    //    four low passes and the high ones again instead (the order of equal
    //    keys, vertex order, is kept by every pass).  A pass whose digit is
    //    the same for every key is skipped.
    auto lsd_pass = [&](int pass) {
      const int shift = 8 * pass;
      if (tid < 256) S.cnt[tid] = 0;
      if (tid == 0) S.trivial = 0;
      __syncthreads();
      for (int k = tid; k < n; k += kBThreads) atomicAdd(&S.cnt[(unsigned int)(kin[k] >> shift) & 255u], 1u);
      __syncthreads();
      if (tid < 256) {
        const unsigned int v = S.cnt[tid];
        unsigned int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
          if (lane >= o) x += y;
        }
        if (lane == 31) S.wsum[warp] = (int)x;
        if (v == (unsigned int)n) S.trivial = 1;
        S.base[tid] = x - v;  // warp-local for now
      }
      __syncthreads();
      if (tid < 256) {
        unsigned int pre = 0;
        for (int w = 0; w < warp; w++) pre += (unsigned int)S.wsum[w];
        S.base[tid] += pre;
      }
      __syncthreads();
      const int trivial = S.trivial;
      __syncthreads();  // S.trivial is rewritten at the start of the next pass
      if (trivial) return;
      for (int tile0 = 0; tile0 < n; tile0 += kSortTile) {
        for (int d = lane; d < 256; d += 32) S.wcnt[warp][d] = 0;
        __syncwarp();
        const int wb = tile0 + warp * (kSortR * 32);
        const unsigned int lt = (1u << lane) - 1u;
        u64 kk[kSortR];
        unsigned int rd[kSortR];  // rank within the warp's keys | digit << 16, digit 256 = none
#pragma unroll
        for (int r = 0; r < kSortR; r++) {
          const int idx = wb + r * 32 + lane;
          const bool valid = idx < n;
          kk[r] = valid ? kin[idx] : 0ull;
          const unsigned int d = valid ? ((unsigned int)(kk[r] >> shift) & 255u) : 256u;
          const unsigned int peers = __match_any_sync(0xffffffffu, d);
          const unsigned int leader = __ffs(peers) - 1;
          unsigned int old = 0;
          if (d < 256u) old = S.wcnt[warp][d];
          __syncwarp();
          if (d < 256u && lane == leader) S.wcnt[warp][d] = old + __popc(peers);
          __syncwarp();
          rd[r] = (old + __popc(peers & lt)) | (d << 16);
        }
        __syncthreads();
        if (tid < 256) {
          unsigned int run = S.base[tid];
#pragma unroll
          for (int w = 0; w < kBWarps; w++) {
            const unsigned int c = S.wcnt[w][tid];
            S.wcnt[w][tid] = run;
            run += c;
          }
          S.base[tid] = run;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kSortR; r++) {
          const unsigned int d = rd[r] >> 16;
          if (d < 256u) {
            const unsigned int p = S.wcnt[warp][d] + (rd[r] & 0xffffu);
            if (p < (unsigned int)n) {
              kout[p] = kk[r];
              vout[p] = vin[wb + r * 32 + lane];
            } else {
              dev_record_error(a.st, DEV_BAD_INDEX);
            }
          }
        }
        __syncthreads();
      }
      u64 *tk = kin;
      kin = kout;
      kout = tk;
      int *tv = vin;
      vin = vout;
      vout = tv;
    };
    for (int pass = 4; pass < 8; pass++) lsd_pass(pass);
    if (tid == 0) S.trivial = 0;  // reused: a run longer than 32 keys
    __syncthreads();
    for (int k = tid; k < n; k += kBThreads) {
      const unsigned int h = (unsigned int)(kin[k] >> 32);
      if (k > 0 && (unsigned int)(kin[k - 1] >> 32) == h) continue;       // not a run start
      if (k + 1 >= n || (unsigned int)(kin[k + 1] >> 32) != h) continue;  // a run of one
      int len = 2;
      while (k + len < n && (unsigned int)(kin[k + len] >> 32) == h && len <= 32) len++;  // bounded
      if (len > 32) {
        S.trivial = 1;
        continue;
      }
      for (int q = k + 1; q < k + len; q++) {  // insertion sort by (key, vertex)
        const u64 kq = kin[q];
        const int vq = vin[q];
        int b = q - 1;
        while (b >= k && (kin[b] > kq || (kin[b] == kq && vin[b] > vq))) {
          kin[b + 1] = kin[b];
          vin[b + 1] = vin[b];
          b--;
        }
        kin[b + 1] = kq;
        vin[b + 1] = vq;
      }
    }
    __syncthreads();
    const int long_run = S.trivial;
    __syncthreads();
    if (long_run)
      for (int pass = 0; pass < 8; pass++) lsd_pass(pass);
    // 4. positions in Morton order
    for (int k = tid; k < n; k += kBThreads) {
      int v = vin[k];
      if ((unsigned int)v >= (unsigned int)n) {
        dev_record_error(a.st, DEV_BAD_INDEX);
        v = 0;
        vin[k] = 0;
      }
      spos[k] = pos[v];
    }
    // 5. breadth-first build of the compressed quadtree (BarnesHut.h:135-189
    //    without its single-child chain nodes)
    if (tid == 0) {
      brange[0] = make_int2(0, n);
      blvl[0] = node_level(kin, 0, n - 1);
      S.lvl_off[0] = 0;
      S.lvl_off[1] = 1;
    }
    __syncthreads();
    int nlev = 0;
    for (int L = 0; L < kMaxBfsLevels; L++) {
      const int q0 = S.lvl_off[L], q1 = S.lvl_off[L + 1];
      if (q1 == q0) break;
      nlev = L + 1;
      int next = q1;
      for (int c0 = q0; c0 < q1; c0 += kBThreads) {
        const int q = c0 + tid;
        int b[5] = {0, 0, 0, 0, 0};
        int lv = 32, nc = 0;
        if (q < q1) {
          const int2 r = brange[q];
          lv = blvl[q];
          b[0] = r.x;
          b[4] = r.y;
          if (lv < 32) {
            const int shift = 62 - 2 * lv;
            for (int d = 1; d < 4; d++) b[d] = digit_bound(kin, b[d - 1], r.y, shift, (unsigned int)d);
            for (int d = 0; d < 4; d++) nc += (b[d + 1] - b[d] >= 2);
          }
        }
        int tot = 0;
        const int off = block_scan_excl(nc, S.wsum, &tot);
        if (q < q1) {
          int kids[4] = {kNoKid, kNoKid, kNoKid, kNoKid};
          if (lv < 32) {
            int id = next + off, m = 0;
            for (int d = 0; d < 4; d++) {
              const int sz = b[d + 1] - b[d];
              if (sz == 1) {
                kids[m++] = ~b[d];
              } else if (sz >= 2) {
                if (id >= n - 1) {  // a tree over n points has at most n - 1 quad nodes
                  dev_record_error(a.st, DEV_BAD_INDEX);
                  continue;
                }
                brange[id] = make_int2(b[d], b[d + 1]);
                blvl[id] = node_level(kin, b[d], b[d + 1] - 1);
                kids[m++] = id++;
              }
            }
          }
          bkids[q] = make_int4(kids[0], kids[1], kids[2], kids[3]);
        }
        next += tot;
      }
      if (tid == 0) S.lvl_off[L + 2] = min(next, n - 1);
      __syncthreads();
    }
    if (nlev == kMaxBfsLevels && tid == 0) dev_record_error(a.st, DEV_BAD_INDEX);
    // 6. centroids and subtree sizes, deepest level first: unweighted mean of
    //    the children summed in quadrant order in FP64 (BarnesHut.h:197-217)
    for (int L = nlev - 1; L >= 0; L--) {
      for (int q = S.lvl_off[L] + tid; q < S.lvl_off[L + 1]; q += kBThreads) {
        double cx = 0.0, cy = 0.0;
        int cnt = 0, size = 1;
        if (blvl[q] == 32) {
          const int2 r = brange[q];
          for (int k = r.x; k < r.y; k++) {
            const float2 v = spos[k];
            cx = __dadd_rn(cx, (double)v.x);
            cy = __dadd_rn(cy, (double)v.y);
            cnt++;
          }
          size += r.y - r.x;
        } else {
          const int4 kk = bkids[q];
          const int kids[4] = {kk.x, kk.y, kk.z, kk.w};
#pragma unroll
          for (int c = 0; c < 4; c++) {
            const int ch = kids[c];
            if (ch == kNoKid) break;
            double vx, vy;
            if (ch < 0) {
              const float2 v = spos[~ch];
              vx = (double)v.x;
              vy = (double)v.y;
              size += 1;
            } else {
              const double2 v = bcen[ch];
              vx = v.x;
              vy = v.y;
              size += bsize[ch];
            }
            cx = __dadd_rn(cx, vx);
            cy = __dadd_rn(cy, vy);
            cnt++;
          }
        }
        bcen[q] = make_double2(div_count(cx, max(cnt, 1)), div_count(cy, max(cnt, 1)));
        bsize[q] = size;
      }
      __syncthreads();
    }
    // 7. pre-order records with skip links, top level first
    if (tid == 0) bidx[0] = 0;
    __syncthreads();
    for (int L = 0; L < nlev; L++) {
      for (int q = S.lvl_off[L] + tid; q < S.lvl_off[L + 1]; q += kBThreads) {
        const int I = bidx[q], sz = bsize[q], lv = blvl[q];
        if (I < 0 || sz < 1 || I + sz > cap) {
          dev_record_error(a.st, DEV_BAD_INDEX);
          continue;
        }
        const double D = ldexp(maxmin, -lv);
        const double2 c = bcen[q];
        nodes[I] = make_float4(d2f_int(c.x), d2f_int(c.y), bh_record_z(D, a.inv_theta2), __int_as_float(I + sz));
        c64[I] = c;
        nlvl[I] = (unsigned char)lv;
        int run = I + 1;
        if (lv == 32) {
          const int2 r = brange[q];
          for (int k = r.x; k < r.y; k++) write_leaf(a, nodes, c64, nlvl, spos, k, run++, cap);
        } else {
          const int4 kk = bkids[q];
          const int kids[4] = {kk.x, kk.y, kk.z, kk.w};
          for (int c = 0; c < 4; c++) {
            const int ch = kids[c];
            if (ch == kNoKid) break;
            if (ch < 0) {
              write_leaf(a, nodes, c64, nlvl, spos, ~ch, run++, cap);
            } else {
              bidx[ch] = run;
              run += bsize[ch];
            }
          }
        }
      }
      __syncthreads();
    }
    // 8. repulsion of every vertex (Morton order) and the attraction of its
    //    neighbours that have not moved yet in this iteration
    {
      int total = __float_as_int(nodes[0].w);
      if (total < 0 || total > cap) {
        if (tid == 0) dev_record_error(a.st, DEV_BAD_INDEX);
        total = 0;
      }
      unsigned int visits = 0, exact = 0;
      for (int k = tid; k < n; k += kBThreads) {
        const float2 rep = bh_repulsion<false>(nodes, c64, nlvl, maxmin, a.theta, total, spos[k], visits,
                                               exact);
        const int v = vin[k];
        f0[v] = bh_minus_repulsion(bh_unmoved_attraction(v, rp, ci, pos, a.batch, a.W), rep);
      }
    }
    __syncthreads();
    // 9. batches in order: attraction of the neighbours moved earlier in this
    //    iteration, then the unit step (algorithms.cpp:1050-1066)
    const float stepf = (float)step;
    for (int lo = 0; lo < n; lo += a.batch) {
      const int cnt = min(a.batch, n - lo);
      for (int t = tid; t < cnt; t += kBThreads) {
        const int i = lo + t;
        const float2 pi = pos[i];
        const float4 f = f0[i];
        float hx = f.x, hy = f.y, lx = f.z, ly = f.w;
        for (int e = rp[i]; e < rp[i + 1]; e++) {
          const int j = ci[e];
          if (j < lo) bh_attract(pos[j], pi, a.W, hx, lx, hy, ly);
        }
        pos[i] = bh_step(pi, hx, lx, hy, ly, stepf);
        if (last) {
          const double fx = (double)hx + (double)lx, fy = (double)hy + (double)ly;
          e_part += fx * fx + fy * fy;
        }
      }
      __syncthreads();
    }
    step = step * 0.999;
  }
  for (int k = tid; k < n; k += kBThreads) {
    a.xy_out[2 * (size_t)(G.voff + k)] = (double)pos[k].x;
    a.xy_out[2 * (size_t)(G.voff + k) + 1] = (double)pos[k].y;
  }
  const double e = block_sum_d(e_part, red);
  if (tid == 0) a.energy[g] = e;
}

__global__ void __launch_bounds__(kBThreads, 2) batched_kernel(BatchedArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_q;
  __shared__ double red[kBWarps];
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_q = (int)atomicAdd(a.queue, 1u);
    __syncthreads();
    const int q = s_q;
    if (q >= a.num_graphs) return;
    const int g = a.order[q];
    const long long t0 = clock64();
    if (a.graphs[g].algo == kAlgoBH) layout_bh(a, g, *reinterpret_cast<BhShared *>(smem), red);
    else layout_small(a, g, smem, red);
    if (a.cycles && threadIdx.x == 0) a.cycles[g] = (unsigned long long)(clock64() - t0);
  }
}

// size bucket of a minibatch graph for the autotuner
int size_bucket(int n) { return n < 512 ? 0 : (n < 2048 ? 1 : 2); }

}  // namespace

// Host state of the batched layout: graphs and workspace stay on the device
// between runs; the launch is a CUDA graph.
struct BatchedState {
  int num_graphs = 0, total_v = 0, max_small = 0, max_bh = 0, grid = 0, ws_grid = 0;
  size_t smem = 0;
  std::vector<BatchedGraph> gs;
  std::vector<int> order;
  int parts[3] = {0, 0, 0};  // autotuned source split per size bucket (0 = not tuned)
  BatchedGraph *d_graphs = nullptr;
  int *d_order = nullptr, *d_rp = nullptr, *d_ci = nullptr;
  double *d_xy_in = nullptr, *d_xy_out = nullptr, *d_energy = nullptr;
  unsigned long long *d_cycles = nullptr;
  unsigned int *d_queue = nullptr;
  void *ws = nullptr;  // Barnes-Hut workspace
  BatchedArgs args{};
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  int key_iterations = -1, key_batch = -1;
  double key_theta = -1.0, key_weight = -1.0;
  bool graph_dirty = true;
  cudaEvent_t ev[2] = {nullptr, nullptr};
};

void batched_free(BatchedState *b) {
  if (!b) return;
  cudaFree(b->d_graphs);
  cudaFree(b->d_order);
  cudaFree(b->d_rp);
  cudaFree(b->d_ci);
  cudaFree(b->d_xy_in);
  cudaFree(b->d_xy_out);
  cudaFree(b->d_energy);
  cudaFree(b->d_cycles);
  cudaFree(b->d_queue);
  cudaFree(b->ws);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (auto e : b->ev)
    if (e) cudaEventDestroy(e);
  delete b;
}

namespace {

int batched_launch(bl_ctx *ctx, BatchedState &B, int num, const int *d_order, unsigned long long *d_cycles,
                   int iterations) {
  BatchedArgs a = B.args;
  a.num_graphs = num;
  a.order = d_order;
  a.cycles = d_cycles;
  a.iterations = iterations;
  BL_CUDA(ctx, cudaMemsetAsync(B.d_queue, 0, sizeof(unsigned int), ctx->stream));
  batched_kernel<<<std::min(num, B.grid), kBThreads, B.smem, ctx->stream>>>(a);
  ctx->launches++;
  BL_CUDA(ctx, cudaGetLastError());
  return 0;
}

template <typename T>
T *carve(char *&p, size_t count) {
  T *r = reinterpret_cast<T *>(p);
  p += ((count * sizeof(T) + 255) / 256) * 256;
  return r;
}

// Launch shape for this batch size: dynamic shared memory, resident grid and
// one Barnes-Hut workspace slot per block of that grid.
int batched_shape(bl_ctx *ctx, BatchedState &B, int batch) {
  int smem_optin = 0;
  BL_CUDA(ctx, cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
  const size_t smem_small = (size_t)(batch + kBThreads + B.max_small) * sizeof(float2);
  const size_t smem = std::max(smem_small, sizeof(BhShared));
  if (smem + 2048 > (size_t)smem_optin)
    return bl_fail(ctx, BL_ERR_TOO_LARGE, "a minibatch graph is too large for one block's shared memory");
  BL_CUDA(ctx, cudaFuncSetAttribute(batched_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 0;
  BL_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batched_kernel, kBThreads, smem));
  if (occ < 1) return bl_fail(ctx, BL_ERR_TOO_LARGE, "batched kernel cannot be resident");
  const int grid = std::min(B.num_graphs, ctx->num_sms * occ);
  if (smem != B.smem || grid != B.grid) B.graph_dirty = true;
  B.smem = smem;
  if (B.max_bh > 0 && grid > B.ws_grid) {
    cudaFree(B.ws);
    B.ws = nullptr;
    B.ws_grid = 0;
    const size_t slot = (size_t)B.max_bh;
    const size_t per_slot = 2 * 8 + 2 * 4 + 8 + 8 + 16 + 8 + 4 + 16 + 4 + 16 + 4 + 2 * 16 + 2 * 16 + 2;
    const size_t bytes = (size_t)grid * slot * per_slot + 14 * 256;
    BL_CUDA(ctx, cudaMalloc(&B.ws, bytes));
    B.ws_grid = grid;
    char *p = reinterpret_cast<char *>(B.ws);
    const size_t S = (size_t)grid * slot;
    BatchedArgs &a = B.args;
    a.slot = (int)slot;
    a.keys = carve<u64>(p, 2 * S);
    a.perm = carve<int>(p, 2 * S);
    a.pos = carve<float2>(p, S);
    a.spos = carve<float2>(p, S);
    a.f0 = carve<float4>(p, S);
    a.brange = carve<int2>(p, S);
    a.blvl = carve<int>(p, S);
    a.bkids = carve<int4>(p, S);
    a.bsize = carve<int>(p, S);
    a.bcen = carve<double2>(p, S);
    a.bidx = carve<int>(p, S);
    a.nodes = carve<float4>(p, 2 * S);
    a.c64 = carve<double2>(p, 2 * S);
    a.nlvl = carve<unsigned char>(p, 2 * S);
    B.graph_dirty = true;
  }
  B.grid = grid;
  return 0;
}

// Per size bucket: time 2 iterations of up to 16 of its minibatch graphs with
// 1, 2 and 4 source ranges per target and keep the fastest (clock64 cycles
// per n^2, summed over the sample).
int batched_autotune(bl_ctx *ctx, BatchedState &B) {
  for (int bk = 0; bk < 3; bk++) {
    if (B.parts[bk] > 0) continue;
    std::vector<int> sample;
    for (int g : B.order)
      if (B.gs[g].algo != kAlgoBH && size_bucket(B.gs[g].n) == bk && (int)sample.size() < 16) sample.push_back(g);
    if (sample.empty()) continue;
    BL_CUDA(ctx, cudaMemcpyAsync(B.d_order, sample.data(), sizeof(int) * sample.size(), cudaMemcpyHostToDevice,
                                 ctx->stream));
    double best = 1e300;
    int best_parts = 2;
    std::vector<unsigned long long> cyc(B.num_graphs);
    for (int parts : {1, 2, 4}) {
      for (int g : sample) B.gs[g].parts = parts;
      BL_CUDA(ctx, cudaMemcpyAsync(B.d_graphs, B.gs.data(), sizeof(BatchedGraph) * B.num_graphs,
                                   cudaMemcpyHostToDevice, ctx->stream));
      if (int rc = batched_launch(ctx, B, (int)sample.size(), B.d_order, B.d_cycles, 2)) return rc;
      BL_CUDA(ctx, cudaMemcpyAsync(cyc.data(), B.d_cycles, sizeof(unsigned long long) * B.num_graphs,
                                   cudaMemcpyDeviceToHost, ctx->stream));
      BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      double cost = 0.0;
      for (int g : sample) cost += (double)cyc[g] / ((double)B.gs[g].n * B.gs[g].n);
      if (cost < best) {
        best = cost;
        best_parts = parts;
      }
    }
    B.parts[bk] = best_parts;
  }
  for (auto &G : B.gs)
    if (G.algo != kAlgoBH) G.parts = B.parts[size_bucket(G.n)] > 0 ? B.parts[size_bucket(G.n)] : 2;
  BL_CUDA(ctx, cudaMemcpyAsync(B.d_order, B.order.data(), sizeof(int) * B.num_graphs, cudaMemcpyHostToDevice,
                               ctx->stream));
  BL_CUDA(ctx, cudaMemcpyAsync(B.d_graphs, B.gs.data(), sizeof(BatchedGraph) * B.num_graphs, cudaMemcpyHostToDevice,
                               ctx->stream));
  return bl_check_status(ctx);
}

}  // namespace
}  // namespace bl

// ---- C ABI ---------------------------------------------------------------------
extern "C" {

bl_ctx *bl_batch_create(int device) try {
  bl_ctx *ctx = new bl_ctx();
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&ctx->s.status, sizeof(DevStatus)) != cudaSuccess ||
      cudaMemset(ctx->s.status, 0, sizeof(DevStatus)) != cudaSuccess) {
    bl_destroy(ctx);
    return nullptr;
  }
  return ctx;
} catch (...) {
  bl_create_exception();
  return nullptr;
}

int bl_batched_prepare(bl_ctx *ctx, int num_graphs, const int *vertex_offset, const long long *edge_offset,
                       const int *rowptr, const int *colids, const int *algo, const double *xy) try {
  using namespace bl;
  if (!ctx) return BL_ERR_ARG;
  if (num_graphs < 1 || !vertex_offset || !edge_offset || !rowptr || !algo || !xy)
    return bl_fail(ctx, BL_ERR_ARG, "bl_batched_prepare: null argument or no graphs");
  if (edge_offset[num_graphs] > 0 && !colids) return bl_fail(ctx, BL_ERR_ARG, "bl_batched_prepare: null colids");
  if (vertex_offset[0] != 0) return bl_fail(ctx, BL_ERR_ARG, "vertex_offset[0] must be 0");
  if (edge_offset[0] != 0) return bl_fail(ctx, BL_ERR_ARG, "edge_offset[0] must be 0");
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  batched_free(ctx->batched);
  ctx->batched = nullptr;
  BatchedState *B = new BatchedState();
  ctx->batched = B;
  B->num_graphs = num_graphs;
  B->gs.resize(num_graphs);
  std::vector<int> erp, eci;
  long long total_v = 0;
  for (int g = 0; g < num_graphs; g++) {
    const std::string gn = "graph " + std::to_string(g) + ": ";
    const int n = vertex_offset[g + 1] - vertex_offset[g];
    const int al = algo[g];
    if (n < 1) return bl_fail(ctx, BL_ERR_ARG, gn + "no vertices");
    if (al != MODEL_FR && al != MODEL_LINLOG && al != MODEL_FA && al != kAlgoBH)
      return bl_fail(ctx, BL_ERR_UNSUPPORTED, gn + "algo must be 2, 3, 4 or 8");
    if (al == kAlgoBH && n < 2) return bl_fail(ctx, BL_ERR_ARG, gn + "Barnes-Hut needs at least two vertices");
    const int *rp = rowptr + vertex_offset[g] + g;
    const long long e0 = edge_offset[g], m = edge_offset[g + 1] - e0;
    if (rp[0] != 0 || (long long)rp[n] != m) return bl_fail(ctx, BL_ERR_ARG, gn + "rowptr does not match edge_offset");
    std::vector<int> lrp(rp, rp + n + 1), lci(colids ? colids + e0 : colids, colids ? colids + e0 + m : colids);
    for (int i = 0; i < n; i++)
      if (lrp[i + 1] < lrp[i]) return bl_fail(ctx, BL_ERR_ARG, gn + "rowptr decreases");
    for (int c : lci)
      if (c < 0 || c >= n) return bl_fail(ctx, BL_ERR_ARG, gn + "colid out of range");
    BatchedGraph &G = B->gs[g];
    G.n = n;
    G.voff = vertex_offset[g];
    G.algo = al;
    G.parts = 2;
    G.pad = 0;
    G.roff = (int)erp.size();
    G.eoff = (long long)eci.size();
    if (al == kAlgoBH) {
      // Barnes-Hut attraction runs over the whole row (algorithms.cpp:1056-1058)
      erp.insert(erp.end(), lrp.begin(), lrp.end());
      eci.insert(eci.end(), lci.begin(), lci.end());
      B->max_bh = std::max(B->max_bh, n);
    } else {
      std::vector<int> mrp, mci;
      cursor_neighbours(n, lrp, lci, mrp, mci);
      erp.insert(erp.end(), mrp.begin(), mrp.end());
      eci.insert(eci.end(), mci.begin(), mci.end());
      B->max_small = std::max(B->max_small, n);
    }
    total_v += n;
    if (total_v != vertex_offset[g + 1] - vertex_offset[0])
      return bl_fail(ctx, BL_ERR_ARG, gn + "vertex_offset must start at 0 and increase");
    if (erp.size() > (size_t)INT_MAX) return bl_fail(ctx, BL_ERR_TOO_LARGE, "too many graphs");
  }
  if (eci.empty()) eci.push_back(0);
  // largest graphs first (work grows like n^2 for minibatch graphs)
  B->order.resize(num_graphs);
  for (int g = 0; g < num_graphs; g++) B->order[g] = g;
  std::stable_sort(B->order.begin(), B->order.end(), [&](int x, int y) { return B->gs[x].n > B->gs[y].n; });
  // device buffers
  cudaStream_t st = ctx->stream;
  B->total_v = (int)total_v;
  BL_CUDA(ctx, cudaMalloc(&B->d_graphs, sizeof(BatchedGraph) * num_graphs));
  BL_CUDA(ctx, cudaMalloc(&B->d_order, sizeof(int) * num_graphs));
  BL_CUDA(ctx, cudaMalloc(&B->d_rp, sizeof(int) * erp.size()));
  BL_CUDA(ctx, cudaMalloc(&B->d_ci, sizeof(int) * eci.size()));
  BL_CUDA(ctx, cudaMalloc(&B->d_xy_in, sizeof(double) * 2 * total_v));
  BL_CUDA(ctx, cudaMalloc(&B->d_xy_out, sizeof(double) * 2 * total_v));
  BL_CUDA(ctx, cudaMalloc(&B->d_energy, sizeof(double) * num_graphs));
  BL_CUDA(ctx, cudaMalloc(&B->d_cycles, sizeof(unsigned long long) * num_graphs));
  BL_CUDA(ctx, cudaMalloc(&B->d_queue, sizeof(unsigned int)));
  BL_CUDA(ctx, cudaMemcpyAsync(B->d_graphs, B->gs.data(), sizeof(BatchedGraph) * num_graphs, cudaMemcpyHostToDevice, st));
  BL_CUDA(ctx, cudaMemcpyAsync(B->d_order, B->order.data(), sizeof(int) * num_graphs, cudaMemcpyHostToDevice, st));
  BL_CUDA(ctx, cudaMemcpyAsync(B->d_rp, erp.data(), sizeof(int) * erp.size(), cudaMemcpyHostToDevice, st));
  BL_CUDA(ctx, cudaMemcpyAsync(B->d_ci, eci.data(), sizeof(int) * eci.size(), cudaMemcpyHostToDevice, st));
  BL_CUDA(ctx, cudaMemcpyAsync(B->d_xy_in, xy, sizeof(double) * 2 * total_v, cudaMemcpyHostToDevice, st));
  BL_CUDA(ctx, cudaMemsetAsync(B->d_energy, 0, sizeof(double) * num_graphs, st));
  BatchedArgs &a = B->args;
  a = BatchedArgs{};
  a.graphs = B->d_graphs;
  a.queue = B->d_queue;
  a.rowptr = B->d_rp;
  a.colids = B->d_ci;
  a.xy_in = B->d_xy_in;
  a.xy_out = B->d_xy_out;
  a.energy = B->d_energy;
  a.st = ctx->s.status;
  BL_CUDA(ctx, cudaStreamSynchronize(st));
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_batched_run(bl_ctx *ctx, int iterations, int batch, double theta, double weight, double *seconds_out) try {
  using namespace bl;
  if (!ctx) return BL_ERR_ARG;
  BatchedState *B = ctx->batched;
  if (!B) return bl_fail(ctx, BL_ERR_STATE, "bl_batched_run before bl_batched_prepare");
  if (iterations < 1 || batch < 1 || batch > kMaxBatch || !(theta > 0.0))
    return bl_fail(ctx, BL_ERR_ARG, "iterations >= 1, 1 <= batch <= 4096 and theta > 0 required");
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  BatchedArgs &a = B->args;
  a.batch = batch;
  a.W = (float)weight;
  a.theta = theta;
  a.inv_theta2 = 1.0 / (theta * theta);
  if (int rc = batched_shape(ctx, *B, batch)) return rc;
  if (int rc = batched_autotune(ctx, *B)) return rc;
  if (B->graph_dirty || B->key_iterations != iterations || B->key_batch != batch || B->key_theta != theta ||
      B->key_weight != weight) {
    if (B->exec) cudaGraphExecDestroy(B->exec);
    if (B->graph) cudaGraphDestroy(B->graph);
    B->exec = nullptr;
    B->graph = nullptr;
    BL_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const long long before = ctx->launches;
    const int rc = batched_launch(ctx, *B, B->num_graphs, B->d_order, B->d_cycles, iterations);
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
    ctx->launches = before;  // counted when the graph runs
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    BL_CUDA(ctx, ce);
    B->graph = graph;
    BL_CUDA(ctx, cudaGraphInstantiate(&B->exec, graph, 0));
    B->key_iterations = iterations;
    B->key_batch = batch;
    B->key_theta = theta;
    B->key_weight = weight;
    B->graph_dirty = false;
  }
  if (!B->ev[0]) {
    BL_CUDA(ctx, cudaEventCreate(&B->ev[0]));
    BL_CUDA(ctx, cudaEventCreate(&B->ev[1]));
  }
  BL_CUDA(ctx, cudaEventRecord(B->ev[0], ctx->stream));
  BL_CUDA(ctx, cudaGraphLaunch(B->exec, ctx->stream));
  ctx->launches++;
  BL_CUDA(ctx, cudaEventRecord(B->ev[1], ctx->stream));
  BL_CUDA(ctx, cudaEventSynchronize(B->ev[1]));
  float ms = 0.f;
  BL_CUDA(ctx, cudaEventElapsedTime(&ms, B->ev[0], B->ev[1]));
  ctx->last_run_ms = ms;
  if (seconds_out) *seconds_out = ms * 1e-3;
  return bl_check_status(ctx);
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_batched_result(bl_ctx *ctx, double *xy, double *energy) try {
  using namespace bl;
  if (!ctx) return BL_ERR_ARG;
  BatchedState *B = ctx->batched;
  if (!B) return bl_fail(ctx, BL_ERR_STATE, "bl_batched_result before bl_batched_prepare");
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  if (xy)
    BL_CUDA(ctx, cudaMemcpyAsync(xy, B->d_xy_out, sizeof(double) * 2 * (size_t)B->total_v, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  if (energy)
    BL_CUDA(ctx, cudaMemcpyAsync(energy, B->d_energy, sizeof(double) * B->num_graphs, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_batched_layout(bl_ctx *ctx, int num_graphs, const int *vertex_offset, const long long *edge_offset,
                      const int *rowptr, const int *colids, const int *algo, double *xy, int iterations, int batch,
                      double theta, double weight, double *energy_out, double *seconds_out) try {
  if (int rc = bl_batched_prepare(ctx, num_graphs, vertex_offset, edge_offset, rowptr, colids, algo, xy)) return rc;
  if (int rc = bl_batched_run(ctx, iterations, batch, theta, weight, seconds_out)) return rc;
  return bl_batched_result(ctx, xy, energy_out);
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_batched_graph_cycles(bl_ctx *ctx, unsigned long long *cycles) try {
  if (!ctx || !cycles) return BL_ERR_ARG;
  if (!ctx->batched) return bl_fail(ctx, BL_ERR_STATE, "bl_batched_graph_cycles before bl_batched_prepare");
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  BL_CUDA(ctx, cudaMemcpyAsync(cycles, ctx->batched->d_cycles, sizeof(unsigned long long) * ctx->batched->num_graphs,
                               cudaMemcpyDeviceToHost, ctx->stream));
  BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_batched_set_parts(bl_ctx *ctx, const int *parts3) try {
  if (!ctx || !parts3) return BL_ERR_ARG;
  if (!ctx->batched) return bl_fail(ctx, BL_ERR_STATE, "bl_batched_set_parts before bl_batched_prepare");
  for (int k = 0; k < 3; k++)
    if (parts3[k] != 0 && parts3[k] != 1 && parts3[k] != 2 && parts3[k] != 4)
      return bl_fail(ctx, BL_ERR_ARG, "parts must be 0 (autotune), 1, 2 or 4");
  for (int k = 0; k < 3; k++) ctx->batched->parts[k] = parts3[k];
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_batched_parts(const bl_ctx *ctx, int *parts3) try {
  if (!ctx || !parts3) return BL_ERR_ARG;
  for (int k = 0; k < 3; k++) parts3[k] = ctx->batched ? ctx->batched->parts[k] : 0;
  return BL_OK;
} catch (...) {
  return bl_host_exception(nullptr);
}

}  // extern "C"

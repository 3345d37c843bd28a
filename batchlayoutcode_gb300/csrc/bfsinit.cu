// bfsinit.cu -- breadth-first greedy start, a GPU alternative to initDFS.
//
// initDFS (sample/algorithms.cpp:29-97) walks the graph depth first from
// vertex 0 and places every newly reached vertex c of a popped vertex u at
// x_u + 0.1 (cos a, sin a) + (r, r), a = k * 360 / deg(u) for the k-th vertex
// u reaches, r drawn from rand(), then scales the layout to a width of
// 2 * MAXMIN.  The walk and the rand() stream are sequential (0.25 s on the
// 1M-vertex benchmark graph, on the host).  This variant keeps the placement
// rule on a breadth-first tree instead:
//   * tree: a level-synchronous BFS from vertex 0; a vertex's parent is the
//     smallest-id vertex of the previous level adjacent to it;
//   * k: the rank of c among u's children, by first occurrence in u's row;
//   * r: a hash of the vertex id (splitmix64, 24 bits) instead of rand();
//   * positions: x_c = offset_c + x_parent summed by pointer jumping
//     (log2(depth) rounds) in FP64;
//   * scale: 2 * MAXMIN / max(x range, y range) over the reached vertices;
//     unreached vertices stay at the origin, as in initDFS's host version.
// Deterministic; not the reference's layout (no reference counterpart, like
// the learned start); its oracle is oracle/bfs_init.py.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <vector>

#include "../../include/batchlayout_gb300.h"
#include "bl_internal.cuh"

namespace bl {
namespace {

constexpr int kThreads = 512;
constexpr int kBuf = 2048;  // new frontier vertices a block gathers per level
constexpr int kNoLevel = INT_MAX;

struct TreeArgs {
  int n;
  const int *rowptr, *colids;
  int *level, *parent;
  int *wl[2];
  unsigned int *cnt;  // [3] list lengths, rotating by level
  DevStatus *st;
};

// One cooperative launch, one level per bounded grid barrier (the pattern of
// the feature BFS): a warp per frontier vertex, a lane per neighbour; the
// first visitor claims a vertex and appends it to the next frontier, and every
// visitor of the level offers itself as parent (atomicMin), so the parent is
// the smallest-id neighbour on the previous level whatever the timing.
__global__ void __launch_bounds__(kThreads) tree_bfs_kernel(TreeArgs a) {
  __shared__ unsigned int s_count, s_n, s_base;
  __shared__ int s_buf[kBuf];
  unsigned int epoch = 0;
  const unsigned int lane = threadIdx.x & 31u;
  const unsigned int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const unsigned int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int L = 1; L <= a.n; L++) {
    const int cb = (L - 1) & 1, nb = L & 1;
    if (threadIdx.x == 0) {
      s_count = ld_acquire_gpu(&a.cnt[(L - 1) % 3]);
      s_n = 0u;
    }
    __syncthreads();
    const unsigned int count = s_count;
    if (count == 0u) break;
    if (blockIdx.x == 0 && threadIdx.x == 0) a.cnt[(L + 1) % 3] = 0u;
    for (unsigned int idx = wid; idx < count; idx += nwarps) {
      const int u = __ldcg(&a.wl[cb][idx]);
      const int e0 = a.rowptr[u], e1 = a.rowptr[u + 1];
      for (int e = e0 + (int)lane; e < e1; e += 32) {
        const int v = a.colids[e];
        int lv = __ldcg(&a.level[v]);
        if (lv == kNoLevel) {
          lv = atomicCAS(&a.level[v], kNoLevel, L);
          if (lv == kNoLevel) {
            lv = L;
            const unsigned int slot = atomicAdd(&s_n, 1u);
            if (slot < (unsigned int)kBuf) s_buf[slot] = v;
            else a.wl[nb][atomicAdd(&a.cnt[L % 3], 1u)] = v;  // rare spill
          }
        }
        if (lv == L) atomicMin(&a.parent[v], u);
      }
    }
    __syncthreads();
    const unsigned int mine = min(s_n, (unsigned int)kBuf);
    if (threadIdx.x == 0 && mine) s_base = atomicAdd(&a.cnt[L % 3], mine);
    __syncthreads();
    for (unsigned int k = threadIdx.x; k < mine; k += blockDim.x) a.wl[nb][s_base + k] = s_buf[k];
    if (!grid_barrier(a.st, epoch)) return;
  }
}

// first CSR position (in the parent's row) of every tree child
__global__ void first_pos_kernel(int n, const int *__restrict__ rowptr, const int *__restrict__ colids,
                                 const int *__restrict__ parent, int *__restrict__ firstpos) {
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= n) return;
  const int u = (int)w;
  for (int e = rowptr[u] + lane; e < rowptr[u + 1]; e += 32) {
    const int c = colids[e];
    if (parent[c] == u) atomicMin(&firstpos[c], e);
  }
}

__device__ __forceinline__ double hash_unit(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  x ^= x >> 31;
  return (double)(x >> 40) * (1.0 / 16777216.0);  // 24 bits, exact in float and double
}

// offsets of u's children (rank by first occurrence) relative to u
__global__ void child_offset_kernel(int n, const int *__restrict__ rowptr, const int *__restrict__ colids,
                                    const int *__restrict__ parent, const int *__restrict__ firstpos,
                                    double2 *__restrict__ off) {
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= n) return;
  const int u = (int)w;
  const int e0 = rowptr[u], e1 = rowptr[u + 1];
  const double step = 360.0 / (double)max(e1 - e0, 1);
  const double kPi = 3.14159265358979323846;
  int before = 0;  // children already ranked in earlier chunks of the row
  for (int base = e0; base < e1; base += 32) {
    const int e = base + lane;
    int c = -1;
    bool child = false;
    if (e < e1) {
      c = colids[e];
      child = parent[c] == u && firstpos[c] == e;
    }
    const unsigned int mask = __ballot_sync(0xffffffffu, child);
    if (child) {
      const int k = before + __popc(mask & ((1u << lane) - 1u));
      const double ang = kPi * (k * step) / 180.0;
      const double r = hash_unit((unsigned long long)c);
      off[c] = make_double2(0.1 * cos(ang) + r, 0.1 * sin(ang) + r);
    }
    before += __popc(mask);
  }
}

// one pointer-jumping round: x_c += x_{jump_c}, jump_c = jump_{jump_c}
__global__ void jump_kernel(int n, const double2 *__restrict__ x, const int *__restrict__ jp, double2 *__restrict__ nx,
                            int *__restrict__ njp, unsigned int *__restrict__ active) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int j = jp[c];
  double2 v = x[c];
  int nj = -1;
  if (j >= 0) {
    const double2 p = x[j];
    v.x += p.x;
    v.y += p.y;
    nj = jp[j];
    if (nj >= 0) atomicOr(active, 1u);
  }
  nx[c] = v;
  njp[c] = nj;
}

__global__ void range_kernel(int n, const double2 *__restrict__ x, const int *__restrict__ level,
                             double *__restrict__ part) {
  __shared__ double s[4][32];
  double mnx = DBL_MAX, mny = DBL_MAX, mxx = -DBL_MAX, mxy = -DBL_MAX;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    if (level[c] == kNoLevel) continue;
    const double2 v = x[c];
    mnx = fmin(mnx, v.x);
    mny = fmin(mny, v.y);
    mxx = fmax(mxx, v.x);
    mxy = fmax(mxy, v.y);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mnx = fmin(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
    mny = fmin(mny, __shfl_xor_sync(0xffffffffu, mny, o));
    mxx = fmax(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
    mxy = fmax(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    s[0][w] = mnx;
    s[1][w] = mny;
    s[2][w] = mxx;
    s[3][w] = mxy;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double r = (threadIdx.x < 2) ? DBL_MAX : -DBL_MAX;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++)
      r = (threadIdx.x < 2) ? fmin(r, s[threadIdx.x][k]) : fmax(r, s[threadIdx.x][k]);
    part[blockIdx.x * 4 + threadIdx.x] = r;
  }
}

__global__ void scale_kernel(int n, const double2 *__restrict__ x, double scale, float2 *__restrict__ pos,
                             double2 *__restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const double2 v = x[c];
  const double2 s = make_double2(v.x * scale, v.y * scale);
  out[c] = s;
  pos[c] = make_float2((float)s.x, (float)s.y);
}

__global__ void init_tree_kernel(int n, int *level, int *parent, int *firstpos, double2 *off) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  level[c] = c == 0 ? 0 : kNoLevel;
  parent[c] = c == 0 ? -1 : INT_MAX;
  firstpos[c] = INT_MAX;
  off[c] = c == 0 ? make_double2(1.0, 1.0) : make_double2(0.0, 0.0);
}

// parents INT_MAX (unreached) become -1
__global__ void parent_fix_kernel(int n, int *parent) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n && parent[c] == INT_MAX) parent[c] = -1;
}

}  // namespace

// Breadth-first greedy start of the context's graph into ctx->pos; the FP64
// coordinates are also left in ctx->stage (the staging buffer of
// bl_get_coordinates).
int bfs_init(bl_ctx *ctx) {
  const int n = ctx->g.n;
  cudaStream_t st = ctx->stream;
  const int blocks = (n + 255) / 256;
  // scratch: level, parent, firstpos, jump[2], lists[2], off[2] (FP64 pairs)
  int *level = nullptr, *parent = nullptr, *firstpos = nullptr, *jp2 = nullptr, *wl0 = nullptr, *wl1 = nullptr;
  double2 *x2 = nullptr;
  unsigned int *cnt = nullptr;
  double *part = nullptr;
  int rc = 0;
  auto ck = [&](cudaError_t e, const char *what) {
    if (e != cudaSuccess && !rc) rc = bl_cuda_fail(ctx, e, what);
  };
  ck(cudaMalloc(&level, sizeof(int) * n), "cudaMalloc");
  ck(cudaMalloc(&parent, sizeof(int) * n), "cudaMalloc");
  ck(cudaMalloc(&firstpos, sizeof(int) * n), "cudaMalloc");
  ck(cudaMalloc(&jp2, sizeof(int) * n), "cudaMalloc");
  ck(cudaMalloc(&wl0, sizeof(int) * n), "cudaMalloc");
  ck(cudaMalloc(&wl1, sizeof(int) * n), "cudaMalloc");
  ck(cudaMalloc(&x2, sizeof(double2) * n), "cudaMalloc");
  ck(cudaMalloc(&cnt, sizeof(unsigned int) * 4), "cudaMalloc");
  ck(cudaMalloc(&part, sizeof(double) * 4 * 1024), "cudaMalloc");
  double2 *off = ctx->stage;  // n FP64 pairs
  if (!rc) {
    init_tree_kernel<<<blocks, 256, 0, st>>>(n, level, parent, firstpos, off);
    const int zero = 0;
    const unsigned int one[3] = {1u, 0u, 0u};
    ck(cudaMemcpyAsync(wl0, &zero, sizeof(int), cudaMemcpyHostToDevice, st), "H2D");
    ck(cudaMemcpyAsync(cnt, one, sizeof(one), cudaMemcpyHostToDevice, st), "H2D");
    ck(cudaMemsetAsync(ctx->s.status, 0, sizeof(DevStatus), st), "memset");
    int occ = 0;
    ck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, tree_bfs_kernel, kThreads, 0), "occupancy");
    TreeArgs a{n, ctx->g.rowptr, ctx->g.colids, level, parent, {wl0, wl1}, cnt, ctx->s.status};
    void *args[] = {&a};
    bl_time_begin(ctx, "tree_bfs_kernel");
    if (!rc && occ > 0)
      ck(cudaLaunchCooperativeKernel((const void *)tree_bfs_kernel, dim3(ctx->num_sms * std::min(occ, 2)),
                                     dim3(kThreads), args, 0, st),
         "BFS launch");
    bl_time_end(ctx, "tree_bfs_kernel");
    ctx->launches += 2;
    parent_fix_kernel<<<blocks, 256, 0, st>>>(n, parent);
    const unsigned int wblocks = (unsigned int)(((long long)n * 32 + 255) / 256);
    first_pos_kernel<<<wblocks, 256, 0, st>>>(n, ctx->g.rowptr, ctx->g.colids, parent, firstpos);
    child_offset_kernel<<<wblocks, 256, 0, st>>>(n, ctx->g.rowptr, ctx->g.colids, parent, firstpos, off);
    ctx->launches += 3;
    ck(cudaGetLastError(), "tree kernels");
  }
  // positions: pointer jumping up the tree, until no pointer is left
  double2 *xa = off, *xb = x2;
  int *ja = parent, *jb = jp2;
  for (int round = 0; round < 40 && !rc; round++) {
    ck(cudaMemsetAsync(cnt + 3, 0, sizeof(unsigned int), st), "memset");
    jump_kernel<<<blocks, 256, 0, st>>>(n, xa, ja, xb, jb, cnt + 3);
    ctx->launches++;
    std::swap(xa, xb);
    std::swap(ja, jb);
    unsigned int more = 0;
    ck(cudaMemcpyAsync(&more, cnt + 3, sizeof(more), cudaMemcpyDeviceToHost, st), "D2H");
    ck(cudaStreamSynchronize(st), "sync");
    if (!more) break;  // every vertex now holds its sum up to the root
  }
  if (!rc) {
    const int rb = std::min(1024, blocks);
    range_kernel<<<rb, 256, 0, st>>>(n, xa, level, part);
    ctx->launches++;
    std::vector<double> hp(4 * (size_t)rb);
    ck(cudaMemcpyAsync(hp.data(), part, sizeof(double) * 4 * rb, cudaMemcpyDeviceToHost, st), "D2H");
    ck(cudaStreamSynchronize(st), "sync");
    double mnx = DBL_MAX, mny = DBL_MAX, mxx = -DBL_MAX, mxy = -DBL_MAX;
    for (int b = 0; b < rb; b++) {
      mnx = std::min(mnx, hp[4 * b]);
      mny = std::min(mny, hp[4 * b + 1]);
      mxx = std::max(mxx, hp[4 * b + 2]);
      mxy = std::max(mxy, hp[4 * b + 3]);
    }
    const double width = std::max(mxx - mnx, mxy - mny);
    const double scale = width > 0 ? 2.0 * 3.0 / width : 1.0;  // 2 * MAXMIN / range
    scale_kernel<<<blocks, 256, 0, st>>>(n, xa, scale, ctx->pos, ctx->stage);
    ctx->launches++;
    ck(cudaGetLastError(), "scale");
    ck(cudaStreamSynchronize(st), "sync");
  }
  if (!rc) rc = bl_check_status(ctx);
  cudaFree(level);
  cudaFree(parent);
  cudaFree(firstpos);
  cudaFree(jp2);
  cudaFree(wl0);
  cudaFree(wl1);
  cudaFree(x2);
  cudaFree(cnt);
  cudaFree(part);
  return rc;
}

}  // namespace bl

extern "C" int bl_bfs_init(bl_ctx *ctx) try {
  if (!ctx) return BL_ERR_ARG;
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  return bl::bfs_init(ctx);
} catch (...) {
  return bl_host_exception(ctx);
}

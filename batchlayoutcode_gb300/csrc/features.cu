// features.cu -- the 16 input features of the learned initializer.
//
// A 3-layer message-passing network sees only 3 hops, so the features have
// to carry the global shape: they are pivot-MDS coordinates (Brandes & Pich,
// "Eigensolver methods for progressive multidimensional scaling of large
// data", 2006) from 16 pivots, plus degree features:
//   f[0..11]  the first 12 component scores of the double-centred squared
//             hop distances to the pivots, scaled so that component 1 has
//             unit mean square;
//   f[12]     log2(1 + deg), f[13] 1 / (1 + deg),
//   f[14]     mean of log2(1 + deg) over the neighbours,
//   f[15]     log2(n) / 20.
// Hop distances come from one multi-source BFS on the device (a 16-bit
// visited mask per vertex, one level per grid-barrier step, the vertices of
// the level's frontier push their new source bits to their neighbours, which
// join the next frontier list the first time a bit reaches them); all graphs
// of a training set run in the same BFS, each with its own pivots.  The work
// of a level is its frontier (the 1M-vertex random geometric graph has 1,430
// levels), and a block gathers its new frontier vertices in shared memory and
// reserves room for them in the global list with one atomic per level.  Distances to pivots that a vertex cannot
// reach count as one more than the pivot's largest finite distance.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/batchlayout_gb300.h"
#include "learned.h"

namespace bl {

namespace {

constexpr int kP = kPivots;
constexpr unsigned short kUnreached = 0xFFFF;

__global__ void bfs_init_kernel(int n, unsigned int *visited, unsigned int *fr0, unsigned int *fr1,
                                unsigned short *dist) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  visited[v] = 0u;
  fr0[v] = 0u;
  fr1[v] = 0u;
#pragma unroll
  for (int s = 0; s < kP; s++) dist[(size_t)v * kP + s] = kUnreached;
}

// pivots[g * 16 + s]: global vertex of pivot s of graph g; the distinct pivot
// vertices form the frontier list of level 0
__global__ void bfs_seed_kernel(int count, const int *pivots, unsigned int *visited, unsigned int *fr0,
                                unsigned short *dist, int *wl0, unsigned int *cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int p = pivots[i], s = i % kP;
  atomicOr(&visited[p], 1u << s);
  dist[(size_t)p * kP + s] = 0;
  if (atomicOr(&fr0[p], 1u << s) == 0u) wl0[atomicAdd(&cnt[0], 1u)] = p;
}

struct BfsArgs {
  int n;
  const int *rowptr, *colids;
  unsigned int *visited;
  unsigned int *fr[2];   // frontier masks: bits that reached the vertex at the level
  int *wl[2];            // frontier lists
  unsigned int *cnt;     // [3] list lengths, rotating by level
  unsigned short *dist;
  DevStatus *st;
  int max_levels;
};

constexpr int kBfsBuf = 2048;  // new frontier vertices a block gathers per level before spilling

// One cooperative launch, one level per bounded grid barrier.  Level L reads
// the list of level L-1 (fr[(L-1)&1], wl[(L-1)&1], cnt[(L-1)%3]) and builds
// the list of level L; a frontier vertex's mask is cleared once pushed, so a
// mask buffer holds only its own list's vertices.  Lists and masks written by
// other blocks are read through L2 (__ldcg) after the barrier.
__global__ void __launch_bounds__(512) msbfs_kernel(BfsArgs a) {
  __shared__ unsigned int s_count, s_n, s_base;
  __shared__ int s_buf[kBfsBuf];
  unsigned int epoch = 0;
  const unsigned int lane = threadIdx.x & 31u;
  const unsigned int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const unsigned int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int L = 1; L <= a.max_levels; L++) {
    const int cb = (L - 1) & 1, nbuf = L & 1;
    // one read per block; all appends preceded the barrier, so every block
    // sees the same value
    if (threadIdx.x == 0) {
      s_count = ld_acquire_gpu(&a.cnt[(L - 1) % 3]);
      s_n = 0u;
    }
    __syncthreads();
    const unsigned int count = s_count;
    if (count == 0u) break;
    if (blockIdx.x == 0 && threadIdx.x == 0) a.cnt[(L + 1) % 3] = 0u;  // untouched during this level
    // a warp per frontier vertex, a lane per neighbour: a level costs one
    // neighbour's chain of dependent L2 round trips, not deg of them
    for (unsigned int idx = wid; idx < count; idx += nwarps) {
      const int u = __ldcg(&a.wl[cb][idx]);
      const unsigned int m = __ldcg(&a.fr[cb][u]);
      const int e0 = a.rowptr[u], e1 = a.rowptr[u + 1];
      __syncwarp();
      if (lane == 0) a.fr[cb][u] = 0u;
      for (int e = e0 + lane; e < e1; e += 32) {
        const int v = a.colids[e];
        const unsigned int got = m & ~atomicOr(&a.visited[v], m);
        if (!got) continue;
        unsigned int b = got;
        while (b) {
          const int s = __ffs(b) - 1;
          b &= b - 1u;
          a.dist[(size_t)v * kP + s] = (unsigned short)min(L, 65534);
        }
        if (atomicOr(&a.fr[nbuf][v], got) == 0u) {
          const unsigned int slot = atomicAdd(&s_n, 1u);
          if (slot < (unsigned int)kBfsBuf) s_buf[slot] = v;
          else a.wl[nbuf][atomicAdd(&a.cnt[L % 3], 1u)] = v;  // rare spill
        }
      }
    }
    __syncthreads();
    const unsigned int mine = min(s_n, (unsigned int)kBfsBuf);
    if (threadIdx.x == 0 && mine) s_base = atomicAdd(&a.cnt[L % 3], mine);
    __syncthreads();
    for (unsigned int k = threadIdx.x; k < mine; k += blockDim.x) a.wl[nbuf][s_base + k] = s_buf[k];
    if (!grid_barrier(a.st, epoch)) return;
  }
}

// ---- pivot MDS of one graph (vertices [v0, v1)) ---------------------------
__device__ __forceinline__ double hop2(const unsigned short *dist, int v, int s, const int *maxd) {
  const unsigned short d = dist[(size_t)v * kP + s];
  const double h = (d == kUnreached) ? (double)(maxd[s] + 1) : (double)d;
  return h * h;
}

// per block: largest finite distance per pivot
__global__ void mds_max_kernel(int v0, int v1, const unsigned short *dist, int *part) {
  __shared__ int smax[kP];
  if (threadIdx.x < kP) smax[threadIdx.x] = 0;
  __syncthreads();
  int m[kP];
#pragma unroll
  for (int s = 0; s < kP; s++) m[s] = 0;
  for (int v = v0 + blockIdx.x * blockDim.x + threadIdx.x; v < v1; v += gridDim.x * blockDim.x)
#pragma unroll
    for (int s = 0; s < kP; s++) {
      const unsigned short d = dist[(size_t)v * kP + s];
      if (d != kUnreached) m[s] = max(m[s], (int)d);
    }
#pragma unroll
  for (int s = 0; s < kP; s++) atomicMax(&smax[s], m[s]);
  __syncthreads();
  if (threadIdx.x < kP) part[blockIdx.x * kP + threadIdx.x] = smax[threadIdx.x];
}

__device__ void block_sum_doubles(double *vals, int count, double *scratch, double *out) {
  // scratch: blockDim.x / 32 * count doubles; out: count doubles (thread 0 writes)
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = 0; k < count; k++) {
    double v = vals[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) scratch[w * count + k] = v;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < count; k += blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < nw; j++) s += scratch[j * count + k];
    out[k] = s;
  }
}

// per block: column sums of the squared distances
__global__ void __launch_bounds__(256) mds_colsum_kernel(int v0, int v1, const unsigned short *dist,
                                                         const int *maxd, double *part) {
  __shared__ double scratch[8 * kP];
  double c[kP];
#pragma unroll
  for (int s = 0; s < kP; s++) c[s] = 0.0;
  for (int v = v0 + blockIdx.x * blockDim.x + threadIdx.x; v < v1; v += gridDim.x * blockDim.x)
#pragma unroll
    for (int s = 0; s < kP; s++) c[s] += hop2(dist, v, s, maxd);
  block_sum_doubles(c, kP, scratch, part + (size_t)blockIdx.x * kP);
}

// per block: Gram matrix sum_v C_v C_v^T of the double-centred rows
// C[v][s] = -0.5 (D2[v][s] - r_v - c_s + g), upper triangle (136 values):
// a tile of 256 rows is staged in shared memory, thread t < 136 owns entry t.
__global__ void __launch_bounds__(256) mds_gram_kernel(int v0, int v1, const unsigned short *dist, const int *maxd,
                                                       const double *colmean, double grand, double *part) {
  __shared__ double cbuf[256][kP + 1];
  const int tid = threadIdx.x;
  int pi = 0, pj = 0;
  if (tid < 136) {
    int k = tid, i = 0;
    while (k >= kP - i) {
      k -= kP - i;
      i++;
    }
    pi = i;
    pj = i + k;
  }
  double acc = 0.0;
  for (int base = v0 + blockIdx.x * 256; base < v1; base += gridDim.x * 256) {
    const int v = base + tid;
    if (v < v1) {
      double d2[kP], r = 0.0;
#pragma unroll
      for (int s = 0; s < kP; s++) {
        d2[s] = hop2(dist, v, s, maxd);
        r += d2[s];
      }
      r *= 1.0 / kP;
#pragma unroll
      for (int s = 0; s < kP; s++) cbuf[tid][s] = -0.5 * (d2[s] - r - colmean[s] + grand);
    } else {
#pragma unroll
      for (int s = 0; s < kP; s++) cbuf[tid][s] = 0.0;
    }
    __syncthreads();
    if (tid < 136)
      for (int rr = 0; rr < 256; rr++) acc = fma(cbuf[rr][pi], cbuf[rr][pj], acc);
    __syncthreads();
  }
  if (tid < 136) part[(size_t)blockIdx.x * 136 + tid] = acc;
}

struct ProjectArgs {
  int v0, v1, n_graph;
  const int *rowptr;  // global CSR
  const int *colids;
  const unsigned short *dist;
  const int *maxd;
  const double *colmean;
  double grand;
  const double *V;  // 16 x 12, column j = eigenvector j
  double inv_scale;
  float *features;  // global n x 16
};

__global__ void mds_project_kernel(ProjectArgs a) {
  const int v = a.v0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= a.v1) return;
  double d2[kP], r = 0.0;
#pragma unroll
  for (int s = 0; s < kP; s++) {
    d2[s] = hop2(a.dist, v, s, a.maxd);
    r += d2[s];
  }
  r *= 1.0 / kP;
  double c[kP];
#pragma unroll
  for (int s = 0; s < kP; s++) c[s] = -0.5 * (d2[s] - r - a.colmean[s] + a.grand);
  float *f = a.features + (size_t)v * kFeat;
#pragma unroll
  for (int j = 0; j < 12; j++) {
    double y = 0.0;
#pragma unroll
    for (int s = 0; s < kP; s++) y = fma(c[s], a.V[s * 12 + j], y);
    f[j] = (float)(y * a.inv_scale);
  }
  const int e0 = a.rowptr[v], e1 = a.rowptr[v + 1];
  const int deg = e1 - e0;
  float m = 0.f;
  for (int e = e0; e < e1; e++) {
    const int u = a.colids[e];
    m += log2f(1.0f + (float)(a.rowptr[u + 1] - a.rowptr[u]));
  }
  f[12] = log2f(1.0f + (float)deg);
  f[13] = 1.0f / (1.0f + (float)deg);
  f[14] = deg > 0 ? m / (float)deg : 0.0f;
  f[15] = log2f((float)a.n_graph) / 20.0f;
}

}  // namespace

// splitmix64 (Steele, Lea & Flood, "Fast splittable pseudorandom number
// generators", 2014)
static uint64_t splitmix64(uint64_t &x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

void choose_pivots(int n, uint64_t seed, int *out) {
  uint64_t x = seed;
  int k = 0;
  if (n <= kP) {
    for (int s = 0; s < kP; s++) out[s] = s % n;
    return;
  }
  while (k < kP) {
    const int p = (int)(splitmix64(x) % (uint64_t)n);
    bool dup = false;
    for (int j = 0; j < k; j++) dup |= out[j] == p;
    if (!dup) out[k++] = p;
  }
}

// Cyclic Jacobi eigenvalue iteration (Golub & Van Loan, "Matrix Computations",
// section 8.5) for a symmetric m x m matrix; eigenvalues descending, column j
// of V the eigenvector of eigenvalue j with its largest-magnitude entry
// positive.
void jacobi_eigen(int m, std::vector<double> A, std::vector<double> &lam, std::vector<double> &V) {
  V.assign(m * m, 0.0);
  for (int i = 0; i < m; i++) V[i * m + i] = 1.0;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < m; i++)
      for (int j = 0; j < m; j++) {
        tot += A[i * m + j] * A[i * m + j];
        if (i != j) off += A[i * m + j] * A[i * m + j];
      }
    if (off <= 1e-30 * tot || off == 0.0) break;
    for (int p = 0; p < m; p++)
      for (int q = p + 1; q < m; q++) {
        const double apq = A[p * m + q];
        if (apq == 0.0) continue;
        const double theta = (A[q * m + q] - A[p * m + p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < m; k++) {
          const double akp = A[k * m + p], akq = A[k * m + q];
          A[k * m + p] = c * akp - s * akq;
          A[k * m + q] = s * akp + c * akq;
        }
        for (int k = 0; k < m; k++) {
          const double apk = A[p * m + k], aqk = A[q * m + k];
          A[p * m + k] = c * apk - s * aqk;
          A[q * m + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < m; k++) {
          const double vkp = V[k * m + p], vkq = V[k * m + q];
          V[k * m + p] = c * vkp - s * vkq;
          V[k * m + q] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> idx(m);
  for (int i = 0; i < m; i++) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return A[x * m + x] > A[y * m + y]; });
  std::vector<double> V2(m * m);
  lam.assign(m, 0.0);
  for (int j = 0; j < m; j++) {
    const int c = idx[j];
    lam[j] = A[c * m + c];
    int arg = 0;
    for (int k = 1; k < m; k++)
      if (std::fabs(V[k * m + c]) > std::fabs(V[arg * m + c])) arg = k;
    const double sg = V[arg * m + c] < 0 ? -1.0 : 1.0;
    for (int k = 0; k < m; k++) V2[k * m + j] = sg * V[k * m + c];
  }
  V = V2;
}

// Features of the graphs [voff[g], voff[g+1]) of a block-diagonal device CSR.
int compute_features(bl_ctx *ctx, int num_graphs, const int *voff, int n, const int *d_rowptr, const int *d_colids,
                     const int *pivots, float *d_features, unsigned short *d_dist) {
  cudaStream_t st = ctx->stream;
  const int P = num_graphs * kP;
  unsigned int *visited = nullptr, *fr0 = nullptr, *fr1 = nullptr, *cnt = nullptr;
  int *d_piv = nullptr, *d_maxd = nullptr, *d_ipart = nullptr, *wl0 = nullptr, *wl1 = nullptr;
  double *d_dpart = nullptr, *d_colmean = nullptr, *d_V = nullptr;
  const int kBlocks = 256;
  int rc = 0;
  auto cleanup = [&]() {
    cudaFree(visited); cudaFree(fr0); cudaFree(fr1); cudaFree(cnt); cudaFree(wl0); cudaFree(wl1);
    cudaFree(d_piv); cudaFree(d_maxd);
    cudaFree(d_ipart); cudaFree(d_dpart); cudaFree(d_colmean); cudaFree(d_V);
  };
  auto ck = [&](cudaError_t e, const char *w) {
    if (e != cudaSuccess && !rc) rc = bl_cuda_fail(ctx, e, w);
    return rc == 0;
  };
  ck(cudaMalloc(&visited, sizeof(unsigned int) * n), "cudaMalloc");
  ck(cudaMalloc(&fr0, sizeof(unsigned int) * n), "cudaMalloc");
  ck(cudaMalloc(&fr1, sizeof(unsigned int) * n), "cudaMalloc");
  ck(cudaMalloc(&cnt, 3 * sizeof(unsigned int)), "cudaMalloc");
  ck(cudaMalloc(&wl0, sizeof(int) * n), "cudaMalloc");
  ck(cudaMalloc(&wl1, sizeof(int) * n), "cudaMalloc");
  ck(cudaMalloc(&d_piv, sizeof(int) * P), "cudaMalloc");
  ck(cudaMalloc(&d_maxd, sizeof(int) * kP), "cudaMalloc");
  ck(cudaMalloc(&d_ipart, sizeof(int) * kBlocks * kP), "cudaMalloc");
  ck(cudaMalloc(&d_dpart, sizeof(double) * kBlocks * 136), "cudaMalloc");
  ck(cudaMalloc(&d_colmean, sizeof(double) * kP), "cudaMalloc");
  ck(cudaMalloc(&d_V, sizeof(double) * kP * 12), "cudaMalloc");
  if (rc) {
    cleanup();
    return rc;
  }
  ck(cudaMemcpyAsync(d_piv, pivots, sizeof(int) * P, cudaMemcpyHostToDevice, st), "H2D");
  ck(cudaMemsetAsync(cnt, 0, 3 * sizeof(unsigned int), st), "memset");
  bfs_init_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, visited, fr0, fr1, d_dist);
  bfs_seed_kernel<<<(P + 255) / 256, 256, 0, st>>>(P, d_piv, visited, fr0, d_dist, wl0, cnt);
  ck(cudaMemsetAsync(&ctx->s.status->barrier, 0, sizeof(unsigned int), st), "memset");
  ctx->launches += 2;
  {
    int occ = 0;
    ck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, msbfs_kernel, 512, 0), "occupancy");
    if (!rc && occ < 1) rc = bl_fail(ctx, BL_ERR_TOO_LARGE, "BFS kernel cannot be resident");
    BfsArgs b{n, d_rowptr, d_colids, visited, {fr0, fr1}, {wl0, wl1}, cnt, d_dist, ctx->s.status, n + 1};
    void *args[] = {&b};
    bl_time_begin(ctx, "msbfs_kernel");
    if (!rc)
      ck(cudaLaunchCooperativeKernel((const void *)msbfs_kernel, dim3(ctx->num_sms * std::min(occ, 2)), dim3(512),
                                     args, 0, st),
         "BFS launch");
    bl_time_end(ctx, "msbfs_kernel");
    ctx->launches++;
  }
  if (!rc) ck(cudaStreamSynchronize(st), "BFS");
  if (!rc) rc = bl_check_status(ctx);
  std::vector<int> ipart(kBlocks * kP);
  std::vector<double> dpart(kBlocks * 136);
  for (int g = 0; g < num_graphs && !rc; g++) {
    const int v0 = voff[g], v1 = voff[g + 1], ng = v1 - v0;
    const int blocks = std::max(1, std::min(kBlocks, (ng + 255) / 256));
    mds_max_kernel<<<blocks, 256, 0, st>>>(v0, v1, d_dist, d_ipart);
    ck(cudaMemcpyAsync(ipart.data(), d_ipart, sizeof(int) * blocks * kP, cudaMemcpyDeviceToHost, st), "D2H");
    ck(cudaStreamSynchronize(st), "sync");
    int maxd[kP] = {0};
    for (int b = 0; b < blocks; b++)
      for (int s = 0; s < kP; s++) maxd[s] = std::max(maxd[s], ipart[b * kP + s]);
    ck(cudaMemcpyAsync(d_maxd, maxd, sizeof(maxd), cudaMemcpyHostToDevice, st), "H2D");
    mds_colsum_kernel<<<blocks, 256, 0, st>>>(v0, v1, d_dist, d_maxd, d_dpart);
    ck(cudaMemcpyAsync(dpart.data(), d_dpart, sizeof(double) * blocks * kP, cudaMemcpyDeviceToHost, st), "D2H");
    ck(cudaStreamSynchronize(st), "sync");
    double colmean[kP], grand = 0.0;
    for (int s = 0; s < kP; s++) {
      double t = 0.0;
      for (int b = 0; b < blocks; b++) t += dpart[b * kP + s];
      colmean[s] = t / ng;
      grand += colmean[s];
    }
    grand /= kP;
    ck(cudaMemcpyAsync(d_colmean, colmean, sizeof(colmean), cudaMemcpyHostToDevice, st), "H2D");
    mds_gram_kernel<<<blocks, 256, 0, st>>>(v0, v1, d_dist, d_maxd, d_colmean, grand, d_dpart);
    ck(cudaMemcpyAsync(dpart.data(), d_dpart, sizeof(double) * blocks * 136, cudaMemcpyDeviceToHost, st), "D2H");
    ck(cudaStreamSynchronize(st), "sync");
    std::vector<double> S(kP * kP, 0.0);
    int k = 0;
    for (int i = 0; i < kP; i++)
      for (int j = i; j < kP; j++, k++) {
        double t = 0.0;
        for (int b = 0; b < blocks; b++) t += dpart[b * 136 + k];
        S[i * kP + j] = S[j * kP + i] = t;
      }
    std::vector<double> lam, V;
    jacobi_eigen(kP, S, lam, V);
    std::vector<double> V12(kP * 12);
    for (int s = 0; s < kP; s++)
      for (int j = 0; j < 12; j++) V12[s * 12 + j] = V[s * kP + j];
    ck(cudaMemcpyAsync(d_V, V12.data(), sizeof(double) * kP * 12, cudaMemcpyHostToDevice, st), "H2D");
    ProjectArgs pa{v0, v1, ng, d_rowptr, d_colids, d_dist, d_maxd, d_colmean, grand, d_V,
                   lam[0] > 0 ? 1.0 / std::sqrt(lam[0] / ng) : 0.0, d_features};
    mds_project_kernel<<<(ng + 255) / 256, 256, 0, st>>>(pa);
    ctx->launches += 4;
    ck(cudaGetLastError(), "MDS kernels");
  }
  if (!rc) ck(cudaStreamSynchronize(st), "features");
  cleanup();
  return rc;
}

}  // namespace bl

extern "C" {

int bl_learned_features(bl_ctx *ctx, int n, const int *rowptr, const int *colids, int seed, const int *pivots,
                        float *features, unsigned short *dist, int *pivots_out) try {
  using namespace bl;
  if (!ctx || n < 1 || !rowptr || !features) return BL_ERR_ARG;
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  const long long nnz = rowptr[n];
  for (int v = 0; v < n; v++)
    if (rowptr[v + 1] < rowptr[v]) return bl_fail(ctx, BL_ERR_ARG, "rowptr decreases");
  for (long long e = 0; e < nnz; e++)
    if (colids[e] < 0 || colids[e] >= n) return bl_fail(ctx, BL_ERR_ARG, "colid out of range");
  int piv[kPivots];
  if (pivots) {
    for (int s = 0; s < kPivots; s++) {
      if (pivots[s] < 0 || pivots[s] >= n) return bl_fail(ctx, BL_ERR_ARG, "pivot out of range");
      piv[s] = pivots[s];
    }
  } else {
    choose_pivots(n, (uint64_t)seed, piv);
  }
  if (pivots_out) std::memcpy(pivots_out, piv, sizeof(piv));
  if (!ctx->s.status) {
    BL_CUDA(ctx, cudaMalloc(&ctx->s.status, sizeof(DevStatus)));
    BL_CUDA(ctx, cudaMemset(ctx->s.status, 0, sizeof(DevStatus)));
  }
  int *d_rp = nullptr, *d_ci = nullptr;
  float *d_f = nullptr;
  unsigned short *d_d = nullptr;
  int rc = 0;
  auto ck = [&](cudaError_t e, const char *w) {
    if (e != cudaSuccess && !rc) rc = bl_cuda_fail(ctx, e, w);
  };
  ck(cudaMalloc(&d_rp, sizeof(int) * (n + 1)), "cudaMalloc");
  ck(cudaMalloc(&d_ci, sizeof(int) * std::max<long long>(nnz, 1)), "cudaMalloc");
  ck(cudaMalloc(&d_f, sizeof(float) * kFeat * (size_t)n), "cudaMalloc");
  ck(cudaMalloc(&d_d, sizeof(unsigned short) * kPivots * (size_t)n), "cudaMalloc");
  if (!rc) {
    ck(cudaMemcpy(d_rp, rowptr, sizeof(int) * (n + 1), cudaMemcpyHostToDevice), "H2D");
    if (nnz) ck(cudaMemcpy(d_ci, colids, sizeof(int) * nnz, cudaMemcpyHostToDevice), "H2D");
  }
  const int voff[2] = {0, n};
  if (!rc) rc = compute_features(ctx, 1, voff, n, d_rp, d_ci, piv, d_f, d_d);
  if (!rc) ck(cudaMemcpy(features, d_f, sizeof(float) * kFeat * (size_t)n, cudaMemcpyDeviceToHost), "D2H");
  if (!rc && dist) ck(cudaMemcpy(dist, d_d, sizeof(unsigned short) * kPivots * (size_t)n, cudaMemcpyDeviceToHost), "D2H");
  cudaFree(d_rp);
  cudaFree(d_ci);
  cudaFree(d_f);
  cudaFree(d_d);
  return rc;
} catch (...) {
  return bl_host_exception(ctx);
}

}  // extern "C"

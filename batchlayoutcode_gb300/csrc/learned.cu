// learned.cu -- training and use of the learned initializer.
//
// The network predicts a correction to the graph's pivot-MDS shape y (input
// features 0 and 1): the start is p = y + net(features), scaled to a
// predicted mean edge length.
//
// Training (bl_learned_train): the graphs of a training set form one
// block-diagonal graph on the device; their features come from one
// multi-source BFS and a pivot MDS per graph (features.cu).  Each target
// layout (what algo 4 produced for that graph) is centred and fitted to y by
// the similarity (scale times the Procrustes rotation or reflection) that
// minimises the squared distance; the network learns the residual
// fit(target) - y.  Full-batch Adam on sum_g mean_v |net_v - residual_v|^2 / G
// with the tcgen05 kernels of mpnn.cu.  A least-squares model
// log l = a + b log n + c log(mean degree) of the targets' mean edge length l
// gives the scale at inference.
//
// Use (bl_learned_init): features, one forward pass, p = y + net, scaled to
// the predicted mean edge length.  bl_learned_layout adds the refinement by Barnes-Hut
// iterations until a target energy is reached, and falls back to the greedy
// DFS start with the plain iteration count when the refined energy stays
// above the target.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/batchlayout_gb300.h"
#include "learned.h"
#include "mpnn.h"

namespace bl {

namespace {

// p = y + net (unscaled start) into pos
__global__ void residual_start_kernel(const float *__restrict__ net, const float *__restrict__ feat, int n,
                                      float2 *__restrict__ pos) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n) pos[v] = make_float2(net[2 * v] + feat[(size_t)v * kFeat], net[2 * v + 1] + feat[(size_t)v * kFeat + 1]);
}

// per block: sum over the CSR entries of |p_v - p_u| (each edge twice)
__global__ void edge_length_kernel(int n, const int *__restrict__ rowptr, const int *__restrict__ colids,
                                   const float2 *__restrict__ pos, double *part) {
  __shared__ double red[8];
  double s = 0.0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const float2 p = pos[v];
    for (int e = rowptr[v]; e < rowptr[v + 1]; e++) {
      const float2 q = pos[colids[e]];
      s += sqrt((double)(p.x - q.x) * (p.x - q.x) + (double)(p.y - q.y) * (p.y - q.y));
    }
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    part[blockIdx.x] = t;
  }
}

// per block: sum_v A_v . R_v and sum_v |A_v|^2 with A_v the FR attraction
// sum_u W |p_u - p_v| (p_u - p_v) (algorithms.cpp:1056-1058) and R_v the
// Barnes-Hut sum of unit vectors towards the cells (BarnesHut.h:69-86)
__global__ void scale_fit_kernel(int n, const int *__restrict__ rowptr, const int *__restrict__ colids,
                                 const float2 *__restrict__ pos, const float2 *__restrict__ rep, float W,
                                 double *part) {
  __shared__ double red[2][8];
  double ar = 0.0, aa = 0.0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const float2 p = pos[v];
    double ax = 0.0, ay = 0.0;
    for (int e = rowptr[v]; e < rowptr[v + 1]; e++) {
      const float2 q = pos[colids[e]];
      const double dx = (double)q.x - p.x, dy = (double)q.y - p.y;
      const double sc = (double)W * sqrt(dx * dx + dy * dy);
      ax += sc * dx;
      ay += sc * dy;
    }
    const float2 r = rep[v];
    ar += ax * r.x + ay * r.y;
    aa += ax * ax + ay * ay;
  }
  for (int o = 16; o > 0; o >>= 1) {
    ar += __shfl_xor_sync(0xffffffffu, ar, o);
    aa += __shfl_xor_sync(0xffffffffu, aa, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = ar;
    red[1][threadIdx.x >> 5] = aa;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0.0, t1 = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
      t0 += red[0][w];
      t1 += red[1][w];
    }
    part[2 * blockIdx.x] = t0;
    part[2 * blockIdx.x + 1] = t1;
  }
}

__global__ void scale_pos_kernel(float2 *pos, int n, float s) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < n) pos[v] = make_float2(pos[v].x * s, pos[v].y * s);
}

__global__ void f32_to_bf16_kernel(const float *__restrict__ in, __nv_bfloat16 *__restrict__ out, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = __float2bfloat16_rn(in[i]);
}

double wall_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// orthogonal R (rotation or reflection) maximising tr(R^T M), M 2x2 row-major
void procrustes2(const double M[4], double R[4]) {
  const double tr = std::atan2(M[2] - M[1], M[0] + M[3]);
  const double vr = std::hypot(M[2] - M[1], M[0] + M[3]);
  const double tf = std::atan2(M[1] + M[2], M[0] - M[3]);
  const double vf = std::hypot(M[1] + M[2], M[0] - M[3]);
  if (vr >= vf) {
    R[0] = std::cos(tr); R[1] = -std::sin(tr);
    R[2] = std::sin(tr); R[3] = std::cos(tr);
  } else {
    R[0] = std::cos(tf); R[1] = std::sin(tf);
    R[2] = std::sin(tf); R[3] = -std::cos(tf);
  }
}

double predict_edge_length(const double *sm, int n, double mean_degree) {
  return std::exp(sm[0] + sm[1] * std::log((double)std::max(n, 1)) + sm[2] * std::log(std::max(mean_degree, 1e-3)));
}

}  // namespace

constexpr int kParts = 256;

// Learned coordinates for the context's graph into ctx->pos.
int learned_init(bl_ctx *ctx, const float *params, const double *scale_model, int seed) {
  const int n = ctx->g.n;
  if (n < 2) return bl_fail(ctx, BL_ERR_ARG, "learned init needs at least two vertices");
  if (int rc = mpnn_set_params_device(ctx, params)) return rc;
  if (int rc = mpnn_prepare(ctx, n)) return rc;
  float *d_f = nullptr;
  unsigned short *d_d = nullptr;
  BL_CUDA(ctx, cudaMalloc(&d_f, sizeof(float) * kFeat * (size_t)n));
  if (cudaMalloc(&d_d, sizeof(unsigned short) * kPivots * (size_t)n) != cudaSuccess) {
    cudaFree(d_f);
    return bl_fail(ctx, BL_ERR_CUDA, "cudaMalloc");
  }
  int piv[kPivots];
  choose_pivots(n, (uint64_t)seed, piv);
  const int voff[2] = {0, n};
  int rc = compute_features(ctx, 1, voff, n, ctx->g.rowptr, ctx->g.colids, piv, d_f, d_d);
  if (!rc) {
    f32_to_bf16_kernel<<<(int)((16LL * n + 255) / 256), 256, 0, ctx->stream>>>(d_f, mpnn_input(ctx), 16LL * n);
    ctx->launches++;
    rc = mpnn_forward(ctx, n, ctx->g.rowptr, ctx->g.colids, false);
  }
  if (!rc) {
    residual_start_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(mpnn_output(ctx), d_f, n, ctx->pos);
    double *d_part = nullptr;
    std::vector<double> part(kParts);
    if (cudaMalloc(&d_part, sizeof(double) * kParts) != cudaSuccess) rc = bl_fail(ctx, BL_ERR_CUDA, "cudaMalloc");
    if (!rc) {
      edge_length_kernel<<<kParts, 256, 0, ctx->stream>>>(n, ctx->g.rowptr, ctx->g.colids, ctx->pos, d_part);
      if (cudaMemcpyAsync(part.data(), d_part, sizeof(double) * kParts, cudaMemcpyDeviceToHost, ctx->stream) !=
              cudaSuccess ||
          cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        rc = bl_fail(ctx, BL_ERR_CUDA, "learned init");
    }
    cudaFree(d_part);
    if (!rc) {
      double tot = 0.0;
      for (double x : part) tot += x;
      const double mean_len = ctx->g.nnz > 0 ? tot / (double)ctx->g.nnz : 0.0;
      const double want = predict_edge_length(scale_model, n, (double)ctx->g.nnz / n);
      const float sc = mean_len > 0.0 ? (float)(want / mean_len) : 1.0f;
      scale_pos_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(ctx->pos, n, sc);
      ctx->launches += 3;
    }
    // Energy-optimal scale of this shape: the Barnes-Hut repulsion R is
    // invariant under scaling (unit vectors, scale-free opening test) while
    // the attraction A grows with the square of the scale, so
    // sum_v |k^2 A_v - R_v|^2 is least at k^2 = sum A.R / sum |A|^2.
    if (!rc) rc = ensure_bh_scratch(ctx);
    if (!rc) rc = bh_build(ctx, ctx->pos, 1.2);
    if (!rc) rc = bh_traverse(ctx, 1.2, false, 0);
    if (!rc) {
      double *d_p2 = nullptr;
      std::vector<double> p2(2 * kParts);
      if (cudaMalloc(&d_p2, sizeof(double) * 2 * kParts) != cudaSuccess) rc = bl_fail(ctx, BL_ERR_CUDA, "cudaMalloc");
      if (!rc) {
        scale_fit_kernel<<<kParts, 256, 0, ctx->stream>>>(n, ctx->g.rowptr, ctx->g.colids, ctx->pos, ctx->s.rep,
                                                          (float)ctx->weight, d_p2);
        ctx->launches++;
        if (cudaMemcpyAsync(p2.data(), d_p2, sizeof(double) * 2 * kParts, cudaMemcpyDeviceToHost, ctx->stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(ctx->stream) != cudaSuccess)
          rc = bl_fail(ctx, BL_ERR_CUDA, "learned init scale");
      }
      cudaFree(d_p2);
      if (!rc) {
        double ar = 0.0, aa = 0.0;
        for (int b = 0; b < kParts; b++) {
          ar += p2[2 * b];
          aa += p2[2 * b + 1];
        }
        if (ar > 0.0 && aa > 0.0) {
          scale_pos_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(ctx->pos, n, (float)std::sqrt(ar / aa));
          ctx->launches++;
        }
      }
    }
    if (!rc && cudaStreamSynchronize(ctx->stream) != cudaSuccess) rc = bl_fail(ctx, BL_ERR_CUDA, "learned init");
  }
  if (!rc) rc = bl_check_status(ctx);
  cudaFree(d_f);
  cudaFree(d_d);
  return rc;
}

}  // namespace bl

extern "C" {

int bl_learned_train(bl_ctx *ctx, int num_graphs, const int *vertex_offset, const long long *edge_offset,
                     const int *rowptr, const int *colids, const double *layouts, int epochs, double lr, int seed,
                     float *params, double *scale_model, double *loss_history) try {
  using namespace bl;
  if (!ctx || num_graphs < 1 || !vertex_offset || !edge_offset || !rowptr || !layouts || !params || !scale_model ||
      epochs < 0 || !(lr > 0))
    return BL_ERR_ARG;
  if (vertex_offset[0] != 0) return bl_fail(ctx, BL_ERR_ARG, "vertex_offset[0] must be 0");
  if (edge_offset[0] != 0 || edge_offset[num_graphs] < 0 || edge_offset[num_graphs] > 2147483647LL)
    return bl_fail(ctx, BL_ERR_ARG, "edge_offset must start at 0 and end within int32");
  if (edge_offset[num_graphs] > 0 && !colids) return bl_fail(ctx, BL_ERR_ARG, "null colids");
  for (int g = 0; g < num_graphs; g++)  // before the offsets size anything
    if ((long long)vertex_offset[g + 1] - vertex_offset[g] < 2)
      return bl_fail(ctx, BL_ERR_ARG, "graph " + std::to_string(g) + " has fewer than two vertices");
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  const int N = vertex_offset[num_graphs];
  std::vector<int> grp(N + 1), gci;
  gci.reserve((size_t)edge_offset[num_graphs]);
  std::vector<int> piv((size_t)num_graphs * kPivots);
  std::vector<double> logn(num_graphs), logd(num_graphs);
  grp[0] = 0;
  for (int g = 0; g < num_graphs; g++) {
    const int v0 = vertex_offset[g], v1 = vertex_offset[g + 1], n = v1 - v0;
    if (n < 2) return bl_fail(ctx, BL_ERR_ARG, "graph " + std::to_string(g) + " has fewer than two vertices");
    const int *rp = rowptr + v0 + g;
    const long long e0 = edge_offset[g], m = edge_offset[g + 1] - e0;
    if (rp[0] != 0 || rp[n] != m) return bl_fail(ctx, BL_ERR_ARG, "rowptr does not match edge_offset");
    for (int v = 0; v < n; v++) {
      if (rp[v + 1] < rp[v]) return bl_fail(ctx, BL_ERR_ARG, "rowptr decreases");
      for (int e = rp[v]; e < rp[v + 1]; e++) {
        const int c = colids[e0 + e];
        if (c < 0 || c >= n) return bl_fail(ctx, BL_ERR_ARG, "colid out of range");
        gci.push_back(v0 + c);
      }
      grp[v0 + v + 1] = (int)gci.size();
    }
    choose_pivots(n, (uint64_t)seed + (uint64_t)g, &piv[(size_t)g * kPivots]);
    for (int s = 0; s < kPivots; s++) piv[(size_t)g * kPivots + s] += v0;
    logn[g] = std::log((double)n);
    logd[g] = std::log(std::max((double)m / n, 1e-3));
  }
  if (gci.empty()) gci.push_back(0);
  if (!ctx->s.status) {
    BL_CUDA(ctx, cudaMalloc(&ctx->s.status, sizeof(DevStatus)));
    BL_CUDA(ctx, cudaMemset(ctx->s.status, 0, sizeof(DevStatus)));
  }
  if (int rc = mpnn_set_params_device(ctx, params)) return rc;
  if (int rc = mpnn_prepare(ctx, N)) return rc;
  int *d_rp = nullptr, *d_ci = nullptr;
  float *d_f = nullptr;
  unsigned short *d_d = nullptr;
  int rc = 0;
  auto ck = [&](cudaError_t e, const char *w) {
    if (e != cudaSuccess && !rc) rc = bl_cuda_fail(ctx, e, w);
  };
  ck(cudaMalloc(&d_rp, sizeof(int) * (N + 1)), "cudaMalloc");
  ck(cudaMalloc(&d_ci, sizeof(int) * gci.size()), "cudaMalloc");
  ck(cudaMalloc(&d_f, sizeof(float) * kFeat * (size_t)N), "cudaMalloc");
  ck(cudaMalloc(&d_d, sizeof(unsigned short) * kPivots * (size_t)N), "cudaMalloc");
  if (!rc) {
    ck(cudaMemcpy(d_rp, grp.data(), sizeof(int) * (N + 1), cudaMemcpyHostToDevice), "H2D");
    ck(cudaMemcpy(d_ci, gci.data(), sizeof(int) * gci.size(), cudaMemcpyHostToDevice), "H2D");
  }
  if (!rc) rc = compute_features(ctx, num_graphs, vertex_offset, N, d_rp, d_ci, piv.data(), d_f, d_d);
  std::vector<float> feat, target, vw;
  std::vector<double> logsig(num_graphs);
  if (!rc) {
    feat.resize((size_t)kFeat * N);
    ck(cudaMemcpy(feat.data(), d_f, sizeof(float) * feat.size(), cudaMemcpyDeviceToHost), "D2H");
    target.resize(2 * (size_t)N);
    vw.resize(N);
    for (int g = 0; g < num_graphs && !rc; g++) {
      const int v0 = vertex_offset[g], v1 = vertex_offset[g + 1], n = v1 - v0;
      double mx = 0, my = 0;
      for (int v = v0; v < v1; v++) {
        mx += layouts[2 * (size_t)v];
        my += layouts[2 * (size_t)v + 1];
      }
      mx /= n;
      my /= n;
      // mean edge length of the target (the scale model's data)
      double el = 0.0;
      for (int v = v0; v < v1; v++)
        for (int e = grp[v]; e < grp[v + 1]; e++) {
          const int u = gci[e];
          el += std::hypot(layouts[2 * (size_t)v] - layouts[2 * (size_t)u],
                           layouts[2 * (size_t)v + 1] - layouts[2 * (size_t)u + 1]);
        }
      const long long m = (long long)grp[v1] - grp[v0];
      logsig[g] = std::log(std::max(m > 0 ? el / (double)m : 1.0, 1e-300));
      // similarity fit of the centred target onto y: t -> s * t R
      double Mx[4] = {0, 0, 0, 0};  // M = t^T y
      for (int v = v0; v < v1; v++) {
        const double tx = layouts[2 * (size_t)v] - mx, ty = layouts[2 * (size_t)v + 1] - my;
        const double y0 = feat[(size_t)v * kFeat], y1 = feat[(size_t)v * kFeat + 1];
        Mx[0] += tx * y0;
        Mx[1] += tx * y1;
        Mx[2] += ty * y0;
        Mx[3] += ty * y1;
      }
      double R[4];
      procrustes2(Mx, R);
      double num = 0.0, den = 0.0;
      for (int v = v0; v < v1; v++) {
        const double tx = layouts[2 * (size_t)v] - mx, ty = layouts[2 * (size_t)v + 1] - my;
        const double rx = tx * R[0] + ty * R[2], ry = tx * R[1] + ty * R[3];
        num += rx * feat[(size_t)v * kFeat] + ry * feat[(size_t)v * kFeat + 1];
        den += rx * rx + ry * ry;
      }
      const double sc = den > 0.0 ? num / den : 0.0;
      for (int v = v0; v < v1; v++) {
        const double tx = layouts[2 * (size_t)v] - mx, ty = layouts[2 * (size_t)v + 1] - my;
        const double rx = sc * (tx * R[0] + ty * R[2]), ry = sc * (tx * R[1] + ty * R[3]);
        target[2 * (size_t)v] = (float)(rx - feat[(size_t)v * kFeat]);
        target[2 * (size_t)v + 1] = (float)(ry - feat[(size_t)v * kFeat + 1]);
        vw[v] = (float)(1.0 / ((double)num_graphs * n));
      }
    }
    ck(cudaMemcpy(mpnn_targets(ctx), target.data(), sizeof(float) * target.size(), cudaMemcpyHostToDevice), "H2D");
    ck(cudaMemcpy(mpnn_vweights(ctx), vw.data(), sizeof(float) * vw.size(), cudaMemcpyHostToDevice), "H2D");
    f32_to_bf16_kernel<<<(int)((16LL * N + 255) / 256), 256, 0, ctx->stream>>>(d_f, mpnn_input(ctx), 16LL * N);
    ctx->launches++;
  }
  for (int e = 0; e < epochs && !rc; e++) {
    const double lr_e = lr * 0.5 * (1.0 + std::cos(M_PI * e / std::max(epochs, 1)));
    rc = mpnn_forward(ctx, N, d_rp, d_ci, true);
    if (!rc) rc = mpnn_backward(ctx, N, d_rp, d_ci);
    double loss = 0.0;
    if (!rc && loss_history) rc = mpnn_loss(ctx, N, &loss);
    if (!rc && loss_history) loss_history[e] = loss;
    if (!rc) rc = mpnn_adam_step(ctx, lr_e);
  }
  if (!rc) ck(cudaStreamSynchronize(ctx->stream), "training");
  if (!rc) rc = bl_check_status(ctx);
  if (!rc) rc = bl_mpnn_get_params(ctx, params);
  if (!rc) {
    // log l = a + b log n + c log(mean degree), least squares (3x3 normal equations)
    double A[9] = {0}, bb[3] = {0};
    for (int g = 0; g < num_graphs; g++) {
      const double x[3] = {1.0, logn[g], logd[g]};
      for (int i = 0; i < 3; i++) {
        bb[i] += x[i] * logsig[g];
        for (int j = 0; j < 3; j++) A[i * 3 + j] += x[i] * x[j];
      }
    }
    for (int i = 0; i < 3; i++) A[i * 3 + i] += 1e-9 * (A[0] + 1.0);  // ridge for singular sets
    // Gaussian elimination with partial pivoting
    int p[3] = {0, 1, 2};
    for (int c = 0; c < 3; c++) {
      int best = c;
      for (int r = c + 1; r < 3; r++)
        if (std::fabs(A[p[r] * 3 + c]) > std::fabs(A[p[best] * 3 + c])) best = r;
      std::swap(p[c], p[best]);
      for (int r = c + 1; r < 3; r++) {
        const double f = A[p[r] * 3 + c] / A[p[c] * 3 + c];
        for (int k = c; k < 3; k++) A[p[r] * 3 + k] -= f * A[p[c] * 3 + k];
        bb[p[r]] -= f * bb[p[c]];
      }
    }
    double sol[3];
    for (int c = 2; c >= 0; c--) {
      double s = bb[p[c]];
      for (int k = c + 1; k < 3; k++) s -= A[p[c] * 3 + k] * sol[k];
      sol[c] = s / A[p[c] * 3 + c];
    }
    for (int i = 0; i < 3; i++) scale_model[i] = sol[i];
  }
  cudaFree(d_rp);
  cudaFree(d_ci);
  cudaFree(d_f);
  cudaFree(d_d);
  return rc;
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_learned_load_model(const char *path, float *params, double *scale_model) try {
  if (!path || !params || !scale_model) return BL_ERR_ARG;
  FILE *f = std::fopen(path, "rb");
  if (!f) return BL_ERR_IO;
  char magic[8];
  unsigned char cnt[4];
  int rc = BL_OK;
  if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, "BLMPNN01", 8) != 0 || std::fread(cnt, 1, 4, f) != 4)
    rc = BL_ERR_IO;
  // little-endian fields, read byte by byte so the host's byte order does not matter
  const unsigned count = cnt[0] | (cnt[1] << 8) | (cnt[2] << 16) | ((unsigned)cnt[3] << 24);
  if (!rc && count != (unsigned)bl::kMpnnParams) rc = BL_ERR_IO;
  for (int i = 0; i < bl::kMpnnParams && !rc; i++) {
    unsigned char b[4];
    if (std::fread(b, 1, 4, f) != 4) {
      rc = BL_ERR_IO;
      break;
    }
    const uint32_t u = b[0] | (b[1] << 8) | (b[2] << 16) | ((uint32_t)b[3] << 24);
    std::memcpy(&params[i], &u, 4);
  }
  for (int i = 0; i < 3 && !rc; i++) {
    unsigned char b[8];
    if (std::fread(b, 1, 8, f) != 8) {
      rc = BL_ERR_IO;
      break;
    }
    uint64_t u = 0;
    for (int k = 7; k >= 0; k--) u = (u << 8) | b[k];
    std::memcpy(&scale_model[i], &u, 8);
  }
  std::fclose(f);
  // a non-finite weight or scale would give a start of NaNs: not a model
  for (int i = 0; i < bl::kMpnnParams && !rc; i++)
    if (!std::isfinite(params[i])) rc = BL_ERR_IO;
  for (int i = 0; i < 3 && !rc; i++)
    if (!std::isfinite(scale_model[i])) rc = BL_ERR_IO;
  return rc;
} catch (...) {
  return bl_host_exception(nullptr);
}

int bl_learned_init(bl_ctx *ctx, const float *params, const double *scale_model, int seed) try {
  if (!ctx || !params || !scale_model) return BL_ERR_ARG;
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  if (ctx->g.n < 2) return bl_fail(ctx, BL_ERR_STATE, "bl_learned_init needs a context with a graph");
  return bl::learned_init(ctx, params, scale_model, seed);
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_learned_layout(bl_ctx *ctx, const float *params, const double *scale_model, int seed, int max_iterations,
                      int batch, double theta, double target_energy, double step0, double *out) try {
  using namespace bl;
  if (!ctx || !params || !scale_model || !out || max_iterations < 1 || batch < 1 || !(theta > 0) || !(step0 > 0))
    return BL_ERR_ARG;
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  if (ctx->g.n < 2) return bl_fail(ctx, BL_ERR_STATE, "bl_learned_layout needs a context with a graph");
  const double t0 = wall_s();
  if (int rc = learned_init(ctx, params, scale_model, seed)) return rc;
  const double t_init = wall_s() - t0;
  double e = HUGE_VAL, step = step0;
  int it = 0;
  while (it < max_iterations) {
    if (int rc = bh_run(ctx, 1, batch, theta, &step, &e)) return rc;  // STEP times 0.999
    it++;
    if (e <= target_energy) break;
  }
  int fell_back = 0;
  if (!(e <= target_energy)) {
    // the plain run: greedy DFS start, STEP from 1 (algorithms.cpp:1020-1072)
    if (int rc = bl_init_dfs(ctx)) return rc;
    step = 1.0;
    if (int rc = bh_run(ctx, max_iterations, batch, theta, &step, &e)) return rc;
    fell_back = 1;
  }
  BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  out[0] = e;
  out[1] = wall_s() - t0;
  out[2] = it;
  out[3] = fell_back;
  out[4] = t_init;
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

}  // extern "C"

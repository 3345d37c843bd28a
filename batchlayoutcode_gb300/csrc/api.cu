// api.cu -- C ABI of the GB300 BatchLayout engine (include/batchlayout_gb300.h).
//
// Mirrors class algorithms (sample/algorithms.h:50-85): the context holds the
// graph and run options given to the constructor (sample/algorithms.cpp:3-15),
// each layout method runs the optional initialiser and then its iterations on
// the device, returning {energy, seconds}.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <exception>
#include <limits>
#include <new>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/batchlayout_gb300.h"
#include "bl_internal.cuh"
#include "host.h"

static thread_local std::string g_create_error;

int bl_fail(bl_ctx *ctx, int code, const std::string &msg) {
  if (ctx) ctx->err = msg;
  return code;
}

// Host code (allocations, worker threads, strings) may throw; no exception
// crosses the C ABI.  Each entry point's handler calls one of these: the
// exception in flight becomes BL_ERR_HOST, its message on the context (or,
// for a constructor, in bl_create_error()).
static void describe_exception(char *buf, size_t cap) {
  try {
    throw;
  } catch (const std::bad_alloc &) {
    std::snprintf(buf, cap, "host exception: memory allocation failed");
  } catch (const std::exception &e) {
    std::snprintf(buf, cap, "host exception: %s", e.what());
  } catch (...) {
    std::snprintf(buf, cap, "host exception");
  }
}

int bl_host_exception(bl_ctx *ctx, char *msg, int msgcap) {
  char buf[256];
  describe_exception(buf, sizeof(buf));
  if (msg && msgcap > 0) std::snprintf(msg, (size_t)msgcap, "%s", buf);
  if (ctx) {
    try {
      ctx->err = buf;
    } catch (...) {
    }
  }
  return BL_ERR_HOST;
}

void bl_create_exception() {
  char buf[256];
  describe_exception(buf, sizeof(buf));
  try {
    g_create_error = buf;
  } catch (...) {
  }
}

int bl_cuda_fail(bl_ctx *ctx, cudaError_t e, const char *what) {
  return bl_fail(ctx, BL_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int bl_check_status(bl_ctx *ctx) {
  DevStatus st;
  cudaError_t e = cudaMemcpy(&st, ctx->s.status, sizeof(st), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return bl_cuda_fail(ctx, e, "read device status");
  if (st.code == DEV_OK) return 0;
  const char *what = st.code == DEV_TIMEOUT_GRID_BARRIER ? "grid barrier timed out"
                     : st.code == DEV_TIMEOUT_TREE        ? "tree build wait timed out"
                     : st.code == DEV_FORCE_RANGE         ? "force beyond the fixed-point range (coincident vertices?)"
                     : st.code == DEV_TIMEOUT_MMA         ? "tensor-core MMA completion wait timed out"
                     : st.code == DEV_TIMEOUT_SWEEP       ? "level sweep wait for a moved neighbour timed out"
                                                          : "device error";
  cudaMemset(ctx->s.status, 0, sizeof(DevStatus));
  return bl_fail(ctx, BL_ERR_DEVICE_TIMEOUT,
                 std::string(what) + " (block " + std::to_string(st.where) + ")");
}

void bl_time_begin(bl_ctx *ctx, const char *kernel) {
  if (ctx->timed_kernel.empty() || ctx->timed_kernel != kernel) return;
  if (ctx->ev_used + 2 > ctx->ev_pool.size()) {
    for (int k = 0; k < 256; k++) {
      cudaEvent_t ev;
      if (cudaEventCreate(&ev) != cudaSuccess) return;
      ctx->ev_pool.push_back(ev);
    }
  }
  cudaEventRecord(ctx->ev_pool[ctx->ev_used], ctx->stream);
}

void bl_time_end(bl_ctx *ctx, const char *kernel) {
  if (ctx->timed_kernel.empty() || ctx->timed_kernel != kernel) return;
  if (ctx->ev_used + 2 > ctx->ev_pool.size()) return;
  cudaEventRecord(ctx->ev_pool[ctx->ev_used + 1], ctx->stream);
  ctx->ev_used += 2;
}

static void collect_timing(bl_ctx *ctx) {
  if (ctx->ev_used == 0) return;
  cudaStreamSynchronize(ctx->stream);
  for (size_t k = 0; k + 1 < ctx->ev_used; k += 2) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ctx->ev_pool[k], ctx->ev_pool[k + 1]) == cudaSuccess) {
      ctx->timed_ms += ms;
      ctx->timed_count++;
    }
  }
  ctx->ev_used = 0;
}

// Neighbours the sorted-CSR cursor of the minibatch sweep matches
// (sample/algorithms.cpp:746, 758-762): the cursor starts at rowptr[i] and
// advances after a match while it is below rowptr[i+1]-1, as the source index
// j increases.  It matches the strictly increasing prefix of the row; for an
// empty row it reads colids[rowptr[i]], the first entry of a later row.
void bl::cursor_neighbours(int n, const std::vector<int> &rp, const std::vector<int> &ci,
                       std::vector<int> &erp, std::vector<int> &eci) {
  const long long nnz = rp[n];
  erp.assign(n + 1, 0);
  eci.clear();
  eci.reserve(ci.size());
  for (int i = 0; i < n; i++) {
    const int k0 = rp[i], k1 = rp[i + 1];
    if (k1 > k0) {
      int last = ci[k0];
      eci.push_back(last);
      for (int k = k0 + 1; k < k1; k++) {
        if (ci[k] <= last) break;
        last = ci[k];
        eci.push_back(last);
      }
    } else if (k0 < nnz) {
      eci.push_back(ci[k0]);
    }
    erp[i + 1] = (int)eci.size();
  }
}

namespace {

double wall() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

__global__ void to_f32_kernel(const double2 *in, float2 *out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_float2((float)in[i].x, (float)in[i].y);
}

__global__ void to_f64_kernel(const float2 *in, double2 *out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_double2((double)in[i].x, (double)in[i].y);
}

void free_ctx(bl_ctx *c) {
  auto fr = [](void *p) { if (p) cudaFree(p); };
  fr(c->g.rowptr); fr(c->g.colids);
  if (c->g.eff_rowptr != c->g.rowptr) fr(c->g.eff_rowptr);
  if (c->g.eff_colids != c->g.colids) fr(c->g.eff_colids);
  if (c->g.srt_rowptr != c->g.rowptr) fr(c->g.srt_rowptr);
  if (c->g.srt_colids != c->g.colids) fr(c->g.srt_colids);
  fr(c->pos); fr(c->force); fr(c->e); fr(c->stage);
  bl::Scratch &s = c->s;
  fr(s.energy_parts); fr(s.energy); fr(s.status); fr(s.partials); fr(s.keys); fr(s.keys_alt);
  fr(s.perm); fr(s.perm_alt); fr(s.hist); fr(s.bbox); fr(s.frame); fr(s.spos); fr(s.bparent);
  fr(s.bchild); fr(s.brange); fr(s.bdelta); fr(s.qkids); fr(s.qpar); fr(s.qnchild); fr(s.span); fr(s.span_stage); fr(s.ztab); fr(s.chain); fr(s.qcen); fr(s.qbelow); fr(s.startcnt);
  fr(s.startbase); fr(s.nodes); fr(s.nodes_c64); fr(s.nodes_lvl); fr(s.rep);
  fr(s.stats); fr(s.pos_alt); fr(s.f0); fr(s.runs); fr(s.bnode); fr(s.cursor); fr(s.cursor_full); fr(s.walk_off); fr(s.walk_pairs);
  fr(s.term_off); fr(s.terms); fr(s.term_tgt); fr(s.greedy_share); fr(s.greedy_pos);
  for (auto &ls : c->schedules) {
    fr(ls.order);
    fr(ls.d_offsets);
    fr(ls.early_off);
    fr(ls.early_col);
  }
  bl::batched_free(c->batched);
  c->batched = nullptr;
  bl::mpnn_free(c->mpnn);
  c->mpnn = nullptr;
  bl::bh_graph_free(c->bh_graph);
  c->bh_graph = nullptr;
  for (auto ev : c->ev_pool) cudaEventDestroy(ev);
  for (auto ev : c->run_ev)
    if (ev) cudaEventDestroy(ev);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->stream) cudaStreamDestroy(c->stream);
}

int init_coordinates(bl_ctx *ctx) {
  if (ctx->init == 0) return bl_init_dfs(ctx);
  if (ctx->init == 4) return bl_bfs_init(ctx);  // breadth-first start on the GPU
  if (ctx->init == 2) return bl_file_initialization(ctx);
  if (ctx->init == 3) {
    // learned start from the model file in initfile (no reference counterpart)
    std::vector<float> params(BL_MPNN_PARAMS);
    double sm[3];
    if (int rc = bl_learned_load_model(ctx->initfile.c_str(), params.data(), sm)) {
      bl_fail(ctx, rc, std::string("cannot read model file ") + ctx->initfile);
      return rc;
    }
    return bl_learned_init(ctx, params.data(), sm, 1);
  }
  return bl_rand_init(ctx);
}

}  // namespace

extern "C" {

const char *bl_create_error(void) { return g_create_error.c_str(); }

static int export_csr(const blhost::MatrixInfo &mi, const std::vector<int> &rp, const std::vector<int> &ci,
                      long long *info, double *seconds, int **rowptr, int **colids) {
  info[0] = mi.rows;
  info[1] = mi.cols;
  info[2] = mi.nnz;
  info[3] = mi.symmetric ? 1 : 0;
  if (seconds) *seconds = mi.seconds;
  *rowptr = static_cast<int *>(std::malloc(sizeof(int) * rp.size()));
  *colids = static_cast<int *>(std::malloc(sizeof(int) * std::max<size_t>(ci.size(), 1)));
  if (!*rowptr || !*colids) {
    std::free(*rowptr);
    std::free(*colids);
    return BL_ERR_ARG;
  }
  std::memcpy(*rowptr, rp.data(), sizeof(int) * rp.size());
  if (!ci.empty()) std::memcpy(*colids, ci.data(), sizeof(int) * ci.size());
  return BL_OK;
}

int bl_read_matrix_market(const char *path, long long *info, double *seconds, int **rowptr,
                          int **colids, char *err, int errcap) try {
  if (!path || !info || !rowptr || !colids) return BL_ERR_ARG;
  blhost::MatrixInfo mi;
  std::vector<int> rp, ci;
  std::string msg;
  if (!blhost::read_matrix_market(path, mi, rp, ci, msg)) {
    if (err && errcap > 0) std::snprintf(err, (size_t)errcap, "%s", msg.c_str());
    return BL_ERR_IO;
  }
  return export_csr(mi, rp, ci, info, seconds, rowptr, colids);
} catch (...) {
  return bl_host_exception(nullptr, err, errcap);
}

int bl_read_matrix_market_cached(const char *path, const char *cache_dir, long long *info, double *seconds,
                                 int **rowptr, int **colids, char *err, int errcap) try {
  if (!path || !info || !rowptr || !colids) return BL_ERR_ARG;
  blhost::MatrixInfo mi;
  std::vector<int> rp, ci;
  std::string msg;
  bool cached = false;
  const bool ok = cache_dir ? blhost::read_matrix_market_cached(path, cache_dir, mi, rp, ci, msg, &cached)
                            : blhost::read_matrix_market(path, mi, rp, ci, msg);
  if (!ok) {
    if (err && errcap > 0) std::snprintf(err, (size_t)errcap, "%s", msg.c_str());
    return BL_ERR_IO;
  }
  info[4] = cached ? 1 : 0;
  return export_csr(mi, rp, ci, info, seconds, rowptr, colids);
} catch (...) {
  return bl_host_exception(nullptr, err, errcap);
}

void bl_free(void *p) { std::free(p); }

// Vertex ids are int, as the reference's INDEXTYPE, and coordinate arrays
// are indexed by 2 * id in int arithmetic: at most 2^30 - 1 vertices.
static constexpr int kMaxVertices = (1 << 30) - 1;

// Checks of a caller's CSR (rowptr[n+1], colids[nnz]) before anything reads
// it by index: null when valid, else the reason.
static const char *csr_error(int n, long long nnz, const int *rowptr, const int *colids) {
  if (n < 1 || nnz < 0 || !rowptr || (nnz > 0 && !colids)) return "invalid graph arguments";
  if (n > kMaxVertices) return "more than 2^30 - 1 vertices";
  if (nnz > 2147483647LL) return "nnz exceeds int32 (the reference's INDEXTYPE)";
  if (rowptr[0] != 0 || rowptr[n] != nnz) return "rowptr must start at 0 and end at nnz";
  for (int i = 0; i < n; i++)
    if (rowptr[i + 1] < rowptr[i]) return "rowptr not monotone";
  for (long long k = 0; k < nnz; k++)
    if (colids[k] < 0 || colids[k] >= n) return "column id out of range";
  return nullptr;
}

bl_ctx *bl_algorithms_create(int device, int n, long long nnz, const int *rowptr,
                             const int *colids, const char *input, const char *outputdir,
                             int init, double weight, double threshold, const char *initfile) try {
  g_create_error.clear();
  if (const char *why = csr_error(n, nnz, rowptr, colids)) {
    g_create_error = std::string("bl_algorithms_create: ") + why;
    return nullptr;
  }
  bl_ctx *ctx = new bl_ctx();
  auto bad = [&](cudaError_t e, const char *what) {
    g_create_error = std::string(what) + ": " + cudaGetErrorString(e);
    free_ctx(ctx);
    delete ctx;
    return (bl_ctx *)nullptr;
  };
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return bad(e, "cudaSetDevice");
  ctx->device = device;
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  // the main stream at the highest priority: work beside it on `side` (the
  // lowest) gives way to it
  int prio_least = 0, prio_greatest = 0;
  cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
  e = cudaStreamCreateWithPriority(&ctx->stream, cudaStreamNonBlocking, prio_greatest);
  if (e != cudaSuccess) return bad(e, "cudaStreamCreate");
  e = cudaStreamCreateWithPriority(&ctx->side, cudaStreamNonBlocking, prio_least);
  if (e != cudaSuccess) return bad(e, "cudaStreamCreate");
  if ((e = cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming)) != cudaSuccess) return bad(e, "cudaEventCreate");
  if ((e = cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming)) != cudaSuccess) return bad(e, "cudaEventCreate");
  ctx->input = input ? input : "";
  ctx->outputdir = outputdir ? outputdir : "";
  ctx->initfile = initfile ? initfile : "";
  ctx->init = init;
  ctx->weight = weight;
  ctx->threshold = threshold;
  ctx->g.n = n;
  ctx->g.nnz = nnz;
  ctx->h_rowptr.assign(rowptr, rowptr + n + 1);
  ctx->h_colids.assign(colids, colids + nnz);
  std::vector<int> erp, eci;
  bl::cursor_neighbours(n, ctx->h_rowptr, ctx->h_colids, erp, eci);
  const size_t cn = std::max<long long>(nnz, 1);
  if ((e = cudaMalloc(&ctx->g.rowptr, (n + 1) * sizeof(int))) != cudaSuccess) return bad(e, "cudaMalloc");
  if ((e = cudaMalloc(&ctx->g.colids, cn * sizeof(int))) != cudaSuccess) return bad(e, "cudaMalloc");
  cudaMemcpy(ctx->g.rowptr, rowptr, (n + 1) * sizeof(int), cudaMemcpyHostToDevice);
  if (nnz) cudaMemcpy(ctx->g.colids, colids, nnz * sizeof(int), cudaMemcpyHostToDevice);
  if (erp == ctx->h_rowptr && eci == ctx->h_colids) {
    ctx->g.eff_rowptr = ctx->g.rowptr;
    ctx->g.eff_colids = ctx->g.colids;
  } else {
    if ((e = cudaMalloc(&ctx->g.eff_rowptr, (n + 1) * sizeof(int))) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = cudaMalloc(&ctx->g.eff_colids, std::max<size_t>(eci.size(), 1) * sizeof(int))) != cudaSuccess)
      return bad(e, "cudaMalloc");
    cudaMemcpy(ctx->g.eff_rowptr, erp.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice);
    if (!eci.empty()) cudaMemcpy(ctx->g.eff_colids, eci.data(), eci.size() * sizeof(int), cudaMemcpyHostToDevice);
  }
  int maxd = 0;
  for (int i = 0; i < n; i++) maxd = std::max(maxd, erp[i + 1] - erp[i]);
  ctx->g.max_eff_degree = maxd;
  const size_t m = std::max(n, 2);
  if ((e = cudaMalloc(&ctx->pos, m * sizeof(float2))) != cudaSuccess) return bad(e, "cudaMalloc");
  if ((e = cudaMalloc(&ctx->force, m * sizeof(double2))) != cudaSuccess) return bad(e, "cudaMalloc");
  if ((e = cudaMalloc(&ctx->e, m * sizeof(double))) != cudaSuccess) return bad(e, "cudaMalloc");
  if ((e = cudaMalloc(&ctx->stage, m * sizeof(double2))) != cudaSuccess) return bad(e, "cudaMalloc");
  if ((e = cudaMalloc(&ctx->s.energy_parts, 1024 * sizeof(double))) != cudaSuccess) return bad(e, "cudaMalloc");
  if ((e = cudaMalloc(&ctx->s.energy, 16 * sizeof(double))) != cudaSuccess) return bad(e, "cudaMalloc");
  if ((e = cudaMalloc(&ctx->s.status, sizeof(DevStatus))) != cudaSuccess) return bad(e, "cudaMalloc");
  if ((e = cudaMalloc(&ctx->s.bbox, 8 * sizeof(unsigned int))) != cudaSuccess) return bad(e, "cudaMalloc");
  if ((e = cudaMalloc(&ctx->s.frame, 4 * sizeof(double))) != cudaSuccess) return bad(e, "cudaMalloc");
  if ((e = cudaMalloc(&ctx->s.stats, 2 * sizeof(unsigned long long))) != cudaSuccess) return bad(e, "cudaMalloc");
  cudaMemset(ctx->pos, 0, m * sizeof(float2));
  cudaMemset(ctx->force, 0, m * sizeof(double2));
  cudaMemset(ctx->e, 0, m * sizeof(double));
  cudaMemset(ctx->s.status, 0, sizeof(DevStatus));
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return bad(e, "cudaDeviceSynchronize");
  return ctx;
} catch (...) {
  bl_create_exception();
  return nullptr;
}

void bl_destroy(bl_ctx *ctx) try {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  free_ctx(ctx);
  delete ctx;
} catch (...) {
}

const char *bl_last_error(const bl_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int bl_num_vertices(const bl_ctx *ctx) { return ctx ? ctx->g.n : 0; }

long long bl_kernel_launches(const bl_ctx *ctx) { return ctx ? ctx->launches : 0; }

// Device address of page-locked host memory the device can read and write
// (a pinned allocation or registered range with a device mapping), else null:
// the conversion kernels then work on the host buffer directly instead of a
// staging copy.
static void *mapped_host(const void *p) {
  cudaPointerAttributes pa;
  if (cudaPointerGetAttributes(&pa, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return pa.type == cudaMemoryTypeHost ? pa.devicePointer : nullptr;
}

int bl_set_coordinates(bl_ctx *ctx, const double *xy, int n) try {
  if (!ctx || !xy || n != ctx->g.n) return bl_fail(ctx, BL_ERR_ARG, "bl_set_coordinates: size mismatch");
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  const double2 *src = static_cast<const double2 *>(mapped_host(xy));
  if (!src) {
    BL_CUDA(ctx, cudaMemcpyAsync(ctx->stage, xy, (size_t)n * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
    src = ctx->stage;
  }
  to_f32_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(src, ctx->pos, n);
  ctx->launches++;
  BL_CUDA(ctx, cudaGetLastError());
  BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_get_coordinates(bl_ctx *ctx, double *xy, int n) try {
  if (!ctx || !xy || n != ctx->g.n) return bl_fail(ctx, BL_ERR_ARG, "bl_get_coordinates: size mismatch");
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  double2 *dst = static_cast<double2 *>(mapped_host(xy));
  to_f64_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(ctx->pos, dst ? dst : ctx->stage, n);
  ctx->launches++;
  if (!dst)
    BL_CUDA(ctx, cudaMemcpyAsync(xy, ctx->stage, (size_t)n * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
  BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_get_forces(bl_ctx *ctx, double *fxy, int n) try {
  if (!ctx || !fxy || n != ctx->g.n) return bl_fail(ctx, BL_ERR_ARG, "bl_get_forces: size mismatch");
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  BL_CUDA(ctx, cudaMemcpyAsync(fxy, ctx->force, (size_t)n * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
  BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

// ---- initialisers ----------------------------------------------------------

int bl_rand_init(bl_ctx *ctx) try {
  if (!ctx) return BL_ERR_ARG;
  std::vector<double> xy;
  blhost::rand_init(ctx->g.n, xy);
  return bl_set_coordinates(ctx, xy.data(), ctx->g.n);
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_init_dfs(bl_ctx *ctx) try {
  if (!ctx) return BL_ERR_ARG;
  std::vector<double> xy;
  blhost::init_dfs(ctx->g.n, ctx->h_rowptr, ctx->h_colids, xy);
  return bl_set_coordinates(ctx, xy.data(), ctx->g.n);
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_file_initialization(bl_ctx *ctx) try {
  if (!ctx) return BL_ERR_ARG;
  std::vector<double> xy(2 * (size_t)ctx->g.n, 0.0);
  std::string msg;
  if (!blhost::file_init(ctx->initfile, ctx->g.n, xy, msg)) return bl_fail(ctx, BL_ERR_IO, msg);
  return bl_set_coordinates(ctx, xy.data(), ctx->g.n);
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_random_coordinates(int n, double *xy) try {
  if (n < 0 || n > kMaxVertices || (n > 0 && !xy)) return BL_ERR_ARG;
  std::vector<double> v;
  blhost::rand_init(n, v);
  std::memcpy(xy, v.data(), v.size() * sizeof(double));
  return BL_OK;
} catch (...) {
  return bl_host_exception(nullptr);
}

int bl_greedy_coordinates(int n, const int *rowptr, const int *colids, double *xy) try {
  if (!xy || !rowptr || n < 1 || n > kMaxVertices || csr_error(n, rowptr[n], rowptr, colids)) return BL_ERR_ARG;
  std::vector<int> rp(rowptr, rowptr + n + 1), ci(colids, colids + rowptr[n]);
  std::vector<double> v;
  blhost::init_dfs(n, rp, ci, v);
  std::memcpy(xy, v.data(), v.size() * sizeof(double));
  return BL_OK;
} catch (...) {
  return bl_host_exception(nullptr);
}

int bl_cursor_neighbours(int n, const int *rowptr, const int *colids, int *matched_rowptr, int *matched_colids) try {
  if (!rowptr || !colids || !matched_rowptr || n < 1 || n > kMaxVertices || csr_error(n, rowptr[n], rowptr, colids))
    return BL_ERR_ARG;
  std::vector<int> rp(rowptr, rowptr + n + 1), ci(colids, colids + rowptr[n]), erp, eci;
  bl::cursor_neighbours(n, rp, ci, erp, eci);
  std::memcpy(matched_rowptr, erp.data(), erp.size() * sizeof(int));
  if (matched_colids && !eci.empty()) std::memcpy(matched_colids, eci.data(), eci.size() * sizeof(int));
  return BL_OK;
} catch (...) {
  return bl_host_exception(nullptr);
}

int bl_write_coordinates(const char *input, const char *outputdir, const char *tag, const double *xy,
                         int n, char *path_out, int path_cap) try {
  if (!input || !outputdir || !tag || (n > 0 && !xy)) return BL_ERR_ARG;
  std::vector<double> v(xy, xy + 2 * (size_t)n);
  std::string path;
  const bool ok = blhost::write_coordinates(input, outputdir, tag, v, path);
  if (path_out && path_cap > 0) std::snprintf(path_out, (size_t)path_cap, "%s", path.c_str());
  return ok ? BL_OK : BL_ERR_IO;
} catch (...) {
  return bl_host_exception(nullptr);
}

// ---- layout methods ----------------------------------------------------------

static int minibatch_method(bl_ctx *ctx, int model, double decay, int iterations, int batch,
                            int flag, bool converged, double *out, double energy_if_none) {
  if (!ctx || !out) return BL_ERR_ARG;
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  const double t0 = wall();
  double step0 = 1.0;
  if (flag == 0) {
    if (int rc = init_coordinates(ctx)) return rc;
  } else {
    step0 = std::pow(0.999, 4 * iterations);
  }
  double energy = energy_if_none;
  long long loops = 0;
  if (converged || iterations > 0) {
    if (int rc = bl::minibatch_run(ctx, model, batch, iterations, step0, decay, converged,
                                   ctx->threshold, 100000000LL, &energy, &loops))
      return rc;
  }
  collect_timing(ctx);
  out[0] = energy;
  out[1] = wall() - t0;
  if (converged) out[2] = (double)loops;
  return BL_OK;
}

int bl_cache_blocking_minibatch(bl_ctx *ctx, int iterations, int threads, int batch, int flag,
                                double *out) try {
  (void)threads;
  return minibatch_method(ctx, bl::MODEL_FR, 0.999, iterations, batch, flag, false, out, 0.0);
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_cache_blocking_minibatch_converged(bl_ctx *ctx, int iterations, int threads, int batch,
                                          int flag, double *out) try {
  (void)threads;
  return minibatch_method(ctx, bl::MODEL_FR, 0.999, iterations, batch, flag, true, out, 0.0);
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_linlog_cache_blocking_minibatch(bl_ctx *ctx, int iterations, int threads, int batch,
                                       double *out) try {
  (void)threads;
  return minibatch_method(ctx, bl::MODEL_LINLOG, 0.99, iterations, batch, 0, false, out,
                          std::numeric_limits<double>::max());
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_fa_cache_blocking_minibatch(bl_ctx *ctx, int iterations, int threads, int batch,
                                   double *out) try {
  (void)threads;
  return minibatch_method(ctx, bl::MODEL_FA, 0.99, iterations, batch, 0, false, out,
                          std::numeric_limits<double>::max());
} catch (...) {
  return bl_host_exception(ctx);
}

static int bh_loop(bl_ctx *ctx, int iterations, int batch, double theta, double *energy) {
  double step = 1.0;
  return bl::bh_run(ctx, iterations, batch, theta, &step, energy);
}

int bl_barnes_hut_approximation(bl_ctx *ctx, int iterations, int threads, int batch,
                                double theta, int flag, double *out) try {
  (void)threads;
  if (!ctx || !out) return BL_ERR_ARG;
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  const double t0 = wall();
  if (flag == 0)
    if (int rc = init_coordinates(ctx)) return rc;
  double energy = std::numeric_limits<double>::max();
  if (int rc = bh_loop(ctx, iterations, batch, theta, &energy)) return rc;
  collect_timing(ctx);
  out[0] = energy;
  out[1] = wall() - t0;
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_approx_cache_block_bh(bl_ctx *ctx, int iterations, int threads, int batch, double *out) try {
  (void)threads;
  if (!ctx || !out) return BL_ERR_ARG;
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  const double t0 = wall();
  if (int rc = init_coordinates(ctx)) return rc;
  const int approx = (int)(iterations * 0.8);
  double e_bh = 0.0;
  if (int rc = bh_loop(ctx, approx, batch, 1.2, &e_bh)) return rc;
  const int rest = iterations - approx;
  double energy = 0.0;
  long long loops = 0;
  if (rest > 0)
    if (int rc = bl::minibatch_run(ctx, bl::MODEL_FR, batch, rest, std::pow(0.999, 4 * rest), 0.999,
                                   false, 0.0, 0, &energy, &loops))
      return rc;
  collect_timing(ctx);
  out[0] = energy;
  out[1] = wall() - t0;
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

// Algo 5 from STEP `step`: iterations 0..(int)(0.8*iterations) are the walk
// phase, the rest the all-pairs phase; STEP *= 0.99 per iteration (:1179).
static int greedy_loop(bl_ctx *ctx, int iterations, int batch, double step, double *energy) {
  const int approx = (int)(iterations * 0.8);  // :1086
  const int first = std::min(iterations, approx + 1);
  const int rest = iterations - first;
  if (first > 0)
    if (int rc = bl::greedy_walk_run(ctx, batch, first, step, 0.99, rest == 0 && energy, energy)) return rc;
  if (rest > 0) {
    double s = step;  // STEP after `first` decays, multiplied as the kernel does
    for (int k = 0; k < first; k++) s = s * 0.99;
    long long loops = 0;
    if (int rc = bl::minibatch_run(ctx, bl::MODEL_GREEDY_EXACT, batch, rest, s, 0.99, false, 0.0, 0, energy, &loops))
      return rc;
  }
  return 0;
}

int bl_approx_force_directed(bl_ctx *ctx, int iterations, int threads, int batch, double *out) try {
  (void)threads;
  if (!ctx || !out) return BL_ERR_ARG;
  if (batch < 1) return bl_fail(ctx, BL_ERR_ARG, "batch must be >= 1");
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  const double t0 = wall();
  if (int rc = init_coordinates(ctx)) return rc;
  double energy = std::numeric_limits<double>::max();
  if (int rc = greedy_loop(ctx, iterations, batch, 1.0, &energy)) return rc;
  collect_timing(ctx);
  out[0] = energy;
  out[1] = wall() - t0;
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_cache_blocking_minibatch_sd(bl_ctx *ctx, int iterations, int threads, int batch, int flag,
                                   double *out) try {
  (void)threads;
  return minibatch_method(ctx, bl::MODEL_SD, 0.999, iterations, batch, flag, false, out,
                          std::numeric_limits<double>::max());
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_write_to_file(bl_ctx *ctx, const char *tag, char *path_out, int path_cap) try {
  if (!ctx || !tag) return BL_ERR_ARG;
  std::vector<double> xy(2 * (size_t)ctx->g.n);
  if (int rc = bl_get_coordinates(ctx, xy.data(), ctx->g.n)) return rc;
  std::string path;
  if (!blhost::write_coordinates(ctx->input, ctx->outputdir, tag, xy, path))
    return bl_fail(ctx, BL_ERR_IO, "cannot write " + path);
  ctx->input = path;  // writeToFile rewrites its `filename` member (:1248)
  if (path_out && path_cap > 0) {
    std::snprintf(path_out, (size_t)path_cap, "%s", path.c_str());
  }
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

// ---- building blocks -----------------------------------------------------------

int bl_minibatch_iteration(bl_ctx *ctx, int model, int batch, double step, double *energy_out) try {
  if (!ctx) return BL_ERR_ARG;
  if (model != 2 && model != 3 && model != 8 && model != 7 && model != 5)
    return bl_fail(ctx, BL_ERR_ARG, "model must be 2, 3, 5, 7 or 8");
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  long long loops = 0;
  double energy = 0.0;
  if (int rc = bl::minibatch_run(ctx, model, batch, 1, step, 1.0, false, 0.0, 0, &energy, &loops)) return rc;
  if (energy_out) *energy_out = energy;
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_greedy_iteration(bl_ctx *ctx, int batch, double step, double *energy_out) try {
  if (!ctx) return BL_ERR_ARG;
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  double energy = 0.0;
  if (int rc = bl::greedy_walk_run(ctx, batch, 1, step, 1.0, true, &energy)) return rc;
  if (energy_out) *energy_out = energy;
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_barnes_hut_iteration(bl_ctx *ctx, int batch, double theta, double step, double *energy_out) try {
  if (!ctx) return BL_ERR_ARG;
  if (batch < 1) return bl_fail(ctx, BL_ERR_ARG, "batch must be >= 1");
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  double energy = 0.0, s = step;
  if (int rc = bl::bh_run(ctx, 1, batch, theta, &s, &energy)) return rc;
  if (energy_out) *energy_out = energy;
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_morton_order(bl_ctx *ctx, double *frame, unsigned long long *keys, int *perm) try {
  if (!ctx || !frame || !keys || !perm) return BL_ERR_ARG;
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  const int n = ctx->g.n;
  if (n < 2) return bl_fail(ctx, BL_ERR_ARG, "need at least two vertices");
  if (int rc = bl::ensure_bh_scratch(ctx)) return rc;
  if (int rc = bl::bh_build(ctx, ctx->pos, 1.2)) return rc;  // (theta enters only the records)
  BL_CUDA(ctx, cudaMemcpyAsync(frame, ctx->s.frame, 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  BL_CUDA(ctx, cudaMemcpyAsync(keys, ctx->s.keys, (size_t)n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  BL_CUDA(ctx, cudaMemcpyAsync(perm, ctx->s.perm, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return bl_check_status(ctx);
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_quadtree(bl_ctx *ctx, int cap, int *lo, int *hi, int *depth, int *nchild, double *centroid) try {
  if (!ctx || cap < 0 || !lo || !hi || !depth || !nchild || !centroid) return BL_ERR_ARG;
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  if (ctx->g.n < 2) return bl_fail(ctx, BL_ERR_ARG, "need at least two vertices");
  return bl::bh_canonical_tree(ctx, cap, lo, hi, depth, nchild, centroid);
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_bh_repulsion(bl_ctx *ctx, double theta, double *out, long long *stats) try {
  if (!ctx || !out) return BL_ERR_ARG;
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  const int n = ctx->g.n;
  if (int rc = bl::ensure_bh_scratch(ctx)) return rc;
  if (int rc = bl::bh_build(ctx, ctx->pos, theta)) return rc;
  if (int rc = bl::bh_traverse(ctx, theta, true, 0)) return rc;
  std::vector<float2> rep(n);
  unsigned long long st[2] = {0, 0};
  BL_CUDA(ctx, cudaMemcpyAsync(rep.data(), ctx->s.rep, (size_t)n * sizeof(float2), cudaMemcpyDeviceToHost, ctx->stream));
  BL_CUDA(ctx, cudaMemcpyAsync(st, ctx->s.stats, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream));
  BL_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (int rc = bl_check_status(ctx)) return rc;
  for (int i = 0; i < n; i++) {
    out[2 * i] = rep[i].x;
    out[2 * i + 1] = rep[i].y;
  }
  if (stats) {
    stats[0] = (long long)st[0];
    stats[1] = (long long)st[1];
  }
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_run_resident(bl_ctx *ctx, int algo, int iterations, int batch, double theta, double step,
                    double *energy_out) try {
  if (!ctx) return BL_ERR_ARG;
  BL_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!ctx->run_ev[0]) {
    BL_CUDA(ctx, cudaEventCreate(&ctx->run_ev[0]));
    BL_CUDA(ctx, cudaEventCreate(&ctx->run_ev[1]));
  }
  BL_CUDA(ctx, cudaEventRecord(ctx->run_ev[0], ctx->stream));
  double energy = 0.0;
  long long loops = 0;
  int rc = 0;
  if (algo == 2 || algo == 3 || algo == 8 || algo == 7) {
    rc = bl::minibatch_run(ctx, algo, batch, iterations, step, (algo == 2 || algo == 7) ? 0.999 : 0.99, false,
                           0.0, 0, &energy, &loops);
  } else if (algo == 5) {
    rc = greedy_loop(ctx, iterations, batch, step, &energy);
  } else if (algo == 4) {
    double s = step;
    rc = bl::bh_run(ctx, iterations, batch, theta, &s, energy_out ? &energy : nullptr);
  } else {
    return bl_fail(ctx, BL_ERR_UNSUPPORTED, "bl_run_resident: algo must be 2, 3, 4, 5, 7 or 8");
  }
  if (rc) return rc;
  BL_CUDA(ctx, cudaEventRecord(ctx->run_ev[1], ctx->stream));
  BL_CUDA(ctx, cudaEventSynchronize(ctx->run_ev[1]));
  float ms = 0.f;
  BL_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->run_ev[0], ctx->run_ev[1]));
  ctx->last_run_ms = ms;
  collect_timing(ctx);
  if (energy_out) *energy_out = energy;
  if (algo == 4 && !energy_out) return bl_check_status(ctx);
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_last_run_ms(bl_ctx *ctx, double *ms) try {
  if (!ctx || !ms) return BL_ERR_ARG;
  *ms = ctx->last_run_ms;
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_set_graph_mode(bl_ctx *ctx, int enabled) try {
  if (!ctx) return BL_ERR_ARG;
  ctx->graph_mode = enabled != 0;
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

int bl_last_kernel_time(bl_ctx *ctx, const char *kernel, double *ms) try {
  if (!ctx || !ms) return BL_ERR_ARG;
  if (kernel && ctx->timed_kernel != kernel) {
    // start timing this kernel family from now on
    collect_timing(ctx);
    ctx->timed_kernel = kernel;
    ctx->timed_ms = 0.0;
    ctx->timed_count = 0;
    ms[0] = 0.0;
    ms[1] = 0.0;
    return BL_OK;
  }
  collect_timing(ctx);
  ms[0] = ctx->timed_ms;
  ms[1] = (double)ctx->timed_count;
  ctx->timed_ms = 0.0;
  ctx->timed_count = 0;
  return BL_OK;
} catch (...) {
  return bl_host_exception(ctx);
}

}  // extern "C"

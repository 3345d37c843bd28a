// bl_internal.cuh -- shared declarations of the GB300 BatchLayout engine.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <deque>
#include <string>
#include <vector>

// ----------------------------------------------------------------------------
// Device-side error record.  Every spin-wait in this library is bounded; when
// a bound runs out the waiting block records the site here and returns, the
// host reads the record after the kernel and reports BL_ERR_DEVICE_TIMEOUT.
// ----------------------------------------------------------------------------
enum : unsigned int {
  DEV_OK = 0,
  DEV_TIMEOUT_GRID_BARRIER = 1,
  DEV_TIMEOUT_TREE = 2,
  DEV_BAD_INDEX = 3,
  DEV_FORCE_RANGE = 4,
  DEV_TIMEOUT_MMA = 5,
  DEV_TIMEOUT_SWEEP = 6,
};

struct DevStatus {
  unsigned int code;     // first error code (0 = none)
  unsigned int where;    // block id that recorded it
  unsigned int barrier;  // grid-barrier generation counter
  unsigned int pad;
};

// Timeouts for device waits (nanoseconds of %globaltimer).
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;  // 2 s
constexpr unsigned long long kMmaTimeoutNs = 1000000000ull;      // 1 s, tensor-core completion

__device__ __forceinline__ unsigned long long dev_globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned int ld_volatile_u32(const unsigned int *p) {
  return *reinterpret_cast<const volatile unsigned int *>(p);
}

// Whether no earlier launch recorded an error: one read per block, shared
// (every thread reading the same word would queue at one L2 slice).  All
// threads of the block must call it, before any early return.
__device__ __forceinline__ bool block_status_ok(const DevStatus *st) {
  __shared__ unsigned int s_code;
  if (threadIdx.x == 0) s_code = ld_volatile_u32(&st->code);
  __syncthreads();
  return s_code == 0u;
}

__device__ __forceinline__ void dev_record_error(DevStatus *st, unsigned int code) {
  if (atomicCAS(&st->code, 0u, code) == 0u) st->where = blockIdx.x;
}

// Grid-wide barrier for a cooperative (co-resident) launch, in two halves so
// that a block can do independent work between announcing its arrival and
// waiting for the others.  `epoch` counts the barriers this block has passed;
// the counter is monotone within one launch and reset by the host before it.
// grid_wait returns false when the grid must stop (timeout here or an error
// recorded elsewhere).
__device__ __forceinline__ void grid_arrive(DevStatus *st, unsigned int &epoch) {
  __syncthreads();
  epoch++;
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(&st->barrier, 1u);
  }
}

__device__ __forceinline__ bool grid_wait(DevStatus *st, unsigned int epoch) {
  __shared__ unsigned int s_ok;
  if (threadIdx.x == 0) {
    const unsigned int target = epoch * gridDim.x;
    const unsigned long long t0 = dev_globaltimer();
    unsigned int ok = 1, polls = 0;
    while (ld_acquire_gpu(&st->barrier) < target) {
      if ((++polls & 127u) == 0u) {
        if (ld_volatile_u32(&st->code) != 0u) {
          ok = 0;
          break;
        }
        if (dev_globaltimer() - t0 > kBarrierTimeoutNs) {
          dev_record_error(st, DEV_TIMEOUT_GRID_BARRIER);
          ok = 0;
          break;
        }
      }
    }
    if (ld_volatile_u32(&st->code) != 0u) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ bool grid_barrier(DevStatus *st, unsigned int &epoch) {
  grid_arrive(st, epoch);
  return grid_wait(st, epoch);
}

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Added to every squared distance in FP32: leaves |d|^2 >= ~1e-23 bit-identical
// and turns the coincident case (d = 0) into a zero contribution 0 * (1/tiny)
// instead of 0 * inf, which is what the reference's `dist > 0` guard yields.
constexpr float kTinyD2 = 1e-30f;

// ----------------------------------------------------------------------------
// Host-side helpers
// ----------------------------------------------------------------------------
struct KernelTimer;  // per-kernel CUDA-event timing (api.cu)

namespace bl {

// Force models of the minibatch sweep (sample/algorithms.cpp:759, :912, :985),
// and the two reference algorithms built on the same sweep: algo 7 (FR over
// every CSR neighbour, :536-590) and the second phase of algo 5 (FR with
// unit-vector repulsion, :1112-1125).
enum Model { MODEL_FR = 2, MODEL_LINLOG = 3, MODEL_FA = 8, MODEL_SD = 7, MODEL_GREEDY_EXACT = 5 };

struct DeviceGraph {
  int n = 0;
  long long nnz = 0;
  int *rowptr = nullptr;      // CSR of the graph
  int *colids = nullptr;
  int *eff_rowptr = nullptr;  // neighbours the minibatch cursor actually matches
  int *eff_colids = nullptr;
  int max_eff_degree = 0;
  // every CSR neighbour, each row sorted ascending with duplicates kept
  // (aliases the CSR when its rows are sorted); built on first use
  int *srt_rowptr = nullptr;
  int *srt_colids = nullptr;
  int max_degree = -1;  // -1 until srt_* is built
};

// Level schedule of the Barnes-Hut attraction sweep for one batch size.
struct LevelSchedule {
  int batch = 0;
  int levels = 0;
  std::vector<int> offsets;  // host copy, levels + 1 entries
  int *order = nullptr;      // device: vertices grouped by level
  int *d_offsets = nullptr;  // device copy of offsets
  int *early_off = nullptr;  // per level-order slot: neighbours in earlier batches
  int *early_col = nullptr;
};

struct Scratch {
  // generic
  double *energy_parts = nullptr;  // per-block energy partials
  double *energy = nullptr;        // per-iteration energies (device)
  DevStatus *status = nullptr;
  // minibatch sweep
  float2 *partials = nullptr;
  size_t partials_bytes = 0;
  int *cursor = nullptr;  // per (block, vertex) neighbour cursor start
  int cursor_grid = 0;
  int *cursor_full = nullptr;  // the same for the full sorted rows (algo 7)
  int cursor_full_grid = 0;
  // algo 5, first phase: repulsion sources per vertex as (vertex, count) pairs
  long long *walk_off = nullptr;  // n + 1
  int2 *walk_pairs = nullptr;
  long long walk_total = -1;      // -1 until built
  long long *term_off = nullptr;  // n + 1: CSR entries then walk pairs per vertex
  int2 *terms = nullptr;          // (source, 0 = attraction | k = k x repulsion)
  int *term_tgt = nullptr;        // target vertex of each term
  std::vector<long long> h_term_off;
  int *greedy_share = nullptr;    // [batches][CTAs + 1] target shares of the cluster's CTAs
  long long greedy_share_key = -1;
  float2 *greedy_pos = nullptr;   // second position array (odd number of moves)
  // Barnes-Hut
  size_t bh_n = 0;
  unsigned long long *keys = nullptr, *keys_alt = nullptr;
  int *perm = nullptr, *perm_alt = nullptr;
  unsigned int *hist = nullptr;  // radix histograms / offsets
  int fk_grid = 0;               // resident blocks of the frame/key kernel
  int4 *bnode = nullptr;         // packed binary radix nodes for the chain walk
  int *runs = nullptr;           // runs of equal high key halves: count, (start, length) pairs, overflow
  int runs_cap = 0;
  size_t hist_entries = 0;
  unsigned int *bbox = nullptr;  // frame/key kernel: box (ordered-uint floats) and arrivals
  double *frame = nullptr;       // minX, minY, MAXMIN
  float2 *spos = nullptr;        // positions in Morton order
  int *bparent = nullptr;        // binary radix tree: parent of node (internal i, leaf n-1+k)
  int2 *bchild = nullptr;        // children of internal node (encoded: >= 0 internal, < 0 leaf ~k)
  int2 *brange = nullptr;        // [first, last] of internal node
  int *bdelta = nullptr;         // common prefix length of internal node
  int4 *qkids = nullptr;         // quad children of a quad node
  int *qpar = nullptr;           // quad parent of a quad node / leaf
  int *qnchild = nullptr;        // number of children of a quad node
  int *span = nullptr;           // centroid pass: spanning quad nodes per level (counts, then lists)
  int span_cap = 0;              // list slots per level (centroid blocks)
  void *span_stage = nullptr;    // staged spanning nodes for the cluster pass
  float *ztab = nullptr;         // pre-order records' z by quad level
  void *chain = nullptr;         // centroid pass: nodes spanning one block boundary, per boundary
  double2 *qcen = nullptr;       // centroid of quad node (indexed by binary internal id)
  int *qbelow = nullptr;         // chain length below a quad node
  int *startcnt = nullptr;       // quad nodes starting at each sorted position (n+1)
  int *startbase = nullptr;      // exclusive scan of startcnt (n+1)
  float4 *nodes = nullptr;       // pre-order records {x, y, D^2, skip}
  double2 *nodes_c64 = nullptr;  // FP64 centroid per pre-order record
  unsigned char *nodes_lvl = nullptr;
  float2 *rep = nullptr;         // BH repulsion per vertex
  float4 *f0 = nullptr;          // unmoved-neighbour attraction minus repulsion (float-float)
  unsigned long long *stats = nullptr;
  float2 *pos_alt = nullptr;     // second position buffer (Gauss-Seidel sweep)
};

}  // namespace bl

namespace bl {
struct BatchedState;
struct MpnnState;
struct BhGraph;
}

struct bl_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  // a second stream for work beside the main one inside an iteration (forked
  // from and joined back to `stream` by the two events)
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  std::string err;
  // run options (reference constructor arguments)
  std::string input, outputdir, initfile;
  int init = 0;
  double weight = 1.0, threshold = 0.01;
  // graph
  bl::DeviceGraph g;
  std::vector<int> h_rowptr, h_colids;
  // layout state
  float2 *pos = nullptr;      // current coordinates (float32)
  double2 *force = nullptr;   // forces of the last iteration
  double *e = nullptr;        // |f|^2 per vertex
  double2 *stage = nullptr;   // FP64 staging for coordinate transfers
  bl::Scratch s;
  std::deque<bl::LevelSchedule> schedules;  // stable addresses
  long long launches = 0;
  bool graph_mode = true;
  // timing of one kernel family for the roofline
  std::string timed_kernel;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  double timed_ms = 0.0;
  long long timed_count = 0;
  cudaEvent_t run_ev[2] = {nullptr, nullptr};
  double last_run_ms = 0.0;
  bl::BatchedState *batched = nullptr;  // many-graph layout (batched.cu)
  bl::MpnnState *mpnn = nullptr;        // learned initializer (mpnn.cu)
  bl::BhGraph *bh_graph = nullptr;      // captured Barnes-Hut iteration (barnes_hut.cu)
};

// ---- helpers implemented in api.cu ---------------------------------------
int bl_fail(bl_ctx *ctx, int code, const std::string &msg);
int bl_cuda_fail(bl_ctx *ctx, cudaError_t e, const char *what);
// inside a catch: BL_ERR_HOST, the message on ctx and in msg (msgcap bytes)
int bl_host_exception(bl_ctx *ctx, char *msg = nullptr, int msgcap = 0);
void bl_create_exception();          // inside a catch: message for bl_create_error()
int bl_check_status(bl_ctx *ctx);
void bl_time_begin(bl_ctx *ctx, const char *kernel);
void bl_time_end(bl_ctx *ctx, const char *kernel);

#define BL_CUDA(ctx, call)                                  \
  do {                                                      \
    cudaError_t _e = (call);                                \
    if (_e != cudaSuccess) return bl_cuda_fail(ctx, _e, #call); \
  } while (0)

// ---- kernels drivers (smu.cu, bh.cu, reduce.cu) ----------------------------
namespace bl {
int ensure_minibatch_scratch(bl_ctx *ctx, int batch, int grid);
int minibatch_run(bl_ctx *ctx, int model, int batch, int iterations, double step0,
                  double decay, bool converged, double engt, long long max_loops,
                  double *energy_out, long long *loops_out);
int ensure_sorted_csr(bl_ctx *ctx);
int greedy_walks_build(bl_ctx *ctx);
int greedy_walk_run(bl_ctx *ctx, int batch, int iterations, double step0, double decay, bool want_energy,
                    double *energy_out);
int ensure_bh_scratch(bl_ctx *ctx);
// theta: folded into the walk records; attract_batch > 0: also the
// attraction of the neighbours not yet moved in an iteration with that batch
// size into the force sums (bh_traverse with the same batch adds the rest)
int bh_build(bl_ctx *ctx, const float2 *pos, double theta, int attract_batch = 0);
int bh_traverse(bl_ctx *ctx, double theta, bool want_stats, int batch);
int bh_iteration(bl_ctx *ctx, int batch, double theta, double step, bool want_energy,
                 double *energy_out);
int bh_canonical_tree(bl_ctx *ctx, int cap, int *lo, int *hi, int *depth, int *nchild,
                      double *centroid);
const LevelSchedule *level_schedule(bl_ctx *ctx, int batch);
void cursor_neighbours(int n, const std::vector<int> &rp, const std::vector<int> &ci, std::vector<int> &erp,
                       std::vector<int> &eci);
struct BatchedState;
void batched_free(BatchedState *b);
void mpnn_free(MpnnState *m);
void bh_graph_free(BhGraph *g);
int bh_graph_iterations(bl_ctx *ctx, int batch, double theta, double *step, int count);
int bh_graph_energy_iteration(bl_ctx *ctx, int batch, double theta, double step, double *energy_out);
int bh_run(bl_ctx *ctx, int iterations, int batch, double theta, double *step, double *energy);
int energy_reduce(bl_ctx *ctx, double *out_host);
}  // namespace bl

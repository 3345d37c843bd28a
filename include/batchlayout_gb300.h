/*
 * batchlayout_gb300.h -- C ABI of the GB300 BatchLayout layout engine.
 *
 * The reference (khaled-rahman/BatchLayoutCode) exposes its layout engine as
 * the C++ class `algorithms` (sample/algorithms.h:50-85): a constructor that
 * takes the CSR graph and the run options, one method per layout algorithm
 * returning {energy, seconds} and mutating the coordinates, and writers for
 * the `x<TAB>y<TAB>id` output file.  This header is the same interface as a
 * plain C ABI: opaque context, plain pointers and sizes, int status codes.
 *
 * Conventions
 *   - Coordinates cross the ABI as interleaved x,y pairs (2*n values), double
 *     like the reference's Coordinate<double> (sample/Coordinate.h:27-85);
 *     the device keeps them as float32.
 *   - Every call returns BL_OK (0) or a negative BL_ERR_* code; the message is
 *     available from bl_last_error().  Nothing exits or throws across the ABI.
 *     (The reference prints and calls exit(1), e.g. sample/algorithms.cpp:104-106.)
 *   - A context is used by one host thread at a time; it owns its CUDA stream
 *     and device buffers.  No caller pointer is retained after a call returns.
 *   - `threads` arguments are accepted for signature compatibility with the
 *     reference (OpenMP thread count) and ignored.
 */
#ifndef BATCHLAYOUT_GB300_H
#define BATCHLAYOUT_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define BL_OK 0
#define BL_ERR_ARG (-1)            /* invalid argument                      */
#define BL_ERR_CUDA (-2)           /* CUDA runtime error                    */
#define BL_ERR_DEVICE_TIMEOUT (-3) /* a device-side wait ran out of time    */
#define BL_ERR_UNSUPPORTED (-4)    /* algorithm not on the GPU path         */
#define BL_ERR_TOO_LARGE (-5)      /* problem exceeds a documented limit    */
#define BL_ERR_IO (-6)             /* file could not be read or written     */
#define BL_ERR_STATE (-7)          /* call order violated (e.g. no graph)   */
#define BL_ERR_HOST (-8)           /* host-side failure (memory, threads)   */

typedef struct bl_ctx bl_ctx;

/* ---- context -------------------------------------------------------------- */

/* Replaces algorithms::algorithms(A_csr, input, outputd, init, weight, th, ifile)
 * (sample/algorithms.cpp:3-15).  Copies the CSR (rowptr[n+1], colids[nnz],
 * zero-based, as built by SetInputMatricesAsCSR, sample/commonutility.h:45-54)
 * to the device; 1 <= n <= 2^30 - 1, rowptr[0] = 0, rowptr[n] = nnz,
 * rowptr non-decreasing, 0 <= colids[k] < n (checked before any device call).
 * init: 0 greedy DFS, 1 random, 2 file (`initfile`).
 * init 3 (an extension): the learned start, `initfile` naming the model file.
 * Returns NULL on failure (bl_create_error() then holds the reason). */
bl_ctx *bl_algorithms_create(int device, int n, long long nnz, const int *rowptr,
                             const int *colids, const char *input,
                             const char *outputdir, int init, double weight,
                             double threshold, const char *initfile);
const char *bl_create_error(void);
void bl_destroy(bl_ctx *ctx);
const char *bl_last_error(const bl_ctx *ctx);
int bl_num_vertices(const bl_ctx *ctx);

/* ---- input (host; the reference's L0 graph IO) ------------------------------ */

/* SetInputMatricesAsCSR (sample/commonutility.h:45-54) = ReadASCII (IO.h:60-155)
 * + CSC(triples) (CSC.h:147-190) + CSR(csc) (CSR.h:155-186): symmetric files are
 * mirrored with self loops dropped, colids ascend within each row, duplicates
 * are kept, values are ignored.  *rowptr / *colids are malloc'ed; release them
 * with bl_free.  info[0..3] = rows, cols, nnz, symmetric; seconds = parse time.
 * On error returns BL_ERR_IO and copies the reason into err (errcap bytes). */
int bl_read_matrix_market(const char *path, long long *info, double *seconds, int **rowptr,
                          int **colids, char *err, int errcap);
/* The same through a binary CSR cache (no reference counterpart): with
 * cache_dir not NULL, <cache_dir>/<basename(path)>.blcsr is read instead of
 * the text when it was made from this very file (same canonical absolute
 * path, device and inode) and records its current size and modification
 * time, else the text is parsed and the cache written (a failed write is
 * ignored).  info[4] = 1 when the cache was used, else 0 (info holds 5
 * values); seconds = load time. */
int bl_read_matrix_market_cached(const char *path, const char *cache_dir, long long *info,
                                 double *seconds, int **rowptr, int **colids, char *err,
                                 int errcap);
void bl_free(void *p);

/* ---- coordinates (the reference's nCoordinates) ---------------------------- */

int bl_set_coordinates(bl_ctx *ctx, const double *xy, int n);
int bl_get_coordinates(bl_ctx *ctx, double *xy, int n);
/* Per-vertex forces of the last iteration run (the reference's prevCoordinates). */
int bl_get_forces(bl_ctx *ctx, double *fxy, int n);

/* ---- initialisers (host; sample/algorithms.cpp:16-119) --------------------- */

/* randInit (:16-28) with a private glibc-compatible rand() stream seeded 1,
 * i.e. the reference's sequence when it runs with one thread. */
int bl_rand_init(bl_ctx *ctx);
/* initDFS (:29-97): greedy DFS placement from vertex 0, same rand() stream. */
int bl_init_dfs(bl_ctx *ctx);
/* fileInitialization (:98-119): `x y id` lines read with "%lf %lf %d". */
int bl_file_initialization(bl_ctx *ctx);

/* Breadth-first greedy start (no reference counterpart): initDFS's placement
 * rule (children of u at 0.1 (cos a, sin a) + (r, r) around it, a stepping by
 * 360/deg(u), then scaled to a width of 2*MAXMIN) on a breadth-first tree from
 * vertex 0 (parent = smallest-id neighbour on the previous level), with r a
 * hash of the vertex id: the whole start on the GPU, deterministic, not the
 * reference's layout.  Also selected by init = 4 in bl_algorithms_create. */
int bl_bfs_init(bl_ctx *ctx);

/* Host-only forms of the same initialisers and of writeToFile: no context or
 * GPU needed (xy holds 2*n doubles; the CSR is checked as in
 * bl_algorithms_create, BL_ERR_ARG when it fails). */
int bl_random_coordinates(int n, double *xy);
int bl_greedy_coordinates(int n, const int *rowptr, const int *colids, double *xy);
int bl_write_coordinates(const char *input, const char *outputdir, const char *tag,
                         const double *xy, int n, char *path_out, int path_cap);
/* The neighbours the reference's sorted-CSR cursor matches (kindex,
 * sample/algorithms.cpp:746,758-762), host only: per row the longest
 * strictly ascending prefix; an empty row i with a non-empty row after it
 * matches colids[rowptr[i]], that row's first entry (the cursor starts there
 * and the reference applies attraction to it); empty rows with no non-empty
 * row after them match nothing.
 * matched_rowptr receives n+1 offsets; matched_colids (may be NULL for a
 * counting call) at least matched_rowptr[n] ids, which is at most
 * rowptr[n] + (number of empty rows).  These are the lists every minibatch
 * method attracts over; bl_minibatch_iteration_noalloc takes them as input. */
int bl_cursor_neighbours(int n, const int *rowptr, const int *colids, int *matched_rowptr,
                         int *matched_colids);

/* ---- layout methods: out[0] = energy of the last iteration, out[1] = seconds
 * (wall time including the init, like omp_get_wtime() in the reference).
 * flag == 0 runs the context's initialiser first (init 0/1/2) and STEP = 1;
 * flag == 1 keeps the current coordinates (and, for the minibatch methods,
 * starts at STEP = 0.999^(4*iterations), sample/algorithms.cpp:737). ------ */

/* algo 2: cacheBlockingminiBatchForceDirectedAlgorithm, sample/algorithms.cpp:715-794 */
int bl_cache_blocking_minibatch(bl_ctx *ctx, int iterations, int threads, int batch,
                                int flag, double *out);
/* algo 2 with -engt: ...Converged, sample/algorithms.cpp:795-871; out[2] = loops run */
int bl_cache_blocking_minibatch_converged(bl_ctx *ctx, int iterations, int threads,
                                          int batch, int flag, double *out);
/* algo 3: LinLogcacheBlockingminiBatchForceDirectedAlgorithm, :874-945 */
int bl_linlog_cache_blocking_minibatch(bl_ctx *ctx, int iterations, int threads,
                                       int batch, double *out);
/* algo 8: FAcacheBlockingminiBatchForceDirectedAlgorithm, :947-1018 */
int bl_fa_cache_blocking_minibatch(bl_ctx *ctx, int iterations, int threads, int batch,
                                   double *out);
/* algo 4: BarnesHutApproximation, :1020-1083 (theta = -bht) */
int bl_barnes_hut_approximation(bl_ctx *ctx, int iterations, int threads, int batch,
                                double theta, int flag, double *out);
/* algo 6: approxCacheBlockBH, :1192-1215 (80% BH at theta 1.2, then algo 2) */
int bl_approx_cache_block_bh(bl_ctx *ctx, int iterations, int threads, int batch,
                             double *out);
/* algo 5: approxForceDirectedAlgorithm, :1085-1190 (iterations up to
 * (int)(0.8*iterations): CSR attraction plus the repulsion of a 200-step
 * depth-first walk; the rest: all pairs with unit-vector repulsion; STEP
 * *= 0.99).  Always runs the context's initialiser first, like the reference. */
int bl_approx_force_directed(bl_ctx *ctx, int iterations, int threads, int batch,
                             double *out);
/* algo 7: cacheBlockingminiBatchForceDirectedAlgorithmSD, :517-598
 * (attraction over every CSR neighbour, repulsion over all other vertices). */
int bl_cache_blocking_minibatch_sd(bl_ctx *ctx, int iterations, int threads, int batch,
                                   int flag, double *out);

/* writeToFile (:1244-1256): outputdir + basename(input) + tag + ".txt",
 * lines "x\ty\tid" at 6 significant digits.  The written path is copied to
 * path_out (if not NULL, up to path_cap bytes). */
int bl_write_to_file(bl_ctx *ctx, const char *tag, char *path_out, int path_cap);

/* ---- building blocks exposed for verification and benchmarking ----------- */

/* One minibatch iteration (the while-loop body of :742-780 / :895-933 /
 * :968-1006) at the given STEP.  model: 2 FR, 3 LinLog, 8 FA, 7 (algo 7's
 * body, :540-590), 5 (algo 5's second-phase body, :1112-1125, :1171-1177).
 * energy_out receives sum |f|^2 of this iteration. */
int bl_minibatch_iteration(bl_ctx *ctx, int model, int batch, double step,
                           double *energy_out);
/* One first-phase iteration of algo 5 (:1126-1177) at the given STEP. */
int bl_greedy_iteration(bl_ctx *ctx, int batch, double step, double *energy_out);
/* The repulsion sources of algo 5's first phase (the depth-first walks of
 * :1126-1170; they depend on the graph only) as (source, count) pairs per
 * vertex: offsets[n+1] (int64), up to `cap` sources and counts; *total =
 * number of pairs.  A source a walk reaches k times appears with count k
 * (possibly split over several pairs); pair order within a vertex is not
 * the walk order. */
int bl_greedy_walks(bl_ctx *ctx, long long *offsets, int *sources, int *counts,
                    long long cap, long long *total);
/* One Barnes-Hut iteration (the loop body of :1039-1071) at the given STEP. */
int bl_barnes_hut_iteration(bl_ctx *ctx, int batch, double theta, double step,
                            double *energy_out);

/* Morton frame and order of the current coordinates (MortonCode.h:42-97,
 * BarnesHut.h:121): frame = {minX, minY, MAXMIN}, keys[n] (y-major bit
 * interleave of the two 32-bit quantised coordinates), perm[n]. */
int bl_morton_order(bl_ctx *ctx, double *frame, unsigned long long *keys, int *perm);
/* Quadtree of the current coordinates (BarnesHut.h:135-220) in canonical form:
 * the nodes with at least two children, depth-first pre-order.  Returns the
 * node count (>= 0) or a BL_ERR_* code; arrays must hold `cap` entries
 * (centroid: 2*cap doubles). */
int bl_quadtree(bl_ctx *ctx, int cap, int *lo, int *hi, int *depth, int *nchild,
                double *centroid);
/* Barnes-Hut repulsion sum (BarnesHut.h:69-86) for every vertex against the
 * tree of the current coordinates; out[2n].  stats[0] = node visits,
 * stats[1] = opening tests settled in FP64 (may be NULL). */
int bl_bh_repulsion(bl_ctx *ctx, double theta, double *out, long long *stats);

/* Device-resident run for throughput measurement: `iterations` iterations of
 * algo (2, 3, 4, 5, 7 or 8) from the current device coordinates, no init, no
 * host copies; STEP starts at `step` and decays as in the reference (algo 5
 * switches phase after (int)(0.8*iterations) iterations).
 * energy_out = energy of the last iteration; for algo 4 it may be NULL, and
 * then no energy is computed. */
int bl_run_resident(bl_ctx *ctx, int algo, int iterations, int batch, double theta,
                    double step, double *energy_out);
/* Device time of the last bl_run_resident call: CUDA events recorded on the
 * context's stream before its first and after its last kernel. */
int bl_last_run_ms(bl_ctx *ctx, double *ms);
/* Barnes-Hut iterations (bl_run_resident with algo 4,
 * bl_barnes_hut_iteration, bl_barnes_hut_approximation and the Barnes-Hut
 * part of bl_approx_cache_block_bh) replay captured CUDA graphs of one
 * iteration (1, the default: the iterations without energy one graph, the
 * last iteration the graph that also reduces its energy), or launch every
 * kernel directly (0).  The graphs are captured on first use for the given
 * batch and theta and kept until they change; the results are the same bits
 * either way.  If an iteration cannot be captured its kernels are launched
 * directly. */
int bl_set_graph_mode(bl_ctx *ctx, int enabled);
/* CUDA events around the dominant kernel of the last bl_run_resident call:
 * ms[0] = total milliseconds of that kernel, ms[1] = number of launches. */
int bl_last_kernel_time(bl_ctx *ctx, const char *kernel, double *ms);
/* Number of kernels this library launched since the context was created. */
long long bl_kernel_launches(const bl_ctx *ctx);

/* ---- many graphs in one launch ----------------------------------------------- */

/* No counterpart in the reference, which lays out one graph per process
 * (Test/BatchLayout.cpp:56-182, one algorithms object per run).  A batch of
 * independent graphs is laid out by one persistent kernel (a device work
 * queue, one block per graph, largest graph first), replayed as a CUDA graph.
 * Each graph uses the reference's per-graph semantics: algo 2, 3 or 8 as
 * cacheBlockingminiBatchForceDirectedAlgorithm / LinLog / FA
 * (sample/algorithms.cpp:715-794, 874-1018; all coordinates of the graph in
 * one block's shared memory, so these graphs are limited to about 26k
 * vertices), algo 4 as BarnesHutApproximation (:1020-1083) with the same bits
 * as bl_barnes_hut_iteration.  Every graph starts from the coordinates given
 * and runs `iterations` iterations with STEP = 1 at the start; energy is the
 * reference's ENERGY of its last iteration. */

/* Context without a graph, for the batched calls (free with bl_destroy). */
bl_ctx *bl_batch_create(int device);
/* Upload the graphs.  Graph g has vertex_offset[g+1] - vertex_offset[g]
 * vertices (vertex_offset[0] = 0); its CSR is rowptr[vertex_offset[g] + g ..
 * vertex_offset[g+1] + g] (n+1 entries starting at 0) over
 * colids[edge_offset[g] .. edge_offset[g+1]) with local vertex ids, as
 * SetInputMatricesAsCSR builds it (sample/commonutility.h:26-54); algo[g] is
 * 2, 3, 4 or 8; xy holds 2 * vertex_offset[num_graphs] doubles (x, y per
 * vertex) of starting coordinates. */
int bl_batched_prepare(bl_ctx *ctx, int num_graphs, const int *vertex_offset, const long long *edge_offset,
                       const int *rowptr, const int *colids, const int *algo, const double *xy);
/* Lay out every prepared graph from its starting coordinates (repeatable).
 * The first run of a prepared set autotunes the source split of the
 * minibatch graphs per size bucket; *seconds_out = device time of the run. */
int bl_batched_run(bl_ctx *ctx, int iterations, int batch, double theta, double weight, double *seconds_out);
/* Coordinates after the last run (2 * total vertices doubles, either may be
 * NULL) and the energy of each graph's last iteration. */
int bl_batched_result(bl_ctx *ctx, double *xy, double *energy);
/* prepare + run + result in one call; xy is read and overwritten. */
int bl_batched_layout(bl_ctx *ctx, int num_graphs, const int *vertex_offset, const long long *edge_offset,
                      const int *rowptr, const int *colids, const int *algo, double *xy, int iterations, int batch,
                      double theta, double weight, double *energy_out, double *seconds_out);
/* Source ranges per target the autotuner chose for minibatch graphs below 512,
 * below 2048 and from 2048 vertices (0 = no graph in that bucket). */
int bl_batched_parts(const bl_ctx *ctx, int *parts3);
/* SM clock cycles (clock64) the block spent on each graph in the last run:
 * the load balance of the launch (num_graphs values). */
int bl_batched_graph_cycles(bl_ctx *ctx, unsigned long long *cycles);
/* Fix those choices (1, 2 or 4; 0 = autotune) for the next runs of the
 * prepared set, e.g. to reproduce a run bit for bit. */
int bl_batched_set_parts(bl_ctx *ctx, const int *parts3);

/* ---- learned initializer: the message-passing network ------------------------ */

/* No counterpart in the reference (its initial layouts are random, greedy DFS
 * or read from a file, sample/algorithms.cpp:16-119).  A 3-layer
 * message-passing network (16 input features, 64 hidden, mean aggregation
 * over the CSR neighbours, ReLU) with a linear 64 -> 2 readout predicts
 * initial coordinates; BF16 weights and activations, FP32 accumulation on
 * the tensor cores.  Parameters are one FP32 vector of BL_MPNN_PARAMS values:
 * W1 (64 x 32), b1 (64), W2 (64 x 128), b2 (64), W3 (64 x 128), b3 (64),
 * Wo (2 x 64), bo (2); row o of W_l holds the weights of output o over
 * [own features | mean of the neighbours' features]. */
#define BL_MPNN_PARAMS 18754
#define BL_MPNN_FEATURES 16

/* Load / read the parameters of the context's network (any context). */
int bl_mpnn_set_params(bl_ctx *ctx, const float *params);
int bl_mpnn_get_params(bl_ctx *ctx, float *params);
/* One forward pass over a graph given as host arrays (CSR rowptr[n+1],
 * colids, features[n*16] row-major): xy[2n] receives the predicted
 * coordinates and, if h is not NULL, h[3*n*64] the BF16 activations of the
 * three layers.  With target != NULL (2n values) and vweight (n values) the
 * loss sum_v vweight[v] * |xy_v - target_v|^2 and its gradient with respect
 * to the parameters (grad[BL_MPNN_PARAMS]) are computed as well. */
int bl_mpnn_run(bl_ctx *ctx, int n, const int *rowptr, const int *colids, const float *features,
                const float *target, const float *vweight, float *xy, unsigned short *h, double *loss,
                float *grad);

/* Input features of the network for one graph (host arrays): multi-source
 * BFS hop distances to 16 pivots (given, or drawn with splitmix64 from seed
 * when pivots is NULL), pivot-MDS component scores 1-12 of the double-centred
 * squared distances scaled to unit mean square of component 1, then
 * log2(1+deg), 1/(1+deg), the neighbours' mean log2(1+deg) and log2(n)/20.
 * features: n*16 floats; dist (optional): n*16 hop distances, 0xFFFF for an
 * unreachable pivot; pivots_out (optional): the 16 pivots used. */
int bl_learned_features(bl_ctx *ctx, int n, const int *rowptr, const int *colids, int seed, const int *pivots,
                        float *features, unsigned short *dist, int *pivots_out);

/* Train the network on graphs and their target layouts (what algo 4 produced
 * for them): graphs as in bl_batched_prepare, layouts 2 * total vertices
 * doubles.  The network learns the residual between each target, fitted to
 * the graph's first two MDS components y by a similarity transform, and y.
 * params holds the starting parameters and receives the trained ones;
 * scale_model[3] receives {a, b, c} of log l = a + b log n + c log(mean
 * degree), l the mean edge length of a target; loss_history (optional) one
 * loss per epoch.  Full-batch Adam, cosine learning rate from lr, pivots
 * drawn from seed + graph index. */
int bl_learned_train(bl_ctx *ctx, int num_graphs, const int *vertex_offset, const long long *edge_offset,
                     const int *rowptr, const int *colids, const double *layouts, int epochs, double lr, int seed,
                     float *params, double *scale_model, double *loss_history);
/* Read a model file (8 bytes "BLMPNN01", uint32 parameter count, the FP32
 * parameters, the three FP64 scale-model coefficients, all little-endian). */
int bl_learned_load_model(const char *path, float *params, double *scale_model);
/* Replace the context's coordinates by the learned start for its graph (the
 * learned counterpart of bl_init_dfs): y + network output, scaled to the mean
 * edge length the scale model predicts. */
int bl_learned_init(bl_ctx *ctx, const float *params, const double *scale_model, int seed);
/* Learned start, then Barnes-Hut iterations (batch, theta; STEP from step0,
 * times 0.999 per iteration, as :1070) until the energy of an iteration is at
 * most target_energy or max_iterations ran; if the target was not reached,
 * the plain run instead: greedy DFS start and max_iterations iterations from
 * STEP = 1.  out[5] = {energy, wall seconds, refinement iterations, 1 if the
 * plain run was used, seconds of the learned start}. */
int bl_learned_layout(bl_ctx *ctx, const float *params, const double *scale_model, int seed, int max_iterations,
                      int batch, double theta, double target_energy, double step0, double *out);

/* ---- bounded device waits --------------------------------------------------- */

/* No counterpart in the reference (which has no device waits).  Runs one of
 * the bounded waits the layout kernels use, with its arrival made
 * (complete = 1) or withheld (complete = 0): site 0 the grid barrier of the
 * cooperative kernels (limit 2 s), site 1 the mbarrier wait for tensor-core
 * completion (limit 1 s).  A withheld arrival lets the wait run to its limit;
 * the kernel then records the site and returns, and the call returns
 * BL_ERR_DEVICE_TIMEOUT with the reason in bl_last_error -- the path every
 * layout call takes when a device wait runs out.  The context stays usable. */
int bl_wait_selftest(bl_ctx *ctx, int site, int complete);

/* ---- allocation-free variant ------------------------------------------------ */

/* No counterpart in the reference.  One minibatch iteration (as
 * bl_minibatch_iteration) for callers that cannot allocate device memory while
 * they run -- services that reserve all GPU memory up front in their own pool,
 * real-time loops that forbid allocation after start-up, code enqueuing on a
 * stream another component owns.  It allocates nothing: its scratch is a fixed
 * 768 KiB device array inside the library, which limits batch to 256 and the
 * launch to 160 blocks (larger requests return BL_ERR_TOO_LARGE).
 * Device pointers, all caller-owned, on the current device:
 *   d_rowptr[n+1], d_colids   neighbour lists the minibatch cursor matches,
 *                             as bl_cursor_neighbours builds them on the host
 *                             (the CSR rows themselves only when every row is
 *                             sorted ascending without duplicates AND no row
 *                             but the last is empty: an empty row matches the
 *                             next row's first neighbour)
 *   d_xy[2n] float32           coordinates, updated in place
 *   d_force[2n], d_vertex_energy[n]  outputs: forces and |f|^2 per vertex
 * stream: cudaStream_t (NULL = default stream); the call returns after the
 * stream has finished it.  The first call on a device fetches the scratch
 * array's device address: make it before any stream capture.  All calls on a
 * device share the scratch, so calls that overlap on the GPU race. */
int bl_minibatch_iteration_noalloc(int n, const int *d_rowptr, const int *d_colids, float *d_xy,
                                   double *d_force, double *d_vertex_energy, int model, int batch,
                                   double weight, double step, double *energy_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* BATCHLAYOUT_GB300_H */

// oracle.cpp -- FP64 CPU restatement of BatchLayout's layout hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: tests/ compare
// the CUDA path against it, __graft_entry__.smoke() checks one small GPU run
// against it, and bench.py times it as the CPU baseline ("port").  The product
// path (batchlayoutcode_gb300/) never links, loads or calls it.
//
// Every routine restates a reference routine in plain FP64 C++ and follows its
// operation order so that a strict (no -ffast-math, -ffp-contract=off) build of
// the reference and this file agree bit for bit.  Reference citations are
// paths inside khaled-rahman/BatchLayoutCode.
//
// Documented deviations (all unreachable on valid, connected, duplicate-free
// inputs, which is what the reference itself assumes):
//   * zero force: the reference's Coordinate::getUnitVector divides 0/0 and
//     writes NaN (sample/Coordinate.h:63-64); here the update is skipped.
//   * kindex read past the end of colids for an isolated last vertex
//     (sample/algorithms.cpp:758 with rowptr[n-1]==nnz): treated as "no
//     neighbour".
//   * coincident quantised points make the reference's build_tree recurse
//     forever (sample/BarnesHut.h:3,156); here recursion stops at level bit 0
//     and the remaining points become leaves of that node.
//   * -engt convergence loop has no iteration cap in the reference
//     (sample/algorithms.cpp:818); here it stops after max_loops.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct P2 {
  double x, y;
};

// ---------------------------------------------------------------------------
// Force laws of the minibatch sweep.  `d` is x_j - x_i.
//   FR     sample/algorithms.cpp:759  f += d * (W * |d|)
//   LinLog sample/algorithms.cpp:912  f += d * log2(1 + W*|d|)
//   FA     sample/algorithms.cpp:985  f += d * W
// Repulsion (all three) sample/algorithms.cpp:764-768: f -= d * (1/|d|^2), |d|^2>0
// ---------------------------------------------------------------------------
enum { MODEL_FR = 2, MODEL_LINLOG = 3, MODEL_FA = 8 };

inline void attraction(int model, double W, double dx, double dy, double &fx,
                       double &fy) {
  if (model == MODEL_FR) {
    double s = W * std::sqrt(dx * dx + dy * dy);
    fx += dx * s;
    fy += dy * s;
  } else if (model == MODEL_LINLOG) {
    double s = std::log2(1.0 + W * std::sqrt(dx * dx + dy * dy));
    fx += dx * s;
    fy += dy * s;
  } else {
    fx += dx * W;
    fy += dy * W;
  }
}

// Minibatch position update + energy, sample/algorithms.cpp:775-779:
//   x_i = x_i + unit(f_i) * STEP ;  E += |f_i|^2
inline void apply_update(P2 &p, double fx, double fy, double step) {
  double mag = std::sqrt(fx * fx + fy * fy);
  if (mag > 0) {
    double ux = fx / mag, uy = fy / mag;
    p.x = p.x + ux * step;
    p.y = p.y + uy * step;
  }
}

// One pass of the iteration body of cacheBlockingminiBatchForceDirectedAlgorithm
// (sample/algorithms.cpp:742-780), LinLog (:895-933) and FA (:968-1006).
// The j loop is blocked by 512 with a fresh accumulator per block (:753-771),
// and the sorted-CSR cursor kindex (:746,758-762) decides whether a source is
// a neighbour (attraction) or not (repulsion).
// `replay` (optional): instead of moving a batch by its own forces, set it to
// replay[i] -- the positions another implementation produced -- so that every
// batch is evaluated from that implementation's batch-start state.
double smu_iteration(int model, int n, const int *rowptr, const int *colids,
                     P2 *pos, int batch, double W, double step, P2 *force_out,
                     int nthreads, const P2 *replay = nullptr) {
  const int blocky = 512;
  const long long nnz = rowptr[n];
  std::vector<P2> prev(n, P2{0.0, 0.0});
  std::vector<long long> kindex(n);
  for (int k = 0; k < n; k++) kindex[k] = rowptr[k];
  double energy = 0.0;
  const int nbatches = (int)std::ceil(1.0 * n / batch);
  for (int b = 0; b < nbatches; b++) {
    const int i0 = b * batch;
    const int i1 = std::min(n, (b + 1) * batch);
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int i = i0; i < i1; i++) {
      const P2 pi = pos[i];
      long long k = kindex[i];
      double px = 0.0, py = 0.0;
      for (int j0 = 0; j0 < n; j0 += blocky) {
        const int j1 = std::min(n, j0 + blocky);
        double fx = 0.0, fy = 0.0;
        for (int j = j0; j < j1; j++) {
          const double dx = pos[j].x - pi.x, dy = pos[j].y - pi.y;
          if (k < nnz && j == colids[k]) {
            attraction(model, W, dx, dy, fx, fy);
            if (k < (long long)rowptr[i + 1] - 1) k++;
          } else {
            const double dist = dx * dx + dy * dy;
            if (dist > 0) {
              const double r = 1.0 / dist;
              fx = fx - dx * r;
              fy = fy - dy * r;
            }
          }
        }
        px += fx;
        py += fy;
      }
      kindex[i] = k;
      prev[i] = P2{px, py};
    }
    for (int i = i0; i < i1; i++) {
      if (replay) pos[i] = replay[i];
      else apply_update(pos[i], prev[i].x, prev[i].y, step);
      energy += prev[i].x * prev[i].x + prev[i].y * prev[i].y;
    }
  }
  if (force_out)
    for (int i = 0; i < n; i++) force_out[i] = prev[i];
  return energy;
}

// ---------------------------------------------------------------------------
// Morton order, sample/MortonCode.h:42-97.
//   q(x) = (uint32)(4294967295.0 * (x - minX) / MAXMIN), likewise y;
//   order = interleaved bits, y more significant at every level.
// The oracle expresses the order as one 64-bit key: bit 2b+1 = qy bit b,
// bit 2b = qx bit b, which compares exactly like the reference comparator.
// ---------------------------------------------------------------------------
struct Frame {
  double minX, minY, maxmin;
};

Frame morton_frame(int n, const P2 *p) {
  double mnx = p[0].x, mxx = p[0].x, mny = p[0].y, mxy = p[0].y;
  for (int i = 1; i < n; i++) {
    mnx = std::min(mnx, p[i].x);
    mxx = std::max(mxx, p[i].x);
    mny = std::min(mny, p[i].y);
    mxy = std::max(mxy, p[i].y);
  }
  Frame f;
  f.minX = mnx;
  f.minY = mny;
  f.maxmin = std::max(mxy - mny, mxx - mnx);  // MortonCode.h:52
  return f;
}

inline uint32_t qscale(double v, double mn, double maxmin) {
  return (uint32_t)(4294967295.0 * (v - mn) / maxmin);  // MortonCode.h:62-67
}

inline uint64_t spread32(uint32_t v) {
  uint64_t x = v;
  x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
  x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
  x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
  x = (x | (x << 2)) & 0x3333333333333333ull;
  x = (x | (x << 1)) & 0x5555555555555555ull;
  return x;
}

inline uint64_t morton_key(const P2 &p, const Frame &f) {
  return (spread32(qscale(p.y, f.minY, f.maxmin)) << 1) |
         spread32(qscale(p.x, f.minX, f.maxmin));
}

// ---------------------------------------------------------------------------
// Quadtree, sample/BarnesHut.h:135-220 (build) and :69-86 (traversal).
// Nodes hold a point range of the Morton-sorted array; a quadrant with one
// point is a leaf point, one with more is a child node; the centroid is the
// unweighted mean of the present children (child centroids or points) summed
// in quadrant order; the root diameter is MAXMIN and halves per level.
// ---------------------------------------------------------------------------
struct Node {
  double cx, cy, diameter;
  int lo, hi;      // sorted point range [lo, hi)
  int depth;       // 0 at the root (level bit 1<<31)
  int child[4];    // node index or -1
  int leaf[4];     // sorted point index or -1
};

struct Tree {
  std::vector<Node> nodes;
  std::vector<P2> pts;        // sorted points
  std::vector<uint64_t> keys; // sorted keys
};

int build_node(Tree &t, int lo, int hi, int depth, double diameter) {
  // quadrant bounds via the 2 key bits of this level (BarnesHut.h:143-146)
  int bounds[5];
  bounds[0] = lo;
  bounds[4] = hi;
  const int shift = 62 - 2 * depth;
  int q = lo;
  for (int quad = 1; quad < 4; quad++) {
    if (depth < 32)
      while (q < hi && (int)((t.keys[q] >> shift) & 3u) < quad) q++;
    else
      q = hi;  // level bit exhausted: every point in quadrant 0
    bounds[quad] = q;
  }
  if (depth >= 32) {
    // coincident quantised points: stop (the reference never terminates)
    bounds[1] = bounds[2] = bounds[3] = hi;
  }
  Node nd;
  nd.lo = lo;
  nd.hi = hi;
  nd.depth = depth;
  nd.diameter = diameter;
  for (int k = 0; k < 4; k++) nd.child[k] = nd.leaf[k] = -1;
  const int idx = (int)t.nodes.size();
  t.nodes.push_back(nd);
  const double sub_diameter = diameter / 2.0;
  int child[4] = {-1, -1, -1, -1}, leaf[4] = {-1, -1, -1, -1};
  for (int k = 0; k < 4; k++) {
    const int c = bounds[k + 1] - bounds[k];
    if (c > 1) {
      if (depth >= 32) {
        // bucket: expose the points as leaves one by one (deviation, see top)
        continue;
      }
      child[k] = build_node(t, bounds[k], bounds[k + 1], depth + 1, sub_diameter);
    } else if (c == 1) {
      leaf[k] = bounds[k];
    }
  }
  double cx = 0.0, cy = 0.0, count = 0;
  for (int k = 0; k < 4; k++) {
    if (child[k] >= 0) {
      cx += t.nodes[child[k]].cx;
      cy += t.nodes[child[k]].cy;
      count++;
    } else if (leaf[k] >= 0) {
      cx += t.pts[leaf[k]].x;
      cy += t.pts[leaf[k]].y;
      count++;
    }
  }
  if (depth >= 32) {
    for (int p = lo; p < hi; p++) {
      cx += t.pts[p].x;
      cy += t.pts[p].y;
      count++;
    }
  }
  if (count > 0) {
    cx /= count;
    cy /= count;
  }
  Node &me = t.nodes[idx];
  me.cx = cx;
  me.cy = cy;
  for (int k = 0; k < 4; k++) {
    me.child[k] = child[k];
    me.leaf[k] = leaf[k];
  }
  return idx;
}

void build_tree(Tree &t, int n, const P2 *p, Frame &frame, std::vector<int> &perm) {
  frame = morton_frame(n, p);
  std::vector<uint64_t> keys(n);
  for (int i = 0; i < n; i++) keys[i] = morton_key(p[i], frame);
  perm.resize(n);
  for (int i = 0; i < n; i++) perm[i] = i;
  std::stable_sort(perm.begin(), perm.end(),
                   [&](int a, int b) { return keys[a] < keys[b]; });
  t.nodes.clear();
  t.nodes.reserve(2 * (size_t)n);
  t.pts.resize(n);
  t.keys.resize(n);
  for (int i = 0; i < n; i++) {
    t.pts[i] = p[perm[i]];
    t.keys[i] = keys[perm[i]];
  }
  build_node(t, 0, n, 0, frame.maxmin / 1.0);  // gridLength(1), BarnesHut.h:128
}

// `visits` (optional) counts the records a stackless pre-order walk of the
// canonical tree (no single-child chain nodes) reads for the same decisions:
// the leaf points reached and the nodes tested, where a chain of
// single-child nodes counts once (its head is tested; the canonical node at
// its foot has the same centroid and a smaller diameter, so it is accepted
// whenever the head is, and is tested in the head's place otherwise).
static int present_children(const Tree &t, const Node &nd) {
  if (nd.depth >= 32) return nd.hi - nd.lo;
  int nc = 0;
  for (int k = 0; k < 4; k++) nc += (nd.child[k] >= 0) || (nd.leaf[k] >= 0);
  (void)t;
  return nc;
}

void bh_force(const Tree &t, int node, const P2 &v, double theta, double &fx,
              double &fy, long long *visits = nullptr, bool counted = true) {
  const Node &nd = t.nodes[node];
  if (visits && counted) ++*visits;
  const double dx = nd.cx - v.x, dy = nd.cy - v.y;
  const double distance = std::sqrt(dx * dx + dy * dy);
  if (nd.diameter / distance < theta) {
    const double r = 1.0 / distance;
    fx = fx + dx * r;
    fy = fy + dy * r;
    return;
  }
  for (int k = 0; k < 4; k++) {
    if (nd.child[k] >= 0) {
      bh_force(t, nd.child[k], v, theta, fx, fy, visits, visits && present_children(t, nd) >= 2);
    } else if (nd.leaf[k] >= 0) {
      if (visits) ++*visits;
      const P2 &q = t.pts[nd.leaf[k]];
      const double ex = q.x - v.x, ey = q.y - v.y;
      const double den = std::sqrt(ex * ex + ey * ey);
      if (den > 0) {
        const double r = 1.0 / den;
        fx = fx + ex * r;
        fy = fy + ey * r;
      }
    }
  }
  if (nd.depth >= 32) {
    for (int p = nd.lo; p < nd.hi; p++) {
      if (visits) ++*visits;
      const P2 &q = t.pts[p];
      const double ex = q.x - v.x, ey = q.y - v.y;
      const double den = std::sqrt(ex * ex + ey * ey);
      if (den > 0) {
        const double r = 1.0 / den;
        fx = fx + ex * r;
        fy = fy + ey * r;
      }
    }
  }
}

// One pass of the BarnesHutApproximation loop body (sample/algorithms.cpp:1039-1071).
double bh_iteration(int n, const int *rowptr, const int *colids, P2 *pos,
                    int batch, double theta, double W, double step,
                    P2 *force_out, int nthreads, const P2 *replay = nullptr) {
  std::vector<P2> prev(n, P2{0.0, 0.0});
  Tree t;
  Frame fr;
  std::vector<int> perm;
  build_tree(t, n, pos, fr, perm);  // snapshot of the iteration start (:1044-1047)
  double energy = 0.0;
  const int nbatches = (int)std::ceil(1.0 * n / batch);
  for (int b = 0; b < nbatches; b++) {
    const int i0 = b * batch, i1 = std::min(n, (b + 1) * batch);
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int i = i0; i < i1; i++) {
      double fx = 0.0, fy = 0.0;
      const P2 pi = pos[i];
      for (int e = rowptr[i]; e < rowptr[i + 1]; e++) {
        const P2 pj = pos[colids[e]];
        const double dx = pj.x - pi.x, dy = pj.y - pi.y;
        const double s = W * std::sqrt(dx * dx + dy * dy);
        fx = fx + dx * s;
        fy = fy + dy * s;
      }
      double rx = 0.0, ry = 0.0;
      bh_force(t, 0, pi, theta, rx, ry);
      prev[i] = P2{fx - rx, fy - ry};
    }
    for (int i = i0; i < i1; i++) {
      if (replay) pos[i] = replay[i];
      else apply_update(pos[i], prev[i].x, prev[i].y, step);
      energy += prev[i].x * prev[i].x + prev[i].y * prev[i].y;
    }
  }
  if (force_out)
    for (int i = 0; i < n; i++) force_out[i] = prev[i];
  return energy;
}

// ---------------------------------------------------------------------------
// Algo 5, greedy approximation (approxForceDirectedAlgorithm,
// sample/algorithms.cpp:1085-1190).
//
// First phase (iterations LOOP <= (int)(0.8 * ITERATIONS), :1110, :1126):
// f_i = attraction W|d|d over every CSR neighbour of i, plus calcRepulsion
// (:128-133, -d/|d|^2 when |d|^2 > 0) for every vertex a depth-first walk
// reaches (:1126-1170): the stack starts with i's neighbours in CSR order;
// popping u scans u's CSR row and, for each entry v outside {i} u N(i),
// adds v's repulsion, pushes v and decrements a budget of 200; the walk stops
// after the row in which the budget reaches 0, or when the stack is empty.
// Visited vertices are not marked, so a vertex can be reached (and repel)
// more than once.  The walk depends on the graph only.
// Second phase (LOOP > approx, :1112-1125): the kindex cursor of algo 2 with
// attraction W|d|d and repulsion -d/|d| (a unit vector) for every other
// vertex with |d| > 0, one accumulator over all j.  STEP *= t = 0.99
// (algorithms.h:44) in both phases.
// ---------------------------------------------------------------------------
constexpr int kGreedyBudget = 200;  // countNodes (:1147)

// Repulsion sources of vertex i in walk order (appended to `out`).
void greedy_walk(int n, const int *rowptr, const int *colids, int i, std::vector<int> &inset,
                 std::vector<int> &stack, std::vector<int> &out) {
  (void)n;
  inset.assign(colids + rowptr[i], colids + rowptr[i + 1]);
  inset.push_back(i);
  std::sort(inset.begin(), inset.end());
  auto member = [&](int v) { return std::binary_search(inset.begin(), inset.end(), v); };
  stack.assign(colids + rowptr[i], colids + rowptr[i + 1]);
  int budget = kGreedyBudget;
  while (!stack.empty()) {
    const int u = stack.back();
    stack.pop_back();
    for (int e = rowptr[u]; e < rowptr[u + 1]; e++) {
      const int v = colids[e];
      if (!member(v)) {
        out.push_back(v);
        stack.push_back(v);
        budget--;
      }
    }
    if (budget <= 0) break;
  }
}

struct Walks {
  std::vector<long long> off;  // n + 1
  std::vector<int> src;
};

void greedy_walks(int n, const int *rowptr, const int *colids, Walks &w) {
  w.off.assign(n + 1, 0);
  w.src.clear();
  std::vector<int> inset, stack;
  for (int i = 0; i < n; i++) {
    greedy_walk(n, rowptr, colids, i, inset, stack, w.src);
    w.off[i + 1] = (long long)w.src.size();
  }
}

// One iteration of the first phase (:1126-1177).
double greedy_walk_iteration(int n, const int *rowptr, const int *colids, const Walks &w, P2 *pos,
                             int batch, double W, double step, P2 *force_out, int nthreads,
                             const P2 *replay = nullptr) {
  std::vector<P2> prev(n, P2{0.0, 0.0});
  double energy = 0.0;
  const int nbatches = (int)std::ceil(1.0 * n / batch);
  for (int b = 0; b < nbatches; b++) {
    const int i0 = b * batch, i1 = std::min(n, (b + 1) * batch);
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int i = i0; i < i1; i++) {
      const P2 pi = pos[i];
      double fx = 0.0, fy = 0.0;
      for (int e = rowptr[i]; e < rowptr[i + 1]; e++) {
        const P2 pj = pos[colids[e]];
        const double dx = pj.x - pi.x, dy = pj.y - pi.y;
        const double s = W * std::sqrt(dx * dx + dy * dy);
        fx += dx * s;
        fy += dy * s;
      }
      for (long long k = w.off[i]; k < w.off[i + 1]; k++) {
        const P2 pj = pos[w.src[k]];
        const double dx = pj.x - pi.x, dy = pj.y - pi.y;
        const double d2 = dx * dx + dy * dy;
        double tx = 0.0, ty = 0.0;
        if (d2 > 0) {
          const double r = 1.0 / d2;
          tx = tx - dx * r;
          ty = ty - dy * r;
        }
        fx += tx;
        fy += ty;
      }
      prev[i] = P2{fx, fy};
    }
    for (int i = i0; i < i1; i++) {
      if (replay) pos[i] = replay[i];
      else apply_update(pos[i], prev[i].x, prev[i].y, step);
      energy += prev[i].x * prev[i].x + prev[i].y * prev[i].y;
    }
  }
  if (force_out)
    for (int i = 0; i < n; i++) force_out[i] = prev[i];
  return energy;
}

// One iteration of the second phase (:1112-1125, :1171-1177).
double greedy_exact_iteration(int n, const int *rowptr, const int *colids, P2 *pos, int batch, double W,
                              double step, P2 *force_out, int nthreads, const P2 *replay = nullptr) {
  const long long nnz = rowptr[n];
  std::vector<P2> prev(n, P2{0.0, 0.0});
  double energy = 0.0;
  const int nbatches = (int)std::ceil(1.0 * n / batch);
  for (int b = 0; b < nbatches; b++) {
    const int i0 = b * batch, i1 = std::min(n, (b + 1) * batch);
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int i = i0; i < i1; i++) {
      const P2 pi = pos[i];
      long long k = rowptr[i];
      double fx = 0.0, fy = 0.0;
      for (int j = 0; j < n; j++) {
        const double dx = pos[j].x - pi.x, dy = pos[j].y - pi.y;
        if (k < nnz && j == colids[k]) {
          const double s = W * std::sqrt(dx * dx + dy * dy);
          fx += dx * s;
          fy += dy * s;
          if (k < (long long)rowptr[i + 1] - 1) k++;
        } else {
          const double dist = std::sqrt(dx * dx + dy * dy);
          if (dist > 0) {
            const double r = 1.0 / dist;
            fx = fx - dx * r;
            fy = fy - dy * r;
          }
        }
      }
      prev[i] = P2{fx, fy};
    }
    for (int i = i0; i < i1; i++) {
      if (replay) pos[i] = replay[i];
      else apply_update(pos[i], prev[i].x, prev[i].y, step);
      energy += prev[i].x * prev[i].x + prev[i].y * prev[i].y;
    }
  }
  if (force_out)
    for (int i = 0; i < n; i++) force_out[i] = prev[i];
  return energy;
}

// ---------------------------------------------------------------------------
// Algo 7, cacheBlockingminiBatchForceDirectedAlgorithmSD
// (sample/algorithms.cpp:517-598): every CSR neighbour adds W|d|d + d/|d|^2,
// then the repulsion d/|d|^2 of every other vertex (j < i, then j > i, no
// distance guard) is subtracted.  STEP *= 0.999.
// Deviation: a coincident pair (|d| = 0) contributes 0 here; the reference
// computes 0 * inf = NaN.
// ---------------------------------------------------------------------------
double sd_iteration(int n, const int *rowptr, const int *colids, P2 *pos, int batch, double W, double step,
                    P2 *force_out, int nthreads, const P2 *replay = nullptr) {
  std::vector<P2> prev(n, P2{0.0, 0.0});
  double energy = 0.0;
  auto inv2 = [](double dx, double dy) {
    const double d2 = dx * dx + dy * dy;
    return d2 > 0 ? 1.0 / d2 : 0.0;
  };
  const int nbatches = (int)std::ceil(1.0 * n / batch);
  for (int b = 0; b < nbatches; b++) {
    const int i0 = b * batch, i1 = std::min(n, (b + 1) * batch);
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int i = i0; i < i1; i++) {
      const P2 pi = pos[i];
      double px = 0.0, py = 0.0;
      for (int e = rowptr[i]; e < rowptr[i + 1]; e++) {
        const P2 pj = pos[colids[e]];
        const double dx = pj.x - pi.x, dy = pj.y - pi.y;
        const double s = W * std::sqrt(dx * dx + dy * dy);
        const double r = inv2(dx, dy);
        px += dx * s + dx * r;
        py += dy * s + dy * r;
      }
      double fx = 0.0, fy = 0.0;
      for (int j = 0; j < n; j++) {
        if (j == i) continue;
        const double dx = pos[j].x - pi.x, dy = pos[j].y - pi.y;
        const double r = inv2(dx, dy);
        fx += dx * r;
        fy += dy * r;
      }
      prev[i] = P2{px - fx, py - fy};
    }
    for (int i = i0; i < i1; i++) {
      if (replay) pos[i] = replay[i];
      else apply_update(pos[i], prev[i].x, prev[i].y, step);
      energy += prev[i].x * prev[i].x + prev[i].y * prev[i].y;
    }
  }
  if (force_out)
    for (int i = 0; i < n; i++) force_out[i] = prev[i];
  return energy;
}

}  // namespace

extern "C" {

// Morton frame, keys and stable sort permutation (MortonCode.h, BarnesHut.h:121).
// frame_out = {minX, minY, MAXMIN}; keys_out/perm_out in sorted order.
int orc_morton_sort(int n, const double *xy, double *frame_out,
                    uint64_t *keys_out, int *perm_out) {
  if (n < 1) return -1;
  const P2 *p = reinterpret_cast<const P2 *>(xy);
  Frame f = morton_frame(n, p);
  std::vector<uint64_t> keys(n);
  for (int i = 0; i < n; i++) keys[i] = morton_key(p[i], f);
  std::vector<int> perm(n);
  for (int i = 0; i < n; i++) perm[i] = i;
  std::stable_sort(perm.begin(), perm.end(),
                   [&](int a, int b) { return keys[a] < keys[b]; });
  frame_out[0] = f.minX;
  frame_out[1] = f.minY;
  frame_out[2] = f.maxmin;
  for (int i = 0; i < n; i++) {
    perm_out[i] = perm[i];
    keys_out[i] = keys[perm[i]];
  }
  return 0;
}

// Canonical (compressed) quadtree: every reference node that has at least two
// children, in depth-first pre-order.  Chain nodes with a single child node
// carry the same centroid as that child and open exactly when it does, so they
// are omitted.  Returns the node count or -needed when cap is too small.
int orc_bh_tree(int n, const double *xy, int cap, int *lo, int *hi, int *depth,
                int *nchild, double *cxy) {
  const P2 *p = reinterpret_cast<const P2 *>(xy);
  Tree t;
  Frame fr;
  std::vector<int> perm;
  build_tree(t, n, p, fr, perm);
  // pre-order walk
  std::vector<int> stack{0};
  int count = 0;
  std::vector<int> order;
  while (!stack.empty()) {
    int v = stack.back();
    stack.pop_back();
    const Node &nd = t.nodes[v];
    int nc = 0;
    for (int k = 0; k < 4; k++) nc += (nd.child[k] >= 0) || (nd.leaf[k] >= 0);
    if (nd.depth >= 32) nc = nd.hi - nd.lo;
    if (nc >= 2) order.push_back(v);
    for (int k = 3; k >= 0; k--)
      if (nd.child[k] >= 0) stack.push_back(nd.child[k]);
  }
  count = (int)order.size();
  if (count > cap) return -count;
  for (int m = 0; m < count; m++) {
    const Node &nd = t.nodes[order[m]];
    int nc = 0;
    for (int k = 0; k < 4; k++) nc += (nd.child[k] >= 0) || (nd.leaf[k] >= 0);
    if (nd.depth >= 32) nc = nd.hi - nd.lo;
    lo[m] = nd.lo;
    hi[m] = nd.hi;
    depth[m] = nd.depth;
    nchild[m] = nc;
    cxy[2 * m] = nd.cx;
    cxy[2 * m + 1] = nd.cy;
  }
  return count;
}

// Barnes-Hut repulsion R(v) = sum of unit vectors (BarnesHut.h:69-86) for
// each query, from the tree built over tree_xy.  The layout step subtracts it.
int orc_bh_repulsion(int n, const double *tree_xy, int nq, const double *q_xy,
                     double theta, double *out, int nthreads, long long *visits_out) {
  const P2 *p = reinterpret_cast<const P2 *>(tree_xy);
  Tree t;
  Frame fr;
  std::vector<int> perm;
  build_tree(t, n, p, fr, perm);
  const P2 *q = reinterpret_cast<const P2 *>(q_xy);
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
  for (int i = 0; i < nq; i++) {
    double fx = 0.0, fy = 0.0;
    long long vis = 0;
    bh_force(t, 0, q[i], theta, fx, fy, visits_out ? &vis : nullptr);
    out[2 * i] = fx;
    out[2 * i + 1] = fy;
    if (visits_out) visits_out[i] = vis;
  }
  return 0;
}

// Whole-run restatement of the layout methods of class algorithms
// (sample/algorithms.h:74-80), starting from coordinates already initialised
// (the init step is separate, see orc_init_*).
//   algo 2 : cacheBlockingminiBatchForceDirectedAlgorithm        (:715-794)
//   algo 2 with engt != 0.01 : ...Converged                       (:795-871)
//   algo 3 : LinLogcacheBlockingminiBatchForceDirectedAlgorithm   (:874-945)
//   algo 4 : BarnesHutApproximation                              (:1020-1083)
//   algo 5 : approxForceDirectedAlgorithm                        (:1085-1190)
//   algo 6 : approxCacheBlockBH                                  (:1192-1215)
//   algo 7 : cacheBlockingminiBatchForceDirectedAlgorithmSD      (:517-598)
//   algo 8 : FAcacheBlockingminiBatchForceDirectedAlgorithm       (:947-1018)
// step_in < 0 means STEP starts at 1.0 (flag == 0); otherwise STEP starts at
// step_in (the flag == 1 entry of algo 6's second phase, :737).
// result_out = {energy of the last iteration, iterations run}.
// force_out (optional, 2n) receives the per-vertex forces of the last iteration.
int orc_layout(int algo, int n, const int *rowptr, const int *colids,
               double *xy, int iterations, int batch, double theta, double W,
               double engt, double step_in, int nthreads, double *force_out,
               double *result_out) {
  if (n < 1 || batch < 1) return -1;
  P2 *pos = reinterpret_cast<P2 *>(xy);
  P2 *fo = reinterpret_cast<P2 *>(force_out);
  double energy = 0.0;
  long long loops = 0;
  if (algo == 2 && std::fabs(engt - 0.01) > 0) {
    double step = step_in < 0 ? 1.0 : step_in;
    double e0 = std::numeric_limits<double>::max();
    double e = 0.0;
    const long long max_loops = 1000000;
    while (std::fabs(e0 - e) / e0 > engt && loops < max_loops) {
      e0 = e;
      e = smu_iteration(MODEL_FR, n, rowptr, colids, pos, batch, W, step, fo,
                        nthreads);
      step = step * 0.999;
      loops++;
    }
    energy = e;
  } else if (algo == 2 || algo == 3 || algo == 8) {
    const double decay = (algo == 2) ? 0.999 : 0.99;  // :781 vs :934 (t=0.99)
    double step = step_in < 0 ? 1.0 : step_in;
    for (int it = 0; it < iterations; it++) {
      energy = smu_iteration(algo, n, rowptr, colids, pos, batch, W, step, fo,
                             nthreads);
      step = step * decay;
      loops++;
    }
  } else if (algo == 4) {
    double step = step_in < 0 ? 1.0 : step_in;
    for (int it = 0; it < iterations; it++) {
      energy = bh_iteration(n, rowptr, colids, pos, batch, theta, W, step, fo,
                            nthreads);
      step = step * 0.999;
      loops++;
    }
  } else if (algo == 6) {
    const int approx = (int)(iterations * 0.8);
    double step = 1.0;
    for (int it = 0; it < approx; it++) {
      energy = bh_iteration(n, rowptr, colids, pos, batch, 1.2, W, step, fo,
                            nthreads);
      step = step * 0.999;
    }
    const int rest = iterations - approx;
    step = std::pow(0.999, 4 * rest);
    energy = 0.0;
    for (int it = 0; it < rest; it++) {
      energy = smu_iteration(MODEL_FR, n, rowptr, colids, pos, batch, W, step,
                             fo, nthreads);
      step = step * 0.999;
    }
    loops = iterations;
  } else if (algo == 5) {
    const int approx = (int)(iterations * 0.8);  // :1086
    Walks w;
    greedy_walks(n, rowptr, colids, w);
    double step = 1.0;
    for (int it = 0; it < iterations; it++) {
      if (it > approx)
        energy = greedy_exact_iteration(n, rowptr, colids, pos, batch, W, step, fo, nthreads);
      else
        energy = greedy_walk_iteration(n, rowptr, colids, w, pos, batch, W, step, fo, nthreads);
      step = step * 0.99;
      loops++;
    }
  } else if (algo == 7) {
    double step = step_in < 0 ? 1.0 : step_in;
    for (int it = 0; it < iterations; it++) {
      energy = sd_iteration(n, rowptr, colids, pos, batch, W, step, fo, nthreads);
      step = step * 0.999;
      loops++;
    }
  } else {
    return -2;
  }
  result_out[0] = energy;
  result_out[1] = (double)loops;
  return 0;
}

// One SMU iteration with an explicit STEP, exposing the forces (test use).
double orc_smu_iteration(int model, int n, const int *rowptr, const int *colids,
                         double *xy, int batch, double W, double step,
                         double *force_out, int nthreads) {
  return smu_iteration(model, n, rowptr, colids, reinterpret_cast<P2 *>(xy),
                       batch, W, step, reinterpret_cast<P2 *>(force_out),
                       nthreads);
}

// One Barnes-Hut iteration with an explicit STEP, exposing the forces.
double orc_bh_iteration(int n, const int *rowptr, const int *colids, double *xy,
                        int batch, double theta, double W, double step,
                        double *force_out, int nthreads) {
  return bh_iteration(n, rowptr, colids, reinterpret_cast<P2 *>(xy), batch,
                      theta, W, step, reinterpret_cast<P2 *>(force_out),
                      nthreads);
}

// Forces of one iteration evaluated on another implementation's trajectory:
// batch b sees xy_end for the batches before it and xy_start for the rest
// (its batch-start state in that implementation).  algo 2/3/8 (minibatch
// models) or 4 (Barnes-Hut, tree and queries from xy_start).  Returns the
// energy; force_out receives 2n values.
double orc_forces_on_trajectory(int algo, int n, const int *rowptr, const int *colids,
                                const double *xy_start, const double *xy_end, int batch,
                                double theta, double W, double *force_out, int nthreads) {
  std::vector<P2> pos(reinterpret_cast<const P2 *>(xy_start),
                      reinterpret_cast<const P2 *>(xy_start) + n);
  const P2 *rep = reinterpret_cast<const P2 *>(xy_end);
  P2 *fo = reinterpret_cast<P2 *>(force_out);
  if (algo == 4)
    return bh_iteration(n, rowptr, colids, pos.data(), batch, theta, W, 1.0, fo, nthreads, rep);
  if (algo == 7) return sd_iteration(n, rowptr, colids, pos.data(), batch, W, 1.0, fo, nthreads, rep);
  if (algo == 5) {
    Walks w;
    greedy_walks(n, rowptr, colids, w);
    return greedy_walk_iteration(n, rowptr, colids, w, pos.data(), batch, W, 1.0, fo, nthreads, rep);
  }
  if (algo == 50)  // algo 5, second phase
    return greedy_exact_iteration(n, rowptr, colids, pos.data(), batch, W, 1.0, fo, nthreads, rep);
  return smu_iteration(algo, n, rowptr, colids, pos.data(), batch, W, 1.0, fo, nthreads, rep);
}

// Repulsion sources of algo 5's first phase for every vertex, in walk order
// (greedy_walk).  off_out: n + 1 offsets; src_out: up to cap sources (may be
// NULL).  Returns the total number of sources.
long long orc_greedy_walks(int n, const int *rowptr, const int *colids, long long *off_out, int *src_out,
                           long long cap) {
  Walks w;
  greedy_walks(n, rowptr, colids, w);
  std::memcpy(off_out, w.off.data(), (n + 1) * sizeof(long long));
  if (src_out) std::memcpy(src_out, w.src.data(), std::min<long long>(cap, (long long)w.src.size()) * sizeof(int));
  return (long long)w.src.size();
}

}  // extern "C"

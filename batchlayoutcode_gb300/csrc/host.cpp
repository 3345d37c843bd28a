// host.cpp -- MatrixMarket reader, initialisers and writer (host side).
#include "host.h"
#include "fmt_g6.h"

#include <stdlib.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <thread>

namespace blhost {

static_assert(sizeof(struct random_data) <= 64, "random_data storage");

RandStream::RandStream() {
  std::memset(state_, 0, sizeof(state_));
  std::memset(data_, 0, sizeof(data_));
  initstate_r(1u, state_, sizeof(state_), reinterpret_cast<struct random_data *>(data_));
}

int RandStream::next() {
  int32_t r = 0;
  random_r(reinterpret_cast<struct random_data *>(data_), &r);
  return (int)r;
}

void rand_init(int n, std::vector<double> &xy) {
  const double kMaxMin = 3.0;  // MAXMIN, sample/algorithms.h:43
  RandStream rs;
  xy.assign(2 * (size_t)n, 0.0);
  for (int i = 0; i < n; i++) {
    double x, y;
    do {
      x = -1.0 + 2.0 * rs.next() / (RAND_MAX + 1.0);
      y = -1.0 + 2.0 * rs.next() / (RAND_MAX + 1.0);
    } while (x * x + y * y > 1.0);
    xy[2 * i] = x * kMaxMin;
    xy[2 * i + 1] = y * kMaxMin;
  }
}

void init_dfs(int n, const std::vector<int> &rowptr, const std::vector<int> &colids,
              std::vector<double> &xy) {
  const double kMaxMin = 3.0, kPi = 3.14159265358979323846, radi = 0.1;
  const int nnz = rowptr[n];
  RandStream rs;
  // unvisited vertices (disconnected inputs) stay at the origin; the
  // reference leaves their memory uninitialised
  xy.assign(2 * (size_t)n, 0.0);
  std::vector<char> visited(n, 0);
  std::vector<int> stack;
  double minX = 1.0, minY = 1.0, maxX = 1.0, maxY = 1.0;
  stack.push_back(0);
  visited[0] = 1;
  xy[0] = 1.0;
  xy[1] = 1.0;
  auto place = [&](int parent, int lo, int hi) {
    const double deg = 360.0 / (hi - lo);
    double degree = 0;
    for (int k = lo; k < hi; k++) {
      const int c = colids[k];
      if (visited[c] == 0) {
        const float r = static_cast<float>(rs.next()) / static_cast<float>(RAND_MAX);
        const double cx = xy[2 * parent] + radi * std::cos(kPi * (degree) / 180.0);
        const double cy = xy[2 * parent + 1] + radi * std::sin(kPi * (degree) / 180.0);
        xy[2 * c] = cx + r;
        xy[2 * c + 1] = cy + r;
        visited[c] = 1;
        stack.push_back(c);
        degree += deg;
        if (minX > xy[2 * c]) minX = xy[2 * c];
        else if (maxX < xy[2 * c]) maxX = xy[2 * c];
        if (minY > xy[2 * c + 1]) minY = xy[2 * c + 1];
        else if (maxY < xy[2 * c + 1]) maxY = xy[2 * c + 1];
      }
    }
  };
  while (!stack.empty()) {
    const int parent = stack.back();
    stack.pop_back();
    if (parent < n - 1 && (rowptr[parent + 1] - rowptr[parent]) > 0) {
      place(parent, rowptr[parent], rowptr[parent + 1]);
    } else {
      // the reference's else branch walks to the end of colids (:65-89)
      if ((nnz - rowptr[parent]) <= 0) continue;
      place(parent, rowptr[parent], nnz);
    }
  }
  const double scalefactor = 2.0 * kMaxMin / std::max(maxX - minX, maxY - minY);
  for (int i = 0; i < n; i++) {
    xy[2 * i] = xy[2 * i] * scalefactor;
    xy[2 * i + 1] = xy[2 * i + 1] * scalefactor;
  }
}

bool file_init(const std::string &path, int n, std::vector<double> &xy, std::string &msg) {
  FILE *f = std::fopen(path.c_str(), "r");
  if (!f) {
    msg = "ERROR in input coordinates file!";
    return false;
  }
  char line[256];
  double x = 0.0, y = 0.0;
  int id = 0, index = 0;
  // like the reference, a line sscanf cannot parse repeats the previous x, y
  while (std::fgets(line, 256, f)) {
    std::sscanf(line, "%lf %lf %d", &x, &y, &id);
    if (index < n) {
      xy[2 * index] = x;
      xy[2 * index + 1] = y;
    }
    index++;
  }
  std::fclose(f);
  return true;
}

// Worker count for the host-side parallel parts: the machine's threads, at
// most 32, and one per `grain` units of work.
static int host_threads(size_t work, size_t grain) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t by_work = std::max<size_t>(1, work / std::max<size_t>(grain, 1));
  return (int)std::min<size_t>({(size_t)hw, (size_t)32, by_work});
}

template <typename F>
static void parallel_for(int threads, F &&body) {
  if (threads <= 1) {
    body(0);
    return;
  }
  std::vector<std::thread> pool;
  pool.reserve(threads - 1);
  for (int k = 1; k < threads; k++) pool.emplace_back(body, k);
  body(0);
  for (auto &t : pool) t.join();
}

bool write_coordinates(const std::string &input, const std::string &outputdir,
                       const std::string &tag, const std::vector<double> &xy,
                       std::string &path_out) {
  std::stringstream data(input);
  std::string lasttok;
  while (std::getline(data, lasttok, '/')) {
  }
  path_out = outputdir + lasttok + tag + ".txt";
  FILE *f = std::fopen(path_out.c_str(), "wb");
  if (!f) return false;
  // "x\ty\tid\n" with the default ostream formatting of doubles (6
  // significant digits, the %g conversion, by fmt_g6), formatted in parallel
  // slices and written in order
  const size_t n = xy.size() / 2;
  const int T = host_threads(n, 65536);
  std::vector<std::string> parts(T);
  parallel_for(T, [&](int k) {
    const size_t lo = n * k / T, hi = n * (k + 1) / T;
    std::string &out = parts[k];
    out.resize((hi - lo) * 72);  // a line is at most 2 x 32 + 2 + 21 bytes
    char *w = &out[0];
    for (size_t i = lo; i < hi; i++) {
      w += bl::fmt_g6(xy[2 * i], w);
      *w++ = '\t';
      w += bl::fmt_g6(xy[2 * i + 1], w);
      *w++ = '\t';
      w += bl::fmt_u64(i + 1, w);
      *w++ = '\n';
    }
    out.resize((size_t)(w - &out[0]));
  });
  bool ok = true;
  for (auto &part : parts)
    if (!part.empty() && std::fwrite(part.data(), 1, part.size(), f) != part.size()) ok = false;
  if (std::fclose(f) != 0) ok = false;
  return ok;
}

namespace {

// strtol-like base-10 integer at p (leading blanks skipped); returns false
// when there are no digits.  Saturates instead of overflowing (a saturated
// value is out of range for any matrix).
inline bool parse_long(const char *&p, const char *end, long long &v) {
  while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\v' || *p == '\f')) p++;
  const char *q = p;
  bool neg = false;
  if (q < end && (*q == '+' || *q == '-')) {
    neg = *q == '-';
    q++;
  }
  if (q >= end || *q < '0' || *q > '9') return false;
  long long x = 0;
  while (q < end && *q >= '0' && *q <= '9') {
    if (x < (1LL << 40)) x = x * 10 + (*q - '0');
    q++;
  }
  v = neg ? -x : x;
  p = q;
  return true;
}

struct ChunkResult {
  std::vector<std::pair<int, int>> entries;  // 0-based (row, col), file order
  long long bad_at = -1;                     // entry index (within the chunk) of the first bad line
  std::string bad_line;
};

}  // namespace

bool read_matrix_market(const std::string &path, MatrixInfo &info, std::vector<int> &rowptr,
                        std::vector<int> &colids, std::string &msg) {
  const auto t0 = std::chrono::steady_clock::now();
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) {
    msg = "cannot open " + path;
    return false;
  }
  std::vector<char> buf;
  {
    struct stat st;
    if (fstat(fileno(f), &st) == 0 && st.st_size > 0) buf.resize((size_t)st.st_size);
    size_t have = std::fread(buf.data(), 1, buf.size(), f);
    buf.resize(have);
    char block[1 << 16];  // anything beyond the size stat reported
    size_t got;
    while ((got = std::fread(block, 1, sizeof(block), f)) > 0) buf.insert(buf.end(), block, block + got);
  }
  std::fclose(f);
  const char *text = buf.data();
  const size_t size = buf.size();
  // header: comment lines (any of them containing "symmetric" marks the
  // matrix symmetric, IO.h:67-75), then the size line
  bool symmetric = false;
  int m = 0, ncol = 0;
  long long nnz = -1;
  size_t pos = 0;
  bool have_size = false;
  while (pos < size) {
    const char *nl = static_cast<const char *>(std::memchr(text + pos, '\n', size - pos));
    const size_t eol = nl ? (size_t)(nl - text) : size;
    std::string line(text + pos, eol - pos);
    pos = nl ? eol + 1 : size;
    if (!line.empty() && line[0] == '%') {
      if (line.find("symmetric") != std::string::npos) symmetric = true;
      continue;
    }
    if (std::sscanf(line.c_str(), "%d %d %lld", &m, &ncol, &nnz) != 3) {
      msg = "bad size line in " + path;
      return false;
    }
    have_size = true;
    break;
  }
  if (!have_size || nnz < 0 || m < 0 || ncol < 0) {
    msg = "missing size line in " + path;
    return false;
  }
  // entry lines, parsed in parallel slices cut at line ends
  const size_t body = pos, blen = size - pos;
  const int T = host_threads(blen, 1 << 20);
  std::vector<size_t> cut(T + 1, size);
  cut[0] = body;
  for (int k = 1; k < T; k++) {
    size_t c = body + blen * k / T;
    c = std::max(c, cut[k - 1]);
    const char *nl = c < size ? static_cast<const char *>(std::memchr(text + c, '\n', size - c)) : nullptr;
    cut[k] = nl ? (size_t)(nl - text) + 1 : size;
  }
  std::vector<ChunkResult> res(T);
  parallel_for(T, [&](int k) {
    ChunkResult &r = res[k];
    r.entries.reserve((cut[k + 1] - cut[k]) / 8 + 1);
    size_t p0 = cut[k];
    while (p0 < cut[k + 1]) {
      const char *nl = static_cast<const char *>(std::memchr(text + p0, '\n', cut[k + 1] - p0));
      const size_t eol = nl ? (size_t)(nl - text) : cut[k + 1];
      const size_t ls = p0;
      const char *p = text + p0, *e = text + eol;
      p0 = eol + 1;
      long long rr, cc;
      if (!parse_long(p, e, rr)) continue;  // blank (or comment) line
      if (!parse_long(p, e, cc) || rr < 1 || cc < 1 || rr > m || cc > ncol) {
        r.bad_at = (long long)r.entries.size();
        r.bad_line.assign(text + ls, eol - ls);
        return;
      }
      r.entries.emplace_back((int)rr - 1, (int)cc - 1);
    }
  });
  // only the first nnz entry lines count (the reference stops reading there)
  long long before = 0;
  std::vector<long long> keep(T, 0);
  for (int k = 0; k < T; k++) {
    const long long have = (long long)res[k].entries.size();
    if (res[k].bad_at >= 0 && before + res[k].bad_at < nnz) {
      msg = "bad entry line in " + path + ": " + res[k].bad_line;
      return false;
    }
    keep[k] = std::max(0LL, std::min(have, nnz - before));
    before += have;
    if (res[k].bad_at >= 0) break;  // lines after a bad one were not parsed
  }
  if (before < nnz) {
    msg = "file ends before nnz entries in " + path;
    return false;
  }
  // CSR: symmetric files mirrored with self loops dropped, general files as
  // they are; rows sorted ascending.  Built without atomics in three
  // parallel passes: every slice counts its (mirrored) entries per block of
  // rows, scatters them into a staging array grouped by block (slice order
  // inside a block), then every block of rows counts, fills and sorts its
  // own rows, whose colids form one contiguous range.
  const int NB = std::max(1, std::min(m, 8 * T));  // row blocks
  const long long bsize = ((long long)m + NB - 1) / NB;
  auto for_kept = [&](int k, auto &&emit) {
    for (long long q = 0; q < keep[k]; q++) {
      const auto &e = res[k].entries[q];
      if (symmetric) {
        if (e.first != e.second) {
          emit(e.first, e.second);
          emit(e.second, e.first);
        }
      } else {
        emit(e.first, e.second);
      }
    }
  };
  std::vector<long long> bcnt((size_t)T * NB, 0);  // [slice][block]
  parallel_for(T, [&](int k) {
    long long *c = &bcnt[(size_t)k * NB];
    for_kept(k, [&](int r, int) { c[r / bsize]++; });
  });
  std::vector<long long> boff((size_t)T * NB), bbase(NB + 1, 0);
  long long total = 0;
  for (int b = 0; b < NB; b++) {
    bbase[b] = total;
    for (int k = 0; k < T; k++) {
      boff[(size_t)k * NB + b] = total;
      total += bcnt[(size_t)k * NB + b];
    }
  }
  bbase[NB] = total;
  if (total > 2147483647LL) {
    msg = "more than 2^31-1 stored entries in " + path;
    return false;
  }
  std::vector<std::pair<int, int>> staged((size_t)total);
  parallel_for(T, [&](int k) {
    long long *o = &boff[(size_t)k * NB];
    for_kept(k, [&](int r, int c) { staged[(size_t)o[r / bsize]++] = std::make_pair(r, c); });
  });
  rowptr.assign((size_t)m + 1, 0);
  colids.assign((size_t)total, 0);
  const int TB = std::min(NB, T);
  parallel_for(TB, [&](int k) {
    for (int b = k; b < NB; b += TB) {
      const int r0 = (int)std::min<long long>(m, (long long)b * bsize);
      const int r1 = (int)std::min<long long>(m, (long long)(b + 1) * bsize);
      std::vector<int> rc(r1 - r0 + 1, 0);
      for (long long q = bbase[b]; q < bbase[b + 1]; q++) rc[staged[q].first - r0 + 1]++;
      for (int i = 0; i < r1 - r0; i++) rc[i + 1] += rc[i];
      for (int i = r0; i < r1; i++) rowptr[i + 1] = (int)(bbase[b] + rc[i - r0 + 1]);
      std::vector<int> cur(rc.begin(), rc.end() - 1);
      for (long long q = bbase[b]; q < bbase[b + 1]; q++)
        colids[(size_t)(bbase[b] + cur[staged[q].first - r0]++)] = staged[q].second;
      // rows of this block only (rowptr[r0] belongs to the block before)
      for (int i = r0; i < r1; i++)
        std::sort(colids.begin() + (bbase[b] + rc[i - r0]), colids.begin() + (bbase[b] + rc[i - r0 + 1]));
    }
  });
  info.rows = m;
  info.cols = ncol;
  info.nnz = (long long)rowptr[m];
  info.symmetric = symmetric;
  info.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return true;
}

// ---- binary CSR cache ---------------------------------------------------------

namespace {
constexpr char kCacheMagic[8] = {'B', 'L', 'C', 'S', 'R', '0', '0', '2'};

// The header is followed by the source's canonical absolute path (path_len
// bytes, zero-padded to a multiple of 8), then rowptr and colids.  A cache is
// used only for the file it was made from: same canonical path, device and
// inode, size and modification time.
struct CacheHeader {
  char magic[8];
  long long src_size;
  long long src_mtime_ns;
  int rows, cols;
  long long nnz;
  int symmetric, pad;
  long long src_dev, src_ino;
  int path_len, pad2;
};

struct SourceStamp {
  long long size = 0, mtime_ns = 0, dev = 0, ino = 0;
  std::string canon;  // realpath of the source
};

// rowptr non-decreasing from 0 to colids.size(), every colid in [0, cols):
// checked in parallel slices of rows.
bool csr_consistent(const std::vector<int> &rowptr, const std::vector<int> &colids, int cols) {
  const int rows = (int)rowptr.size() - 1;
  if (rows < 0 || rowptr[0] != 0 || (size_t)rowptr[rows] != colids.size()) return false;
  const int T = host_threads(colids.size() + (size_t)rows, 1 << 20);
  std::vector<char> good(T, 1);
  parallel_for(T, [&](int k) {
    const int lo = (int)((long long)rows * k / T), hi = (int)((long long)rows * (k + 1) / T);
    for (int i = lo; i < hi; i++)
      if (rowptr[i + 1] < rowptr[i]) {
        good[k] = 0;
        return;
      }
    for (int e = rowptr[lo]; e < rowptr[hi]; e++)
      if (colids[e] < 0 || colids[e] >= cols) {
        good[k] = 0;
        return;
      }
  });
  for (char g : good)
    if (!g) return false;
  return true;
}

bool source_stamp(const std::string &path, SourceStamp &s) {
  struct stat st;
  if (stat(path.c_str(), &st) != 0) return false;
  s.size = (long long)st.st_size;
  s.mtime_ns = (long long)st.st_mtim.tv_sec * 1000000000LL + (long long)st.st_mtim.tv_nsec;
  s.dev = (long long)st.st_dev;
  s.ino = (long long)st.st_ino;
  char *rp = realpath(path.c_str(), nullptr);
  if (!rp) return false;
  s.canon = rp;
  std::free(rp);
  return s.canon.size() < 65536;
}

long long padded_path_bytes(long long len) { return (len + 7) & ~7LL; }
}  // namespace

std::string csr_cache_path(const std::string &path, const std::string &cache_dir) {
  std::string base = path;
  const size_t slash = base.find_last_of('/');
  if (slash != std::string::npos) base = base.substr(slash + 1);
  std::string dir = cache_dir;
  if (!dir.empty() && dir.back() != '/') dir += '/';
  return dir + base + ".blcsr";
}

bool read_matrix_market_cached(const std::string &path, const std::string &cache_dir, MatrixInfo &info,
                               std::vector<int> &rowptr, std::vector<int> &colids, std::string &msg,
                               bool *from_cache) {
  const auto t0 = std::chrono::steady_clock::now();
  if (from_cache) *from_cache = false;
  SourceStamp src;
  const bool stamped = source_stamp(path, src);
  const std::string cpath = csr_cache_path(path, cache_dir);
  const long long plen = (long long)src.canon.size();
  if (stamped) {
    if (FILE *f = std::fopen(cpath.c_str(), "rb")) {
      CacheHeader h;
      struct stat cst;
      // the header's sizes must account for the file's length exactly before
      // anything is sized from them; the arrays are checked after the read,
      // and a cache that fails either check is parsed again and rewritten
      bool ok = std::fread(&h, sizeof(h), 1, f) == 1 && std::memcmp(h.magic, kCacheMagic, 8) == 0 &&
                h.src_size == src.size && h.src_mtime_ns == src.mtime_ns && h.src_dev == src.dev &&
                h.src_ino == src.ino && h.path_len == plen && h.rows >= 0 && h.cols >= 0 && h.nnz >= 0 &&
                h.nnz <= 2147483647LL && fstat(fileno(f), &cst) == 0 &&
                (long long)cst.st_size == (long long)sizeof(h) + padded_path_bytes(plen) +
                                              4LL * ((long long)h.rows + 1) + 4LL * h.nnz;
      if (ok) {
        std::string stored((size_t)padded_path_bytes(plen), '\0');
        ok = std::fread(&stored[0], 1, stored.size(), f) == stored.size() &&
             std::memcmp(stored.data(), src.canon.data(), (size_t)plen) == 0;
      }
      if (ok) {
        rowptr.assign((size_t)h.rows + 1, 0);
        colids.assign((size_t)h.nnz, 0);
        ok = std::fread(rowptr.data(), sizeof(int), rowptr.size(), f) == rowptr.size() &&
             (h.nnz == 0 || std::fread(colids.data(), sizeof(int), colids.size(), f) == colids.size()) &&
             csr_consistent(rowptr, colids, h.cols);
      }
      std::fclose(f);
      if (ok) {
        info.rows = h.rows;
        info.cols = h.cols;
        info.nnz = h.nnz;
        info.symmetric = h.symmetric != 0;
        info.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (from_cache) *from_cache = true;
        return true;
      }
    }
  }
  if (!read_matrix_market(path, info, rowptr, colids, msg)) return false;
  if (stamped) {
    // written to a temporary name and renamed, so a reader never sees half a file
    const std::string tmp = cpath + ".tmp" + std::to_string((long long)getpid());
    if (FILE *f = std::fopen(tmp.c_str(), "wb")) {
      CacheHeader h;
      std::memset(&h, 0, sizeof(h));
      std::memcpy(h.magic, kCacheMagic, 8);
      h.src_size = src.size;
      h.src_mtime_ns = src.mtime_ns;
      h.rows = info.rows;
      h.cols = info.cols;
      h.nnz = info.nnz;
      h.symmetric = info.symmetric ? 1 : 0;
      h.src_dev = src.dev;
      h.src_ino = src.ino;
      h.path_len = (int)plen;
      std::string stored((size_t)padded_path_bytes(plen), '\0');
      std::memcpy(&stored[0], src.canon.data(), (size_t)plen);
      bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 &&
                std::fwrite(stored.data(), 1, stored.size(), f) == stored.size() &&
                std::fwrite(rowptr.data(), sizeof(int), rowptr.size(), f) == rowptr.size() &&
                (colids.empty() || std::fwrite(colids.data(), sizeof(int), colids.size(), f) == colids.size());
      ok = (std::fclose(f) == 0) && ok;
      if (ok) ok = std::rename(tmp.c_str(), cpath.c_str()) == 0;
      if (!ok) std::remove(tmp.c_str());
    }
  }
  return true;
}

}  // namespace blhost

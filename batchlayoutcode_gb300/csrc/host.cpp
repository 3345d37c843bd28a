// host.cpp -- MatrixMarket reader, initialisers and writer (host side).
#include "host.h"

#include <stdlib.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>

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

bool write_coordinates(const std::string &input, const std::string &outputdir,
                       const std::string &tag, const std::vector<double> &xy,
                       std::string &path_out) {
  std::stringstream data(input);
  std::string lasttok;
  while (std::getline(data, lasttok, '/')) {
  }
  path_out = outputdir + lasttok + tag + ".txt";
  std::ofstream output(path_out);
  if (!output) return false;
  const size_t n = xy.size() / 2;
  for (size_t i = 0; i < n; i++) output << xy[2 * i] << "\t" << xy[2 * i + 1] << "\t" << i + 1 << "\n";
  return (bool)output;
}

bool read_matrix_market(const std::string &path, MatrixInfo &info, std::vector<int> &rowptr,
                        std::vector<int> &colids, std::string &msg) {
  const auto t0 = std::chrono::steady_clock::now();
  std::ifstream in(path);
  if (!in) {
    msg = "cannot open " + path;
    return false;
  }
  std::string line;
  bool symmetric = false;
  int m = 0, ncol = 0;
  long long nnz = -1;
  while (std::getline(in, line)) {
    if (!line.empty() && line[0] == '%') {
      // the reference tests every comment line for "symmetric" (IO.h:67-75)
      if (line.find("symmetric") != std::string::npos) symmetric = true;
      continue;
    }
    if (std::sscanf(line.c_str(), "%d %d %lld", &m, &ncol, &nnz) != 3) {
      msg = "bad size line in " + path;
      return false;
    }
    break;
  }
  if (nnz < 0 || m < 0 || ncol < 0) {
    msg = "missing size line in " + path;
    return false;
  }
  std::vector<std::pair<int, int>> rc;
  rc.reserve(symmetric ? 2 * nnz : nnz);
  long long read = 0;
  while (read < nnz && std::getline(in, line)) {
    const char *p = line.c_str();
    char *end = nullptr;
    const long r = std::strtol(p, &end, 10);
    if (end == p) continue;  // blank line
    p = end;
    const long c = std::strtol(p, &end, 10);
    if (end == p || r < 1 || c < 1 || r > m || c > ncol) {
      msg = "bad entry line in " + path + ": " + line;
      return false;
    }
    read++;
    const int ri = (int)r - 1, ci = (int)c - 1;
    if (symmetric) {
      if (ri != ci) {
        rc.emplace_back(ri, ci);
        rc.emplace_back(ci, ri);
      }
    } else {
      rc.emplace_back(ri, ci);
    }
  }
  if (read < nnz) {
    msg = "file ends before nnz entries in " + path;
    return false;
  }
  std::vector<int> cnt(m + 1, 0);
  for (auto &e : rc) cnt[e.first + 1]++;
  for (int i = 0; i < m; i++) cnt[i + 1] += cnt[i];
  rowptr = cnt;
  colids.assign(rc.size(), 0);
  std::vector<int> fill(cnt.begin(), cnt.end() - 1);
  for (auto &e : rc) colids[fill[e.first]++] = e.second;
  for (int i = 0; i < m; i++) std::sort(colids.begin() + rowptr[i], colids.begin() + rowptr[i + 1]);
  info.rows = m;
  info.cols = ncol;
  info.nnz = (long long)rc.size();
  info.symmetric = symmetric;
  info.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return true;
}

}  // namespace blhost

// host.h -- host-side parts of the layout path: MatrixMarket reader,
// initialisers and the coordinate writer (all CPU work in the reference too).
#pragma once

#include <string>
#include <vector>

namespace blhost {

// glibc-compatible rand() stream (additive feedback generator, 128-byte state)
// with its own state, seeded 1: the sequence the reference draws from rand()
// when nothing calls srand().  Implemented with random_r so the process-wide
// rand() state is untouched.
class RandStream {
 public:
  RandStream();
  int next();

 private:
  alignas(8) char state_[128];
  alignas(8) char data_[64];  // struct random_data
};

// randInit, sample/algorithms.cpp:16-28 (one-thread order).
void rand_init(int n, std::vector<double> &xy);
// initDFS, sample/algorithms.cpp:29-97.
void init_dfs(int n, const std::vector<int> &rowptr, const std::vector<int> &colids,
              std::vector<double> &xy);
// fileInitialization, sample/algorithms.cpp:98-119.  False when the file
// cannot be opened.
bool file_init(const std::string &path, int n, std::vector<double> &xy, std::string &msg);
// writeToFile, sample/algorithms.cpp:1244-1256; lines formatted in parallel
// slices and written in order.
bool write_coordinates(const std::string &input, const std::string &outputdir,
                       const std::string &tag, const std::vector<double> &xy,
                       std::string &path_out);

struct MatrixInfo {
  int rows = 0, cols = 0;
  long long nnz = 0;     // after mirroring and self-loop removal
  bool symmetric = false;
  double seconds = 0.0;  // parse time (the reference prints it)
};

// ReadASCII + CSC(triples) + CSR(csc) (IO.h:60-155, CSC.h:147-190,
// CSR.h:155-186): symmetric files are mirrored with self loops dropped,
// general files are taken as they are; colids ascend within each row and
// duplicates are kept.  Values are ignored (the layout never reads them).
// The file is read whole and its entry lines parsed in parallel slices (one
// thread per MB, at most 32); the CSR is filled and its rows sorted in
// parallel.
bool read_matrix_market(const std::string &path, MatrixInfo &info, std::vector<int> &rowptr,
                        std::vector<int> &colids, std::string &msg);

// The same CSR through a binary cache: <cache_dir>/<basename>.blcsr holds the
// CSR and the source file's canonical absolute path, device, inode, size and
// modification time; a cache made from this very file, unchanged, is read
// instead of the text (no parsing), otherwise the text is
// parsed and the cache (re)written (write failures are ignored).
// *from_cache (may be null) tells which happened.
bool read_matrix_market_cached(const std::string &path, const std::string &cache_dir, MatrixInfo &info,
                               std::vector<int> &rowptr, std::vector<int> &colids, std::string &msg,
                               bool *from_cache);
std::string csr_cache_path(const std::string &path, const std::string &cache_dir);

}  // namespace blhost

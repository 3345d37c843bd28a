// ref_driver.cpp -- drives the reference BatchLayout code (compiled from its
// own sources by oracle/build_ref.sh) and prints its results at full
// precision, so that golden vectors can pin the oracle restatement.
//
// TEST INFRASTRUCTURE ONLY: built into oracle/_ref/, used by
// tests/golden/make_golden.py in a container that has the reference sources.
// It calls only public reference interfaces:
//   SetInputMatricesAsCSR     sample/commonutility.h:45
//   class algorithms          sample/algorithms.h:50-85
//   BarnesHut / calcRepForce  sample/BarnesHut.h:114-228
//
// usage:
//   ref_driver csr    <mtx>                                  -> rowptr/colids
//   ref_driver layout <mtx> <initf> <algo> <iter> <batch> <bht> <weight> <engt> <outdir>
//   ref_driver bh     <mtx> <initf> <theta>                  -> sorted points, tree, repulsion
//   ref_driver init   <mtx> <init 0|1>                       -> initial coordinates
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "sample/algorithms.h"

static void dump_coords(const char *tag, Coordinate<double> *c, int n) {
  printf("%s %d\n", tag, n);
  for (int i = 0; i < n; i++) printf("%.17g %.17g\n", c[i].getX(), c[i].getY());
}

static std::vector<Coordinate<double>> read_initf(const char *path) {
  std::vector<Coordinate<double>> v;
  FILE *f = fopen(path, "r");
  if (!f) {
    fprintf(stderr, "cannot open %s\n", path);
    exit(2);
  }
  char line[256];
  while (fgets(line, 256, f)) {
    double x, y;
    int id;
    if (sscanf(line, "%lf %lf %d", &x, &y, &id) >= 2) v.push_back(Coordinate<double>(x, y));
  }
  fclose(f);
  return v;
}

int main(int argc, char **argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: see source\n");
    return 2;
  }
  std::string mode = argv[1];
  // The reference reader prints progress lines to stdout; keep them out of
  // the golden stream.
  std::streambuf *saved = std::cout.rdbuf();
  std::ostringstream sink;
  std::cout.rdbuf(sink.rdbuf());
  CSR<int, double> A;
  SetInputMatricesAsCSR(A, std::string(argv[2]));
  std::cout.rdbuf(saved);
  fflush(stdout);

  if (mode == "csr") {
    printf("rows %d nnz %d\n", A.rows, A.nnz);
    for (int i = 0; i <= A.rows; i++) printf("%d\n", A.rowptr[i]);
    for (int k = 0; k < A.nnz; k++) printf("%d\n", A.colids[k]);
    return 0;
  }
  if (mode == "layout") {
    const char *initf = argv[3];
    int algo = atoi(argv[4]), iter = atoi(argv[5]), batch = atoi(argv[6]);
    double bht = atof(argv[7]), weight = atof(argv[8]), engt = atof(argv[9]);
    std::string outdir = argv[10];
    algorithms al(A, std::string(argv[2]), outdir, 2, weight, engt, std::string(initf));
    std::vector<double> r;
    std::cout.rdbuf(sink.rdbuf());
    if (algo == 2 && engt != 0.01)
      r = al.cacheBlockingminiBatchForceDirectedAlgorithmConverged(iter, 1, batch, 0);
    else if (algo == 2)
      r = al.cacheBlockingminiBatchForceDirectedAlgorithm(iter, 1, batch, 0);
    else if (algo == 3)
      r = al.LinLogcacheBlockingminiBatchForceDirectedAlgorithm(iter, 1, batch);
    else if (algo == 8)
      r = al.FAcacheBlockingminiBatchForceDirectedAlgorithm(iter, 1, batch);
    else if (algo == 4)
      r = al.BarnesHutApproximation(iter, 1, batch, bht, 0);
    else if (algo == 6)
      r = al.approxCacheBlockBH(iter, 1, batch);
    else if (algo == 5)
      r = al.approxForceDirectedAlgorithm(iter, 1, batch);
    else if (algo == 7)
      r = al.cacheBlockingminiBatchForceDirectedAlgorithmSD(iter, 1, batch, 0);
    std::cout.rdbuf(saved);
    std::string log = sink.str();
    // the converged variant reports its loop count in the output file tag
    printf("energy %.17g\n", r.size() ? r[0] : 0.0);
    size_t p = log.rfind("PARAOUT");
    if (p != std::string::npos) printf("tag %s", log.substr(p).c_str());
    else printf("tag none\n");
    dump_coords("coords", al.nCoordinates, A.rows);
    dump_coords("forces", al.prevCoordinates, A.rows);
    return 0;
  }
  if (mode == "bh") {
    std::vector<Coordinate<double>> pts = read_initf(argv[3]);
    double theta = atof(argv[4]);
    int n = (int)pts.size();
    std::vector<Coordinate<double>> work(pts);
    BarnesHut bh(work.data(), n, theta);
    dump_coords("sorted", work.data(), n);
    std::vector<Coordinate<double>> rep(n);
    for (int i = 0; i < n; i++) rep[i] = bh.calcRepForce(pts[i]);
    dump_coords("repulsion", rep.data(), n);
    // the public tree printer, at full precision
    std::ostringstream tree;
    std::cout.rdbuf(tree.rdbuf());
    std::cout.precision(17);
    bh.print_t(0);
    std::cout.rdbuf(saved);
    printf("tree\n%s", tree.str().c_str());
    return 0;
  }
  if (mode == "init") {
    int init = atoi(argv[3]);
    algorithms al(A, std::string(argv[2]), std::string("/tmp/"), init, 1.0, 0.01, std::string(""));
    if (init == 0) al.initDFS();
    else {
      omp_set_num_threads(1);
      al.randInit();
    }
    dump_coords("coords", al.nCoordinates, A.rows);
    return 0;
  }
  fprintf(stderr, "unknown mode\n");
  return 2;
}

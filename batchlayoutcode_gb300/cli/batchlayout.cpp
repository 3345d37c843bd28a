// batchlayout.cpp -- command-line tool with the reference BatchLayout CLI surface
// (Test/BatchLayout.cpp:26-188): same flags, defaults, clamps, stdout lines,
// output file names and Results.txt row; the layout runs on the GPU through
// the C ABI.  -threads is accepted and reported but the GPU ignores it.
//
// Algorithms on the GPU path: 2 (and 2 with -engt), 3, 4, 5, 6, 7, 8.
// Algorithms 0 and 1 of the reference (sequential and naive) are not on it;
// they exit with an error message instead of running elsewhere.  As in the
// reference, -algo outside 0..8 (its 9 and 100 included) becomes 2.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <thread>
#include <vector>

#include "batchlayout_gb300.h"

static void helpmessage() {
  printf("\n");
  printf("Usage of BatchLayout tool:\n");
  printf("-input <string>, full path of input file (required).\n");
  printf("-output <string>, directory where output file will be stored.\n");
  printf("-batch <int>, size of minibatch.\n");
  printf("-init <int>, any of 0 or 1, 1 - random initialization, 0 - greedy initialization.\n");
  printf("-initf <string>, this will overwrite -init and initialize coordinates from a given file.\n");
  printf("-learned <string>, learned initialization with the model file given (overwrites -init and -initf).\n");
  printf("-iter <int>, number of iteration.\n");
  printf("-threads <int>, number of threads, default value is maximum available threads in the machine.\n");
  printf("-algo <int>, an integer among 0, 1, 2, 3, 4, 5 and 6.\n");
  printf("        0 - for sequential layout generation.\n");
  printf("        1 - for naive parallel approach for layout generation.\n");
  printf("        2 - for parallel layout generation using cache blocking stochastic minibatch update.\n");
  printf("        3 - for parallel layout generation using linlog mode, (0,-1)-energy model.\n");
  printf("        4 - for parallel layout generation using barnes-hut repulsive force approximation.\n");
  printf("        5 - for parallel layout generation using greedy force approximation approach.\n");
  printf("        6 - for parallel layout generation, 80%% time in -algo 4 and last 20%% time in -algo 2.\n");
  printf("        7 - for parallel layout generation, this will calculate forces using linear algebric format.\n");
  printf("        8 - for parallel layout generation, (1,-1)-energy model.\n");
  printf("-bht <float>, barnes-hut threshold parameter.\n");
  printf("-engt <float>, convergenece criteria. It should be a floating point number between 0 to 1 exclusive.\n");
  printf("It indicates if energy value is improved less than this percenrages then optimization will stop and return layout. If this value is set, then number of iteration will be overwritten.\n");
  printf("-weight <float>, a real number to include edge weight.\n");
  printf("-bfsinit, breadth-first greedy initialization on the GPU (overwritten by -initf and -learned).\n");
  printf("-csrcache <string>, directory of a binary CSR cache of the input (read when it matches the input file, else written).\n");
  printf("-h, show help message.\n");
  printf("default: -weight 1.0 -bht 1.2 -engt 0.01 -batch 256 -iter 600 -threads MAX -algo 2 -init 0\n\n");
}

static void banner() {
  printf("\n");
  printf("@@@@@                   @      @                                     \n");
  printf("@    @                  @      @                                     \n");
  printf("@  @   @@@@@@ @  @@@@@@ @      @      @@@@@@ @    @ @@@@@@ @    @ @  \n");
  printf("@@@         @ @@ @    @ @@@@@@ @           @ @    @ @    @ @    @ @@ \n");
  printf("@  @   @@@@@@ @  @      @    @ @      @@@@@@ @@@@@@ @    @ @    @ @  \n");
  printf("@    @ @    @ @  @      @    @ @      @    @      @ @    @ @    @ @  \n");
  printf("@@@@@  @@@@@@ @@ @@@@@@ @    @ @@@@@@ @@@@@@ @@@@@@ @@@@@@ @@@@@@ @@ \n\n");
}

static int max_threads() {
  if (const char *s = getenv("OMP_NUM_THREADS")) {
    int v = atoi(s);
    if (v > 0) return v;
  }
  unsigned h = std::thread::hardware_concurrency();
  return h ? (int)h : 1;
}

static void die(bl_ctx *ctx, const char *what) {
  fprintf(stderr, "%s failed: %s\n", what, ctx ? bl_last_error(ctx) : bl_create_error());
  exit(2);
}

static void write_out(bl_ctx *ctx, const std::string &tag) {
  char path[4096];
  if (bl_write_to_file(ctx, tag.c_str(), path, sizeof(path)) != BL_OK) die(ctx, "writeToFile");
  std::cout << "Creating output file in following directory:" << path << std::endl;
}

int main(int argc, char *argv[]) {
  double energyThreshold = 0.01, bhThreshold = 1.2, weight = 1.0;
  int init = 0, batchsize = 256, iterations = 600, numberOfThreads = max_threads(), algoOption = 2;
  std::string inputfile, initfile, outputfile, algoname = "CACHE", initname = "GREEDY", csrcache;
  auto arg = [&](int p) -> const char * { return p + 1 < argc ? argv[p + 1] : ""; };
  for (int p = 0; p < argc; p++) {
    if (strcmp(argv[p], "-input") == 0) inputfile = arg(p);
    if (strcmp(argv[p], "-output") == 0) outputfile = arg(p);
    if (strcmp(argv[p], "-batch") == 0) batchsize = atoi(arg(p));
    if (strcmp(argv[p], "-init") == 0 && init != 2 && init != 3) {
      init = atoi(arg(p));
      if (init < 0 || init > 1) init = 1;
    }
    if (strcmp(argv[p], "-iter") == 0) iterations = atoi(arg(p));
    if (strcmp(argv[p], "-threads") == 0) numberOfThreads = atoi(arg(p));
    if (strcmp(argv[p], "-algo") == 0) algoOption = atoi(arg(p));
    if (strcmp(argv[p], "-bht") == 0) bhThreshold = atof(arg(p));
    if (strcmp(argv[p], "-initf") == 0 && init != 3) {
      initfile = arg(p);
      init = 2;
    }
    if (strcmp(argv[p], "-learned") == 0) {
      initfile = arg(p);
      init = 3;
    }
    if (strcmp(argv[p], "-engt") == 0) {
      energyThreshold = atof(arg(p));
      if (energyThreshold < 0.0 || energyThreshold > 1.0) energyThreshold = 0.01;
    }
    if (strcmp(argv[p], "-weight") == 0) weight = atof(arg(p));
    if (strcmp(argv[p], "-csrcache") == 0) csrcache = arg(p);
    if (strcmp(argv[p], "-bfsinit") == 0 && init != 2 && init != 3) init = 4;
    if (strcmp(argv[p], "-h") == 0) {
      helpmessage();
      exit(1);
    }
  }
  if (inputfile.size() < 1 || argc < 2) {
    helpmessage();
    exit(1);
  }
  if (init == 1) initname = "RANDOM";
  if (init == 2) initname = "FILE";
  if (init == 3) initname = "LEARNED";
  if (init == 4) initname = "BFS";
  banner();
  // SetInputMatricesAsCSR prints these lines (sample/commonutility.h:31-32, IO.h:72-150)
  std::cout << "Reading input matrices in text (ascii)... " << std::endl;
  std::cout << "Input File Directory:" << inputfile << std::endl;
  long long info[5];
  double secs = 0.0;
  int *rowptr = nullptr, *colids = nullptr;
  char err[512];
  if (bl_read_matrix_market_cached(inputfile.c_str(), csrcache.empty() ? nullptr : csrcache.c_str(), info, &secs,
                                   &rowptr, &colids, err, sizeof(err)) != BL_OK) {
    fprintf(stderr, "%s\n", err);
    exit(1);
  }
  if (info[3]) std::cout << "Matrix is symmetric" << std::endl;
  printf("Converting matrix data from ASCII to COO format: %.16g seconds\n", secs);
  printf("Input Matrix: Rows = %d, Columns= %d, nnz = %d\n", (int)info[0], (int)info[1], (int)info[2]);
  fflush(stdout);
  std::cout << "Converting to csc ... " << std::endl << std::endl;
  if (algoOption < 0 || algoOption > 8) algoOption = 2;
  if (max_threads() < numberOfThreads) {
    numberOfThreads = max_threads();
    if (info[0] < 1000000 && numberOfThreads > 32) numberOfThreads = 32;
  }
  if (algoOption == 0 || algoOption == 1) {
    fprintf(stderr, "-algo %d is not on the GPU layout path (available: 2, 3, 4, 5, 6, 7, 8)\n", algoOption);
    exit(3);
  }
  const int n = (int)info[0];
  bl_ctx *ctx = bl_algorithms_create(0, n, info[2], rowptr, colids, inputfile.c_str(), outputfile.c_str(), init,
                                     weight, energyThreshold, initfile.c_str());
  bl_free(rowptr);
  bl_free(colids);
  if (!ctx) die(nullptr, "bl_algorithms_create");
  double out[3] = {0, 0, 0};
  const std::string B = std::to_string(batchsize);
  if (algoOption == 2) {
    algoname = "CACHE";
    if (std::fabs(energyThreshold - 0.01) > 0) {
      if (bl_cache_blocking_minibatch_converged(ctx, iterations, numberOfThreads, batchsize, 0, out) != BL_OK)
        die(ctx, "cacheBlockingminiBatchForceDirectedAlgorithmConverged");
      std::cout << "Cache Blocking (converged) Minibatch Size:" << batchsize << std::endl;
      std::cout << "Cache Blocking (converged)  Minbatch Energy:" << out[0] << std::endl;
      std::cout << "Cache Blocking (converged) Minibatch Parallel Wall time required:" << out[1] << std::endl;
      write_out(ctx, "CACHEMINB" + B + "PARAOUT" + std::to_string((long long)out[2]));
    } else {
      if (bl_cache_blocking_minibatch(ctx, iterations, numberOfThreads, batchsize, 0, out) != BL_OK)
        die(ctx, "cacheBlockingminiBatchForceDirectedAlgorithm");
      std::cout << "Cache Blocking Minibatch Size:" << batchsize << std::endl;
      std::cout << "Cache Blocking Minbatch Energy:" << out[0] << std::endl;
      std::cout << "Cache Blocking Minibatch Parallel Wall time required:" << out[1] << std::endl;
      write_out(ctx, "CACHEMINB" + B + "PARAOUT" + std::to_string(iterations));
    }
  } else if (algoOption == 3) {
    algoname = "LINLOG";
    if (bl_linlog_cache_blocking_minibatch(ctx, iterations, numberOfThreads, batchsize, out) != BL_OK)
      die(ctx, "LinLogcacheBlockingminiBatchForceDirectedAlgorithm");
    std::cout << "LinLog Batch Size:" << batchsize << std::endl;
    std::cout << "LinLog Minbatch Energy:" << out[0] << std::endl;
    std::cout << "LinLog Minibatch Parallel Wall time required:" << out[1] << std::endl;
    write_out(ctx, "LLCACHEMINB" + B + "PARAOUT" + std::to_string(iterations));
  } else if (algoOption == 4) {
    algoname = "BHCACHE";
    if (bl_barnes_hut_approximation(ctx, iterations, numberOfThreads, batchsize, bhThreshold, 0, out) != BL_OK)
      die(ctx, "BarnesHutApproximation");
    std::cout << "Barnes-Hut Minibatch Size:" << batchsize << std::endl;
    std::cout << "Barnes-Hut Minbatch Energy:" << out[0] << std::endl;
    std::cout << "Barnes-Hut Minibatch Parallel Wall time required:" << out[1] << std::endl;
    write_out(ctx, "BHMINB" + B + "PARAOUT" + std::to_string(iterations));
  } else if (algoOption == 5) {
    algoname = "GREEDY";
    if (bl_approx_force_directed(ctx, iterations, numberOfThreads, batchsize, out) != BL_OK)
      die(ctx, "approxForceDirectedAlgorithm");
    std::cout << "Greedy Approximation" << std::endl;
    std::cout << "Greedy Approximation Energy:" << out[0] << std::endl;
    std::cout << "Greedy Approximation Wall time required:" << out[1] << std::endl;
    write_out(ctx, "GAPPROX" + B + "PARAOUT" + std::to_string(iterations));
  } else if (algoOption == 7) {
    algoname = "CACHESD";
    if (bl_cache_blocking_minibatch_sd(ctx, iterations, numberOfThreads, batchsize, 0, out) != BL_OK)
      die(ctx, "cacheBlockingminiBatchForceDirectedAlgorithmSD");
    std::cout << "Cache BlockingSD Minibatch Size:" << batchsize << std::endl;
    std::cout << "Cache BlockingSD Minbatch Energy:" << out[0] << std::endl;
    std::cout << "Cache BlockingSD Minibatch Parallel Wall time required:" << out[1] << std::endl;
    write_out(ctx, "CACHESDMINB" + B + "PARAOUT" + std::to_string(iterations));
  } else if (algoOption == 6) {
    algoname = "BCGRDY";
    if (bl_approx_cache_block_bh(ctx, iterations, numberOfThreads, batchsize, out) != BL_OK)
      die(ctx, "approxCacheBlockBH");
    std::cout << "80%% - 20%% BH - CB" << std::endl;  // the doubled % as printed by algorithms.cpp:1209
    std::cout << "BH-CACHE Approximation Energy:" << out[0] << std::endl;
    std::cout << "BH-CACHE Approximation Wall time required:" << out[1] << std::endl;
    write_out(ctx, "BCAPPROX" + B + "PARAOUT" + std::to_string(iterations));
  } else if (algoOption == 8) {
    algoname = "FA";
    if (bl_fa_cache_blocking_minibatch(ctx, iterations, numberOfThreads, batchsize, out) != BL_OK)
      die(ctx, "FAcacheBlockingminiBatchForceDirectedAlgorithm");
    std::cout << "FA Batch Size:" << batchsize << std::endl;
    std::cout << "FA Minbatch Energy:" << out[0] << std::endl;
    std::cout << "FA Minibatch Parallel Wall time required:" << out[1] << std::endl;
    write_out(ctx, "FACACHEMINB" + B + "PARAOUT" + std::to_string(iterations));
  }
  bl_destroy(ctx);
  std::ofstream output("Results.txt", std::ofstream::app);
  output << algoname << "\t" << initname << "\t";
  output << iterations << "\t" << numberOfThreads << "\t" << batchsize << "\t";
  output << out[0] << "\t" << out[1];
  output << std::endl;
  return 0;
}

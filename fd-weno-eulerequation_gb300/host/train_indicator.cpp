// Trains the learned troubled-cell indicator through the C ABI alone (no
// Python, no PyTorch): solver runs at training seeds produce the data
// (wenofd_indicator_sample: a balanced sample of cells, formed on the GPU),
// wenofd_mlp_init gives the initial parameters and wenofd_mlp_train runs the
// FP32 forward / backward / Adam kernels.  The parameters are written as
// WENOFD_MLP_PARAMS float32 values, ready for wenofd_set_indicator.  The
// steps and defaults are those of the Python workflow
// (python/wenofd/learned.py: generate_dataset + train), which gives the same
// parameters bit for bit.
//
//   wenofd_train <out.bin> [--n N] [--snapshots a,b,..] [--per-snapshot K]
//                [--epochs E] [--batch B] [--lr L] [--seed S] [--init-seed I]
//                [--sample-seed T] [--label-deviation D] [--device G]
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "wenofd.h"

namespace {

struct Options {
  std::string out;
  int n = 512;
  std::vector<long long> snapshots = {40, 120, 240, 400};
  long long per_snapshot = 125000;
  int epochs = 30, batch = 4096;
  float lr = 3e-3f;
  unsigned long long seed = 1, init_seed = 0, sample_seed = 0;
  double label_deviation = 1e-2;
  int device = 0;
};

// (testcase, seed) of the training runs: two shear layers, two seeded
// four-quadrant Riemann problems.
const int kRuns[4][2] = {{5, 11}, {5, 12}, {4, 13}, {4, 14}};

void die(const std::string &what) {
  std::fprintf(stderr, "wenofd_train: %s: %s\n", what.c_str(), wenofd_last_error());
  std::exit(1);
}
void check(int rc, const char *what) {
  if (rc != WENOFD_OK) die(what);
}
void check_cuda(cudaError_t e, const char *what) {
  if (e != cudaSuccess) {
    std::fprintf(stderr, "wenofd_train: %s: %s\n", what, cudaGetErrorString(e));
    std::exit(1);
  }
}

Options parse(int argc, char **argv) {
  Options o;
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s <out.bin> [options]\n", argv[0]);
    std::exit(2);
  }
  o.out = argv[1];
  for (int a = 2; a < argc; ++a) {
    const std::string k = argv[a];
    if (a + 1 >= argc) {
      std::fprintf(stderr, "missing value for %s\n", k.c_str());
      std::exit(2);
    }
    const char *v = argv[++a];
    if (k == "--n") o.n = std::atoi(v);
    else if (k == "--per-snapshot") o.per_snapshot = std::atoll(v);
    else if (k == "--epochs") o.epochs = std::atoi(v);
    else if (k == "--batch") o.batch = std::atoi(v);
    else if (k == "--lr") o.lr = float(std::atof(v));
    else if (k == "--seed") o.seed = std::strtoull(v, nullptr, 10);
    else if (k == "--init-seed") o.init_seed = std::strtoull(v, nullptr, 10);
    else if (k == "--sample-seed") o.sample_seed = std::strtoull(v, nullptr, 10);
    else if (k == "--label-deviation") o.label_deviation = std::atof(v);
    else if (k == "--device") o.device = std::atoi(v);
    else if (k == "--snapshots") {
      o.snapshots.clear();
      for (const char *p = v; *p;) {
        o.snapshots.push_back(std::atoll(p));
        p = std::strchr(p, ',');
        if (!p) break;
        ++p;
      }
    } else {
      std::fprintf(stderr, "unknown option %s\n", k.c_str());
      std::exit(2);
    }
  }
  return o;
}

// Seed of the sampler for one snapshot of one run (learned.py sample_seed_of).
unsigned long long sample_seed_of(unsigned long long base, int run, int snapshot) {
  return base * 1000003ull + (unsigned long long)run * 1009ull + (unsigned long long)snapshot;
}

}  // namespace

int main(int argc, char **argv) {
  const Options o = parse(argc, argv);
  check_cuda(cudaSetDevice(o.device), "cudaSetDevice");
  const long long per_cap = (long long)(o.per_snapshot * 1.05 + 1024);  // the sampler's count varies
  const long long cap = 4 * (long long)o.snapshots.size() * per_cap;
  float *X = nullptr, *y = nullptr, *params = nullptr;
  check_cuda(cudaMalloc(&X, size_t(cap) * WENOFD_MLP_INPUTS * sizeof(float)), "cudaMalloc X");
  check_cuda(cudaMalloc(&y, size_t(cap) * sizeof(float)), "cudaMalloc y");
  check_cuda(cudaMalloc(&params, WENOFD_MLP_PARAMS * sizeof(float)), "cudaMalloc params");

  long long rows = 0;
  const std::string n = std::to_string(o.n), dev = std::to_string(o.device), dv = std::to_string(o.label_deviation);
  for (int r = 0; r < 4; ++r) {
    const std::string tc = std::to_string(kRuns[r][0]), seed = std::to_string(kRuns[r][1]);
    const char *keys[] = {"TESTCASE", "ELEMNUMX", "ELEMNUMY", "RKMETH", "CFL", "SCHEME", "SEED", "PRECISION",
                          "DEVICE", "TEND", "LABEL_DEVIATION"};
    const char *vals[] = {tc.c_str(), n.c_str(), n.c_str(), "2", "0.7", "1", seed.c_str(), "1", dev.c_str(),
                          "1.0e9", dv.c_str()};
    wenofd_solver *s = nullptr;
    check(wenofd_create(keys, vals, 11, &s), "wenofd_create");
    check(wenofd_initialize(s), "wenofd_initialize");
    long long done = 0;
    for (size_t k = 0; k < o.snapshots.size(); ++k) {
      check(wenofd_advance(s, o.snapshots[k] - done, nullptr), "wenofd_advance");
      done = o.snapshots[k];
      long long got = 0;
      check(wenofd_indicator_sample(s, o.per_snapshot, sample_seed_of(o.sample_seed, r, int(k)),
                                    X + rows * WENOFD_MLP_INPUTS, y + rows, cap - rows, &got),
            "wenofd_indicator_sample");
      rows += got;
    }
    wenofd_destroy(s);
  }

  std::vector<float> host(WENOFD_MLP_PARAMS), losses(o.epochs);
  check(wenofd_mlp_init(host.data(), o.init_seed), "wenofd_mlp_init");
  check_cuda(cudaMemcpy(params, host.data(), host.size() * sizeof(float), cudaMemcpyHostToDevice), "upload");
  check(wenofd_mlp_train(params, X, y, rows, o.epochs, o.batch, o.lr, o.seed, losses.data(), nullptr),
        "wenofd_mlp_train");
  check_cuda(cudaMemcpy(host.data(), params, host.size() * sizeof(float), cudaMemcpyDeviceToHost), "download");
  FILE *f = std::fopen(o.out.c_str(), "wb");
  if (!f || std::fwrite(host.data(), sizeof(float), host.size(), f) != host.size() || std::fclose(f) != 0) {
    std::fprintf(stderr, "wenofd_train: cannot write %s\n", o.out.c_str());
    return 1;
  }
  std::printf("%lld samples, %d epochs: loss %.4f -> %.4f; parameters in %s\n", rows, o.epochs, losses.front(),
              losses.back(), o.out.c_str());
  cudaFree(X);
  cudaFree(y);
  cudaFree(params);
  return 0;
}

// ref_probes.cpp — dumps the PGURE probe stream produced by the reference's
// own vendored PCG engine (src/pcg/pcg_random.hpp) and libstdc++'s
// std::bernoulli_distribution, the same calls as pgure.hpp:52-59,167-186.
// Test infrastructure: built by oracle/build.py only where the reference tree
// is mounted, to generate tests/golden/probes_*.bin.  Usage:
//   ref_probes <seed> <n> <out.bin>   writes n int8 delta1 then n f64 delta2
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "pcg_random.hpp"

int main(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: %s seed n out\n", argv[0]);
    return 2;
  }
  const int64_t seed = std::strtoll(argv[1], nullptr, 10);
  const size_t n = std::strtoull(argv[2], nullptr, 10);
  pcg64 rng;
  rng.seed(seed);
  const double kappa = 1.;
  const double vP = 0.5 + 0.5 * kappa / std::sqrt(kappa * kappa + 4);
  const double vQ = 1 - vP;
  const double vQvP = std::sqrt(vQ / vP);
  const double vPvQ = std::sqrt(vP / vQ);
  std::bernoulli_distribution b1(0.5), b2(vP);
  std::vector<int8_t> d1(n);
  std::vector<double> d2(n);
  for (size_t i = 0; i < n; ++i) d1[i] = b1(rng) ? -1 : 1;
  for (size_t i = 0; i < n; ++i) d2[i] = b2(rng) ? -1 * vQvP : vPvQ;
  FILE* f = std::fopen(argv[3], "wb");
  if (!f) return 1;
  std::fwrite(d1.data(), 1, n, f);
  std::fwrite(d2.data(), sizeof(double), n, f);
  std::fclose(f);
  return 0;
}

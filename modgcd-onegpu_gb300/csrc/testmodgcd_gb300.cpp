// testmodgcd_gb300.cpp -- correctness/timing driver of the drop-in API, after the
// reference's testmodgcd (testmodgcd.cpp): every GPU result is compared with mpz_gcd.
//
//   testmodgcd_gb300 file <path> [--batch]
//       pairs from a file in the reference's test-vector format: base-62 mpz_out_str
//       lines, u then v (testmodgcd.cpp:190-259)
//   testmodgcd_gb300 rand <num_bits> <gcd_bits> <reps> [seed] [--batch]
//       u = g*a, v = g*b from gmp_randinit_mt (seeded), like testmodgcd.cpp:219-229
//
// Prints one JSON line: pairs, mismatches, errors, mean GPU and GMP milliseconds.
#include <gmp.h>
#include <time.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "GmpCuda.h"

static double now_ms()
{
  timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return t.tv_sec * 1e3 + t.tv_nsec * 1e-6;
}

int main(int argc, char** argv)
{
  if (argc < 3) {
    std::printf("usage: %s file <path> [--batch] | rand <bits> <gcd_bits> <reps> [seed] [--batch]\n", argv[0]);
    return 1;
  }
  bool batch = false;
  std::vector<char*> args;
  for (int i = 1; i < argc; ++i) {
    if (!std::strcmp(argv[i], "--batch")) batch = true; else args.push_back(argv[i]);
  }
  std::vector<__mpz_struct> U, V;
  auto push = [&](mpz_srcptr u, mpz_srcptr v) {
    U.emplace_back(); V.emplace_back();
    mpz_init(&U.back()); mpz_init(&V.back());
    mpz_set(&U.back(), u); mpz_set(&V.back(), v);
  };
  mpz_t u, v, g;
  mpz_init(u); mpz_init(v); mpz_init(g);
  if (!std::strcmp(args[0], "file")) {
    FILE* f = std::fopen(args[1], "r");
    if (!f) { std::fprintf(stderr, "cannot open %s\n", args[1]); return 3; }
    while (mpz_inp_str(u, f, 62) && mpz_inp_str(v, f, 62)) push(u, v);
    std::fclose(f);
  } else if (!std::strcmp(args[0], "rand") && args.size() >= 4) {
    const unsigned bits = std::atoi(args[1]), gbits = std::atoi(args[2]);
    const int reps = std::atoi(args[3]);
    gmp_randstate_t st;
    gmp_randinit_mt(st);
    if (args.size() >= 5) gmp_randseed_ui(st, std::strtoul(args[4], nullptr, 10));
    for (int i = 0; i < reps; ++i) {
      do mpz_urandomb(u, st, bits - gbits); while (mpz_cmp_ui(u, 0) == 0);
      do mpz_urandomb(v, st, bits - gbits); while (mpz_cmp_ui(v, 0) == 0);
      do mpz_urandomb(g, st, gbits); while (mpz_cmp_ui(g, 0) == 0);
      mpz_mul(u, g, u);
      mpz_mul(v, g, v);
      push(u, v);
    }
  } else {
    return 1;
  }
  const size_t n = U.size();
  int mismatches = 0, errors = 0;
  double gpu_ms = 0, gmp_ms = 0;
  std::string err;
  try {
    GmpCuda::GmpCudaDevice::setDevice(0);
    GmpCuda::GmpCudaDevice dev;
    std::vector<__mpz_struct> G(n), R(n);
    for (size_t i = 0; i < n; ++i) { mpz_init(&G[i]); mpz_init(&R[i]); }
    for (size_t i = 0; i < n; ++i) {
      const double t0 = now_ms();
      mpz_gcd(&R[i], &U[i], &V[i]);
      gmp_ms += now_ms() - t0;
    }
    if (batch) {
      dev.gcdBatch(n, G.data(), U.data(), V.data());   // warm-up
      const double t0 = now_ms();
      dev.gcdBatch(n, G.data(), U.data(), V.data());
      gpu_ms = now_ms() - t0;
    } else {
      if (n) dev.gcd(&G[0], &U[0], &V[0]);              // warm-up, as testmodgcd.cpp:447-451
      for (size_t i = 0; i < n; ++i) {
        const double t0 = now_ms();
        try {
          dev.gcd(&G[i], &U[i], &V[i]);
        } catch (std::runtime_error& e) {
          ++errors;
          err = e.what();
          continue;
        }
        gpu_ms += now_ms() - t0;
      }
    }
    for (size_t i = 0; i < n; ++i)
      if (mpz_cmp(&G[i], &R[i]) != 0) ++mismatches;
  } catch (std::runtime_error& e) {
    err = e.what();
    errors = (int)n;
  }
  std::printf("{\"pairs\": %zu, \"mismatches\": %d, \"errors\": %d, \"gpu_ms_mean\": %.4f, \"gmp_ms_mean\": %.4f, "
              "\"mode\": \"%s\", \"gmp\": \"%s\", \"error\": \"%s\"}\n",
              n, mismatches, errors, n ? gpu_ms / n : 0.0, n ? gmp_ms / n : 0.0,
              batch ? "batch" : "plain", gmp_version, err.c_str());
  return (mismatches || errors) ? 4 : 0;
}

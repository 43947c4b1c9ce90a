// createModuli.cpp -- prints the moduli table as C++ source in the reference's format.
//
//   createModuli [L [count]] [--inverses]
//
// Output (stdout) is what the reference's createModuli prints (createModuli.cpp:131-169):
// a comment header, #include "GmpCuda.h", and
//     const uint32_t GmpCuda::moduli[] = { D, ... };
// one usable L-bit prime per line, largest first.  With --inverses it also prints the
// multiply-by-inverse constants J = floor(2^(W+L-1) / D) + 1 (W = 64) that the reference
// recomputes in every kernel launch (getModulus, GmpCudaDevice-getGcdKernel.cu:326-340):
//     const uint64_t GmpCuda::moduliInverse[] = { J, ... };
// Defaults: L = 32, count = 131072.  Exit status 2 if fewer than count moduli exist
// (createModuli.cpp:171-178), 1 for bad arguments.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "mgcd_moduli.h"

int main(int argc, char** argv)
{
  int L = 32;
  size_t count = 131072;
  bool inverses = false;
  int pos = 0;
  for (int i = 1; i < argc; ++i) {
    if (!std::strcmp(argv[i], "--inverses")) { inverses = true; continue; }
    if (pos == 0) L = std::atoi(argv[i]);
    else if (pos == 1) count = (size_t)std::strtoull(argv[i], nullptr, 10);
    ++pos;
  }
  if (L < 3 || L > 32) {
    std::fprintf(stderr, "L = %d is invalid.", L);
    return 1;
  }
  std::vector<uint32_t> q(count);
  const size_t got = mgcd::gen_moduli(L, q.data(), count);
  std::printf("//  AUTOMATICALLY GENERATED by createModuli: do not edit\n\n");
  std::printf("//  A list of %d-bit primes, selected so that DBM_a(N, J) will always be accurate.\n", L);
  std::printf("//  See Cavagnino & Werbrouck,\n");
  std::printf("//      Efficient Algorithms for Integer Division by Constants Using Multiplication,\n");
  std::printf("//      The Computer Journal, Vol. 51 No. 4, 2008.\n\n");
  std::printf("#include \"GmpCuda.h\"\n");
  std::printf("const uint32_t GmpCuda::moduli[] = \n{\n");
  for (size_t i = 0; i < got; ++i) std::printf("\t%u,\n", q[i]);
  std::printf("};\n");
  if (inverses) {
    std::printf("const uint64_t GmpCuda::moduliInverse[] = \n{\n");
    for (size_t i = 0; i < got; ++i) {
      const unsigned __int128 F = (unsigned __int128)1 << (64 + L - 1);
      const uint64_t J = (uint64_t)(F / q[i] + 1);
      std::printf("\t%lluull,\n", (unsigned long long)J);
    }
    std::printf("};\n");
  }
  if (got < count) {
    std::fprintf(stderr, "There are %zu usable %d-bit moduli, and %zu moduli are called for.\n", got, L, count);
    return 2;
  }
  std::fprintf(stderr, "%zu moduli were generated.\n", count);
  return 0;
}

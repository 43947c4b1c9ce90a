// mgcd_moduli.cpp -- the moduli table: createModuli-compatible prime list and the
// per-modulus constants the kernels use.
//
// The table is the reference's: the largest L-bit primes, descending, keeping only those
// for which the Cavagnino-Werbrouck multiply-by-inverse remainder DBM_a is exact for every
// W = 64 bit dividend (createModuli.cpp:143-167).  The reference sieves all 2^(L-2) odd
// numbers of [2^(L-1), 2^L) into a 1 GiB array at L = 32 and takes ~25 s; here a segmented
// sieve walks down from 2^L only as far as the requested count needs (milliseconds).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "mgcd_moduli.h"

namespace mgcd {

// bitlen(ceil(J / (D*J - 2^(W+L-1))) * D - 1) > W with J = floor(2^(W+L-1) / D) + 1.
static bool dbm_usable(uint32_t D, int L)
{
  constexpr int W = 64;
  using u128 = unsigned __int128;
  const u128 F = (u128)1 << (W + L - 1);
  const u128 J = F / D + 1;
  const u128 excess = (u128)D * J - F;                 // in (0, D]
  const u128 Qcr = J / excess + (J % excess != 0);
  const u128 Ncr = Qcr * D - 1;
  return (Ncr >> W) != 0;
}

size_t gen_moduli(int L, uint32_t* out, size_t count)
{
  if (L < 3 || L > 32 || (!out && count)) return 0;
  const uint64_t top = uint64_t{1} << L, floor_ = uint64_t{1} << (L - 1);
  const uint32_t root = (uint32_t)std::sqrt((double)top) + 1;

  // odd primes up to sqrt(2^L)
  std::vector<uint8_t> comp(root + 1, 0);
  std::vector<uint32_t> small;
  for (uint32_t i = 3; i <= root; i += 2) {
    if (comp[i]) continue;
    small.push_back(i);
    for (uint64_t k = (uint64_t)i * i; k <= root; k += 2 * (uint64_t)i) comp[k] = 1;
  }

  // Blocks of odd candidates, walking down: block covers odd x in [base, base + 2*len).
  constexpr uint64_t BLOCK = uint64_t{1} << 18;
  std::vector<uint8_t> mark(BLOCK);
  size_t n = 0;
  uint64_t end = top;                                  // exclusive upper bound of this block
  while (n < count && end > floor_ + 1) {
    uint64_t base = end > floor_ + 2 * BLOCK ? end - 2 * BLOCK : floor_ + 1;
    base |= 1;                                         // first odd >= base
    if (base >= end) break;
    const uint64_t len = (end - base + 1) / 2;         // odd numbers base, base+2, ..., < end
    std::memset(mark.data(), 0, len);
    for (uint32_t p : small) {
      const uint64_t pp = (uint64_t)p * p;
      if (pp >= end) break;
      uint64_t m = (base + p - 1) / p * p;             // first multiple of p >= base
      if (m < pp) m = pp;
      if ((m & 1) == 0) m += p;                        // odd multiples only
      for (; m < end; m += 2 * (uint64_t)p) mark[(m - base) / 2] = 1;
    }
    for (uint64_t i = len; i-- > 0 && n < count;) {   // descending within the block
      if (mark[i]) continue;
      const uint32_t x = (uint32_t)(base + 2 * i);
      if (dbm_usable(x, L)) out[n++] = x;
    }
    end = base;
  }
  return n;
}

int moduli_needed(int L, size_t bits)
{
  // numModuliNeededFor (GmpCudaDevice-gcd.cu:49-55), in float as the reference evaluates it.
  const float C_L = (float)(1.6 - 0.015 * L);
  if (bits < 2) return 256;
  const int n = (int)std::ceil(C_L * (float)bits / std::log((float)bits));
  return ((n - 1) / 256 + 1) * 256;
}

void mod_constants(const uint32_t* q, size_t n, ModConstHost* out)
{
  for (size_t i = 0; i < n; ++i) {
    const uint32_t m = q[i];
    uint32_t x = m;                                    // Newton: x = m^-1 mod 2^32
    for (int k = 0; k < 5; ++k) x *= 2u - m * x;
    const uint64_t r1 = (uint64_t{1} << 32) % m;
    out[i].q = m;
    out[i].qinv = 0u - x;
    out[i].r2 = (uint32_t)((r1 * r1) % m);
    out[i].r1 = (uint32_t)r1;
  }
}

}  // namespace mgcd

// mgcd_moduli.h -- host-side moduli table helpers.
#pragma once
#include <cstddef>
#include <cstdint>

namespace mgcd {

// Host mirror of the device ModConst record (mgcd_device.cuh): q, -q^-1 mod 2^32,
// 2^64 mod q, 2^32 mod q.
struct ModConstHost {
  uint32_t q, qinv, r2, r1;
};

// The first `count` usable L-bit primes, descending (createModuli order).  Returns the
// number written.
size_t gen_moduli(int L, uint32_t* out, size_t count);

// numModuliNeededFor (GmpCudaDevice-gcd.cu:49-55) for modulus width L.
int moduli_needed(int L, size_t bits);

// q, -q^-1 mod 2^32, 2^64 mod q for each modulus.
void mod_constants(const uint32_t* q, size_t n, ModConstHost* out);

}  // namespace mgcd

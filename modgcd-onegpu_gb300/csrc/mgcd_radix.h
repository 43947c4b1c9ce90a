// mgcd_radix.h -- mixed-radix digits to binary (host, GMP).
#pragma once
#include <gmp.h>

#include <cstddef>
#include <cstdint>

#include "../../include/modgcd.h"

namespace mgcd {

// |g| for digits d[0..n): g = d[n-1].value, then g = g * d[i].modulus + d[i].value.
void mixed_radix_to_mpz(const mgcd_pair* d, size_t n, mpz_ptr g);

// The same as little-endian 32-bit limbs; -1 if cap is too small.
int mixed_radix_to_limbs(const mgcd_pair* d, size_t n, uint32_t* out, size_t cap, size_t* len);

}  // namespace mgcd

// mgcd_radix.cpp -- signed mixed-radix digits to a binary integer, on the host with GMP.
//
// The reference converts with a Horner loop of mpz_mul_ui / mpz_add_ui / mpz_sub_ui over
// the digits (GmpCudaDevice-gcd.cu:116-129), O(k^2) limb work for k digits.  The same
// value is built here by splitting the digit list in halves:
//     value(lo, hi) = value(lo, mid) + prod(lo, mid) * value(mid, hi),
//     prod(lo, hi)  = prod(lo, mid) * prod(mid, hi),
// so the large products go through GMP's subquadratic multiplication; short runs use the
// reference's Horner directly.
#include <gmp.h>

#include <cstdint>
#include <cstring>

#include "mgcd_radix.h"

namespace mgcd {

namespace {

constexpr size_t LEAF = 24;

void leaf(const mgcd_pair* d, size_t lo, size_t hi, mpz_ptr val, mpz_ptr prod)
{
  mpz_set_si(val, d[hi - 1].value);
  for (size_t i = hi - 1; i-- > lo;) {
    mpz_mul_ui(val, val, d[i].modulus);
    const int32_t x = d[i].value;
    if (x < 0)
      mpz_sub_ui(val, val, (unsigned long)(0u - (uint32_t)x));
    else
      mpz_add_ui(val, val, (unsigned long)x);
  }
  if (prod) {
    mpz_set_ui(prod, d[lo].modulus);
    for (size_t i = lo + 1; i < hi; ++i) mpz_mul_ui(prod, prod, d[i].modulus);
  }
}

void split(const mgcd_pair* d, size_t lo, size_t hi, mpz_ptr val, mpz_ptr prod)
{
  if (hi - lo <= LEAF) {
    leaf(d, lo, hi, val, prod);
    return;
  }
  const size_t mid = lo + (hi - lo) / 2;
  mpz_t vh, pl;
  mpz_init(vh);
  mpz_init(pl);
  split(d, lo, mid, val, pl);
  split(d, mid, hi, vh, prod);
  mpz_mul(vh, vh, pl);
  mpz_add(val, val, vh);
  if (prod) mpz_mul(prod, prod, pl);
  mpz_clear(vh);
  mpz_clear(pl);
}

}  // namespace

void mixed_radix_to_mpz(const mgcd_pair* d, size_t n, mpz_ptr g)
{
  if (n == 0) {
    mpz_set_ui(g, 0);
    return;
  }
  split(d, 0, n, g, nullptr);
  mpz_abs(g, g);
}

int mixed_radix_to_limbs(const mgcd_pair* d, size_t n, uint32_t* out, size_t cap, size_t* len)
{
  mpz_t g;
  mpz_init(g);
  mixed_radix_to_mpz(d, n, g);
  size_t words = mpz_sgn(g) == 0 ? 0 : (mpz_sizeinbase(g, 2) + 31) / 32;
  int rc = 0;
  if (words > cap) {
    rc = -1;
  } else if (words) {
    size_t cnt = 0;
    mpz_export(out, &cnt, -1, sizeof(uint32_t), 0, 0, g);
    words = cnt;
  }
  if (len) *len = rc ? 0 : words;
  mpz_clear(g);
  return rc;
}

}  // namespace mgcd

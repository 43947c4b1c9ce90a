// mgcd_radix_dev.cu -- signed mixed-radix digits to binary on the device.
//
// The reference turns the kernel's digits into an integer on the host with a Horner loop
// of mpz_mul_ui / mpz_add_ui / mpz_sub_ui (GmpCudaDevice-gcd.cu:116-129):
//     g = d[n-1];  g = g * m_i + d_i  for i = n-2 .. 0;  result |g|.
// Here one CTA converts one pair:
//   1. sign: with symmetric digits |d_i| <= (m_i - 1) / 2 the lower digits are worth less
//      than half of one unit of the top digit, so sign(g) = sign(d[n-1]); the digits are
//      negated when it is negative, which yields |g| directly;
//   2. the digits become nonnegative (e_i in [0, m_i)) by a borrow pass from the bottom;
//   3. Horner on the limbs in a carry-deferred form: limb j holds V_j <= 2^33 - 2 and the
//      value is sum V_j 2^(32 j).  Normalising a limb, w_j = (V_j mod 2^32) + (V_{j-1} >> 32)
//      <= 2^32, needs only its lower neighbour, so a step g <- g * m + e is, for every limb
//      at once, p_j = w_j m (+ e at j = 0) < 2^64 and V'_j = lo(p_j) + hi(p_{j-1}): one
//      barrier per digit, no carry chain.  After s steps the value is below 2^(32 (s+1)),
//      so only limbs 0..s can be nonzero;
//   4. one carry pass gives the canonical limbs.
// Pairs with more than RADIX_MAX digits (gcds above ~127,000 bits) are left to the host.
#include <cstdint>
#include <cuda_runtime.h>

#include "mgcd_internal.h"

namespace mgcd {

namespace {

constexpr int RT = 256;   // threads per CTA

__global__ void __launch_bounds__(RT) radix_kernel(const PairDesc* __restrict__ pairs, uint32_t npairs,
                                                   const mgcd_pair* __restrict__ digits,
                                                   const uint32_t* __restrict__ count,
                                                   const int32_t* __restrict__ status, uint32_t* __restrict__ glimbs,
                                                   uint32_t* __restrict__ glen)
{
  extern __shared__ __align__(16) unsigned long long rsm[];
  unsigned long long* V0 = rsm;                          // 2 x (RADIX_MAX + 2) limbs
  unsigned long long* V1 = rsm + (RADIX_MAX + 2);
  uint32_t* E = reinterpret_cast<uint32_t*>(rsm + 2 * (RADIX_MAX + 2));   // RADIX_MAX digits
  uint32_t* Mq = E + RADIX_MAX;                                            // RADIX_MAX moduli
  __shared__ uint32_t s_len;
  const unsigned long long LO = 0xFFFFFFFFull;

  for (uint32_t k = blockIdx.x; k < npairs; k += gridDim.x) {
    const PairDesc d = pairs[k];
    const uint32_t n = count[k];
    if (status[k] != ST_OK || n > RADIX_MAX) {      // failed pair, or converted on the host
      if (threadIdx.x == 0) glen[k] = RADIX_HOST;
      continue;
    }
    if (n == 0) {
      if (threadIdx.x == 0) glen[k] = 0;
      continue;
    }
    const mgcd_pair* dg = digits + d.out_off;
    const bool neg = dg[n - 1].value < 0;
    // 1-2. digits (sign-corrected) into shared memory, then the borrow pass (one thread)
    for (uint32_t i = threadIdx.x; i < n; i += RT) {
      const mgcd_pair x = dg[i];
      E[i] = (uint32_t)(neg ? -x.value : x.value);
      Mq[i] = x.modulus;
    }
    for (uint32_t j = threadIdx.x; j < n + 2; j += RT) V0[j] = V1[j] = 0ull;
    __syncthreads();
    if (threadIdx.x == 0) {
      int32_t c = 0;
      for (uint32_t i = 0; i + 1 < n; ++i) {
        const int32_t x = (int32_t)E[i] + c;     // in (-m/2 - 1, m/2)
        c = x < 0 ? -1 : 0;
        E[i] = x < 0 ? (uint32_t)x + Mq[i] : (uint32_t)x;
      }
      E[n - 1] = (uint32_t)((int32_t)E[n - 1] + c);
      V0[0] = E[n - 1];
    }
    __syncthreads();
    // 3. Horner, carry-deferred, one barrier per digit
    unsigned long long* src = V0;
    unsigned long long* dst = V1;
    for (uint32_t s = 1; s < n; ++s) {
      const uint32_t i = n - 1 - s;                   // digit folded in at this step
      const unsigned long long m = Mq[i], e = E[i];
      for (uint32_t j = threadIdx.x; j <= s; j += RT) {
        const unsigned long long vj = src[j];
        const unsigned long long vj1 = j >= 1 ? src[j - 1] : 0ull;
        const unsigned long long vj2 = j >= 2 ? src[j - 2] : 0ull;
        const unsigned long long wj = (vj & LO) + (vj1 >> 32);
        const unsigned long long wj1 = (vj1 & LO) + (vj2 >> 32);
        const unsigned long long pj = wj * m + (j == 0 ? e : 0ull);
        const unsigned long long pj1 = j >= 1 ? wj1 * m + (j == 1 ? e : 0ull) : 0ull;
        dst[j] = (pj & LO) + (pj1 >> 32);
      }
      __syncthreads();
      unsigned long long* t = src;
      src = dst;
      dst = t;
    }
    // 4. carry pass and output (one thread; the result has at most n limbs)
    if (threadIdx.x == 0) {
      unsigned long long carry = 0;
      uint32_t len = 0;
      uint32_t* out = glimbs + d.g_off;
      for (uint32_t j = 0; j < n; ++j) {
        const unsigned long long x = src[j] + carry;
        const uint32_t limb = (uint32_t)x;
        carry = x >> 32;
        if (j < d.g_cap) out[j] = limb;
        if (limb) len = j + 1;
      }
      s_len = (carry != 0 || len > d.g_cap) ? RADIX_HOST : len;
      glen[k] = s_len;
    }
    __syncthreads();
  }
}

}  // namespace

size_t radix_smem_bytes()
{
  return 2 * (RADIX_MAX + 2) * sizeof(unsigned long long) + 2 * RADIX_MAX * sizeof(uint32_t);
}

cudaError_t launch_radix(const PairDesc* pairs, uint32_t npairs, const mgcd_pair* digits, const uint32_t* count,
                         const int32_t* status, uint32_t* glimbs, uint32_t* glen, int grid, cudaStream_t s)
{
  if (npairs == 0) return cudaSuccess;
  const size_t smem = radix_smem_bytes();
  cudaError_t e = cudaFuncSetAttribute(radix_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  radix_kernel<<<grid, RT, smem, s>>>(pairs, npairs, digits, count, status, glimbs, glen);
  return cudaGetLastError();
}

}  // namespace mgcd

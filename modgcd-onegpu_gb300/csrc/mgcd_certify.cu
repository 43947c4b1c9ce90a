// mgcd_certify.cu -- exhaustive certification of the float quotient steps of inv_mod on
// the device it runs on (the reference certifies its quoRem<QUASI> the same way, per
// device, certifyQuoRemQuasi.cu:25-48).
//
// Each Euclid step of inv_mod takes a nearest-integer quotient estimate Q from a float
// reciprocal and the exact remainder r = r0 - Q r1; the step makes progress (|r| < r1) iff
// Q is within 1 of r0 / r1:
//   phase A (2^22 <= r1 < r0 < 2^32): Q = rn(rn(r0) * rcp(rn(r1)));
//   phase A of inv_mod_narrow (2^22 <= r1 < r0 < 2^30): Q from
//                                      fma_rn(rn(r0), rcp(rn(r1)), 1.5 * 2^23);
//   phase C (2 <= r1 < r0 < 2^22):    Q from fma_rn(r0, rcp(r1), 1.5 * 2^23), remainder
//                                      fma_rn(-Q, r1, r0);
//   phase C with r0 < r1 (the step after inv_mod_narrow's phase B may start there):
//                                      Q of 0 or 1, exact remainder.
// On [k r1, (k+1) r1 - 1] the allowed quotients are k at r0 = k r1 and {k, k + 1} above.
// For a fixed r1 both estimates are non-decreasing in r0 (every operation is monotone and
// rcp(r1) is fixed), so the estimate is allowed on the whole interval iff it is at the two
// ends: checking both ends of every interval, for every r1, covers every (r0, r1) of the
// phase.  Phase A: ~6e10 end points; phase C: ~1.3e8 (where the remainder is also checked).
// inv_mod runs phase C on signed remainders; its estimate is odd in each operand (a
// reciprocal and round-to-nearest-even products), so the positive operands checked here
// cover the negative ones too.
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/modgcd.h"
#include "mgcd_device.cuh"
#include "mgcd_plan.h"

namespace mgcd {

namespace {

struct CertOut {
  unsigned long long checked;
  unsigned long long failures;
  uint32_t first_r0, first_r1;
};

// Q allowed for r0 in [k r1, (k+1) r1): k at the bottom end, k or k + 1 above it.
__device__ __forceinline__ bool quot_ok(uint64_t r0, uint32_t r1, uint32_t k, uint32_t Q)
{
  return r0 == (uint64_t)k * r1 ? Q == k : (Q == k || Q == k + 1u);
}

// Phase C step as inv_mod runs it: an allowed quotient and the exact signed remainder.
__device__ __forceinline__ bool step_c_ok(uint32_t r0, uint32_t r1, uint32_t k)
{
  const float f0 = (float)r0, f1 = (float)r1;
  const float qm = inv_quot_c(f0, f1);
  const uint32_t Q = __float_as_uint(qm) - INV_MAGIC_BITS;
  if (!quot_ok(r0, r1, k, Q)) return false;
  const float rem = __fmaf_rn(INV_MAGIC - qm, f1, f0);
  return rem == (float)((int32_t)r0 - (int32_t)(Q * r1));
}

__device__ void fail(CertOut* o, uint32_t r0, uint32_t r1)
{
  if (atomicAdd(&o->failures, 1ull) == 0ull) {
    o->first_r0 = r0;
    o->first_r1 = r1;
  }
}

__global__ void __launch_bounds__(256) certify_kernel(CertOut* out)
{
  const uint32_t stride = gridDim.x * blockDim.x;
  unsigned long long n = 0;
  // phase C: 2 <= r1 < r0 < 2^22
  constexpr uint32_t C_TOP = (1u << 22) - 1u;
  for (uint32_t r1 = 2u + blockIdx.x * blockDim.x + threadIdx.x; r1 < (1u << 22); r1 += stride) {
    for (uint32_t k = 1; k <= C_TOP / r1; ++k) {
      const uint32_t lo = k == 1 ? r1 + 1u : k * r1;
      const uint32_t hi = min((k + 1) * r1 - 1u, C_TOP);
      if (lo > hi) continue;
      n += 2;
      if (!step_c_ok(lo, r1, k)) fail(out, lo, r1);
      if (!step_c_ok(hi, r1, k)) fail(out, hi, r1);
    }
    n += 2;                                            // k = 0: r0 in [1, r1 - 1]
    if (!step_c_ok(1u, r1, 0u)) fail(out, 1u, r1);
    if (!step_c_ok(r1 - 1u, r1, 0u)) fail(out, r1 - 1u, r1);
  }
  // phase A of inv_mod_narrow: 2^22 <= r1 < r0 < 2^30
  constexpr uint32_t AN_TOP = (1u << 30) - 1u;
  for (uint32_t r1 = (1u << 22) + blockIdx.x * blockDim.x + threadIdx.x; r1 < AN_TOP; r1 += stride) {
    const float g1 = __uint2float_rn(r1);
    for (uint32_t k = 1; k <= AN_TOP / r1; ++k) {
      const uint32_t lo = k == 1 ? r1 + 1u : k * r1;
      const uint32_t hi = min((k + 1) * r1 - 1u, AN_TOP);
      if (lo > hi) continue;
      n += 2;
      if (!quot_ok(lo, r1, k, inv_quot_an(__uint2float_rn(lo), g1))) fail(out, lo, r1);
      if (!quot_ok(hi, r1, k, inv_quot_an(__uint2float_rn(hi), g1))) fail(out, hi, r1);
    }
  }
  // phase A: 2^22 <= r1 < r0 < 2^32
  constexpr uint64_t A_TOP = 0xFFFFFFFFull;
  for (uint64_t r1w = (1ull << 22) + blockIdx.x * blockDim.x + threadIdx.x; r1w < A_TOP; r1w += stride) {
    const uint32_t r1 = (uint32_t)r1w;
    const uint32_t kmax = (uint32_t)(A_TOP / r1w);
    for (uint32_t k = 1; k <= kmax; ++k) {
      const uint64_t lo = k == 1 ? r1w + 1 : (uint64_t)k * r1w;
      const uint64_t hi = min((uint64_t)(k + 1) * r1w - 1, A_TOP);
      if (lo > hi) continue;
      n += 2;
      if (!quot_ok(lo, r1, k, inv_quot_a((uint32_t)lo, r1))) fail(out, (uint32_t)lo, r1);
      if (!quot_ok(hi, r1, k, inv_quot_a((uint32_t)hi, r1))) fail(out, (uint32_t)hi, r1);
    }
  }
  atomicAdd(&out->checked, n);
}

}  // namespace

}  // namespace mgcd

extern "C" int mgcd_certify_inverse(mgcd_context* c, uint64_t* checked, uint64_t* failures, uint32_t* first_r0,
                                    uint32_t* first_r1)
{
  using namespace mgcd;
  if (!c || !checked || !failures) return MGCD_ERR_INVALID_ARG;
  if (c->serving) return MGCD_ERR_BUSY;
  if (cudaSetDevice(c->device) != cudaSuccess) return MGCD_ERR_CUDA;
  cudaStream_t s = c->main.stream;
  DevBuf buf;
  if (buf.grow(sizeof(CertOut), c->pool, s) != cudaSuccess) return MGCD_ERR_CUDA;
  CertOut h = {};
  int rc = MGCD_OK;
  if (cudaMemsetAsync(buf.p, 0, sizeof(CertOut), s) != cudaSuccess) rc = MGCD_ERR_CUDA;
  if (rc == MGCD_OK) {
    certify_kernel<<<c->sms * 8, 256, 0, s>>>(buf.as<CertOut>());
    if (cudaGetLastError() != cudaSuccess) rc = MGCD_ERR_CUDA;
  }
  if (rc == MGCD_OK && (cudaMemcpyAsync(&h, buf.p, sizeof(CertOut), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                        cudaStreamSynchronize(s) != cudaSuccess))
    rc = MGCD_ERR_CUDA;
  buf.release(s);
  cudaStreamSynchronize(s);
  if (rc != MGCD_OK) return rc;
  *checked = h.checked;
  *failures = h.failures;
  if (first_r0) *first_r0 = h.first_r0;
  if (first_r1) *first_r1 = h.first_r1;
  return MGCD_OK;
}

// mgcd_device.cuh -- device arithmetic of the modular GCD kernels (sm_103a).
//
// Per-modulus arithmetic is done in Montgomery form with R = 2^32 (REDC), and modular
// inverses by the extended Euclidean algorithm with float-reciprocal quotient estimates
// followed by an exact integer correction.  Everything here is bit-exact integer math;
// floats only ever produce a quotient estimate that is corrected, and every inverse is
// checked (x * x^-1 == 1) before it is used.
#pragma once
#include <cstdint>

namespace mgcd {

// Per-modulus constants, one 16-byte record per table entry.
//   q    : the prime modulus (table order = createModuli order, descending)
//   qinv : -q^{-1} mod 2^32 (Montgomery)
//   r2   : 2^64 mod q
//   r1   : 2^32 mod q (the Montgomery form of 1)
struct __align__(16) ModConst {
  uint32_t q, qinv, r2, r1;
};

// State of one modulus during the reduction loop: t = u_q / v_q mod q, or a marker.
constexpr uint32_t T_INF = 0xFFFFFFFFu;      // v == 0 (mod q), u != 0
constexpr uint32_t T_DEGEN = 0xFFFFFFFEu;    // u == v == 0 (mod q): q divides both
constexpr uint32_t T_RETIRED = 0xFFFFFFFDu;  // q was used as a pivot
constexpr uint32_t T_MARK = T_RETIRED;       // t >= T_MARK: not a finite ratio
constexpr uint32_t U_RETIRED = 0xFFFFFFFFu;  // recovery: modulus consumed by a digit
constexpr int32_t MOD_INFINITY = INT32_MIN;  // reference MOD_INFINITY (GmpCudaDevice-getGcdKernel.cu:46)
constexpr uint32_t KEY_INF_HI = 0x80000000u; // |MOD_INFINITY| as the key's high word

// T * 2^-32 mod q for T < q * 2^32; result in [0, q).
__device__ __forceinline__ uint32_t redc(uint64_t T, uint32_t q, uint32_t qinv)
{
  const uint32_t lo = (uint32_t)T, hi = (uint32_t)(T >> 32);
  const uint32_t m = lo * qinv;                   // T + m*q == 0 (mod 2^32)
  const uint32_t mh = __umulhi(m, q);
  const uint64_t t = (uint64_t)hi + mh + (lo != 0u);   // (T + m*q) / 2^32 < 2q
  return (uint32_t)(t >= q ? t - q : t);
}

// a * b * 2^-32 mod q, a, b < q.
__device__ __forceinline__ uint32_t mont_mul(uint32_t a, uint32_t b, uint32_t q, uint32_t qinv)
{
  return redc((uint64_t)a * b, q, qinv);
}

__device__ __forceinline__ uint32_t mod_sub(uint32_t a, uint32_t b, uint32_t q)
{
  return a - b + ((a < b) ? q : 0u);
}

// Symmetric residue with the reference's boundary (toSigned, GmpCudaDevice-getGcdKernel.cu:273-281):
// x >= q/2 maps to x - q.
__device__ __forceinline__ int32_t to_signed(uint32_t x, uint32_t q)
{
  return (x >= (q >> 1)) ? (int32_t)(x - q) : (int32_t)x;
}

// fromSigned (GmpCudaDevice-getGcdKernel.cu:264-271) for |x| < q.
__device__ __forceinline__ uint32_t from_signed(int32_t x, uint32_t q)
{
  return (uint32_t)x + ((x < 0) ? q : 0u);
}

__device__ __forceinline__ float rcp_approx(float y)
{
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(y));
  return r;
}

// Exact inverse by integer-only extended Euclid (64-bit division); the fallback that
// runs only if the fast routine's self-check ever fails.
static __device__ __noinline__ uint32_t inv_mod_slow(uint32_t x, uint32_t q)
{
  int64_t r0 = q, r1 = x, s0 = 0, s1 = 1;
  while (r1 != 0) {
    const int64_t Q = r0 / r1;
    int64_t t = r0 - Q * r1; r0 = r1; r1 = t;
    t = s0 - Q * s1; s0 = s1; s1 = t;
  }
  return (uint32_t)(s0 < 0 ? s0 + q : s0);
}

// Quotient estimates of inv_mod's Euclid steps (also run by the certification kernel).
// Phase A (2^22 <= r1 < r0 < 2^32): nearest integer to r0 / r1 from a float reciprocal.
__device__ __forceinline__ uint32_t inv_quot_a(uint32_t r0, uint32_t r1)
{
  return __float2uint_rn(__fmul_rn(__uint2float_rn(r0), rcp_approx(__uint2float_rn(r1))));
}

// Phase C (r1 < r0 < 2^22, both exact in float): Q = rint(f0 * rcp(f1)) read from the
// mantissa of Q + 1.5 * 2^23; returns the float whose low mantissa bits hold Q.
constexpr float INV_MAGIC = 12582912.0f;     // 1.5 * 2^23
constexpr uint32_t INV_MAGIC_BITS = 0x4B400000u;
__device__ __forceinline__ float inv_quot_c(float f0, float f1)
{
  return __fmaf_rn(f0, rcp_approx(f1), INV_MAGIC);
}

// x^{-1} mod q for 0 < x < q, q an odd prime < 2^32.
//
// Extended Euclid on (r0, r1) = (q, x) with nearest-integer quotients (remainders of
// either sign, their magnitudes kept; about 13 steps for 32-bit operands instead of 19),
// tracking the cofactor s_k modulo 2^32 with s_k * x == r_k (mod q):
//   phase A (r1 >= 2^22): operands rounded to float, quotient < 2^10, estimate within
//            2^-11 of r0/r1, so the rounded quotient is within 1 of it and |r| < r1;
//   phase B (r0 >= 2^22 > r1): one exact integer division at the transition;
//   phase C (|r0|, |r1| < 2^22): operands exact in float, quotient below 2^22 in magnitude
//            and within 1/2 of r0/r1 before rounding, remainder exact by FMA (an integer
//            below 2^22 in magnitude); remainders and quotients keep their signs.
// The bounds assume rcp.approx.ftz.f32's documented error (1 ulp).  At the end |s| < q,
// so s is either the 32-bit value read as unsigned or that minus 2^32 (possible only for
// q > 2^31); the candidate whose product with x is 1 is taken, and if neither is (never
// observed), the integer-only routine recomputes it, so no float error can reach a result.
__device__ __forceinline__ uint32_t inv_mod(uint32_t x, uint32_t q, uint32_t qinv)
{
  uint32_t r0 = q, r1 = x, s0 = 0, s1 = 1;
  while (r1 >= (1u << 22)) {
    const uint32_t Q = inv_quot_a(r0, r1);
    const uint64_t m = (uint64_t)Q * r1;
    const bool neg = m > r0;
    const uint32_t d = r0 - (uint32_t)m;        // r0 - Q r1 modulo 2^32, |r0 - Q r1| < r1
    const uint32_t s = s0 - Q * s1;
    r0 = r1; s0 = s1;
    r1 = neg ? 0u - d : d;
    s1 = neg ? 0u - s : s;
  }
  if (r1 > 1u) {
    if (r0 >= (1u << 22)) {
      const uint32_t Q = r0 / r1;
      const uint32_t r = r0 - Q * r1;
      const uint32_t s = s0 - Q * s1;
      r0 = r1; r1 = r; s0 = s1; s1 = s;
    }
    // remainders keep their sign here (quotients of either sign, read from the mantissa
    // as two's complement), so s_k x == r_k holds without a sign fix per step
    float f0 = (float)r0, f1 = (float)r1;
    int guard = 64;
    while (fabsf(f1) > 1.0f && --guard) {
      const float qm = inv_quot_c(f0, f1);
      const float rem = __fmaf_rn(INV_MAGIC - qm, f1, f0);   // r0 - Q r1, exact
      const uint32_t Q = __float_as_uint(qm) - INV_MAGIC_BITS;
      const uint32_t s = s0 - Q * s1;
      f0 = f1; s0 = s1;
      f1 = rem; s1 = s;
    }
    if (f1 < 0.0f) s1 = 0u - s1;                   // s1 x == -1
  }
  // inv * x == 1 (mod q)  <=>  redc(inv * x) == redc(1)
  const uint32_t one = redc(1ull, q, qinv);
  if (q < 0x80000000u) {
    const uint32_t inv = (int32_t)s1 < 0 ? s1 + q : s1;
    if (redc((uint64_t)inv * x, q, qinv) == one) return inv;
  } else {
    // candidates s1 mod q and (s1 - 2^32) mod q = that - (2^32 - q); redc of the second's
    // product with x is the first's minus x
    const uint32_t inv = s1 >= q ? s1 - q : s1;
    const uint32_t c = redc((uint64_t)inv * x, q, qinv);
    if (c == one) return inv;
    if (mod_sub(c, x, q) == one) return mod_sub(inv, 0u - q, q);
  }
  return inv_mod_slow(x, q);
}

// Phase A quotient of inv_mod_narrow (2^22 <= r1 < r0 < 2^30, so Q < 2^8): the nearest
// integer to rn(r0) * rcp(rn(r1)), read from the mantissa (one rounding) instead of a
// float-to-integer conversion; g0, g1 are the operands already converted.
__device__ __forceinline__ uint32_t inv_quot_an(float g0, float g1)
{
  return __float_as_uint(__fmaf_rn(g0, rcp_approx(g1), INV_MAGIC)) - INV_MAGIC_BITS;
}

// x^{-1} mod q for 0 < x < q < 2^30 (the moduli of widths up to 30 bits): inv_mod's Euclid
// with cheaper steps where the narrower operands allow them.
//   phase A (r1 >= 2^22): quotient estimate as inv_quot_an, each remainder converted once;
//            |r0 - Q r1| < r1 < 2^30, so the remainder and its sign come from 32-bit
//            wrapping arithmetic read as signed;
//   phase B (r0 >= 2^22 > r1): a float quotient estimate instead of an integer division.
//            Its error is below (r0 / r1) 2^-22 + 1/2 (operand rounding 2^-24, reciprocal
//            2^-23, product 2^-24), so the exact signed remainder r0 - Q r1 is below
//            2^8 + r1 / 2 < 2^22 in magnitude: exact in float, as phase C requires (its
//            first step may then see |r0| < |r1|, a quotient of 0 or +-1);
//   phase C: inv_mod's, two steps per loop trip with the roles of the registers
//            alternating, at most 64 steps (never reached: 22-bit operands take ~32 at most).
// The result is checked as inv_mod's is, with the same integer-only fallback.
__device__ __forceinline__ uint32_t inv_mod_narrow(uint32_t x, uint32_t q, uint32_t qinv)
{
  uint32_t r0 = q, r1 = x, s0 = 0, s1 = 1;
  float g0 = __uint2float_rn(r0), g1 = __uint2float_rn(r1);
  while (r1 >= (1u << 22)) {
    const uint32_t Q = inv_quot_an(g0, g1);
    const uint32_t d = r0 - Q * r1;
    const uint32_t s = s0 - Q * s1;
    const bool neg = (int32_t)d < 0;
    r0 = r1; s0 = s1; g0 = g1;
    r1 = neg ? 0u - d : d;
    s1 = neg ? 0u - s : s;
    g1 = __uint2float_rn(r1);
  }
  if (r1 > 1u) {
    int32_t i0 = (int32_t)r0, i1 = (int32_t)r1;
    if (r0 >= (1u << 22)) {
      const uint32_t Q = __float2uint_rn(__fmul_rn(g0, rcp_approx(g1)));
      const int32_t r = (int32_t)(r0 - Q * r1);
      const uint32_t s = s0 - Q * s1;
      i0 = i1; i1 = r; s0 = s1; s1 = s;
    }
    float f0 = (float)i0, f1 = (float)i1;
    for (int trips = 32; trips > 0 && fabsf(f1) > 1.0f; --trips) {
      {
        const float qm = inv_quot_c(f0, f1);
        f0 = __fmaf_rn(INV_MAGIC - qm, f1, f0);
        s0 = s0 - (__float_as_uint(qm) - INV_MAGIC_BITS) * s1;
      }
      if (!(fabsf(f0) > 1.0f)) { f1 = f0; s1 = s0; break; }
      {
        const float qm = inv_quot_c(f1, f0);
        f1 = __fmaf_rn(INV_MAGIC - qm, f0, f1);
        s1 = s1 - (__float_as_uint(qm) - INV_MAGIC_BITS) * s0;
      }
    }
    if (f1 < 0.0f) s1 = 0u - s1;                   // s1 x == -1
  }
  const uint32_t one = redc(1ull, q, qinv);
  const uint32_t inv = (int32_t)s1 < 0 ? s1 + q : s1;
  if (redc((uint64_t)inv * x, q, qinv) == one) return inv;
  return inv_mod_slow(x, q);
}

// Register arrays indexed by a runtime slot number, without spilling them to memory.
template <int K, class V>
__device__ __forceinline__ V pick(const V (&a)[K], int s)
{
  V r = a[0];
#pragma unroll
  for (int t = 1; t < K; ++t)
    if (t == s) r = a[t];
  return r;
}

template <int K, class V>
__device__ __forceinline__ void put(V (&a)[K], int s, V v)
{
#pragma unroll
  for (int t = 0; t < K; ++t)
    if (t == s) a[t] = v;
}

// Key of the reduction loop's pivot choice (postMinPair, GmpCudaDevice-getGcdKernel.cu:152-154):
// high word |value| (0x80000000 for MOD_INFINITY), low word modulus - (value >= 0).
__device__ __forceinline__ void t_key(uint32_t t, uint32_t q, uint32_t& hi, uint32_t& lo)
{
  if (t >= T_MARK) { hi = KEY_INF_HI; lo = q; return; }
  const bool neg = t >= (q >> 1);
  hi = neg ? q - t : t;
  lo = neg ? q : q - 1u;
}

__device__ __forceinline__ bool key_less(uint32_t h1, uint32_t l1, uint32_t h2, uint32_t l2)
{
  return h1 < h2 || (h1 == h2 && l1 < l2);
}

// (p, b) from a key (collectMinPair, GmpCudaDevice-getGcdKernel.cu:214-219).
__device__ __forceinline__ void key_pair(uint32_t hi, uint32_t lo, uint32_t& p, int32_t& b)
{
  p = lo | 1u;
  b = (lo & 1u) ? (int32_t)(0u - hi) : (int32_t)hi;
}

// Lexicographic (hi, lo) minimum over the warp, result in every lane.
__device__ __forceinline__ void warp_min_key(uint32_t& hi, uint32_t& lo)
{
  const uint32_t mh = __reduce_min_sync(0xFFFFFFFFu, hi);
  const uint32_t ml = __reduce_min_sync(0xFFFFFFFFu, hi == mh ? lo : 0xFFFFFFFFu);
  hi = mh;
  lo = ml;
}

// One reduction-loop update of a modulus state t for pivot (p, b):
//   t' = p / (t - b)  (mod q)   since t' = u'/v' = v / ((u - b v)/p)
// with t = INF -> 0 (v was 0: u' = 0, v' = u/p), t == b -> INF (v' = 0), degenerate and
// retired states fixed; the pivot's own modulus retires.
// narrow: q < 2^30 (the shorter inverse, inv_mod_narrow).
__device__ __forceinline__ uint32_t t_update(uint32_t t, uint32_t q, uint32_t qinv, uint32_t p, int32_t b,
                                             bool narrow)
{
  if (t >= T_MARK) return (t == T_INF) ? 0u : t;
  if (q == p) return T_RETIRED;
  const uint32_t pm = (p > q) ? p - q : p;
  const uint32_t d = mod_sub(t, from_signed(b, q), q);
  if (d == 0u) return T_INF;
  // redc(d) = d/R, inv = R/d, mont_mul(pm, R/d) = pm/d
  const uint32_t x = redc((uint64_t)d, q, qinv);
  return mont_mul(pm, narrow ? inv_mod_narrow(x, q, qinv) : inv_mod(x, q, qinv), q, qinv);
}

// The same update for K pairs that share the modulus q (slot s uses pivot (p[s], b[s]);
// slots outside `mask` are left alone).  The K inverses are all mod q, so Montgomery's
// trick replaces them by one: with x_s = d_s and prefix products P_s = x_0..x_s R^-s,
// Z = R P_{K-1}^{-1} = R^K (x_0..x_{K-1})^{-1}; walking back, mont_mul(Z, P_{s-1}) = R / x_s
// and Z <- mont_mul(Z, x_s).  Slots that need no inverse contribute R mod q (the
// Montgomery one).  Then t'_s = mont_mul(pm_s, R / x_s) = pm_s / d_s.
template <int K>
__device__ __forceinline__ void t_update_k(uint32_t (&t)[K], const ModConst& c, const uint32_t (&p)[K],
                                           const int32_t (&b)[K], uint32_t mask)
{
  const uint32_t q = c.q, qinv = c.qinv, r1 = c.r1;
  uint32_t x[K];
  uint32_t need = 0;
#pragma unroll
  for (int s = 0; s < K; ++s) {
    x[s] = r1;
    if (!((mask >> s) & 1u)) continue;
    const uint32_t ts = t[s];
    if (ts >= T_MARK) { t[s] = (ts == T_INF) ? 0u : ts; continue; }
    if (q == p[s]) { t[s] = T_RETIRED; continue; }
    const uint32_t d = mod_sub(ts, from_signed(b[s], q), q);
    if (d == 0u) { t[s] = T_INF; continue; }
    x[s] = d;
    need |= 1u << s;
  }
  if (!need) return;
  // one slot needing an inverse (common where the slots' live moduli differ): no batch
  const bool one = (need & (need - 1u)) == 0u;
  const int s1 = __ffs((int)need) - 1;
  uint32_t P[K];
  P[0] = x[0];
  if (!one) {
#pragma unroll
    for (int s = 1; s < K; ++s) P[s] = mont_mul(P[s - 1], x[s], q, qinv);
  }
  const uint32_t xin = one ? pick<K>(x, s1) : P[K - 1];
  uint32_t Z = mont_mul(inv_mod(xin, q, qinv), c.r2, q, qinv);   // times R
  if (one) {
    const uint32_t ps = pick<K>(p, s1);
    put<K>(t, s1, mont_mul(ps > q ? ps - q : ps, Z, q, qinv));
    return;
  }
#pragma unroll
  for (int s = K - 1; s >= 1; --s) {
    const uint32_t y = mont_mul(Z, P[s - 1], q, qinv);
    Z = mont_mul(Z, x[s], q, qinv);
    if ((need >> s) & 1u) t[s] = mont_mul(p[s] > q ? p[s] - q : p[s], y, q, qinv);
  }
  if (need & 1u) t[0] = mont_mul(p[0] > q ? p[0] - q : p[0], Z, q, qinv);
}

// Moduli below 2^30 (widths up to 30 bits): 4q < R, so the REDC of a product of two
// operands below 2q is below 2q again without the final subtraction ((T + m q)/R < T/R + q
// and T < 4q^2 < qR), and every sum fits 32 bits.  Values kept "lazy" in [0, 2q) only
// where no comparison, key or inverse reads them.
__device__ __forceinline__ uint32_t mont_mul_lazy(uint32_t a, uint32_t b, uint32_t q, uint32_t qinv)
{
  const uint64_t T = (uint64_t)a * b;
  const uint32_t lo = (uint32_t)T, hi = (uint32_t)(T >> 32);
  return hi + __umulhi(lo * qinv, q) + (lo != 0u);      // < 2q < 2^31
}

// [0, 2q) -> [0, q): x - q wraps to a large value when x < q.
__device__ __forceinline__ uint32_t mod_canon(uint32_t x, uint32_t q)
{
  return min(x, x - q);
}

// t_update_k for moduli below 2^30: the prefix products, the scaled inverse and the walk
// back stay lazy; the inverse's input and the new states are canonical.  Every modulus of a
// width-L table is an L-bit prime, so a pivot p < 2^L <= 2q enters the products as it is,
// and |b| <= p / 2 < q puts t - b in (-q, 2q): one conditional add of q makes it a lazy
// value in [0, 2q), which is 0 mod q exactly at 0 and q.
template <int K>
__device__ __forceinline__ void t_update_k_narrow(uint32_t (&t)[K], const ModConst& c, const uint32_t (&p)[K],
                                                  const int32_t (&b)[K], uint32_t mask)
{
  const uint32_t q = c.q, qinv = c.qinv, r1 = c.r1;
  uint32_t x[K];
  uint32_t need = 0;
#pragma unroll
  for (int s = 0; s < K; ++s) {
    x[s] = r1;
    if (!((mask >> s) & 1u)) continue;
    const uint32_t ts = t[s];
    if (ts >= T_MARK) { t[s] = (ts == T_INF) ? 0u : ts; continue; }
    if (q == p[s]) { t[s] = T_RETIRED; continue; }
    const uint32_t dr = ts - (uint32_t)b[s];
    const uint32_t d = min(dr, dr + q);               // dr < 0 wraps above 2^31; dr + q < 3q
    if (d == 0u || d == q) { t[s] = T_INF; continue; }
    x[s] = d;
    need |= 1u << s;
  }
  if (!need) return;
  // one slot needing an inverse (common where the slots' live moduli differ): no batch
  const bool one = (need & (need - 1u)) == 0u;
  const int s1 = __ffs((int)need) - 1;
  uint32_t P[K];
  P[0] = x[0];
  if (!one) {
#pragma unroll
    for (int s = 1; s < K; ++s) P[s] = mont_mul_lazy(P[s - 1], x[s], q, qinv);
  }
  const uint32_t xin = one ? pick<K>(x, s1) : P[K - 1];
  uint32_t Z = mont_mul_lazy(inv_mod_narrow(mod_canon(xin, q), q, qinv), c.r2, q, qinv);   // times R
  if (one) {
    put<K>(t, s1, mod_canon(mont_mul_lazy(pick<K>(p, s1), Z, q, qinv), q));
    return;
  }
#pragma unroll
  for (int s = K - 1; s >= 1; --s) {
    const uint32_t y = mont_mul_lazy(Z, P[s - 1], q, qinv);
    Z = mont_mul_lazy(Z, x[s], q, qinv);
    if ((need >> s) & 1u) t[s] = mod_canon(mont_mul_lazy(p[s], y, q, qinv), q);
  }
  if (need & 1u) t[0] = mod_canon(mont_mul_lazy(p[0], Z, q, qinv), q);
}

// Size bounds of the reduction loop, for certifying its result: lu >= log2|u_i| and
// lv >= log2|v_i| in fixed point (BOUND_ONE = 1 bit), stepped by
// |v_{i+1}| <= (|u_i| + |b| |v_i|) / p.  Integer arithmetic except for the logarithms
// (log2f, exp2f: within a few ulp, at most 2^-18 bits here), each rounded outward by
// BOUND_SLACK = 2^-17 bits, so the bounds stay upper bounds.
constexpr int BOUND_FRAC = 24;
constexpr long long BOUND_ONE = 1ll << BOUND_FRAC;
constexpr long long BOUND_SLACK = 1ll << (BOUND_FRAC - 17);

__device__ __forceinline__ long long bound_log2(float x)
{
  return (long long)(log2f(x) * (float)BOUND_ONE);
}

// Bit length of the operand limbs (an upper bound of log2 |x|) in bound units.
__device__ __forceinline__ long long bound_init(const uint32_t* limbs, uint32_t len)
{
  return (long long)(((int)len - 1) * 32 + (32 - __clz(limbs[len - 1]))) << BOUND_FRAC;
}

__device__ __forceinline__ void bound_step(long long& lu, long long& lv, uint32_t p, int32_t b)
{
  const uint32_t ab = b < 0 ? 0u - (uint32_t)b : (uint32_t)b;
  long long s = lu;                                 // log2(|u| + |b| |v|) <= s
  if (ab != 0u) {
    const long long y = lv + bound_log2((float)ab) + BOUND_SLACK;
    const long long m = y > lu ? y : lu, d = y > lu ? y - lu : lu - y;
    s = m + BOUND_SLACK;                            // log2(1 + 2^-d) < 2^-17 for d >= 40
    if (d < 40 * BOUND_ONE) s += bound_log2(1.0f + exp2f(-(float)d * (1.0f / (float)BOUND_ONE)));
  }
  lu = lv;
  lv = s - bound_log2((float)p) + BOUND_SLACK;
}

// Certified iff the surviving moduli (each > 2^(L-1)) multiply to more than |v| (so v = 0)
// and more than 2|u| (so the symmetric digits are exact).
__device__ __forceinline__ bool bound_certified(int remaining, int L, long long lu, long long lv)
{
  const long long cap = (long long)remaining * (L - 1) * BOUND_ONE;
  return cap > lu + 2 * BOUND_ONE && cap > lv + BOUND_ONE;
}

// Initial state t = u/v mod q from the residues.
__device__ __forceinline__ uint32_t t_init(uint32_t u, uint32_t v, uint32_t q, uint32_t qinv)
{
  if (v == 0u) return (u == 0u) ? T_DEGEN : T_INF;
  return mont_mul(u, inv_mod(redc((uint64_t)v, q, qinv), q, qinv), q, qinv);
}

}  // namespace mgcd

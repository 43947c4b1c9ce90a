/*  modgcd_oracle.c -- CPU restatement of the reference modular-GCD path.

    TEST INFRASTRUCTURE ONLY.  This file is the oracle: tests, the smoke check and the
    CPU-baseline leg of the benchmark load it to verify the CUDA path.  The product never
    links or calls it.

    It restates, in plain C and with the straightforward per-modulus arithmetic (exact
    (u_q, v_q) residues, one extended-Euclid inverse per division), the algorithm of the
    reference (mountunion/ModGCD-OneGPU):

      - moduli table          createModuli.cpp:104-179   (descending L-bit primes that pass
                                                          the Cavagnino-Werbrouck DBM_a test)
      - moduli count N_Q      GmpCudaDevice-gcd.cu:49-55
      - residues (MGCD2)      GmpCudaDevice-getGcdKernel.cu:294-324, 357-361
      - reduction (MGCD3)     GmpCudaDevice-getGcdKernel.cu:363-402, selection key :146-220
      - recovery (MGCD4)      GmpCudaDevice-getGcdKernel.cu:404-443, selection :54-116
      - result to integer     GmpCudaDevice-gcd.cu:116-129

    Every choice the reference makes deterministically (which modulus is retired, which
    digit is emitted next, when the run reports "ran out of moduli") is reproduced, so the
    (p, b) sequence and the digit list can be compared element by element with the GPU.

    Parity pin: the final integer is checked against GMP mpz_gcd (the reference's own
    oracle, testmodgcd.cpp:441) and Python's exact gcd on the committed golden inputs, which
    were generated by the reference's own test driver; the moduli table is checked against
    the output of the reference's createModuli.
*/
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

typedef struct { uint32_t modulus; int32_t value; } orc_pair_t;   /* GmpCuda.h:112 */

enum {
  ORC_OK           = 0,
  ORC_ERR_REDUX    = 1,   /* "Ran out of moduli in the reduction loop."  GmpCudaDevice-gcd.cu:107 */
  ORC_ERR_RECOVERY = 2,   /* "Ran out of moduli in the recovery loop."   GmpCudaDevice-gcd.cu:108 */
  ORC_ERR_ARG      = 3,
  ORC_ERR_CAPACITY = 4,   /* caller's output buffer too small */
  ORC_ERR_NOMEM    = 5
};

#define ORC_MOD_INFINITY INT32_MIN   /* GmpCudaDevice-getGcdKernel.cu:46 */

/* ------------------------------------------------------------------ moduli table ---- */

/* Cavagnino-Werbrouck DBM_a usability test with W = 64 (createModuli.cpp:143-164):
   J = floor(2^(W+L-1)/D) + 1, Ncr = ceil(J / (D*J - 2^(W+L-1))) * D - 1, usable iff
   bitlen(Ncr) > W. */
static int cw_usable(uint32_t D, int L)
{
  const int W = 64;
  unsigned __int128 FC = (unsigned __int128)1 << (W + L - 1);
  unsigned __int128 J = FC / D + 1;
  unsigned __int128 DJ = (unsigned __int128)D * J - FC;
  unsigned __int128 Qcr = (J + DJ - 1) / DJ;
  unsigned __int128 Ncr = Qcr * D - 1;
  return (Ncr >> W) != 0;
}

/* Fill out[0..count) with the largest usable L-bit primes in descending order -- the same
   list, in the same order, that createModuli prints (createModuli.cpp:150-167).  A
   segmented sieve over the top of [2^(L-1), 2^L) replaces the reference's full 2^(L-2)-byte
   sieve.  Returns the number written (< count if the range runs out). */
size_t orc_gen_moduli(int L, uint32_t *out, size_t count)
{
  if (L < 3 || L > 32 || !out)
    return 0;
  const uint64_t top = (uint64_t)1 << L, bottom = (uint64_t)1 << (L - 1);
  uint32_t lim = (uint32_t)sqrt((double)top) + 2;
  char *small = calloc(lim + 1, 1);
  uint32_t *primes = malloc(sizeof(uint32_t) * (lim / 2 + 16));
  if (!small || !primes) { free(small); free(primes); return 0; }
  size_t np = 0;
  for (uint32_t i = 3; i <= lim; i += 2)
    if (!small[i]) {
      primes[np++] = i;
      for (uint64_t j = (uint64_t)i * i; j <= lim; j += 2 * i) small[j] = 1;
    }
  free(small);

  const uint64_t SEG = (uint64_t)1 << 20;   /* odd numbers per segment */
  char *seg = malloc(SEG);
  if (!seg) { free(primes); return 0; }
  size_t got = 0;
  uint64_t hi = top - 1;                    /* largest odd candidate of this segment */
  while (got < count && hi > bottom) {
    /* segment holds odd x in (hi - 2*SEG, hi]; index i <-> x = hi - 2*i */
    uint64_t n = SEG;
    if (hi - bottom < 2 * n) n = (hi - bottom + 1) / 2;
    memset(seg, 0, n);
    uint64_t lo = hi - 2 * (n - 1);
    for (size_t k = 0; k < np; k++) {
      uint64_t p = primes[k];
      if (p * p > hi) break;
      /* largest odd multiple of p that is <= hi */
      uint64_t m = hi - hi % p;
      if ((m & 1) == 0) { if (m < p) continue; m -= p; }
      for (; m >= lo && m >= p * p; m -= 2 * p) {
        seg[(hi - m) / 2] = 1;
        if (m < 2 * p) break;
      }
    }
    for (uint64_t i = 0; i < n && got < count; i++) {
      uint64_t x = hi - 2 * i;
      if (x <= bottom) break;
      if (seg[i]) continue;
      if (cw_usable((uint32_t)x, L)) out[got++] = (uint32_t)x;
    }
    hi = lo - 2;
  }
  free(seg);
  free(primes);
  return got;
}

/* Moduli count for an operand of numBits bits (GmpCudaDevice-gcd.cu:49-55), evaluated in
   float exactly as the reference does: roundUp(ceil(C_L*bits/logf(bits)), 256) with
   C_L = 1.6 - 0.015*L.  bits < 2 (where the reference divides by logf(1) = 0) gives 256. */
int orc_num_moduli_needed(size_t numBits, int L)
{
  const float C_L = (float)(1.6 - 0.015 * L);
  if (numBits < 2) return 256;
  float x = ceilf(C_L * (float)numBits / logf((float)numBits));
  int n = (int)x;
  return ((n - 1) / 256 + 1) * 256;
}

/* ------------------------------------------------------------- modular helpers ---- */

static inline uint32_t mulmod(uint32_t a, uint32_t b, uint32_t m) { return (uint32_t)((uint64_t)a * b % m); }
static inline uint32_t submod(uint32_t a, uint32_t b, uint32_t m) { return a >= b ? a - b : a + (m - b); }

/* 1/v mod m for 0 < v < m, gcd(v, m) = 1 (the value modInv.h:137-188 computes). */
static uint32_t invmod(uint32_t v, uint32_t m)
{
  int64_t r0 = m, r1 = v, s0 = 0, s1 = 1;
  while (r1 != 0) {
    int64_t q = r0 / r1, t;
    t = r0 - q * r1; r0 = r1; r1 = t;
    t = s0 - q * s1; s0 = s1; s1 = t;
  }
  if (s0 < 0) s0 += m;
  return (uint32_t)s0;
}

/* toSigned / fromSigned (GmpCudaDevice-getGcdKernel.cu:264-281): symmetric residue with
   the reference's boundary: x >= m/2 maps to x - m. */
static inline int32_t to_signed(uint32_t x, uint32_t m) { return (x >= m / 2) ? (int32_t)(x - m) : (int32_t)x; }
static inline uint32_t from_signed(int32_t x, uint32_t m) { return (x < 0) ? (uint32_t)(x + (int64_t)m) : (uint32_t)x; }

/* Selection key of postMinPair (GmpCudaDevice-getGcdKernel.cu:152-154):
   (|value| << 32) | (modulus - (value >= 0)); MOD_INFINITY keeps 0x80000000 as |value|. */
static inline uint64_t min_key(int32_t value, uint32_t modulus)
{
  uint32_t a = (value == ORC_MOD_INFINITY) ? 0x80000000u : (uint32_t)(value < 0 ? -value : value);
  return ((uint64_t)a << 32) | (uint32_t)(modulus - (value >= 0));
}

/* Inverse of min_key (collectMinPair, GmpCudaDevice-getGcdKernel.cu:214-219). */
static inline orc_pair_t key_pair(uint64_t x)
{
  orc_pair_t p;
  p.modulus = (uint32_t)x;
  p.value = (int32_t)(uint32_t)(x >> 32);
  if (p.modulus & 1) p.value = (int32_t)(0u - (uint32_t)p.value);
  p.modulus |= 1;
  return p;
}

/* x mod q for a little-endian array of 32-bit limbs (modMP, GmpCudaDevice-getGcdKernel.cu:294-324). */
uint32_t orc_residue(const uint32_t *x, size_t n, uint32_t q)
{
  uint64_t r = 0;
  for (size_t i = n; i-- != 0;)
    r = ((r << 32) | x[i]) % q;
  return (uint32_t)r;
}

void orc_residues(const uint32_t *x, size_t n, const uint32_t *moduli, size_t nq, uint32_t *out)
{
  for (size_t j = 0; j < nq; j++) out[j] = orc_residue(x, n, moduli[j]);
}

/* --------------------------------------------------------------- the algorithm ---- */

/*  Modular gcd of u (uSz limbs) and v (vSz limbs), u >= v > 0, with the first nq entries of
    moduli[], following kernel<QRTYPE> (GmpCudaDevice-getGcdKernel.cu:342-444).

    Outputs:
      digits[0..*ndigits)  the signed mixed-radix digits (modulus, value) in emission order,
                           i.e. the pair_t records the reference kernel writes at buf+1.
      trace[0..*ntrace)    optional: the (p, b) pair collected by each reduction iteration,
                           the terminating (MOD_INFINITY) pair included.
      *iters               number of reduction iterations (moduli retired by MGCD3).
    Returns ORC_OK, ORC_ERR_REDUX or ORC_ERR_RECOVERY with the reference's rules. */
int orc_modgcd(const uint32_t *u, size_t uSz, const uint32_t *v, size_t vSz, int L,
               const uint32_t *moduli, size_t nq,
               orc_pair_t *digits, size_t digits_cap, size_t *ndigits,
               orc_pair_t *trace, size_t trace_cap, size_t *ntrace, size_t *iters)
{
  if (!moduli || nq == 0 || !digits || !ndigits) return ORC_ERR_ARG;
  uint32_t *uq = malloc(nq * 4), *vq = malloc(nq * 4);
  int32_t *val = malloc(nq * 4);
  char *active = malloc(nq);
  if (!uq || !vq || !val || !active) { free(uq); free(vq); free(val); free(active); return ORC_ERR_NOMEM; }
  int status = ORC_OK;
  size_t nt = 0, nd = 0, it = 0;

  long remaining = (long)nq;                      /* :350 */
  long ubits = (long)(uSz + 1) * 32;              /* :351 */
  long vbits = (long)(vSz + 1) * 32;              /* :352 */

  /* MGCD2 + the initial value (:359-369) */
  for (size_t j = 0; j < nq; j++) {
    uint32_t q = moduli[j];
    uq[j] = orc_residue(u, uSz, q);
    vq[j] = orc_residue(v, vSz, q);
    active[j] = 1;
    val[j] = (vq[j] == 0) ? ORC_MOD_INFINITY : to_signed(mulmod(uq[j], invmod(vq[j], q), q), q);
  }

#define COLLECT_MIN(pairvar)                                              \
  do {                                                                    \
    uint64_t best = UINT64_MAX;                                           \
    for (size_t j = 0; j < nq; j++) {                                     \
      uint64_t k = min_key(val[j], moduli[j]);                            \
      if (k < best) best = k;                                             \
    }                                                                     \
    pairvar = key_pair(best);                                             \
  } while (0)

  orc_pair_t pair;
  COLLECT_MIN(pair);
  if (trace && nt < trace_cap) trace[nt] = pair;
  nt++;

  /* MGCD3 (:373-402) */
  do {
    for (size_t j = 0; j < nq; j++) {
      uint32_t q = moduli[j];
      if (pair.modulus == q) { active[j] = 0; val[j] = ORC_MOD_INFINITY; }
      if (active[j]) {
        uint32_t p = pair.modulus;
        if (p > q) p -= q;
        uint32_t d = submod(uq[j], mulmod(from_signed(pair.value, q), vq[j], q), q);
        uint32_t tq = mulmod(d, invmod(p, q), q);
        val[j] = (tq == 0) ? ORC_MOD_INFINITY : to_signed(mulmod(vq[j], invmod(tq, q), q), q);
        uq[j] = vq[j];
        vq[j] = tq;
      }
    }
    it++;
    remaining -= 1;
    {
      uint32_t absb = (pair.value < 0) ? 0u - (uint32_t)pair.value : (uint32_t)pair.value;
      long tbits = ubits - (L - 1) + __builtin_ffs((int)absb);     /* :391 */
      ubits = vbits;
      vbits = tbits;
    }
    if (remaining * (L - 2) <= ubits) { status = ORC_ERR_REDUX; goto done; }   /* :393-399 */
    COLLECT_MIN(pair);
    if (trace && nt < trace_cap) trace[nt] = pair;
    nt++;
  } while (pair.value != ORC_MOD_INFINITY);

  /* MGCD4 (:406-433): the next digit comes from the lowest-indexed modulus whose value is
     nonzero (findAnyNonZero's ballot order over threads, warps, then blocks); when every
     value is zero the pair of modulus 0 is taken, which ends the loop. */
#define COLLECT_ANY(pairvar)                                              \
  do {                                                                    \
    size_t w = 0;                                                         \
    for (size_t j = 0; j < nq; j++) if (val[j] != 0) { w = j; break; }    \
    pairvar.modulus = moduli[w];                                          \
    pairvar.value = val[w];                                               \
  } while (0)

  for (size_t j = 0; j < nq; j++) val[j] = active[j] ? to_signed(uq[j], moduli[j]) : 0;
  COLLECT_ANY(pair);
  do {
    for (size_t j = 0; j < nq; j++) {
      uint32_t q = moduli[j];
      if (pair.modulus == q) { active[j] = 0; val[j] = 0; }
      if (active[j]) {
        uint32_t p = pair.modulus;
        if (p > q) p -= q;
        uq[j] = mulmod(submod(uq[j], from_signed(pair.value, q), q), invmod(p, q), q);
        val[j] = to_signed(uq[j], q);
      }
    }
    if (nd < digits_cap) digits[nd] = pair; else status = ORC_ERR_CAPACITY;
    nd++;
    remaining -= 1;
    if (remaining <= 0) break;
    COLLECT_ANY(pair);
  } while (pair.value != 0);
  if (status == ORC_OK && pair.value != 0) status = ORC_ERR_RECOVERY;   /* :440-441 */

done:
  *ndigits = nd;
  if (ntrace) *ntrace = nt;
  if (iters) *iters = it;
  free(uq); free(vq); free(val); free(active);
  return status;
#undef COLLECT_MIN
#undef COLLECT_ANY
}

/* ------------------------------------------------- mixed radix to binary (Horner) ---- */

/*  |g| from the signed mixed-radix digits (GmpCudaDevice-gcd.cu:116-129):
    g = d[n-1]; for i = n-2 .. 0: g = g * d[i].modulus + d[i].value;  result |g|.
    out receives the magnitude as little-endian 32-bit limbs; returns the limb count
    (0 for g = 0), or -1 when out_cap is too small. */
long orc_mixed_radix_to_limbs(const orc_pair_t *d, size_t n, uint32_t *out, size_t out_cap)
{
  if (n == 0) return 0;
  size_t len = 0;
  int neg = 0;                                  /* sign of g; magnitude in out[0..len) */
  int32_t top = d[n - 1].value;
  if (top != 0) {
    if (out_cap < 1) return -1;
    out[0] = (top < 0) ? 0u - (uint32_t)top : (uint32_t)top;
    neg = top < 0;
    len = 1;
  }
  for (size_t i = n - 1; i-- != 0;) {
    uint32_t m = d[i].modulus;
    uint64_t carry = 0;
    for (size_t k = 0; k < len; k++) {
      uint64_t t = (uint64_t)out[k] * m + carry;
      out[k] = (uint32_t)t;
      carry = t >> 32;
    }
    if (carry) { if (len >= out_cap) return -1; out[len++] = (uint32_t)carry; }
    int32_t dv = d[i].value;
    if (dv == 0) continue;
    uint32_t a = (dv < 0) ? 0u - (uint32_t)dv : (uint32_t)dv;
    int dneg = dv < 0;
    if (len == 0) { if (out_cap < 1) return -1; out[0] = a; len = 1; neg = dneg; continue; }
    if (dneg == neg) {                          /* |g| += a */
      uint64_t c = a;
      for (size_t k = 0; k < len && c; k++) { uint64_t t = (uint64_t)out[k] + c; out[k] = (uint32_t)t; c = t >> 32; }
      if (c) { if (len >= out_cap) return -1; out[len++] = (uint32_t)c; }
    } else if (len > 1 || out[0] >= a) {        /* |g| -= a, sign kept */
      uint64_t b = a;
      for (size_t k = 0; k < len && b; k++) {
        uint64_t cur = out[k];
        if (cur >= b) { out[k] = (uint32_t)(cur - b); b = 0; }
        else { out[k] = (uint32_t)(cur + ((uint64_t)1 << 32) - b); b = 1; }
      }
      while (len && out[len - 1] == 0) len--;
    } else {                                    /* |g| < a: sign flips */
      out[0] = a - out[0];
      neg = dneg;
      if (out[0] == 0) len = 0;
    }
  }
  return (long)len;
}

/* ------------------------------------------------ moduli grown on demand (batches) ---- */

/*  The reduction loop with moduli grown on demand, as this project's batched K-slot kernel
    runs it (a policy of this project; the reference's count is fixed per call,
    GmpCudaDevice-gcd.cu:49-55).  The steps of the loop and of the recovery are the
    reference's (orc_modgcd above); what differs:

      - the pair starts with the first nq0 moduli and may take the next ones, up to nq_cap,
        step = ceil(nq_cap * step_permille / 1000) rounded up to a multiple of 32 (>= 32)
        at a time;
      - when a pivot's bookkeeping finds the loop out of moduli (the reference's check,
        GmpCudaDevice-getGcdKernel.cu:393-399), or fewer than GROW_LOW surviving moduli,
        and nq < nq_cap, the set grows before that pivot is applied; out of moduli with
        nq = nq_cap, the run fails with ORC_ERR_REDUX;
      - when the loop ends (every value infinite) with a result the surviving moduli less
        one cannot certify (their product, each modulus counted as 2^(L-1), must exceed
        2|u| and |v| by the size bounds below; the one to spare lets the recovery reach its
        all-zero round), the set grows and the next pivot is chosen over it; a result the
        survivors cannot certify at nq = nq_cap is ORC_ERR_UNCERTIFIED (the host reruns
        such a pair with the reference's count, orc_modgcd);
      - a modulus that joins takes the exact residues (u_i, v_i) mod q of the current pair:
        the operands' residues with every applied pivot replayed, (u, v) <- (v, (u - b v)/p).

    Size bounds (the kernel's certification): lu >= log2|u_i|, lv >= log2|v_i| in fixed point
    with 24 fraction bits, from the operands' bit lengths, stepped per pivot by
    |v'| <= (|u| + |b||v|)/p with log2f/exp2f rounded outward by 2^-17 bits.

    *nq_final receives the moduli count at the end; other outputs as orc_modgcd's. */
enum { ORC_ERR_UNCERTIFIED = 6 };
#define GROW_LOW 64

#define BOUND_FRAC 24
#define BOUND_ONE (1ll << BOUND_FRAC)
#define BOUND_SLACK (1ll << (BOUND_FRAC - 17))

static long long bound_log2(float x) { return (long long)(log2f(x) * (float)BOUND_ONE); }

static long long bound_init(const uint32_t *limbs, size_t len)
{
  return (long long)((long long)(len - 1) * 32 + (32 - __builtin_clz(limbs[len - 1]))) << BOUND_FRAC;
}

static void bound_step(long long *lu, long long *lv, uint32_t p, int32_t b)
{
  uint32_t ab = b < 0 ? 0u - (uint32_t)b : (uint32_t)b;
  long long s = *lu;
  if (ab != 0u) {
    long long y = *lv + bound_log2((float)ab) + BOUND_SLACK;
    long long m = y > *lu ? y : *lu, d = y > *lu ? y - *lu : *lu - y;
    s = m + BOUND_SLACK;
    if (d < 40 * BOUND_ONE) s += bound_log2(1.0f + exp2f(-(float)d * (1.0f / (float)BOUND_ONE)));
  }
  *lu = *lv;
  *lv = s - bound_log2((float)p) + BOUND_SLACK;
}

static int bound_certified(long remaining, int L, long long lu, long long lv)
{
  long long cap = (long long)remaining * (L - 1) * BOUND_ONE;
  return cap > lu + 2 * BOUND_ONE && cap > lv + BOUND_ONE;
}

static uint32_t grow_step(size_t cap, unsigned permille)
{
  uint64_t n = ((uint64_t)cap * permille + 999) / 1000;
  return n < 32 ? 32u : (uint32_t)((n + 31) & ~(uint64_t)31);
}

int orc_modgcd_grow(const uint32_t *u, size_t uSz, const uint32_t *v, size_t vSz, int L,
                    const uint32_t *moduli, size_t nq0, size_t nq_cap, unsigned step_permille,
                    orc_pair_t *digits, size_t digits_cap, size_t *ndigits,
                    orc_pair_t *trace, size_t trace_cap, size_t *ntrace, size_t *iters, size_t *nq_final)
{
  if (!moduli || nq0 == 0 || nq_cap < nq0 || !digits || !ndigits) return ORC_ERR_ARG;
  uint32_t *uq = malloc(nq_cap * 4), *vq = malloc(nq_cap * 4);
  int32_t *val = malloc(nq_cap * 4);
  char *active = malloc(nq_cap);
  orc_pair_t *hist = malloc(sizeof(orc_pair_t) * (nq_cap + 1));
  if (!uq || !vq || !val || !active || !hist) {
    free(uq); free(vq); free(val); free(active); free(hist);
    return ORC_ERR_NOMEM;
  }
  int status = ORC_OK;
  size_t nq = nq0, nt = 0, nd = 0, it = 0;
  long remaining = (long)nq;
  long ubits = (long)(uSz + 1) * 32, vbits = (long)(vSz + 1) * 32;
  long long lu = bound_init(u, uSz), lv = bound_init(v, vSz);

  /* residues of moduli [from, to), with the first nrep pivots of hist applied */
#define JOIN(from, to, nrep)                                                              \
  do {                                                                                  \
    for (size_t j = (from); j < (to); j++) {                                            \
      uint32_t q = moduli[j];                                                           \
      uint32_t a = orc_residue(u, uSz, q), c = orc_residue(v, vSz, q);                  \
      for (size_t h = 0; h < (nrep); h++) {                                             \
        uint32_t p = hist[h].modulus;                                                   \
        if (p > q) p -= q;                                                              \
        uint32_t t = mulmod(submod(a, mulmod(from_signed(hist[h].value, q), c, q), q), invmod(p, q), q); \
        a = c; c = t;                                                                   \
      }                                                                                 \
      uq[j] = a; vq[j] = c; active[j] = 1;                                              \
      val[j] = (c == 0) ? ORC_MOD_INFINITY : to_signed(mulmod(a, invmod(c, q), q), q);  \
    }                                                                                   \
  } while (0)
#define COLLECT_MIN(pairvar)                                                              \
  do {                                                                                  \
    uint64_t best = UINT64_MAX;                                                         \
    for (size_t j = 0; j < nq; j++) {                                                   \
      uint64_t k = min_key(val[j], moduli[j]);                                          \
      if (k < best) best = k;                                                           \
    }                                                                                   \
    pairvar = key_pair(best);                                                           \
  } while (0)

  JOIN(0, nq, 0);
  orc_pair_t pair;
  COLLECT_MIN(pair);
  for (;;) {
    if (pair.value == ORC_MOD_INFINITY) {               /* the loop ended */
      if (trace && nt < trace_cap) trace[nt] = pair;
      nt++;
      if (nq < nq_cap && !bound_certified(remaining - 1, L, lu, lv)) {
        size_t n1 = nq + grow_step(nq_cap, step_permille);
        if (n1 > nq_cap) n1 = nq_cap;
        JOIN(nq, n1, it);
        remaining += (long)(n1 - nq);
        nq = n1;
        COLLECT_MIN(pair);
        continue;
      }
      break;
    }
    /* the pivot's bookkeeping (GmpCudaDevice-getGcdKernel.cu:389-399) */
    if (trace && nt < trace_cap) trace[nt] = pair;
    nt++;
    hist[it] = pair;
    remaining -= 1;
    {
      uint32_t absb = (pair.value < 0) ? 0u - (uint32_t)pair.value : (uint32_t)pair.value;
      long tbits = ubits - (L - 1) + __builtin_ffs((int)absb);
      ubits = vbits;
      vbits = tbits;
    }
    if (remaining * (L - 2) <= ubits || (nq < nq_cap && remaining < GROW_LOW)) {
      if (nq >= nq_cap) { status = ORC_ERR_REDUX; it++; goto done; }
      size_t n1 = nq + grow_step(nq_cap, step_permille);
      if (n1 > nq_cap) n1 = nq_cap;
      JOIN(nq, n1, it);                                 /* before this pivot is applied */
      remaining += (long)(n1 - nq);
      nq = n1;
    }
    /* the update (GmpCudaDevice-getGcdKernel.cu:373-386) */
    for (size_t j = 0; j < nq; j++) {
      uint32_t q = moduli[j];
      if (pair.modulus == q) { active[j] = 0; val[j] = ORC_MOD_INFINITY; }
      if (active[j]) {
        uint32_t p = pair.modulus;
        if (p > q) p -= q;
        uint32_t d = submod(uq[j], mulmod(from_signed(pair.value, q), vq[j], q), q);
        uint32_t tq = mulmod(d, invmod(p, q), q);
        val[j] = (tq == 0) ? ORC_MOD_INFINITY : to_signed(mulmod(vq[j], invmod(tq, q), q), q);
        uq[j] = vq[j];
        vq[j] = tq;
      }
    }
    bound_step(&lu, &lv, pair.modulus, pair.value);
    it++;
    COLLECT_MIN(pair);
  }
  if (!bound_certified(remaining, L, lu, lv)) { status = ORC_ERR_UNCERTIFIED; goto done; }

  /* MGCD4, as orc_modgcd */
#define COLLECT_ANY(pairvar)                                                              \
  do {                                                                                  \
    size_t w = 0;                                                                       \
    for (size_t j = 0; j < nq; j++) if (val[j] != 0) { w = j; break; }                  \
    pairvar.modulus = moduli[w];                                                        \
    pairvar.value = val[w];                                                             \
  } while (0)
  for (size_t j = 0; j < nq; j++) val[j] = active[j] ? to_signed(uq[j], moduli[j]) : 0;
  COLLECT_ANY(pair);
  do {
    for (size_t j = 0; j < nq; j++) {
      uint32_t q = moduli[j];
      if (pair.modulus == q) { active[j] = 0; val[j] = 0; }
      if (active[j]) {
        uint32_t p = pair.modulus;
        if (p > q) p -= q;
        uq[j] = mulmod(submod(uq[j], from_signed(pair.value, q), q), invmod(p, q), q);
        val[j] = to_signed(uq[j], q);
      }
    }
    if (nd < digits_cap) digits[nd] = pair; else status = ORC_ERR_CAPACITY;
    nd++;
    remaining -= 1;
    if (remaining <= 0) break;
    COLLECT_ANY(pair);
  } while (pair.value != 0);
  if (status == ORC_OK && pair.value != 0) status = ORC_ERR_RECOVERY;

done:
  *ndigits = nd;
  if (ntrace) *ntrace = nt;
  if (iters) *iters = it;
  if (nq_final) *nq_final = nq;
  free(uq); free(vq); free(val); free(active); free(hist);
  return status;
#undef JOIN
#undef COLLECT_MIN
#undef COLLECT_ANY
}

/*  cpu_gmp_gcd.c -- GMP mpz_gcd over a batch of pairs on the host cores.

    TEST INFRASTRUCTURE ONLY: this is the correctness oracle (GMP mpz_gcd, which the
    reference itself compares against at testmodgcd.cpp:441 and times as its CPU
    baseline in the -DNO_GPU build, Makefile:61-62) and the timed CPU baseline of the
    benchmark.  The product never links or calls it.

    Batch layout (shared with the GPU C ABI): all operand limbs live in one array of
    little-endian 32-bit words; pair i has u at limbs[u_off[i] .. u_off[i]+u_len[i]) and v
    at limbs[v_off[i] .. v_off[i]+v_len[i]).  The gcd of pair i is written as little-endian
    32-bit limbs at g[g_off[i]..] (capacity g_cap[i] words) and its length to g_len[i].

    Threads pull pair indices from a shared atomic counter, one pthread per requested core.
*/
#define _POSIX_C_SOURCE 200809L
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <time.h>
#include <gmp.h>

typedef struct {
  size_t n;
  const uint32_t *limbs;
  const uint64_t *u_off, *v_off;
  const uint32_t *u_len, *v_len;
  uint32_t *g;
  const uint64_t *g_off;
  const uint32_t *g_cap;
  uint32_t *g_len;
  mpz_t *U, *V, *G;          /* pre-imported operands, so only mpz_gcd is timed */
  volatile size_t next;
  int err;
} job_t;

static void *worker(void *arg)
{
  job_t *J = (job_t *)arg;
  for (;;) {
    size_t i = __atomic_fetch_add(&J->next, 1, __ATOMIC_RELAXED);
    if (i >= J->n) break;
    mpz_gcd(J->G[i], J->U[i], J->V[i]);
  }
  return NULL;
}

static double now_s(void)
{
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return t.tv_sec + 1e-9 * t.tv_nsec;
}

/*  Computes all gcds with nthreads threads.  *seconds receives the wall time of the
    mpz_gcd calls alone (import of the operands and export of the results excluded, as in
    testmodgcd.cpp:440-442).  Returns 0, or -1 if an output capacity is too small. */
int cpu_gmp_gcd_batch(size_t n, const uint32_t *limbs,
                      const uint64_t *u_off, const uint32_t *u_len,
                      const uint64_t *v_off, const uint32_t *v_len,
                      uint32_t *g, const uint64_t *g_off, const uint32_t *g_cap, uint32_t *g_len,
                      int nthreads, double *seconds)
{
  job_t J;
  memset(&J, 0, sizeof J);
  J.n = n; J.limbs = limbs; J.u_off = u_off; J.v_off = v_off; J.u_len = u_len; J.v_len = v_len;
  J.g = g; J.g_off = g_off; J.g_cap = g_cap; J.g_len = g_len;
  J.U = malloc(sizeof(mpz_t) * (n ? n : 1));
  J.V = malloc(sizeof(mpz_t) * (n ? n : 1));
  J.G = malloc(sizeof(mpz_t) * (n ? n : 1));
  for (size_t i = 0; i < n; i++) {
    mpz_init(J.U[i]); mpz_init(J.V[i]); mpz_init(J.G[i]);
    mpz_import(J.U[i], u_len[i], -1, 4, 0, 0, limbs + u_off[i]);
    mpz_import(J.V[i], v_len[i], -1, 4, 0, 0, limbs + v_off[i]);
  }
  if (nthreads < 1) nthreads = 1;
  pthread_t *th = malloc(sizeof(pthread_t) * nthreads);
  double t0 = now_s();
  for (int k = 0; k < nthreads; k++) pthread_create(&th[k], NULL, worker, &J);
  for (int k = 0; k < nthreads; k++) pthread_join(th[k], NULL);
  double t1 = now_s();
  if (seconds) *seconds = t1 - t0;
  int rc = 0;
  for (size_t i = 0; i < n; i++) {
    size_t cnt = 0;
    if (g) {
      size_t words = (mpz_sizeinbase(J.G[i], 2) + 31) / 32;
      if (mpz_sgn(J.G[i]) == 0) words = 0;
      if (words > g_cap[i]) { rc = -1; g_len[i] = 0; }
      else { if (words) mpz_export(g + g_off[i], &cnt, -1, 4, 0, 0, J.G[i]); g_len[i] = (uint32_t)cnt; }
    }
    mpz_clear(J.U[i]); mpz_clear(J.V[i]); mpz_clear(J.G[i]);
  }
  free(th); free(J.U); free(J.V); free(J.G);
  return rc;
}

const char *cpu_gmp_version(void) { return gmp_version; }

/*  modgcd.h -- C ABI of the GB300 modular integer GCD library (libmodgcd.so).

    Weber's modular integer GCD on one GPU.  Operands and results cross this boundary as
    little-endian arrays of 32-bit limbs (the layout the reference stages with
    mpz_export(buf, &n, -1, sizeof(uint32_t), 0, 0, x), GmpCudaDevice-gcd.cu:71-73), plain
    pointers and sizes, and every entry point returns a status code (no exceptions cross
    the ABI).  The C++ drop-in GmpCuda::GmpCudaDevice (GmpCuda.h) is implemented on top of
    these calls.

    Reference interfaces replaced (paths within mountunion/ModGCD-OneGPU):
      mgcd_device_count / mgcd_set_device   GmpCudaDevice::setDevice      GmpCudaDevice.cu:96-103
      mgcd_create / mgcd_destroy            GmpCudaDevice(), ~GmpCudaDevice  GmpCudaDevice.cu:107-144
      mgcd_max_grid_size                    GmpCudaDevice::getMaxGridSize GmpCuda.h:118
      mgcd_moduli_needed                    numModuliNeededFor           GmpCudaDevice-gcd.cu:49-55
      mgcd_gcd_digits                       GmpCudaDevice::gcd up to the kernel's pair_t result
                                                                          GmpCudaDevice-gcd.cu:59-114
      mgcd_gcd                              GmpCudaDevice::gcd            GmpCudaDevice-gcd.cu:59-132
      mgcd_moduli / mgcd_gen_moduli         GmpCuda::moduli[] / createModuli GmpCuda.h:126,
                                                                          createModuli.cpp:104-179
      mgcd_batch_* , mgcd_serve_*           no counterpart (batching and serving are new)
*/
#ifndef MODGCD_H
#define MODGCD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference's std::runtime_error messages map to these
   (GmpCudaDevice-gcd.cu:78, 82, 107-109); mgcd_status_string() returns the same text. */
#define MGCD_OK                    0
#define MGCD_ERR_INVALID_ARG       1
#define MGCD_ERR_NO_DEVICE         2   /* "Invalid device number." */
#define MGCD_ERR_CUDA              3
#define MGCD_ERR_NOT_ENOUGH_MODULI 4   /* "Not enough moduli available for given input." */
#define MGCD_ERR_GRID              5   /* "Cannot allocate enough threads to support computation." */
#define MGCD_ERR_REDUX             6   /* "Ran out of moduli in the reduction loop." */
#define MGCD_ERR_RECOVERY          7   /* "Ran out of moduli in the recovery loop." */
#define MGCD_ERR_KERNEL            8   /* "Unknown error in the gcd kernel." */
#define MGCD_ERR_TIMEOUT           9   /* a bounded device-side wait expired */
#define MGCD_ERR_CAPACITY         10   /* caller's output buffer is too small, or a batch needs
                                          more than 2^32 - 1 digit slots (split it) */
#define MGCD_ERR_BUDGET           11   /* serving: request larger than the admission budget */
#define MGCD_ERR_BUSY             12   /* serving: queue full, retry later */

/* One signed mixed-radix digit: the reference's pair_t (GmpCuda.h:112). */
typedef struct mgcd_pair {
  uint32_t modulus;
  int32_t value;
} mgcd_pair;

typedef struct mgcd_context mgcd_context;

const char *mgcd_status_string(int status);

/* Number of CUDA devices (0 when none is usable). */
int mgcd_device_count(int *count);

/* Checks devNo like GmpCudaDevice::setDevice and makes it current for this host thread.
   MGCD_ERR_NO_DEVICE for an invalid number. */
int mgcd_set_device(int devNo);

/* Creates a context on device `device` (-1: the current device) for modulus width L
   (22, 27 or 32; the reference fixes L = 32 at GmpCuda.h:121).  Builds the L-bit moduli
   table (createModuli order) and uploads it with its Montgomery constants. */
int mgcd_create(int device, int L, mgcd_context **ctx);
int mgcd_destroy(mgcd_context *ctx);

/* Largest number of 256-modulus groups one pair may use (the reference's grid cap). */
int mgcd_max_grid_size(const mgcd_context *ctx, int *out);
/* Number of moduli in the context's table (the reference's NUM_MODULI). */
int mgcd_num_moduli(const mgcd_context *ctx, size_t *out);
/* Copies the first n moduli of the context's table. */
int mgcd_moduli(const mgcd_context *ctx, uint32_t *out, size_t n);
/* Moduli the reference would use for an operand of `bits` bits at width L. */
int mgcd_moduli_needed(int L, size_t bits);
/* The first `count` usable L-bit primes in descending order, as createModuli prints
   them.  Returns the number written. */
size_t mgcd_gen_moduli(int L, uint32_t *out, size_t count);

/* gcd of one pair, as the signed mixed-radix digits the reference kernel returns
   (buf[1..count) of GmpCudaDevice-gcd.cu:113-116): |g| = d[n-1], then g = g*d[i].modulus +
   d[i].value for i = n-2..0.  u and v need not be ordered; both must be nonzero.
   *count receives the digit count (<= cap). */
int mgcd_gcd_digits(mgcd_context *ctx, const uint32_t *u, size_t uSz, const uint32_t *v, size_t vSz,
                    mgcd_pair *digits, size_t cap, size_t *count);

/* gcd of one pair as little-endian 32-bit limbs: g = gcd(u, v) >= 0 (gcd(x, 0) = x,
   gcd(0, 0) = 0).  g_cap >= min(uSz, vSz) (or >= the nonzero operand's size) always
   suffices; *g_len receives the limb count (0 for g = 0). */
int mgcd_gcd(mgcd_context *ctx, const uint32_t *u, size_t uSz, const uint32_t *v, size_t vSz,
             uint32_t *g, size_t g_cap, size_t *g_len);

/* ----------------------------------------------------------------------- batches ----
   Batch layout: all operand limbs in one array; pair i has u at limbs[u_off[i] ..
   u_off[i]+u_len[i]) and v at limbs[v_off[i] .. +v_len[i]).  Results: g of pair i at
   g[g_off[i] ..] with capacity g_cap[i] limbs, length in g_len[i], per-pair status in
   status[i] (MGCD_OK or an error code).  The call returns MGCD_OK when every pair
   succeeded, else the first failing pair's code.  When the result slots are contiguous
   (g_off[i+1] = g_off[i] + g_cap[i]), mgcd_gcd_batch writes them straight from the device:
   the limbs of a slot past g_len[i] are then unspecified, as are a failed pair's. */
int mgcd_gcd_batch(mgcd_context *ctx, size_t npairs, const uint32_t *limbs,
                   const uint64_t *u_off, const uint32_t *u_len,
                   const uint64_t *v_off, const uint32_t *v_len,
                   uint32_t *g, const uint64_t *g_off, const uint32_t *g_cap, uint32_t *g_len,
                   int32_t *status);

/* The same in three steps, so that the device part can be timed and replayed with inputs
   resident on the device:
     mgcd_batch_upload   validates and orders the pairs on the host and copies the batch
                         to the device (the plan stays valid until the next upload);
     mgcd_batch_run      runs the GPU work only (queue reset + persistent kernels) on the
                         context's stream, asynchronously; mgcd_batch_sync waits;
     mgcd_batch_download copies the digits back and converts them to binary. */
int mgcd_batch_upload(mgcd_context *ctx, size_t npairs, const uint32_t *limbs,
                      const uint64_t *u_off, const uint32_t *u_len,
                      const uint64_t *v_off, const uint32_t *v_len);
int mgcd_batch_run(mgcd_context *ctx);
int mgcd_batch_sync(mgcd_context *ctx);
int mgcd_batch_download(mgcd_context *ctx, uint32_t *g, const uint64_t *g_off, const uint32_t *g_cap,
                        uint32_t *g_len, int32_t *status);
/* Batches may use fewer moduli per pair than the reference's count (less work per
   reduction iteration): scale in [0.5, 1], 1 = the reference's count (default).  Every
   result is certified on the device (the surviving moduli must bound both operands); a pair
   that cannot be certified is rerun with the reference's count, so results do not change.
   Single-pair calls always use the reference's count. */
int mgcd_set_nq_scale(mgcd_context *ctx, float scale);
/* Moduli grown on demand in batches (pairs of up to 16,384 moduli that run K per CTA):
   each pair starts its reduction loop with `start` times the reference's count (rounded up
   to a multiple of 32, at least 64) and, whenever the loop runs out of moduli (the
   reference's check, GmpCudaDevice-getGcdKernel.cu:393-399), has fewer than 64 surviving
   moduli, or ends with a result that the surviving moduli less one cannot certify, takes
   the next step_permille / 1000 of its cap from the table, up to the cap (the reference's
   count plus a sixteenth, rounded up to 32, at most 16,384).  A new modulus joins in the
   state it would have had from the start (residues of the operands, then the pivots so far
   replayed on it), so the result is the pair's gcd as before; the pivots after a growth may
   differ from a run with the larger set from the start.  A pair that still fails is rerun
   with the reference's count.  start in [0.1, 1] with step_permille in [10, 500], or
   start = 0 (off: the class fractions of mgcd_set_nq_scale apply).  Default 0.4, 50.
   No counterpart in the reference (its count is fixed per call, GmpCudaDevice-gcd.cu:49-55). */
int mgcd_set_growth(mgcd_context *ctx, float start, unsigned step_permille);
int mgcd_get_growth(const mgcd_context *ctx, float *start, unsigned *step_permille);
/* Launch shape of single pairs too large for one CTA:
     MGCD_SINGLE_AUTO              a thread-block cluster of up to 16 CTAs (pivot exchange
                                   through distributed shared memory) while the pair's
                                   moduli fit 16 x 512 threads, else a cooperative grid
                                   with at most one CTA per SM and a leader exchange of
                                   tagged per-CTA slots (default);
     MGCD_SINGLE_REFERENCE_SHAPE   the reference's launch shape: a cooperative grid of
                                   256-thread CTAs with 256 moduli each, one grid-wide
                                   exchange per iteration (GmpCudaDevice-gcd.cu:80-96). */
#define MGCD_SINGLE_AUTO            0
#define MGCD_SINGLE_REFERENCE_SHAPE 1
/*   MGCD_SINGLE_CLUSTER_GRID      above 16 x 512 moduli: a cooperative grid of 8-CTA
                                   clusters; keys meet in each cluster through DSMEM and one
                                   leader per cluster joins a global exchange of atomic
                                   minimum and arrival counter (measured 20-40 % slower than
                                   the default on GB300). */
#define MGCD_SINGLE_CLUSTER_GRID    2
int mgcd_set_single_pair_policy(mgcd_context *ctx, int policy);
/* Bound of every wait a cooperative-grid pair makes on the other CTAs (default 2,000 ms).
   When it runs out, every CTA returns and the pair fails with MGCD_ERR_TIMEOUT; the
   context stays usable.  (The reference's grid barrier spins without a bound,
   GmpCuda.h:68-83.) */
int mgcd_set_wait_timeout_ms(mgcd_context *ctx, unsigned ms);
/* Test hook for the bounded waits: CTA `cta` of the next cooperative-grid pairs never
   publishes its minimum, so the other CTAs' waits run out (-1 turns the hook off). */
int mgcd_test_withhold_cta(mgcd_context *ctx, int cta);
/* Test hook for the operand-staging failure path: the CTA with block index `cta` of every
   later kernel (batched, cluster or grid) reports that its bulk copies of the operand limbs
   did not complete (after they did, so nothing is left in flight); every CTA of the pairs it
   works on stops at the first exchange and those pairs fail with MGCD_ERR_TIMEOUT, while the
   other pairs of a batch are unaffected (-1 turns the hook off).  No reference interface:
   the reference stages limbs with plain loads. */
int mgcd_test_fail_staging(mgcd_context *ctx, int cta);
/* Test hook for the "ran out of moduli" paths: every following pair uses exactly nq
   moduli (a multiple of 256; 0 restores the reference's count) and is not rerun. */
int mgcd_test_force_moduli(mgcd_context *ctx, unsigned nq);
/* Launch configuration of one size class of the batched path: class 0 = pairs needing
   <= 1,024 moduli, 1 = <= 4,096, 2 = <= 16,384 (one CTA per pair), 3 = larger (one
   thread-block cluster per k pairs).  threads: CTA size (256, 512, 1024); k: pairs one CTA
   (class 3: one cluster) runs in lockstep, sharing one modular inverse per modulus and
   iteration (1, 2, 4, or 8 with threads = 512 outside class 3; a bucket whose k largest
   pairs would not fit one CTA's shared memory runs with fewer pairs per CTA); nq_scale as
   above.  The autotuner writes these. */
#define MGCD_NUM_SIZE_CLASSES 4
int mgcd_set_size_class(mgcd_context *ctx, int cls, int threads, int k, float nq_scale);
int mgcd_get_size_class(const mgcd_context *ctx, int cls, int *threads, int *k, float *nq_scale);
/* CTAs per thread-block cluster of size class 3 (2..16, default 8; raised automatically
   when a pair's share of moduli would not fit one CTA's shared memory). */
int mgcd_set_cluster_size(mgcd_context *ctx, int ctas);
int mgcd_get_cluster_size(const mgcd_context *ctx, int *ctas);
/* The same for any size class: classes 0-2 run one pair (k pairs) per CTA by default
   (ctas = 0); with ctas in 2..16 their pairs are spread over clusters of that many CTAs,
   which shortens the longest pairs of a batch (k <= 4 then). */
int mgcd_set_class_cluster(mgcd_context *ctx, int cls, int ctas);
int mgcd_get_class_cluster(const mgcd_context *ctx, int cls, int *ctas);
/* Tuning table (the autotuner's output, modgcd-onegpu_gb300/tune.py): a text file with one
   line per size class, "class threads k nq_scale cluster_ctas" (cluster_ctas 0 except for
   class 3), '#' comments.  Load checks every line before applying any (MGCD_ERR_INVALID_ARG
   for a missing file or a bad line); save writes the context's current table. */
int mgcd_load_tuning(mgcd_context *ctx, const char *path);
int mgcd_save_tuning(const mgcd_context *ctx, const char *path);
/* Records the GPU work of a batch (status reset, queue resets, one persistent kernel per
   size class on its own stream) into a CUDA graph at the first mgcd_batch_run after an
   upload; every later mgcd_batch_run of the same upload is one graph launch.  The graph
   is rebuilt after the next upload (or a change of the wait bound); enable = 0 returns to
   direct launches.  Per-kernel times (mgcd_batch_kernel_stats) exist only for direct
   launches. */
int mgcd_batch_use_graph(mgcd_context *ctx, int enable);
/* Per kernel of the last run (i < number of size classes present, largest first): its
   size class, pair count and device time (the time includes waiting for SMs that other
   concurrently running classes hold). */
int mgcd_batch_kernel_stats(const mgcd_context *ctx, int i, int *cls, int *pairs, float *ms);
/* Work of kernel i of the last downloaded batch by the cost model of mgcd_batch_work. */
int mgcd_batch_kernel_work(const mgcd_context *ctx, int i, double *residue_steps, double *euclid_updates,
                           double *recovery_updates, double *operand_bytes);
/* Pairs the last run had to rerun with the reference's moduli count. */
int mgcd_batch_retried(const mgcd_context *ctx, int *pairs);
/* Kernel launches the last mgcd_batch_run issued. */
int mgcd_batch_launches(const mgcd_context *ctx, int *launches);
/* Device time of the last mgcd_batch_run (CUDA events on the context's stream around
   the run's GPU work), after mgcd_batch_sync.  Also the time of the dominant launch (the
   bucket kernel with the most work). */
int mgcd_batch_elapsed_ms(const mgcd_context *ctx, float *run_ms, float *dominant_ms, int *dominant_threads);
/* Bytes the last upload copied host->device and the last download device->host. */
int mgcd_batch_transfer_bytes(const mgcd_context *ctx, uint64_t *h2d, uint64_t *d2h);
/* Integer-pipe throughput of this GPU measured by a microbenchmark (independent 32-bit
   IMAD chains on every SM): instructions per second. */
int mgcd_int_peak(mgcd_context *ctx, double *int_ops_per_s);
/* Certifies, on this device, the float-reciprocal quotient steps of the modular inverse
   for every operand pair they can see (replaces certifyQuoRemQuasi.cu:25-48, which checks
   the reference's quoRem<QUASI> per device): the estimate must be the true quotient or one
   less, so that the single exact correction step is always right.  The estimate is
   monotone in the dividend for a fixed divisor, so checking both ends of every quotient
   interval of every divisor covers all pairs: *checked end points (about 6e10), *failures
   of them (0 on a certified device), the first failing (r0, r1). */
int mgcd_certify_inverse(mgcd_context *ctx, uint64_t *checked, uint64_t *failures, uint32_t *first_r0,
                         uint32_t *first_r1);

/* ------------------------------------------------------------------------ serving ----
   No counterpart in the reference (one blocking GmpCudaDevice::gcd call per pair).  A
   request server on a context: callers submit single gcd requests from any thread and take
   the results later.  A server thread batches the queued requests continuously: each size
   class (lane, as in mgcd_set_size_class) turns its queue into a wave -- a batch with its
   own streams and buffers -- whenever one of its wave slots (2; 8 for class 3) is free and the admission
   budget allows, and launches it while earlier waves are still on the GPU, so requests
   that arrive later overlap with earlier ones on the device.  The moduli table and the
   inverse tables stay resident; a wave holds only its operands, scratch and digits.
   Admission budget: the device bytes admitted, unanswered requests occupy (operands,
   descriptors, digit slots and their share of the reduction scratch, about
   24 x moduli + 4 x limbs bytes per request) never exceed budget_bytes; a request larger
   than the budget on its own is refused with MGCD_ERR_BUDGET, a full queue (4M requests)
   with MGCD_ERR_BUSY.  While a server runs, the context's own calls return MGCD_ERR_BUSY. */
typedef struct mgcd_server mgcd_server;
int mgcd_serve_start(mgcd_context *ctx, size_t budget_bytes, mgcd_server **server);
/* Continuous lanes (the default) for requests of size classes 0-1 (up to 4,096 reference
   moduli): each class has a ring in pinned, mapped host memory and persistent kernels that
   take new requests from it into the slots that free up while they run (no wave has to
   form or drain); CTAs that stay idle for 0.3 ms leave.  Larger requests take waves.
   enable = 0 routes every request through waves.  Only while no request is queued or in
   flight (else MGCD_ERR_BUSY). */
int mgcd_serve_set_continuous(mgcd_server *server, int enable);
/* Answers every submitted request, then stops the server thread and frees the server. */
int mgcd_serve_stop(mgcd_server *server);
/* Queues gcd(u, v) (operands copied; either order; zero operands allowed). */
int mgcd_serve_submit(mgcd_server *server, const uint32_t *u, size_t uSz, const uint32_t *v, size_t vSz,
                      uint64_t *ticket);
/* *done = 1 once the ticket's result is ready. */
int mgcd_serve_poll(mgcd_server *server, uint64_t ticket, int *done);
/* Waits up to timeout_ms (0: no limit; MGCD_ERR_TIMEOUT keeps the ticket) for the result,
   copies g (little-endian limbs, *g_len of them) and the latency from submission to the
   answer, releases the ticket and returns the request's status. */
int mgcd_serve_take(mgcd_server *server, uint64_t ticket, unsigned timeout_ms, uint32_t *g, size_t g_cap,
                    size_t *g_len, double *latency_s);
/* Open-loop load: submits pair i (batch layout as in mgcd_gcd_batch) at arrival_s[i]
   seconds after the call starts, waits for every answer and returns each request's status,
   result and latency (scheduled arrival to answer); *makespan_s = last answer - start. */
int mgcd_serve_replay(mgcd_server *server, size_t npairs, const uint32_t *limbs,
                      const uint64_t *u_off, const uint32_t *u_len,
                      const uint64_t *v_off, const uint32_t *v_len, const double *arrival_s,
                      uint32_t *g, const uint64_t *g_off, const uint32_t *g_cap, uint32_t *g_len,
                      int32_t *status, double *latency_s, double *makespan_s);
/* Waves launched, kernel launches, peak admitted bytes, requests answered. */
int mgcd_serve_stats(mgcd_server *server, uint64_t *waves, uint64_t *launches, uint64_t *peak_bytes,
                     uint64_t *completed);
/* One record per wave (the first 2^20 waves), times in seconds since the server started:
   formed from the queue, its GPU work enqueued, its completion seen by the server thread,
   its requests answered (digits copied back and converted). */
typedef struct mgcd_wave_trace {
  int32_t lane;            /* size class */
  uint32_t requests;
  double t_admit, t_launched, t_gpu_done, t_answered;
} mgcd_wave_trace;
/* Copies up to cap records; *n receives the number recorded so far. */
int mgcd_serve_trace(mgcd_server *server, mgcd_wave_trace *out, size_t cap, size_t *n);

/* ------------------------------------------------------------ allocation-free call ----
   No counterpart in the reference.  For callers that cannot allocate device memory when
   they need a gcd: a real-time or callback context that must not wait on the allocator
   or risk its failure, an application whose device memory is budgeted and owned by its
   own pool.  The digits of gcd(u, v) (as mgcd_gcd_digits returns them, 32-bit moduli),
   with every buffer supplied by the caller and no allocation at all: no context, no
   cudaMalloc, no cudaFree.  All pointers are device pointers: u at d_limbs[0 .. uSz), v at
   d_limbs[uSz .. uSz + vSz), either order, both nonzero; d_digits holds cap >= the moduli
   count of the larger operand (mgcd_moduli_needed(32, 32 * max(uSz, vSz)) suffices);
   *d_count receives the digit count and *d_status an MGCD_* code.  The kernel is launched
   on `stream` (a cudaStream_t, 0 for the default stream) and the call returns without
   waiting; results are valid once the stream reaches that point.
   Limit: 4,096 moduli (operands of up to about 38,000 bits); larger sizes return
   MGCD_ERR_NOT_ENOUGH_MODULI and launch nothing.  The working memory is one static device
   array of 64 KiB (plus a 64 KiB moduli table) that every GPU loading the library keeps
   until exit.  The first call in a CUDA context (on each device, and again after a device
   reset) sets it up (a synchronous copy of the table): make it before any stream capture.
   All calls share the array: calls that overlap on the GPU race and must be serialised by
   the caller. */
int mgcd_gcd_digits_noalloc(const uint32_t *d_limbs, size_t uSz, size_t vSz, mgcd_pair *d_digits, size_t cap,
                            uint32_t *d_count, int32_t *d_status, void *stream);
/* Total work of the uploaded batch by the algorithmic cost model, after a run completed:
   residue limb steps (N_Q x operand limbs), reduction-loop updates (sum over iterations of
   the surviving moduli), recovery updates (the same over digits) and operand bytes. */
int mgcd_batch_work(const mgcd_context *ctx, double *residue_steps, double *euclid_updates,
                    double *recovery_updates, double *operand_bytes);
/* Occupancy trace of the batched kernels (no counterpart in the reference, whose single
   kernel has no such accounting): when enabled, every CTA of the next runs' size-class
   kernels records its SM, its start and end times (the GPU's global timer) and the pairs
   it took from its queue; mgcd_batch_cta_trace copies the last run's records (launch
   order; times in ms from the earliest CTA start) after waiting for the run.  Off by
   default; switching it drops a recorded graph. */
typedef struct {
  int32_t size_class;
  uint32_t sm, pairs;
  int32_t ran;         /* 0: the CTA never started (or the run has not completed) */
  double t_start_ms, t_end_ms;
  /* K-slot CTAs (0 elsewhere): SM clock cycles in set-up (residues, first pivot), the
     reduction-loop updates, the pivot choice and bookkeeping (including the wait for the
     slowest warp of the update), and finish (certification, replay, recovery); reduction
     iterations; moduli rounds (sum over iterations of the update loop's trips per thread);
     the part of finish spent in certification and replay; summed over the CTA's threads:
     update rounds (one position of every slot), the rounds in which some slot needed an
     inverse, and the slot states updated through the inverse; clock cycles spent re-laying
     out the positions (sorted by the slots live there, so that dead positions leave the
     update loop); clock cycles spent growing moduli sets and the number of growth steps
     (mgcd_set_growth) */
  uint64_t cycles_setup, cycles_update, cycles_pivot, cycles_finish, iterations, rounds, cycles_replay;
  uint64_t update_rounds, rounds_with_inverse, finite_slot_updates, cycles_layout;
  uint64_t cycles_grow, grow_steps;
} mgcd_cta_record;
int mgcd_set_cta_trace(mgcd_context *ctx, int enable);
/* Digits of pair i of the last downloaded batch (the pair_t list the reference kernel
   writes, GmpCudaDevice-getGcdKernel.cu:437-443): *n digits into out (MGCD_ERR_CAPACITY,
   with *n set, when cap is too small), and in *nq_final the moduli count the pair ended
   with (grown sets included).  Diagnostics and tests; copies from the device. */
int mgcd_batch_pair_digits(mgcd_context *ctx, size_t i, mgcd_pair *out, size_t cap, size_t *n, uint32_t *nq_final);
int mgcd_batch_cta_trace(mgcd_context *ctx, mgcd_cta_record *out, size_t cap, size_t *n);
/* Algorithmic bytes of the last downloaded batch, the unit of the memory roofline: per
   pair, its operand limbs (4 bytes each), a prime and an 8-byte constant for every modulus
   it used (12 bytes each; the reference reads the prime, GmpCudaDevice-getGcdKernel.cu:335,
   and derives the constant) and its k + 1 result digits (8 bytes each, the pair_t list of
   GmpCudaDevice-getGcdKernel.cu:437-443).  No counterpart in the reference. */
int mgcd_batch_alg_bytes(const mgcd_context *ctx, double *alg_bytes);

#ifdef __cplusplus
}
#endif

#endif /* MODGCD_H */

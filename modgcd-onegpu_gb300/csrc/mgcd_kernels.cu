// mgcd_kernels.cu -- the modular GCD kernels for sm_103a.
//
// One gcd pair is processed by one CTA (batched, persistent kernels pulling pairs from a
// size-ordered queue, K pairs per CTA in lockstep), or, when its moduli do not fit one CTA,
// by a thread-block cluster or a cooperative grid.
// Stages, with the reference's labels (GmpCudaDevice-getGcdKernel.cu:342-444):
//   MGCD2  residues of u and v for every modulus: limb tiles brought into shared memory by
//          bulk copies (cp.async.bulk, double-buffered), Montgomery Horner per modulus
//          (z <- REDC(z * 2^64 mod q + limb));
//   MGCD3  reduction loop: per modulus only t = u/v mod q is kept; each iteration picks
//          the pivot (p, b) = argmin of the reference's key (|t|, q - sign) with warp
//          redux.sync minima and one barrier (plus a DSMEM or grid exchange across CTAs),
//          then updates t' = p / (t - b) (one modular inverse per update, shared by the K
//          pairs of a CTA; the reference needs two per pair) and records (p, b);
//   replay the surviving moduli rebuild u mod q by applying the recorded (p, b) sequence
//          to their initial residues projectively (three Montgomery products per step, no
//          inverse) and dividing out the accumulated scale once;
//   MGCD4  recovery: signed mixed-radix digits, next digit from the lowest-indexed
//          modulus with a nonzero value, exactly as the reference selects it (in panels of
//          up to 32 digits when the pair spans several CTAs).
// The (p, b) sequence and the digits are identical to the reference algorithm's.
#include <cstdint>
#include <cstdlib>
#include <cuda_runtime.h>

#include "mgcd_device.cuh"
#include "mgcd_internal.h"
#include "mgcd_pair.cuh"

namespace mgcd {

// Start and end of every CTA of a batch kernel: the occupancy trace (BatchArgs::trace: when
// and where each CTA ran and how many pairs it took), the kernel's span (BatchArgs::span:
// the earliest start and, as its complement, the latest end, globaltimer ns) and the launch
// of the batch's next bucket kernel.  The bucket kernels of a batch are launched largest
// class first on one stream, each a programmatic dependent of the one before: it may start
// once every CTA of that one has started (griddepcontrol.launch_dependents) and does not
// wait for its results, so the kernels still run side by side, but every persistent CTA of
// a larger class is placed before a smaller class's CTAs can fill the SMs.
__device__ __forceinline__ void cta_begin(const BatchArgs& a)
{
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  if (threadIdx.x == 0 && (a.trace || a.span)) {
    const unsigned long long t = globaltimer_ns();
    if (a.trace) {
      uint32_t sm;
      asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
      a.trace[4 * blockIdx.x] = t;
      a.trace[4 * blockIdx.x + 2] = sm;
    }
    if (a.span) atomicMin(a.span, t);
  }
}

__device__ __forceinline__ void cta_end(const BatchArgs& a, uint32_t pairs)
{
  if (threadIdx.x == 0 && (a.trace || a.span)) {
    const unsigned long long t = globaltimer_ns();
    if (a.trace) {
      a.trace[4 * blockIdx.x + 1] = t;
      a.trace[4 * blockIdx.x + 3] = pairs;
    }
    if (a.span) atomicMin(a.span + 1, ~t);
  }
}

// ---- continuous serving: the ring of a lane kernel (StreamRing)
constexpr uint32_t NO_ENTRY = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t ld_acquire_sys_u32(const uint32_t* p)
{
  uint32_t v;
  asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_sys_u32(uint32_t* p, uint32_t v)
{
  asm volatile("st.release.sys.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

// Thread 0: the next published entry (claimed through the head counter below the acquired
// tail), or NO_ENTRY.  With `wait`, polls (bounded by a.idle_ns, or until the host asks
// the lane to stop) while nothing is published.
__device__ uint32_t stream_claim(const BatchArgs& a, bool wait)
{
  const unsigned long long t0 = globaltimer_ns();
  for (;;) {
    const uint32_t tail = ld_acquire_sys_u32(&a.ring->tail);
    uint32_t h = *reinterpret_cast<volatile uint32_t*>(a.ring_head);
    while ((int32_t)(tail - h) > 0) {
      const uint32_t got = atomicCAS(a.ring_head, h, h + 1u);
      if (got == h) return h;
      h = got;
    }
    if (!wait || ld_acquire_sys_u32(&a.ring->stop) != 0u) return NO_ENTRY;
    if (globaltimer_ns() - t0 > a.idle_ns) return NO_ENTRY;
    __nanosleep(256);
  }
}

// Thread 0, after the entry's results (written by this thread) are out.
__device__ __forceinline__ void stream_done(const BatchArgs& a, uint32_t k)
{
  st_release_sys_u32(&a.ring->done[k % STREAM_RING], k + 1u);
}

// Persistent batched kernel: each CTA repeatedly takes the next pair of the queue (pairs
// ordered largest first) and computes its gcd alone.
template <int T>
__global__ void __launch_bounds__(T) batch_kernel(const BatchArgs a)
{
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ RedSmem rs;
  __shared__ uint32_t next;
  __shared__ unsigned long long stage_bar[2];
  __shared__ uint32_t stage_state;
  const Stage stg{smem, stage_bar, &stage_state, blockIdx.x == a.stage_fail};   // at dynamic smem start
  stage_init(stg);
  uint32_t* st = smem + STAGE_SMEM_WORDS;
  uint32_t* acc2 = st + a.nq_max;
  uint32_t* scr = a.scratch + (size_t)blockIdx.x * a.scratch_words;
  uint32_t* u0 = scr;
  uint32_t* v0 = scr + a.nq_max;
  int2* hist = reinterpret_cast<int2*>(scr + 2 * (size_t)a.nq_max);
  cta_begin(a);
  uint32_t taken = 0;
  for (;;) {
    if (threadIdx.x == 0) next = atomicAdd(a.queue, 1u);
    __syncthreads();
    const uint32_t k = next;
    __syncthreads();
    if (k >= a.npairs) break;
    ++taken;
    const uint32_t pi = a.order[k];
    const PairDesc d = a.pairs[pi];
    run_pair<T, SYNC_CTA>(a.limbs, d, a.mods, a.L, 0u, d.nq, st, acc2, stg, rs, u0, v0, hist, nullptr,
                       a.digits, a.count + pi, a.iters + pi, a.status + pi, a.inv);
    __syncthreads();
  }
  cta_end(a, taken);
}

// ------------------------------------------------------- K pairs per CTA, lockstep ----
//
// The reduction loops of K pairs run side by side in one CTA; thread i owns modulus index
// i (+ multiples of T) in every pair, so its K inverses per iteration are all mod the same
// prime and t_update_k turns them into one.  Each pair keeps its own pivot sequence,
// exactly as if it ran alone; a pair whose loop has ended simply drops out of the update.
// Set-up (residues) and finish (certification, replay, recovery) run pair by pair: when a
// pair's loop ends, the CTA finishes it and loads the next pair of the queue into that
// slot while the other slots keep their state, so the slots stay occupied.

template <int K>
struct SlotSmem {
  unsigned long long key[2][K][32];  // per-warp minima per slot, double-buffered
  PairDesc d[K];
  uint32_t pi[K];                    // pair index of each slot (~0: empty)
  long long lu[K], lv[K];            // certification bounds (bound_step)
};

template <int T, int K>
__device__ __forceinline__ void block_min_keys(uint32_t (&kh)[K], uint32_t (&kl)[K], SlotSmem<K>& ss,
                                               uint32_t& parity)
{
  constexpr int NW = T / 32;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int s = 0; s < K; ++s) {
    warp_min_key(kh[s], kl[s]);
    if (lane == 0) ss.key[parity][s][w] = ((unsigned long long)kh[s] << 32) | kl[s];
  }
  __syncthreads();
#pragma unroll
  for (int s = 0; s < K; ++s) {
    const unsigned long long k = (lane < NW) ? ss.key[parity][s][lane] : ~0ull;
    kh[s] = (uint32_t)(k >> 32);
    kl[s] = (uint32_t)k;
    warp_min_key(kh[s], kl[s]);
  }
  parity ^= 1u;
}

// Per-slot loop state of batchk_kernel in shared memory.  Warp s owns slot s's entries
// during the pivot step; every thread reads them only after a barrier that follows the
// writes, and the next writes come only after a barrier that follows the reads.  Keeping it
// out of the registers leaves the K pivots and the K running minima as the only per-slot
// registers of the update loop.
template <int K>
struct SlotState {
  unsigned long long key[K][32];     // per-warp minima per slot (read by warp s after the barrier)
  PairDesc d[K];
  uint32_t pi[K];                    // pair index of each slot
  long long lu[K], lv[K];            // certification bounds (bound_step)
  uint32_t p[K];                     // current pivot (modulus, signed value) of each slot
  int32_t b[K];
  int32_t rem[K], ubits[K], vbits[K];  // surviving moduli and the reference's size estimates
  uint32_t iters[K];
  uint32_t res[K];                   // slot_step's result for the slot's last pivot
  uint32_t seq[K];                   // ring mode: the slot's entry number
  unsigned long long upd[K];         // surviving moduli summed over the slot's iterations (work)
  uint32_t stop;                     // set-up: slot_step's result for the first pivot
};

// Words of a K-slot CTA's phase record (BatchArgs::phases, PHASE_WORDS per CTA): clock cycles
// of thread 0 per phase, loop iterations, moduli rounds, pairs taken, the replay's share of
// the finish; words 8-10 are the update loop's liveness counters (every thread).
// Word 11: cycles spent re-laying out the positions.
// Word 12: cycles spent growing moduli sets; word 13: growth steps.
enum { PH_LOAD = 0, PH_UPDATE, PH_PIVOT, PH_FINISH, PH_ITERS, PH_ROUNDS, PH_TAKEN, PH_REPLAY, PH_LAYOUT, PH_GROW,
       PH_GROWS };
constexpr int PH_WORDS_T0 = 11;         // words kept by thread 0

// Iterations between two re-layouts of a K-slot CTA's positions (besides those after a pair
// finishes, is loaded or grows).  Each iteration retires one position per slot, so a layout
// stays close to sorted; one re-layout moves (K + 1) x nq_max words twice.  Measured on the
// mixed batch with moduli growth (27 bits): every 8 iterations 80.4 ms, 16 76.3, 32 74.6.
#ifndef MGCD_RELAYOUT_EVERY
#define MGCD_RELAYOUT_EVERY 32
#endif
constexpr uint32_t RELAYOUT_EVERY = MGCD_RELAYOUT_EVERY;

// Largest K whose update loop loads each position's modulus constants a round ahead
// (batchk_kernel's update loop).
#ifndef MGCD_PREFETCH_MAX_K
#define MGCD_PREFETCH_MAX_K 2
#endif

// A pair that may grow its moduli set grows whenever fewer than GROW_LOW of its moduli
// survive: near the end of a set each iteration reduces the operands by only about
// log2(survivors) bits, so a set run down to a handful costs iterations that do little.
#ifndef MGCD_GROW_LOW
#define MGCD_GROW_LOW 64
#endif
constexpr int GROW_LOW = MGCD_GROW_LOW;

// One reduction-loop step of slot s's bookkeeping for its current pivot (the reference's
// per-iteration checks, GmpCudaDevice-getGcdKernel.cu:365-402): records (p, b) in the
// history; returns 0 (continue), 1 (loop ended: b = INF), 3 (ran out of moduli) or 4 (ran
// out, or fewer than GROW_LOW moduli survive, and the pair may grow its moduli set: grow
// before the update that applies this pivot).  One thread per slot.  The certification
// bounds are stepped for this pivot during the update that uses it, by the last warp
// (below), off the path between the two barriers.
template <int K>
__device__ __forceinline__ uint32_t slot_step(SlotState<K>& ss, int s, int2* hist, int L)
{
  const uint32_t p = ss.p[s];
  const int32_t b = ss.b[s];
  if (b == MOD_INFINITY) return 1u;
  hist[ss.iters[s]] = make_int2((int)p, b);
  ss.iters[s] += 1u;
  const int rem = ss.rem[s] - 1;
  ss.rem[s] = rem;
  ss.upd[s] += (unsigned long long)rem;
  const uint32_t ab = b < 0 ? 0u - (uint32_t)b : (uint32_t)b;
  const int tbits = ss.ubits[s] - (L - 1) + __ffs((int)ab);
  const int ub = ss.vbits[s];
  ss.ubits[s] = ub;
  ss.vbits[s] = tbits;
  const bool can_grow = ss.d[s].nq_cap > ss.d[s].nq;
  if (rem * (L - 2) <= ub) return can_grow ? 4u : 3u;
  return can_grow && rem < GROW_LOW ? 4u : 0u;
}

// Moduli added to a pair's set by one growth step: `permille` thousandths of its cap,
// rounded up to a warp (32).
__device__ __forceinline__ uint32_t grow_step_for(uint32_t cap, uint32_t permille)
{
  const uint32_t n = (uint32_t)(((unsigned long long)cap * permille + 999ull) / 1000ull);
  return n < 32u ? 32u : (n + 31u) & ~31u;
}

// Position layout.  The K slots share every modulus's inverse, so their states sit at common
// positions: slot s's state of modulus pmod[pos] at tS[s][pos].  A slot's states die as the
// loop retires its pivots (about one per iteration; most of its moduli by the end) and
// beyond its own moduli count, and a warp pays for a slot's work wherever one of its lanes
// needs it.  So the CTA re-lays its positions out, sorted by the set of slots that are live
// there (finite or infinite ratio): warps then see one live set, skip a dead slot's work
// together, and positions dead in every slot go to the end, where the update loop no longer
// visits them.  Dead states never change, so the loop result is the same; the pivot is the
// minimum key, whose tie-break is the modulus, not the position.  A slot's states are put
// back into modulus order before its pair finishes (the replay and recovery index moduli),
// and a newly loaded pair's states, computed in modulus order, are taken in by the next
// re-layout (`fresh`).
//
// NARROW: moduli below 2^30 (widths up to 30 bits), lazily reduced Montgomery products.
// RING: continuous serving -- pairs come from a.ring instead of the batch queue, empty
// slots take newly published entries while the others run, and a CTA whose slots stay
// empty for a.idle_ns leaves.
template <int T, int K, bool NARROW = false, bool RING = false>
__global__ void __launch_bounds__(T) batchk_kernel(const BatchArgs a)
{
  constexpr int NW = T / 32;
  static_assert(NW >= K, "one warp per slot reduces the slot's pivot");
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ SlotState<K> ss;
  __shared__ RedSmem rs;
  __shared__ uint32_t next;
  __shared__ unsigned long long stage_bar[2];
  __shared__ uint32_t stage_state;
  // at dynamic smem start; in ring mode the operands are in host memory: plain coherent loads
  // (built where it is used: its fields are cheap to form and would otherwise stay in
  // registers through the update loop)
  auto stage = [&]() {
    return RING ? Stage{smem, nullptr, nullptr, 0u, 1u}
                : Stage{smem, stage_bar, &stage_state, blockIdx.x == a.stage_fail, 0u};
  };
  stage_init(stage());
  const uint32_t NQS = a.nq_max;
  uint32_t* const tS = smem + STAGE_SMEM_WORDS;       // K x NQS states
  uint32_t* const acc2 = tS + (size_t)K * NQS;        // residues of v during set-up; the
                                                      // re-layout's and un-permute's buffer
  uint16_t* const pmod = reinterpret_cast<uint16_t*>(acc2 + NQS);   // modulus at each position
  uint16_t* const aux = pmod + NQS;                   // re-layout: live set, then new position
  uint32_t* const scr = a.scratch + (size_t)blockIdx.x * a.scratch_words;   // per slot u0, v0, hist
  const int L = a.L;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t rparity = 0, repoch = 0;
  uint32_t valid = 0, active = 0, redux = 0;          // slots holding a pair / in the loop / ran out (uniform)
  cta_begin(a);
  uint32_t taken = 0;
  auto hist_of = [&](int s) { return reinterpret_cast<int2*>(scr + (size_t)s * 4 * NQS + 2 * (size_t)NQS); };
  // phase accounting (a.phases): thread 0's clock in each phase; the phases end at barriers,
  // so thread 0's timeline is the CTA's
  // (in shared memory, so that no thread carries them in registers through the loop)
  const bool prof = a.phases != nullptr && threadIdx.x == 0;
  __shared__ unsigned long long phs[PH_WORDS_T0];   // PH_*; PH_REPLAY is the part of PH_FINISH
  __shared__ long long ph_t;                        // spent in certification and replay
  if (prof) {
#pragma unroll
    for (int i = 0; i < PH_WORDS_T0; ++i) phs[i] = 0ull;
    ph_t = clock64();
  }
  __shared__ unsigned long long lvs[3];   // liveness of the update loop: thread-rounds, those with
                                          // a finite slot state, finite slot states (per-iteration
                                          // warp sums, so no counter is carried through the loop)
  if (a.phases && threadIdx.x == 0) lvs[0] = lvs[1] = lvs[2] = 0ull;
  auto ph_mark = [&](int i) {
    if (prof) { const long long t = clock64(); phs[i] += (unsigned long long)(t - ph_t); ph_t = t; }
  };

  // Takes the next pair of the queue (ring mode: of the ring; `wait` = poll, bounded, while
  // nothing is published) into slot s: residues, initial ratios, first pivot and its
  // bookkeeping step (bits 1, 3 of the result as slot_step's; bit 4: a pair was loaded).
  // A pair whose operands could not be staged is answered with ST_TIMEOUT.
  auto load = [&](int s, bool wait) -> uint32_t {
    uint32_t* ts = tS + (size_t)s * NQS;
    for (;;) {
      if (threadIdx.x == 0) {
        if constexpr (RING) next = stream_claim(a, wait);
        else next = atomicAdd(a.queue, 1u);
      }
      __syncthreads();
      const uint32_t k = next;
      __syncthreads();
      if (RING ? k == NO_ENTRY : k >= a.npairs) return 0u;
      ++taken;
      if (threadIdx.x == 0) {
        if constexpr (RING) {                         // volatile: the host rewrites ring entries
          const volatile PairDesc* e = &a.ring->desc[k % STREAM_RING];
          PairDesc d;
          d.u_off = e->u_off; d.v_off = e->v_off; d.u_len = e->u_len; d.v_len = e->v_len;
          d.nq = e->nq; d.out_off = e->out_off; d.g_off = e->g_off; d.g_cap = e->g_cap; d.nq_cap = 0u;
          ss.pi[s] = k % STREAM_RING;
          ss.seq[s] = k;
          ss.d[s] = d;
        } else {
          ss.pi[s] = a.order[k];
          ss.d[s] = a.pairs[ss.pi[s]];
        }
      }
      __syncthreads();
      const PairDesc& d = ss.d[s];
      const Stage stg = stage();
      const bool staged = residues<T>(a.limbs + d.u_off, d.u_len, a.mods, d.nq, ts, stg, NARROW);
      if (residues<T>(a.limbs + d.v_off, d.v_len, a.mods, d.nq, acc2, stg, NARROW) && staged) break;
      if (threadIdx.x == 0) {
        a.status[ss.pi[s]] = ST_TIMEOUT; a.count[ss.pi[s]] = 0; a.iters[ss.pi[s]] = 0;
        if constexpr (RING) stream_done(a, ss.seq[s]);
      }
      __syncthreads();
    }
    const PairDesc& d = ss.d[s];
    uint32_t* u0 = scr + (size_t)s * 4 * NQS;
    uint32_t h0 = 0xFFFFFFFFu, l0 = 0xFFFFFFFFu;
    for (uint32_t j = threadIdx.x; j < d.nq; j += T) {
      const ModConst c = a.mods[j];
      const uint32_t u = ts[j], v = acc2[j];
      u0[j] = u;
      u0[NQS + j] = v;
      const uint32_t t = t_init(u, v, c.q, c.qinv);
      ts[j] = t;
      uint32_t h, l;
      t_key(t, c.q, h, l);
      if (key_less(h, l, h0, l0)) { h0 = h; l0 = l; }
    }
    block_min_key<T>(h0, l0, rs, rparity);
    if (threadIdx.x == 0) {
      uint32_t p0;
      int32_t b0;
      key_pair(h0, l0, p0, b0);
      ss.p[s] = p0;
      ss.b[s] = b0;
      ss.rem[s] = (int)d.nq;
      ss.ubits[s] = ((int)d.u_len + 1) * 32;
      ss.vbits[s] = ((int)d.v_len + 1) * 32;
      ss.iters[s] = 0u;
      ss.upd[s] = 0ull;
      ss.lu[s] = bound_init(a.limbs + d.u_off, d.u_len);
      ss.lv[s] = bound_init(a.limbs + d.v_off, d.v_len);
      ss.stop = 16u | slot_step<K>(ss, s, hist_of(s), L);
    }
    __syncthreads();
    const uint32_t r = ss.stop;
    __syncthreads();                                  // everyone has read it before it changes
    return r;
  };
  uint32_t npos = 0, fresh = 0, since = 0;             // positions visited; slots in modulus order
  uint32_t grow = 0, failed = 0;                      // slots to grow before the next update; slots
                                                      // whose growth could not stage its operands
  auto take_slot = [&](int s, bool wait) {
    ph_mark(PH_FINISH);
    const uint32_t r = load(s, wait);
    ph_mark(PH_LOAD);
    if (r & 16u) {
      valid |= 1u << s;
      fresh |= 1u << s;
      if (!(r & 1u)) active |= 1u << s;
      if ((r & 3u) == 3u) redux |= 1u << s;
      if (r & 4u) grow |= 1u << s;
    }
  };
  // Slot s's states back into modulus order (ts[m] for the modulus of table index m < nq).
  auto to_modulus_order = [&](int s) {
    if ((fresh >> s) & 1u) return;
    const uint32_t nq = ss.d[s].nq;
    uint32_t* ts = tS + (size_t)s * NQS;
    for (uint32_t pos = threadIdx.x; pos < NQS; pos += T) {
      const uint32_t m = pmod[pos];
      if (m < nq) acc2[m] = ts[pos];
    }
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < nq; j += T) ts[j] = acc2[j];
    __syncthreads();
  };

  // ---- moduli grown on demand (batches; not in ring mode).  A pair starts with fewer moduli
  // than the reference's count and takes the next table entries, up to its nq_cap, when its
  // loop runs out of moduli (the reference's check) or ends without a certified result.  A
  // new modulus q joins in the state it would have had from the start: the operands'
  // residues, then the first nrep pivots of the history replayed projectively,
  // (U, V) <- (p V, U - b V) (the ratio U/V is all a state holds; the replay reaches the
  // same INF, degenerate and zero states as the loop's updates), then t = U/V.  The slot is
  // put into modulus order and the next re-layout takes the new states in (`fresh`).  Its
  // moduli count, survivors and the operands' residues (u0, v0, for the final replay) grow
  // with it.  Every thread calls it; returns this thread's minimum key over the new states
  // in (h0, l0), or false (nothing added) if an operand tile could not be staged.
  auto grow_slot = [&](int s, uint32_t nrep, uint32_t& h0, uint32_t& l0) -> bool {
    const PairDesc& d = ss.d[s];
    const uint32_t n0 = d.nq;
    const uint32_t n1 = min(d.nq_cap, n0 + grow_step_for(d.nq_cap, a.grow_permille));
    const uint32_t dn = n1 - n0;
    uint32_t* ts = tS + (size_t)s * NQS;
    uint32_t* u0 = scr + (size_t)s * 4 * NQS;
    to_modulus_order(s);
    const Stage stg = stage();
    bool ok = residues<T>(a.limbs + d.u_off, d.u_len, a.mods + n0, dn, acc2, stg, NARROW);
    for (uint32_t j = threadIdx.x; j < dn; j += T) u0[n0 + j] = acc2[j];
    ok = residues<T>(a.limbs + d.v_off, d.v_len, a.mods + n0, dn, acc2, stg, NARROW) && ok;
    for (uint32_t j = threadIdx.x; j < dn; j += T) u0[NQS + n0 + j] = acc2[j];
    if (!ok) return false;
    const int2* hist = hist_of(s);
    int2* const hb = reinterpret_cast<int2*>(smem);   // the staging buffers (free again)
    for (uint32_t base = 0; base < dn; base += T) {
      const bool have = base + threadIdx.x < dn;
      const uint32_t j = n0 + base + threadIdx.x;
      const ModConst c = a.mods[have ? j : n0];
      const uint32_t q = c.q, qi = c.qinv;
      uint32_t U = have ? u0[j] : 0u, V = have ? u0[NQS + j] : 0u;
      for (uint32_t c0 = 0; c0 < nrep; c0 += REPLAY_CHUNK) {
        const uint32_t n = nrep - c0 < REPLAY_CHUNK ? nrep - c0 : REPLAY_CHUNK;
        __syncthreads();                              // the previous chunk is consumed
        for (uint32_t e = threadIdx.x; e < n; e += T) hb[e] = hist[c0 + e];
        __syncthreads();
        if (!have) continue;
#pragma unroll 4
        for (uint32_t e = 0; e < n; ++e) {
          const int2 h = hb[e];
          if constexpr (NARROW) {                    // lazily in [0, 2q), as the final replay:
            const uint32_t pm = (uint32_t)h.x;       // p < 2^L <= 2q as it is, and q - b in
            const uint32_t bn = q - (uint32_t)h.y;   // (0, 2q) since |b| <= p/2 < q
            const uint64_t T2 = (uint64_t)bn * V + U;
            const uint32_t U2 = mont_mul_lazy(V, pm, q, qi);
            const uint32_t lo = (uint32_t)T2, hi = (uint32_t)(T2 >> 32);
            V = hi + __umulhi(lo * qi, q) + (lo != 0u);
            U = U2;
          } else {
            const uint32_t pp = (uint32_t)h.x;
            const uint32_t pm = pp > q ? pp - q : pp;
            const uint32_t bn = from_signed(-h.y, q);   // -b mod q
            const uint32_t U2 = mont_mul(V, pm, q, qi);
            V = redc((uint64_t)bn * V + U, q, qi);
            U = U2;
          }
        }
      }
      if (have) {
        if constexpr (NARROW) { U = mod_canon(U, q); V = mod_canon(V, q); }
        const uint32_t t = t_init(U, V, q, qi);
        ts[j] = t;
        uint32_t h, l;
        t_key(t, q, h, l);
        if (key_less(h, l, h0, l0)) { h0 = h; l0 = l; }
      }
    }
    __syncthreads();                                  // hb, the new states
    if (threadIdx.x == 0) {
      ss.d[s].nq = n1;
      ss.rem[s] += (int)dn;
      if (prof) phs[PH_GROWS] += 1u;
    }
    __syncthreads();
    fresh |= 1u << s;
    return true;
  };

  // ---- position layout
  __shared__ uint32_t bucket[1u << K];
  __shared__ uint32_t live_pos;
  for (uint32_t pos = threadIdx.x; pos < NQS; pos += T) pmod[pos] = (uint16_t)pos;
  auto state_at = [&](int s, uint32_t pos, uint32_t m) -> uint32_t {
    const uint32_t* ts = tS + (size_t)s * NQS;
    if ((fresh >> s) & 1u) return m < ss.d[s].nq ? ts[m] : T_RETIRED;
    return ts[pos];
  };
  // Counting sort of the positions by live set (full sets first, the empty set last);
  // warp-aggregated shared-memory atomics give the ranks.  Every thread calls it.
  auto relayout = [&]() {
    // without a fresh slot only [0, npos) needs sorting: positions past it are dead in every
    // active slot, and dead states stay dead (a slot becomes active again only as a fresh one)
    const uint32_t lim = fresh ? NQS : npos;
    if (threadIdx.x < (1u << K)) bucket[threadIdx.x] = 0u;
    __syncthreads();
    const uint32_t below = (1u << lane) - 1u;
    for (uint32_t base = 0; base < lim; base += T) {
      const uint32_t pos = base + threadIdx.x;
      const bool in = pos < lim;
      uint32_t set = 0xFFFFu;
      if (in) {
        const uint32_t m = pmod[pos];
        set = 0u;
#pragma unroll
        for (int s = 0; s < K; ++s) {
          if (!((active >> s) & 1u)) continue;
          const uint32_t v = state_at(s, pos, m);
          set |= (uint32_t)(v < T_MARK || v == T_INF) << s;
        }
        aux[pos] = (uint16_t)set;
      }
      const uint32_t grp = __match_any_sync(0xFFFFFFFFu, set);
      if (in && lane == __ffs((int)grp) - 1) atomicAdd(&bucket[set], (uint32_t)__popc(grp));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t off = 0;
      for (uint32_t m = (1u << K) - 1u; m >= 1u; --m) { const uint32_t c = bucket[m]; bucket[m] = off; off += c; }
      live_pos = off;
      bucket[0] = off;
    }
    __syncthreads();
    for (uint32_t base = 0; base < lim; base += T) {
      const uint32_t pos = base + threadIdx.x;
      const bool in = pos < lim;
      const uint32_t set = in ? aux[pos] : 0xFFFFu;
      const uint32_t grp = __match_any_sync(0xFFFFFFFFu, set);
      const int lead = __ffs((int)grp) - 1;
      uint32_t r0 = 0u;
      if (in && lane == lead) r0 = atomicAdd(&bucket[set], (uint32_t)__popc(grp));
      r0 = __shfl_sync(0xFFFFFFFFu, r0, lead);
      if (in) aux[pos] = (uint16_t)(r0 + __popc(grp & below));
    }
    __syncthreads();
#pragma unroll 1
    for (int s = 0; s < K; ++s) {
      if (!((valid >> s) & 1u)) continue;
      for (uint32_t pos = threadIdx.x; pos < lim; pos += T) acc2[aux[pos]] = state_at(s, pos, pmod[pos]);
      __syncthreads();
      uint32_t* ts = tS + (size_t)s * NQS;
      for (uint32_t pos = threadIdx.x; pos < lim; pos += T) ts[pos] = acc2[pos];
      __syncthreads();
    }
    for (uint32_t pos = threadIdx.x; pos < lim; pos += T) acc2[aux[pos]] = pmod[pos];
    __syncthreads();
    for (uint32_t pos = threadIdx.x; pos < lim; pos += T) pmod[pos] = (uint16_t)acc2[pos];
    __syncthreads();
    npos = live_pos;
    fresh = 0u;
  };

#pragma unroll 1
  for (int s = 0; s < K; ++s) {
    take_slot(s, RING && s == 0);
    if (RING && !((valid >> s) & 1u)) break;         // nothing more published now
  }

  for (;;) {
    // ---- pairs whose reduction loop ended: finish them and refill their slots
    const uint32_t done = valid & ~active;
    bool changed = fresh != 0u;
#pragma unroll 1
    for (int s = 0; s < K; ++s) {
      if (!((done >> s) & 1u)) continue;
      if constexpr (!RING) {
        // the loop ended: a result that the surviving moduli cannot certify grows the set
        // (replayed through the whole history) and goes on with the pivot chosen over it
        while (!((redux | failed) >> s & 1u) && ss.d[s].nq_cap > ss.d[s].nq) {
          // one modulus to spare: the recovery stops at the first all-zero round, so it
          // needs one survivor more than it has digits
          if (threadIdx.x == 0) ss.stop = bound_certified(ss.rem[s] - 1, L, ss.lu[s], ss.lv[s]) ? 1u : 0u;
          __syncthreads();
          const bool cert = ss.stop != 0u;
          __syncthreads();
          if (cert) break;
          ph_mark(PH_FINISH);
          uint32_t h0 = 0xFFFFFFFFu, l0 = 0xFFFFFFFFu;
          const bool ok = grow_slot(s, ss.iters[s], h0, l0);
          if (!ok) {
            failed |= 1u << s;
            ph_mark(PH_GROW);
            break;
          }
          block_min_key<T>(h0, l0, rs, rparity);
          if (threadIdx.x == 0) {
            if (h0 == 0xFFFFFFFFu) { h0 = KEY_INF_HI; l0 = 0xFFFFFFFFu; }
            key_pair(h0, l0, ss.p[s], ss.b[s]);
            ss.stop = slot_step<K>(ss, s, hist_of(s), L);
          }
          __syncthreads();
          const uint32_t r = ss.stop;
          __syncthreads();
          ph_mark(PH_GROW);
          if (r & 2u) redux |= 1u << s;
          if (r & 4u) grow |= 1u << s;
          if (!(r & 1u)) { active |= 1u << s; break; }
        }
        if ((active >> s) & 1u) { changed = true; continue; }   // back in the loop
      }
      const uint32_t pi = ss.pi[s];
      const uint32_t it = ss.iters[s];
      if (threadIdx.x == 0) {
        a.iters[pi] = it;
        if (a.nq_final) a.nq_final[pi] = ss.d[s].nq;
        if (a.updates) a.updates[pi] = ss.upd[s];
      }
      if ((failed >> s) & 1u) {
        if (threadIdx.x == 0) { a.status[pi] = ST_TIMEOUT; a.count[pi] = 0; }
      } else if ((redux >> s) & 1u) {
        if (threadIdx.x == 0) { a.status[pi] = ST_REDUX; a.count[pi] = 0; }
      } else {
        to_modulus_order(s);
        uint32_t* u0 = scr + (size_t)s * 4 * NQS;
        finish_pair<T, SYNC_CTA>(a.mods, ss.d[s], L, 0u, ss.d[s].nq, tS + (size_t)s * NQS, rs, rparity, repoch, nullptr,
                              u0, u0 + NQS, reinterpret_cast<const int2*>(u0 + 2 * (size_t)NQS), it, ss.rem[s],
                              ss.lu[s], ss.lv[s], a.digits, a.count + pi, a.status + pi, a.inv, smem, acc2,
                              a.phases ? &phs[PH_REPLAY] : nullptr);
      }
      if (RING && threadIdx.x == 0) stream_done(a, ss.seq[s]);   // results written by this thread
      __syncthreads();
      valid &= ~(1u << s);
      redux &= ~(1u << s);
      fresh &= ~(1u << s);
      grow &= ~(1u << s);
      failed &= ~(1u << s);
      changed = true;
      if (!RING) take_slot(s, false);
    }
    if constexpr (RING) {
      // empty slots take newly published entries while the others run; with every slot
      // empty, wait (bounded) for one, else leave
#pragma unroll 1
      for (int s = 0; s < K; ++s) {
        if ((valid >> s) & 1u) continue;
        take_slot(s, valid == 0u);
        if (!((valid >> s) & 1u)) break;
        changed = true;
      }
    }
    if (!valid) break;
    ph_mark(PH_FINISH);
    if constexpr (!RING) {
      // slots that ran out of moduli at their current pivot: the set grows before the update
      // that applies it (the new moduli replay the history without it)
#pragma unroll 1
      for (int s = 0; s < K; ++s) {
        if (!((grow >> s) & 1u)) continue;
        grow &= ~(1u << s);
        uint32_t h0 = 0xFFFFFFFFu, l0 = 0xFFFFFFFFu;
        if (!grow_slot(s, ss.iters[s] - 1u, h0, l0)) {   // the pair ends: a failed staging
          failed |= 1u << s;
          active &= ~(1u << s);
        }
        changed = true;
      }
      ph_mark(PH_GROW);
    }
    if (changed || since >= RELAYOUT_EVERY) {
      relayout();
      since = 0;
      ph_mark(PH_LAYOUT);
    }
    ++since;

    // ---- one update of every active pair with its current pivot
    uint32_t p[K], kh[K], kl[K];
    int32_t b[K];
#pragma unroll
    for (int s = 0; s < K; ++s) {
      p[s] = ss.p[s];
      b[s] = ss.b[s];
      kh[s] = kl[s] = 0xFFFFFFFFu;
    }
    if (prof) { phs[PH_ITERS] += 1u; phs[PH_ROUNDS] += (npos + T - 1) / T; lvs[0] += npos; }
    uint32_t lv_any = 0, lv_fin = 0;
    // size bounds for this update's pivots (log2f/exp2f on one lane per slot): the last warp
    // has the fewest moduli rounds whenever npos is not a multiple of T
    if (w == NW - 1 && lane < K && ((active >> lane) & 1u)) bound_step(ss.lu[lane], ss.lv[lane], ss.p[lane], ss.b[lane]);
    // with K <= MGCD_PREFETCH_MAX_K, each position's constants are loaded one round ahead (a
    // global load from a table that the shared memory leaves little L1 for: its latency
    // overlaps a round's update); the K = 4 loop has no registers to spare for them (mixed
    // batch: none 72.6 ms, K <= 2 72.1, every K 75.6: the K = 4 loop's spills double)
    constexpr bool PREFETCH = K <= MGCD_PREFETCH_MAX_K;
    ModConst cn{};
    if constexpr (PREFETCH) cn = a.mods[pmod[threadIdx.x < npos ? threadIdx.x : 0u]];
    for (uint32_t j = threadIdx.x; j < npos; j += T) {
      ModConst c;
      if constexpr (PREFETCH) {
        c = cn;
        if (j + T < npos) cn = a.mods[pmod[j + T]];
      } else {
        c = a.mods[pmod[j]];
      }
      uint32_t m = 0, tv[K];
#pragma unroll
      for (int s = 0; s < K; ++s) {                   // (states beyond a pair's moduli are retired)
        const bool on = (active >> s) & 1u;
        m |= (uint32_t)on << s;
        tv[s] = on ? tS[(size_t)s * NQS + j] : T_RETIRED;
      }
      if (a.phases) {                                 // liveness accounting (thread-rounds)
        uint32_t fin = 0;
#pragma unroll
        for (int s = 0; s < K; ++s) fin += ((m >> s) & 1u) && tv[s] < T_MARK;
        lv_any += fin != 0u;
        lv_fin += fin;
      }
      if (!m) continue;
      if constexpr (NARROW) t_update_k_narrow<K>(tv, c, p, b, m);
      else t_update_k<K>(tv, c, p, b, m);
#pragma unroll
      for (int s = 0; s < K; ++s) {
        if (!((m >> s) & 1u)) continue;
        tS[(size_t)s * NQS + j] = tv[s];
        uint32_t h, l;
        t_key(tv[s], c.q, h, l);
        if (key_less(h, l, kh[s], kl[s])) { kh[s] = h; kl[s] = l; }
      }
    }
    if (a.phases) {
      const uint32_t wa = __reduce_add_sync(0xFFFFFFFFu, lv_any), wf = __reduce_add_sync(0xFFFFFFFFu, lv_fin);
      if (lane == 0 && wf) { atomicAdd(&lvs[1], (unsigned long long)wa); atomicAdd(&lvs[2], (unsigned long long)wf); }
    }
    ph_mark(PH_UPDATE);
    // ---- the next pivots (GmpCudaDevice-getGcdKernel.cu:365-402): warp minima, one
    // barrier, then warp s reduces slot s's minima, stores its pivot and steps its
    // bookkeeping (the K slots in parallel)
#pragma unroll
    for (int s = 0; s < K; ++s) {
      warp_min_key(kh[s], kl[s]);
      if (lane == 0) ss.key[s][w] = ((unsigned long long)kh[s] << 32) | kl[s];
    }
    __syncthreads();
    if (w < K && ((active >> w) & 1u)) {
      const unsigned long long k = (lane < NW) ? ss.key[w][lane] : ~0ull;
      uint32_t h = (uint32_t)(k >> 32), l = (uint32_t)k;
      warp_min_key(h, l);
      if (lane == 0) {
        // no position visited holds the slot's states (every ratio retired or degenerate):
        // the infinite key, which ends the slot's loop
        if (h == 0xFFFFFFFFu) { h = KEY_INF_HI; l = 0xFFFFFFFFu; }
        key_pair(h, l, ss.p[w], ss.b[w]);
        ss.res[w] = slot_step<K>(ss, w, hist_of(w), L);
      }
    }
    __syncthreads();
    // ss.res changes next after the next iteration's first barrier (or inside a refill,
    // after its barriers): every thread has read it by then
#pragma unroll
    for (int s = 0; s < K; ++s) {
      if (!((active >> s) & 1u)) continue;
      const uint32_t r = ss.res[s];
      if (r & 1u) active &= ~(1u << s);
      if (r & 2u) redux |= 1u << s;
      if (r & 4u) grow |= 1u << s;
    }
    ph_mark(PH_PIVOT);
  }
  ph_mark(PH_FINISH);
  if (prof) {
    unsigned long long* o = a.phases + PHASE_WORDS * (size_t)blockIdx.x;
#pragma unroll
    for (int i = 0; i < 8; ++i) o[i] = phs[i];
    o[PH_TAKEN] = taken;
    o[8] = lvs[0]; o[9] = lvs[1]; o[10] = lvs[2];      // every warp's sums are in (barriers since)
    o[11] = phs[PH_LAYOUT];
    o[12] = phs[PH_GROW];
    o[13] = phs[PH_GROWS];
  }
  cta_end(a, taken);
}

// ------------------------------------------- K pairs per thread-block cluster, lockstep ----
//
// The cluster analogue of batchk_kernel for pairs larger than one CTA (size class 3).  A
// cluster of C CTAs holds K pairs; CTA r owns global moduli [r * per, (r + 1) * per) of every
// pair (per = ceil(nq_max / C), the same slice for all slots, so a thread's K updates share
// one modulus and one inverse).  Pivot keys: each CTA reduces its K minima (one
// __syncthreads), warp 0 stores them into every CTA of the cluster (DSMEM), one cluster
// barrier, then every warp reduces the C values per slot.  Queue pops are made by CTA 0 and
// broadcast the same way.  Set-up and finish of one slot run the cluster single-pair code
// on the CTA's slice while the other slots wait.

template <int K>
struct ClusterSlotKeys {
  unsigned long long key[2][K][MAX_CLUSTER];   // per slot: each CTA's minimum, double-buffered
  uint32_t next;                               // queue index broadcast by CTA 0
  uint32_t nloc[K];                            // this CTA's moduli of each slot's pair
};

template <int T, int K>
__device__ __forceinline__ void cluster_min_keys(uint32_t (&kh)[K], uint32_t (&kl)[K], SlotSmem<K>& ss,
                                                 ClusterSlotKeys<K>& ck, uint32_t& kparity, uint32_t& cparity)
{
  block_min_keys<T, K>(kh, kl, ss, kparity);
  const uint32_t lane = threadIdx.x & 31u, me = cluster_rank(), nc = cluster_size();
  if (threadIdx.x < 32u && lane < nc) {
#pragma unroll
    for (int s = 0; s < K; ++s)
      st_cluster_u64(&ck.key[cparity][s][me], lane, ((unsigned long long)kh[s] << 32) | kl[s]);
  }
  cluster_sync_all();
#pragma unroll
  for (int s = 0; s < K; ++s) {
    const unsigned long long k = lane < nc ? ck.key[cparity][s][lane] : ~0ull;
    kh[s] = (uint32_t)(k >> 32);
    kl[s] = (uint32_t)k;
    warp_min_key(kh[s], kl[s]);
  }
  cparity ^= 1u;
}

template <int T, int K>
__global__ void __launch_bounds__(T) cluster_batchk_kernel(const BatchArgs a)
{
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ SlotSmem<K> ss;
  __shared__ ClusterSlotKeys<K> ck;
  __shared__ ClusterSmem cs;                          // single-slot exchanges (set-up, finish)
  __shared__ RedSmem rs;
  __shared__ unsigned long long stage_bar[2];
  __shared__ uint32_t stage_state;
  const Stage stg{smem, stage_bar, &stage_state, blockIdx.x == a.stage_fail};   // at dynamic smem start
  stage_init(stg);
  const uint32_t C = cluster_size(), r = cluster_rank();
  const uint32_t per = (a.nq_max + C - 1) / C;        // slice of every slot's moduli
  const uint32_t j0 = r * per;
  uint32_t* const tS = smem + STAGE_SMEM_WORDS;       // K x per states
  uint32_t* const acc2 = tS + (size_t)K * per;        // residues of v during set-up
  uint32_t* const scr = a.scratch + (size_t)(blockIdx.x / C) * a.scratch_words;   // per slot u0, v0, hist
  const uint32_t NQS = a.nq_max;
  const int L = a.L;
  GridSync* const gcs = reinterpret_cast<GridSync*>(&cs);
  // parities of the double-buffered exchanges: slot keys in the CTA (ss) and across the
  // cluster (ck), single keys in the CTA (rs) and across the cluster (cs)
  uint32_t kparity = 0, cparity = 0, bparity = 0, rparity = 0, repoch = 0;
  uint32_t valid = 0, active = 0, redux = 0;
  int rem[K], ubits[K], vbits[K];
  uint32_t iters[K], p[K], kh[K], kl[K];
  int32_t b[K];
  cta_begin(a);
  uint32_t taken = 0;

  cluster_sync_all();
  // Takes the next pair of the queue into slot s.  A CTA whose operands could not be staged
  // contributes the key (0, 0) (no modulus produces it), so the whole cluster answers that
  // pair with ST_TIMEOUT and takes the next one together.
  auto load = [&](int s) -> bool {
    uint32_t h0, l0;
    for (;;) {
      if (r == 0 && threadIdx.x < C) {
        const uint32_t k = __shfl_sync(0xFFFFFFFFu >> (32 - C), threadIdx.x == 0 ? atomicAdd(a.queue, 1u) : 0u, 0);
        const uint32_t ad = (uint32_t)__cvta_generic_to_shared(&ck.next);
        uint32_t ra;
        asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(ad), "r"(threadIdx.x));
        asm volatile("st.shared::cluster.u32 [%0], %1;" :: "r"(ra), "r"(k) : "memory");
      }
      cluster_sync_all();
      const uint32_t k = ck.next;
      cluster_sync_all();                             // everyone has read next before it changes
      if (k >= a.npairs) return false;
      ++taken;
      if (threadIdx.x == 0) {
        ss.pi[s] = a.order[k];
        ss.d[s] = a.pairs[ss.pi[s]];
        const uint32_t nq = ss.d[s].nq;
        ck.nloc[s] = j0 >= nq ? 0u : (nq - j0 < per ? nq - j0 : per);
      }
      __syncthreads();
      const PairDesc& d = ss.d[s];
      const uint32_t nloc = ck.nloc[s];
      uint32_t* ts = tS + (size_t)s * per;
      uint32_t* u0 = scr + (size_t)s * 4 * NQS;
      const ModConst* my = a.mods + j0;
      const bool staged = residues<T>(a.limbs + d.u_off, d.u_len, my, nloc, ts, stg, L <= 30);
      const bool ok = residues<T>(a.limbs + d.v_off, d.v_len, my, nloc, acc2, stg, L <= 30) && staged;
      h0 = 0xFFFFFFFFu;
      l0 = 0xFFFFFFFFu;
      for (uint32_t j = threadIdx.x; j < nloc; j += T) {
        const ModConst c = my[j];
        const uint32_t u = ts[j], v = acc2[j];
        u0[j0 + j] = u;
        u0[NQS + j0 + j] = v;
        const uint32_t t = t_init(u, v, c.q, c.qinv);
        ts[j] = t;
        uint32_t h, l;
        t_key(t, c.q, h, l);
        if (key_less(h, l, h0, l0)) { h0 = h; l0 = l; }
      }
      if (threadIdx.x == 32u * s) {
        ss.lu[s] = bound_init(a.limbs + d.u_off, d.u_len);
        ss.lv[s] = bound_init(a.limbs + d.v_off, d.v_len);
      }
      if (!ok) h0 = l0 = 0u;
      block_min_key<T>(h0, l0, rs, bparity);
      cluster_min_key<T>(h0, l0, cs, rparity, [] {});
      if (h0 != 0u || l0 != 0u) break;
      if (r == 0 && threadIdx.x == 0) {
        a.status[ss.pi[s]] = ST_TIMEOUT;
        a.count[ss.pi[s]] = 0;
        a.iters[ss.pi[s]] = 0;
      }
      __syncthreads();
    }
    const PairDesc& d = ss.d[s];
    uint32_t p0;
    int32_t b0;
    key_pair(h0, l0, p0, b0);
    put(p, s, p0);
    put(b, s, b0);
    put(rem, s, (int)d.nq);
    put(ubits, s, ((int)d.u_len + 1) * 32);
    put(vbits, s, ((int)d.v_len + 1) * 32);
    put(iters, s, 0u);
    return true;
  };

#pragma unroll 1
  for (int s = 0; s < K; ++s)
    if (load(s)) { valid |= 1u << s; active |= 1u << s; }

  for (;;) {
    const uint32_t done = valid & ~active;
#pragma unroll 1
    for (int s = 0; s < K; ++s) {
      if (!((done >> s) & 1u)) continue;
      const uint32_t pi = ss.pi[s];
      const uint32_t it = pick(iters, s);
      if (threadIdx.x == 0 && r == 0) a.iters[pi] = it;
      if ((redux >> s) & 1u) {
        if (threadIdx.x == 0 && r == 0) { a.status[pi] = ST_REDUX; a.count[pi] = 0; }
      } else {
        uint32_t* u0 = scr + (size_t)s * 4 * NQS;
        finish_pair<T, SYNC_CLUSTER>(a.mods, ss.d[s], L, j0, ck.nloc[s], tS + (size_t)s * per, rs, rparity, repoch,
                                     gcs, u0 + j0, u0 + NQS + j0, reinterpret_cast<const int2*>(u0 + 2 * (size_t)NQS),
                                     it, pick(rem, s), ss.lu[s], ss.lv[s], a.digits, a.count + pi, a.status + pi,
                                     a.inv, smem, acc2);
      }
      cluster_sync_all();                             // the slot's scratch is free in every CTA
      valid &= ~(1u << s);
      redux &= ~(1u << s);
      if (load(s)) { valid |= 1u << s; active |= 1u << s; }
    }
    if (!valid) break;

#pragma unroll
    for (int s = 0; s < K; ++s) {
      if (!((active >> s) & 1u)) continue;
      if (b[s] == MOD_INFINITY) { active &= ~(1u << s); continue; }
      if (threadIdx.x == 32u * s) {
        if (r == 0) {
          int2* hist = reinterpret_cast<int2*>(scr + (size_t)s * 4 * NQS + 2 * (size_t)NQS);
          hist[iters[s]] = make_int2((int)p[s], b[s]);
        }
        bound_step(ss.lu[s], ss.lv[s], p[s], b[s]);
      }
      ++iters[s];
      rem[s] -= 1;
      const uint32_t ab = b[s] < 0 ? 0u - (uint32_t)b[s] : (uint32_t)b[s];
      const int tbits = ubits[s] - (L - 1) + __ffs((int)ab);
      ubits[s] = vbits[s];
      vbits[s] = tbits;
      if (rem[s] * (L - 2) <= ubits[s]) { redux |= 1u << s; active &= ~(1u << s); }
    }
    if (!active) continue;

    uint32_t nmax = 0;
#pragma unroll
    for (int s = 0; s < K; ++s) {
      if ((active >> s) & 1u) nmax = max(nmax, ck.nloc[s]);
      kh[s] = kl[s] = 0xFFFFFFFFu;
    }
    for (uint32_t j = threadIdx.x; j < nmax; j += T) {
      uint32_t m = 0, tv[K];
#pragma unroll
      for (int s = 0; s < K; ++s) {
        const bool on = ((active >> s) & 1u) && j < ck.nloc[s];
        m |= (uint32_t)on << s;
        tv[s] = on ? tS[(size_t)s * per + j] : T_RETIRED;
      }
      if (!m) continue;
      const ModConst c = a.mods[j0 + j];
      t_update_k<K>(tv, c, p, b, m);
#pragma unroll
      for (int s = 0; s < K; ++s) {
        if (!((m >> s) & 1u)) continue;
        tS[(size_t)s * per + j] = tv[s];
        uint32_t h, l;
        t_key(tv[s], c.q, h, l);
        if (key_less(h, l, kh[s], kl[s])) { kh[s] = h; kl[s] = l; }
      }
    }
    cluster_min_keys<T, K>(kh, kl, ss, ck, kparity, cparity);
#pragma unroll
    for (int s = 0; s < K; ++s)
      if ((active >> s) & 1u) key_pair(kh[s], kl[s], p[s], b[s]);
  }
  cluster_sync_all();   // no CTA leaves while others may still address its shared memory
  cta_end(a, taken);
}

// One pair over a cooperative grid of GRID_THREADS-thread CTAs; CTA c owns moduli
// [c * per_cta, min(nq, (c + 1) * per_cta)).
template <int T>
__global__ void __launch_bounds__(T) grid_kernel(const GridArgs a)
{
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ RedSmem rs;
  __shared__ unsigned long long stage_bar[2];
  __shared__ uint32_t stage_state;
  const Stage stg{smem, stage_bar, &stage_state, blockIdx.x == a.stage_fail};   // at dynamic smem start
  stage_init(stg);
  const uint32_t nq = a.pair.nq;
  const uint32_t j0 = blockIdx.x * a.per_cta;
  const uint32_t nloc = j0 >= nq ? 0u : (nq - j0 < a.per_cta ? nq - j0 : a.per_cta);
  uint32_t* st = smem + STAGE_SMEM_WORDS;
  uint32_t* acc2 = st + a.per_cta;
  uint32_t* u0 = a.scratch + j0;
  uint32_t* v0 = a.scratch + nq + j0;
  int2* hist = reinterpret_cast<int2*>(a.scratch + 2 * (size_t)nq);
  run_pair<T, SYNC_GRID>(a.limbs, a.pair, a.mods, a.L, j0, nloc, st, acc2, stg, rs, u0, v0, hist,
                               a.sync, a.digits, a.count, a.iters, a.status, a.inv);
}

// One pair over a thread-block cluster (up to 16 CTAs, one per SM); CTA r owns moduli
// [r * per_cta, min(nq, (r + 1) * per_cta)).  Pivot keys travel through distributed shared
// memory; each reduction is one hardware cluster barrier (no global-memory round trip).
template <int T>
__global__ void __launch_bounds__(T) cluster_kernel(const GridArgs a)
{
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ RedSmem rs;
  __shared__ ClusterSmem cs;
  __shared__ unsigned long long stage_bar[2];
  __shared__ uint32_t stage_state;
  const Stage stg{smem, stage_bar, &stage_state, blockIdx.x == a.stage_fail};   // at dynamic smem start
  stage_init(stg);
  const uint32_t nq = a.pair.nq;
  const uint32_t j0 = cluster_rank() * a.per_cta;
  const uint32_t nloc = j0 >= nq ? 0u : (nq - j0 < a.per_cta ? nq - j0 : a.per_cta);
  uint32_t* st = smem + STAGE_SMEM_WORDS;
  uint32_t* acc2 = st + a.per_cta;
  uint32_t* u0 = a.scratch + j0;
  uint32_t* v0 = a.scratch + nq + j0;
  int2* hist = reinterpret_cast<int2*>(a.scratch + 2 * (size_t)nq);
  cluster_sync_all();   // every CTA of the cluster is running before remote stores begin
  run_pair<T, SYNC_CLUSTER>(a.limbs, a.pair, a.mods, a.L, j0, nloc, st, acc2, stg, rs, u0, v0, hist,
                            reinterpret_cast<GridSync*>(&cs), a.digits, a.count, a.iters, a.status, a.inv);
  cluster_sync_all();   // no CTA leaves while others may still address its shared memory
}

// One pair over a cooperative grid of thread-block clusters: CTA b owns moduli
// [b * per_cta, ...); pivot keys meet inside each cluster through DSMEM and only one
// leader per cluster joins the global exchange (fewer atomics on one address than one per
// CTA).
template <int T>
__global__ void __launch_bounds__(T) cgrid_kernel(const GridArgs a)
{
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ RedSmem rs;
  __shared__ CGridSmem cg;
  __shared__ unsigned long long stage_bar[2];
  __shared__ uint32_t stage_state;
  const Stage stg{smem, stage_bar, &stage_state, blockIdx.x == a.stage_fail};   // at dynamic smem start
  stage_init(stg);
  const uint32_t nq = a.pair.nq;
  const uint32_t j0 = blockIdx.x * a.per_cta;
  const uint32_t nloc = j0 >= nq ? 0u : (nq - j0 < a.per_cta ? nq - j0 : a.per_cta);
  uint32_t* st = smem + STAGE_SMEM_WORDS;
  uint32_t* acc2 = st + a.per_cta;
  uint32_t* u0 = a.scratch + j0;
  uint32_t* v0 = a.scratch + nq + j0;
  int2* hist = reinterpret_cast<int2*>(a.scratch + 2 * (size_t)nq);
  if (threadIdx.x == 0) cg.g = a.sync;
  __syncthreads();
  cluster_sync_all();   // every CTA of the cluster is running before remote stores begin
  run_pair<T, SYNC_CGRID>(a.limbs, a.pair, a.mods, a.L, j0, nloc, st, acc2, stg, rs, u0, v0, hist,
                          reinterpret_cast<GridSync*>(&cg), a.digits, a.count, a.iters, a.status, a.inv);
  cluster_sync_all();   // no CTA leaves while others may still address its shared memory
}

// Persistent batched kernel for pairs too large for one CTA: each thread-block cluster of
// C CTAs takes the next pair of the queue and computes it with the cluster path above
// (pair moduli split into C contiguous ranges).  The queue is popped by CTA 0 of the
// cluster, which writes the index into every CTA's shared memory.  Scratch per cluster:
// u0[nq_max], v0[nq_max], hist[2 * nq_max].
template <int T>
__global__ void __launch_bounds__(T) cluster_batch_kernel(const BatchArgs a)
{
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ RedSmem rs;
  __shared__ ClusterSmem cs;
  __shared__ uint32_t next;
  __shared__ unsigned long long stage_bar[2];
  __shared__ uint32_t stage_state;
  const Stage stg{smem, stage_bar, &stage_state, blockIdx.x == a.stage_fail};   // at dynamic smem start
  stage_init(stg);
  const uint32_t C = cluster_size(), r = cluster_rank();
  const uint32_t per_max = (a.nq_max + C - 1) / C;
  uint32_t* st = smem + STAGE_SMEM_WORDS;
  uint32_t* acc2 = st + per_max;
  uint32_t* scr = a.scratch + (size_t)(blockIdx.x / C) * a.scratch_words;
  cta_begin(a);
  uint32_t taken = 0;
  cluster_sync_all();
  for (;;) {
    if (r == 0 && threadIdx.x < C) {
      const uint32_t k = __shfl_sync(0xFFFFFFFFu >> (32 - C), threadIdx.x == 0 ? atomicAdd(a.queue, 1u) : 0u, 0);
      const uint32_t ad = (uint32_t)__cvta_generic_to_shared(&next);
      uint32_t ra;
      asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(ad), "r"(threadIdx.x));
      asm volatile("st.shared::cluster.u32 [%0], %1;" :: "r"(ra), "r"(k) : "memory");
    }
    cluster_sync_all();
    const uint32_t k = next;
    if (k >= a.npairs) break;
    ++taken;
    const uint32_t pi = a.order[k];
    const PairDesc d = a.pairs[pi];
    const uint32_t per = (d.nq + C - 1) / C;
    const uint32_t j0 = r * per;
    const uint32_t nloc = j0 >= d.nq ? 0u : (d.nq - j0 < per ? d.nq - j0 : per);
    run_pair<T, SYNC_CLUSTER>(a.limbs, d, a.mods, a.L, j0, nloc, st, acc2, stg, rs, scr + j0, scr + d.nq + j0,
                              reinterpret_cast<int2*>(scr + 2 * (size_t)d.nq), reinterpret_cast<GridSync*>(&cs),
                              a.digits, a.count + pi, a.iters + pi, a.status + pi, a.inv);
    cluster_sync_all();   // every CTA is done with `next` and with the pair's scratch
  }
  cluster_sync_all();     // no CTA leaves while others may still address its shared memory
  cta_end(a, taken);
}

// Integer-pipe microbenchmark: eight independent IMAD chains per thread.
__global__ void __launch_bounds__(256) int_peak_kernel(uint32_t* out, int iters)
{
  uint32_t a0 = threadIdx.x, a1 = a0 ^ 1u, a2 = a0 ^ 2u, a3 = a0 ^ 3u;
  uint32_t a4 = a0 ^ 4u, a5 = a0 ^ 5u, a6 = a0 ^ 6u, a7 = a0 ^ 7u;
  const uint32_t c = blockIdx.x | 1u;
  uint32_t m = 0x9E3779B9u ^ (uint32_t)iters;
#pragma unroll 4
  for (int i = 0; i < iters; ++i) {
    a0 = a0 * m + c; a1 = a1 * m + c; a2 = a2 * m + c; a3 = a3 * m + c;
    a4 = a4 * m + c; a5 = a5 * m + c; a6 = a6 * m + c; a7 = a7 * m + c;
  }
  if ((a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7) == 0x2545F491u) out[0] = 1u;
}

__global__ void __launch_bounds__(256) gridsync_init_kernel(GridSync* gs, unsigned long long timeout_ns,
                                                             uint32_t withhold)
{
  for (uint32_t i = threadIdx.x; i < 2u * MAX_GRID_CTAS; i += blockDim.x) (&gs->keys[0][0])[i] = 0ull;
  if (threadIdx.x < 32u) (&gs->bcast[0][0])[threadIdx.x] = 0ull;
  if (threadIdx.x == 0) {
    gs->slot[0] = gs->slot[1] = gs->slot[2] = ~0ull;
    gs->arrive = 0u;
    gs->error = 0u;
    gs->withhold_cta = withhold;
    gs->timeout_ns = timeout_ns;
  }
}

cudaError_t launch_gridsync_init(GridSync* gs, unsigned long long timeout_ns, uint32_t withhold, cudaStream_t s)
{
  gridsync_init_kernel<<<1, 256, 0, s>>>(gs, timeout_ns, withhold);
  return cudaGetLastError();
}

cudaError_t launch_int_peak(uint32_t* out, int blocks, int iters, cudaStream_t s)
{
  int_peak_kernel<<<blocks, 256, 0, s>>>(out, iters);
  return cudaGetLastError();
}

// tab[i * n + j] = R / q_i mod q_j (Montgomery form of q_i^{-1}); moduli of one width
// satisfy q_i < 2 q_j, so q_i mod q_j is one conditional subtraction.
__global__ void __launch_bounds__(256) build_invtab_kernel(const ModConst* __restrict__ mods, uint32_t n,
                                                           uint32_t* __restrict__ tab)
{
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t i = blockIdx.y;
  if (j >= n) return;
  const ModConst c = mods[j];
  const uint32_t p = mods[i].q;
  uint32_t v = 0u;
  if (i != j) v = inv_mod(redc((uint64_t)(p > c.q ? p - c.q : p), c.q, c.qinv), c.q, c.qinv);
  tab[(size_t)i * n + j] = v;
}

cudaError_t launch_build_invtab(const ModConst* mods, uint32_t n, uint32_t* tab, cudaStream_t s)
{
  build_invtab_kernel<<<dim3((n + 255) / 256, n), 256, 0, s>>>(mods, n, tab);
  return cudaGetLastError();
}

// ------------------------------------------------------------------- launchers ----

size_t batch_smem_bytes(int /*threads*/, int k, uint32_t nq_max)
{
  // K-slot kernels: K state arrays, the set-up / re-layout buffer and two 16-bit position arrays
  return sizeof(uint32_t) * ((size_t)(k > 1 ? k + 2 : 2) * nq_max + STAGE_SMEM_WORDS);
}

template <bool NARROW>
static const void* batchk_fn_for(int threads, int k)
{
  if (k == 2) {
    switch (threads) {
      case 256: return reinterpret_cast<const void*>(&batchk_kernel<256, 2, NARROW>);
      case 512: return reinterpret_cast<const void*>(&batchk_kernel<512, 2, NARROW>);
      case 1024: return reinterpret_cast<const void*>(&batchk_kernel<1024, 2, NARROW>);
      default: return nullptr;
    }
  }
  if (k == 4) {
    switch (threads) {
      case 256: return reinterpret_cast<const void*>(&batchk_kernel<256, 4, NARROW>);
      case 512: return reinterpret_cast<const void*>(&batchk_kernel<512, 4, NARROW>);
      case 1024: return reinterpret_cast<const void*>(&batchk_kernel<1024, 4, NARROW>);   // 64 registers, 32 warps/SM
      default: return nullptr;
    }
  }
  if (k == 8) {
    switch (threads) {
      case 512: return reinterpret_cast<const void*>(&batchk_kernel<512, 8, NARROW>);
      case 1024: return reinterpret_cast<const void*>(&batchk_kernel<1024, 8, NARROW>);
      default: return nullptr;
    }
  }
  return nullptr;
}

// narrow: the context's moduli are below 2^30 (width <= 30)
static const void* batch_fn_for(int threads, int k, bool narrow)
{
  if (k == 1) {
    switch (threads) {
      case 256: return reinterpret_cast<const void*>(&batch_kernel<256>);
      case 512: return reinterpret_cast<const void*>(&batch_kernel<512>);
      case 1024: return reinterpret_cast<const void*>(&batch_kernel<1024>);
      default: return nullptr;
    }
  }
  return narrow ? batchk_fn_for<true>(threads, k) : batchk_fn_for<false>(threads, k);
}

cudaError_t batch_max_blocks_per_sm(int threads, int k, bool narrow, size_t smem, int* blocks)
{
  const void* fn = batch_fn_for(threads, k, narrow);
  if (!fn) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, fn, threads, smem);
}

static const void* ring_fn_for(int threads, int k, bool narrow)
{
  if (threads == 1024 && k == 4)
    return narrow ? reinterpret_cast<const void*>(&batchk_kernel<1024, 4, true, true>)
                  : reinterpret_cast<const void*>(&batchk_kernel<1024, 4, false, true>);
  if (threads == 1024 && k == 2)
    return narrow ? reinterpret_cast<const void*>(&batchk_kernel<1024, 2, true, true>)
                  : reinterpret_cast<const void*>(&batchk_kernel<1024, 2, false, true>);
  if (threads == 512 && k == 4)
    return narrow ? reinterpret_cast<const void*>(&batchk_kernel<512, 4, true, true>)
                  : reinterpret_cast<const void*>(&batchk_kernel<512, 4, false, true>);
  if (threads == 512 && k == 2)
    return narrow ? reinterpret_cast<const void*>(&batchk_kernel<512, 2, true, true>)
                  : reinterpret_cast<const void*>(&batchk_kernel<512, 2, false, true>);
  return nullptr;
}

cudaError_t launch_ring(const BatchArgs& a, int threads, int k, int grid, size_t smem, cudaStream_t s)
{
  const void* fn = ring_fn_for(threads, k, a.L <= 30);
  if (!fn || !a.ring) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<BatchArgs*>(&a)};
  return cudaLaunchKernel(fn, dim3(grid), dim3(threads), args, smem, s);
}

cudaError_t launch_batch(const BatchArgs& a, int threads, int k, int grid, size_t smem, cudaStream_t s, bool after)
{
  const void* fn = batch_fn_for(threads, k, a.L <= 30);
  if (!fn) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<BatchArgs*>(&a)};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = after ? 1 : 0;
  return cudaLaunchKernelExC(&cfg, fn, args);
}

static const void* cluster_fn(int threads)
{
  switch (threads) {
    case 256: return reinterpret_cast<const void*>(&cluster_kernel<256>);
    case 512: return reinterpret_cast<const void*>(&cluster_kernel<512>);
    case 1024: return reinterpret_cast<const void*>(&cluster_kernel<1024>);
    default: return nullptr;
  }
}

static const void* cluster_batch_fn(int threads)
{
  switch (threads) {
    case 256: return reinterpret_cast<const void*>(&cluster_batch_kernel<256>);
    case 512: return reinterpret_cast<const void*>(&cluster_batch_kernel<512>);
    case 1024: return reinterpret_cast<const void*>(&cluster_batch_kernel<1024>);
    default: return nullptr;
  }
}

static cudaLaunchConfig_t cluster_config(int ctas, int threads, int csize, size_t smem, cudaStream_t s,
                                         cudaLaunchAttribute* attr)
{
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ctas);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

static cudaError_t prepare_cluster_fn(const void* fn, int csize, size_t smem)
{
  if (!fn || csize < 1 || csize > MAX_CLUSTER) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess && csize > 8) e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  return e;
}

static const void* cluster_batch_fn_k(int threads, int k)
{
  if (k == 1) return cluster_batch_fn(threads);
  if (k == 2) {
    switch (threads) {
      case 256: return reinterpret_cast<const void*>(&cluster_batchk_kernel<256, 2>);
      case 512: return reinterpret_cast<const void*>(&cluster_batchk_kernel<512, 2>);
      case 1024: return reinterpret_cast<const void*>(&cluster_batchk_kernel<1024, 2>);
      default: return nullptr;
    }
  }
  if (k == 4) {
    switch (threads) {
      case 256: return reinterpret_cast<const void*>(&cluster_batchk_kernel<256, 4>);
      case 512: return reinterpret_cast<const void*>(&cluster_batchk_kernel<512, 4>);
      case 1024: return reinterpret_cast<const void*>(&cluster_batchk_kernel<1024, 4>);
      default: return nullptr;
    }
  }
  return nullptr;
}

size_t cluster_batch_smem_bytes(int csize, uint32_t nq_max, int k)
{
  const size_t per = (nq_max + csize - 1) / csize;
  return sizeof(uint32_t) * ((size_t)(k > 1 ? k + 1 : 2) * per + STAGE_SMEM_WORDS);
}

cudaError_t cluster_batch_max_clusters(int threads, int k, int csize, size_t smem, int* clusters)
{
  const void* fn = cluster_batch_fn_k(threads, k);
  cudaError_t e = prepare_cluster_fn(fn, csize, smem);
  if (e != cudaSuccess) return e;
  cudaLaunchAttribute attr[1];
  const cudaLaunchConfig_t cfg = cluster_config(csize, threads, csize, smem, nullptr, attr);
  return cudaOccupancyMaxActiveClusters(clusters, fn, &cfg);
}

cudaError_t launch_cluster(const GridArgs& a, int threads, int ctas, size_t smem, cudaStream_t s)
{
  const void* fn = cluster_fn(threads);
  cudaError_t e = prepare_cluster_fn(fn, ctas, smem);
  if (e != cudaSuccess) return e;
  cudaLaunchAttribute attr[1];
  const cudaLaunchConfig_t cfg = cluster_config(ctas, threads, ctas, smem, s, attr);
  void* args[] = {const_cast<GridArgs*>(&a)};
  return cudaLaunchKernelExC(&cfg, fn, args);
}

cudaError_t launch_cluster_batch(const BatchArgs& a, int threads, int k, int csize, int clusters, size_t smem,
                                 cudaStream_t s, bool after)
{
  const void* fn = cluster_batch_fn_k(threads, k);
  cudaError_t e = prepare_cluster_fn(fn, csize, smem);
  if (e != cudaSuccess) return e;
  cudaLaunchAttribute attr[2];
  cudaLaunchConfig_t cfg = cluster_config(clusters * csize, threads, csize, smem, s, attr);
  if (after) {
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.numAttrs = 2;
  }
  void* args[] = {const_cast<BatchArgs*>(&a)};
  return cudaLaunchKernelExC(&cfg, fn, args);
}

static const void* cgrid_fn(int threads)
{
  switch (threads) {
    case 256: return reinterpret_cast<const void*>(&cgrid_kernel<256>);
    case 512: return reinterpret_cast<const void*>(&cgrid_kernel<512>);
    case 1024: return reinterpret_cast<const void*>(&cgrid_kernel<1024>);
    default: return nullptr;
  }
}

cudaError_t cgrid_max_clusters(int threads, int csize, size_t smem, int* clusters)
{
  const void* fn = cgrid_fn(threads);
  cudaError_t e = prepare_cluster_fn(fn, csize, smem);
  if (e != cudaSuccess) return e;
  cudaLaunchAttribute attr[1];
  const cudaLaunchConfig_t cfg = cluster_config(csize, threads, csize, smem, nullptr, attr);
  return cudaOccupancyMaxActiveClusters(clusters, fn, &cfg);
}

cudaError_t launch_cgrid(const GridArgs& a, int threads, int csize, int clusters, size_t smem, cudaStream_t s)
{
  const void* fn = cgrid_fn(threads);
  cudaError_t e = prepare_cluster_fn(fn, csize, smem);
  if (e != cudaSuccess) return e;
  cudaLaunchAttribute attr[2];
  cudaLaunchConfig_t cfg = cluster_config(clusters * csize, threads, csize, smem, s, attr);
  attr[1].id = cudaLaunchAttributeCooperative;   // all clusters resident at once
  attr[1].val.cooperative = 1;
  cfg.numAttrs = 2;
  void* args[] = {const_cast<GridArgs*>(&a)};
  return cudaLaunchKernelExC(&cfg, fn, args);
}

size_t grid_smem_bytes(uint32_t per_cta)
{
  return sizeof(uint32_t) * (2 * (size_t)per_cta + STAGE_SMEM_WORDS);
}

static const void* grid_fn(int threads)
{
  switch (threads) {
    case 256: return reinterpret_cast<const void*>(&grid_kernel<256>);
    case 512: return reinterpret_cast<const void*>(&grid_kernel<512>);
    case 1024: return reinterpret_cast<const void*>(&grid_kernel<1024>);
    default: return nullptr;
  }
}

cudaError_t grid_max_blocks_per_sm(int threads, size_t smem, int* blocks)
{
  const void* fn = grid_fn(threads);
  if (!fn) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, fn, threads, smem);
}

cudaError_t launch_grid(const GridArgs& a, int threads, int grid, size_t smem, cudaStream_t s)
{
  const void* fn = grid_fn(threads);
  if (!fn) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<GridArgs*>(&a)};
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(threads), args, smem, s);
}

}  // namespace mgcd

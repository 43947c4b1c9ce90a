// mgcd_pair.cuh -- the per-pair gcd body shared by the kernels (CTA scope or cooperative
// grid): reductions, residues, the reduction loop, replay and recovery.
// See mgcd_kernels.cu for the stage overview.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mgcd_device.cuh"
#include "mgcd_internal.h"

namespace mgcd {

constexpr int CHUNK = 1024;  // operand limbs staged per residue pass
constexpr uint32_t REPLAY_CHUNK = 512;   // history entries per replay chunk (2 x 512 words of
                                         // the operand staging area, which every kernel has)

// How the CTAs that share one pair synchronise.
enum SyncMode : int {
  SYNC_CTA = 0,      // the pair lives in one CTA
  SYNC_CLUSTER = 1,  // the pair spans a thread-block cluster: DSMEM exchange + barrier.cluster
  SYNC_GRID = 2,     // the pair spans a cooperative grid: global-memory exchange, bounded wait
  SYNC_CGRID = 3     // a cooperative grid of clusters: DSMEM inside each cluster, one
                     // leader per cluster in the global exchange
};

struct RedSmem {
  unsigned long long key[2][32];  // per-warp minima, double-buffered by parity
  unsigned long long bcast;       // grid mode: the grid-wide result
  uint32_t bad;                   // grid mode: a bounded wait expired
  uint32_t cert;                  // the result could not be certified (more moduli needed)
};

// Cluster mode: every warp's minimum lands in every CTA of the cluster, so one cluster
// barrier per reduction suffices.  Double-buffered by parity.
struct ClusterSmem {
  unsigned long long key[2][MAX_CLUSTER][32];
};

// Cluster-grid mode: the global exchange state and, per CTA, the cluster's slots.
struct CGridSmem {
  GridSync* g;                                  // global exchange (one arrival per cluster)
  unsigned long long key[2][MAX_CLUSTER];       // each CTA's minimum, double-buffered
  unsigned long long res[2];                    // the grid-wide minimum, from the leader
  uint32_t bad[2];                              // the leader's wait expired
};

__device__ __forceinline__ uint32_t cluster_rank()
{
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ uint32_t cluster_size()
{
  uint32_t n;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(n));
  return n;
}

__device__ __forceinline__ void cluster_sync_all()
{
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// The two halves of cluster_sync_all, for work that overlaps the wait.
__device__ __forceinline__ void cluster_arrive()
{
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}

__device__ __forceinline__ void cluster_wait()
{
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Stores v at the same shared-memory offset as *local in CTA `rank` of this cluster.
__device__ __forceinline__ void st_cluster_u64(unsigned long long* local, uint32_t rank, unsigned long long v)
{
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(local);
  uint32_t ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
  asm volatile("st.shared::cluster.u64 [%0], %1;" :: "r"(ra), "l"(v) : "memory");
}

// Minimum over the whole cluster: each warp's minimum is written into every CTA's
// slots, one cluster barrier, then each warp reduces all slots locally.
template <int T, class F>
__device__ __forceinline__ void cluster_min_key(uint32_t& hi, uint32_t& lo, ClusterSmem& cs, uint32_t& parity,
                                                F&& during)
{
  constexpr int NW = T / 32;
  const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
  const uint32_t me = cluster_rank(), nc = cluster_size();
  warp_min_key(hi, lo);
  const unsigned long long k = ((unsigned long long)hi << 32) | lo;
  if (lane < nc) st_cluster_u64(&cs.key[parity][me][w], lane, k);   // lane r writes into CTA r
  cluster_arrive();
  during();
  cluster_wait();
  unsigned long long m = ~0ull;
  for (uint32_t e = lane; e < nc * NW; e += 32) {
    const unsigned long long x = cs.key[parity][e / NW][e % NW];
    m = x < m ? x : m;
  }
  hi = (uint32_t)(m >> 32);
  lo = (uint32_t)m;
  warp_min_key(hi, lo);
  parity ^= 1u;
}

static __device__ __forceinline__ unsigned long long globaltimer_ns()
{
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Arrival that publishes this thread's earlier writes (the atomic min, CTA 0's slot reset)
// to any thread that acquires the counter: one fire-and-forget reduction, no fence.
static __device__ __forceinline__ void red_release_add_u32(unsigned int* p, unsigned int v)
{
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

static __device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p)
{
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

static __device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p)
{
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

static __device__ __forceinline__ unsigned int ld_relaxed_u32(const unsigned int* p)
{
  unsigned int v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// The CTA that writes a pair's results: the only one (CTA scope), cluster rank 0, or CTA 0
// of the cooperative grid.
template <int MODE>
__device__ __forceinline__ bool lead_cta()
{
  if constexpr (MODE == SYNC_CTA) return true;
  else if constexpr (MODE == SYNC_CLUSTER) return cluster_rank() == 0;
  else return blockIdx.x == 0;   // the grid's first CTA (also in the cluster grid)
}

// Lexicographic (hi, lo) minimum over the CTA; every thread gets the result.
// One __syncthreads; the two slot buffers alternate so the next call cannot overwrite
// slots still being read.
template <int T>
__device__ __forceinline__ void block_min_key(uint32_t& hi, uint32_t& lo, RedSmem& rs, uint32_t& parity)
{
  constexpr int NW = T / 32;
  warp_min_key(hi, lo);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) rs.key[parity][w] = ((unsigned long long)hi << 32) | lo;
  __syncthreads();
  const unsigned long long k = (lane < NW) ? rs.key[parity][lane] : ~0ull;
  hi = (uint32_t)(k >> 32);
  lo = (uint32_t)k;
  warp_min_key(hi, lo);
  parity ^= 1u;
}

// Minimum over the CTA and, with several CTAs, over the cluster (DSMEM + cluster barrier),
// the cooperative grid (leader exchange over tagged slots) or the cluster grid (atomic
// minimum and arrival counter per cluster leader); the grid protocols are described at
// GridSync.  Every wait is bounded by timeout_ns; returns false if one expired (the grid
// then unwinds; the host sees ST_TIMEOUT).
// `during()` is called by every thread while the CTA waits for the others (after its own
// contribution is out), so per-iteration bookkeeping of one thread (BOUND_THREAD, not the
// thread that carries the CTA's part of the exchange) overlaps the exchange.
constexpr uint32_t BOUND_THREAD = 32;

// 63-bit form of a key for the tagged grid exchange, in the same order: |value| keys stay
// below 2^31 - 1, MOD_INFINITY (0x80000000) and "no key" (0xFFFFFFFF, 0xFFFFFFFF) share the
// high word 2^31 - 1 and differ in the low word.  Bit 63 carries the exchange tag.
constexpr unsigned long long KEY_TAG = 1ull << 63;

__device__ __forceinline__ unsigned long long pack_key(uint32_t hi, uint32_t lo)
{
  const uint32_t h = hi >= 0x7FFFFFFFu ? 0x7FFFFFFFu : hi;
  return ((unsigned long long)h << 32) | lo;
}

__device__ __forceinline__ void unpack_key(unsigned long long k, uint32_t& hi, uint32_t& lo)
{
  lo = (uint32_t)k;
  const uint32_t h = (uint32_t)(k >> 32) & 0x7FFFFFFFu;
  hi = h != 0x7FFFFFFFu ? h : (lo == 0xFFFFFFFFu ? 0xFFFFFFFFu : KEY_INF_HI);
}

__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v)
{
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" :: "l"(p), "l"(v) : "memory");
}

template <int T, int MODE, bool PUB = false, class F>
__device__ __forceinline__ bool reduce_min(uint32_t& hi, uint32_t& lo, RedSmem& rs, uint32_t& parity,
                                           GridSync* gs, uint32_t& epoch, F&& during)
{
  if constexpr (MODE == SYNC_CLUSTER) {
    ClusterSmem& cs = *reinterpret_cast<ClusterSmem*>(gs);
    const uint32_t nc = cluster_size();
    if (nc * (T / 32) <= 64) {
      cluster_min_key<T>(hi, lo, cs, parity, during);
      return true;
    }
    // Large clusters: the CTA's minimum first (one __syncthreads), then one key per CTA
    // into every CTA (slot [me][0] of the buffer chosen by the exchange count), one cluster
    // barrier, and a 16-entry reduction instead of one over every warp of the cluster.
    block_min_key<T>(hi, lo, rs, parity);
    const uint32_t cb = epoch & 1u, lane = threadIdx.x & 31u, me = cluster_rank();
    if (threadIdx.x < 32u && lane < nc) st_cluster_u64(&cs.key[cb][me][0], lane, ((unsigned long long)hi << 32) | lo);
    cluster_arrive();
    during();
    cluster_wait();
    const unsigned long long k = lane < nc ? cs.key[cb][lane][0] : ~0ull;
    hi = (uint32_t)(k >> 32);
    lo = (uint32_t)k;
    warp_min_key(hi, lo);
    epoch += 1u;
    return true;
  }
  if constexpr (MODE == SYNC_CTA) {
    during();
    block_min_key<T>(hi, lo, rs, parity);
    return true;
  }
  block_min_key<T>(hi, lo, rs, parity);
  if constexpr (MODE == SYNC_CGRID) {
    // CTA minima -> every CTA of the cluster (DSMEM), one cluster barrier; the cluster's
    // rank-0 thread 0 takes part in the global exchange (atomic min, release arrival,
    // bounded acquire wait) and stores the result into every CTA; one more cluster barrier.
    CGridSmem& cg = *reinterpret_cast<CGridSmem*>(gs);
    GridSync* g = cg.g;
    const uint32_t cb = epoch & 1u, lane = threadIdx.x & 31u, me = cluster_rank(), nc = cluster_size();
    if (threadIdx.x < 32u && lane < nc) st_cluster_u64(&cg.key[cb][me], lane, ((unsigned long long)hi << 32) | lo);
    cluster_sync_all();
    if (me == 0u && threadIdx.x < 32u) {
      unsigned long long k = lane < nc ? cg.key[cb][lane] : ~0ull;
      hi = (uint32_t)(k >> 32);
      lo = (uint32_t)k;
      warp_min_key(hi, lo);
      k = ((unsigned long long)hi << 32) | lo;
      unsigned long long res = ~0ull;
      uint32_t bad = 0;
      if (lane == 0) {
        const uint32_t cid = blockIdx.x / nc, ncl = gridDim.x / nc;
        const uint32_t s = epoch % 3u;
        if (cid != g->withhold_cta) {
          atomicMin(&g->slot[s], k);
          if (cid == 0) g->slot[(epoch + 1u) % 3u] = ~0ull;
          red_release_add_u32(&g->arrive, 1u);
        }
        const unsigned int target = (epoch + 1u) * ncl;
        const unsigned long long t0 = globaltimer_ns();
        while (ld_acquire_u32(&g->arrive) < target) {
          if (ld_relaxed_u32(&g->error)) { bad = 1; break; }
          if (globaltimer_ns() - t0 > g->timeout_ns) { atomicExch(&g->error, 1u); bad = 1; break; }
        }
        res = bad ? ~0ull : ld_relaxed_u64(&g->slot[s]);
      }
      __syncwarp();
      res = __shfl_sync(0xFFFFFFFFu, res, 0);
      bad = __shfl_sync(0xFFFFFFFFu, bad, 0);
      if (lane < nc) {
        st_cluster_u64(&cg.res[cb], lane, res);
        const uint32_t ad = (uint32_t)__cvta_generic_to_shared(&cg.bad[cb]);
        uint32_t ra;
        asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(ad), "r"(lane));
        asm volatile("st.shared::cluster.u32 [%0], %1;" :: "r"(ra), "r"(bad) : "memory");
      }
    }
    during();
    cluster_sync_all();
    const unsigned long long k = cg.res[cb];
    const bool ok = cg.bad[cb] == 0u;
    hi = (uint32_t)(k >> 32);
    lo = (uint32_t)k;
    epoch += 1u;
    return ok;
  } else {
    // Leader exchange (GridSync): tagged slots, relaxed stores and loads, bounded polls.
    // PUB adds release fences before the stores and acquire fences after the polls, for
    // exchanges that also publish data written before them.
    const uint32_t b = epoch & 1u;
    const unsigned long long tag = (unsigned long long)(((epoch >> 1) + 1u) & 1u) << 63;
    unsigned long long* const keys = gs->keys[b];
    unsigned long long k = pack_key(hi, lo);
    uint32_t bad = 0;
    if (blockIdx.x != 0) {
      if (threadIdx.x == 0) {
        if constexpr (PUB) __threadfence();
        if (blockIdx.x != gs->withhold_cta) st_relaxed_u64(keys + blockIdx.x, tag | k);
        const unsigned long long t0 = globaltimer_ns();
        unsigned long long v;
        for (;;) {
          v = ld_relaxed_u64(&gs->bcast[b][0]);
          if ((v & KEY_TAG) == tag) break;
          if (ld_relaxed_u32(&gs->error)) { bad = 1; break; }
          if (globaltimer_ns() - t0 > gs->timeout_ns) { atomicExch(&gs->error, 1u); bad = 1; break; }
        }
        if constexpr (PUB) __threadfence();
        rs.bcast = v & ~KEY_TAG;
        rs.bad = bad;
      }
      during();
      __syncthreads();
      k = rs.bcast;
      bad = rs.bad;
    } else {
      during();
      unsigned long long m = threadIdx.x == 0 ? k : ~0ull;
      const unsigned long long t0 = globaltimer_ns();
      for (uint32_t i = threadIdx.x == 0 ? T : threadIdx.x; i < gridDim.x && !bad; i += T) {
        unsigned long long v;
        for (;;) {
          v = ld_relaxed_u64(keys + i);
          if ((v & KEY_TAG) == tag) break;
          if (globaltimer_ns() - t0 > gs->timeout_ns) { atomicExch(&gs->error, 1u); bad = 1; break; }
        }
        v &= ~KEY_TAG;
        m = v < m ? v : m;
      }
      if constexpr (PUB) __threadfence();
      bad = __syncthreads_or(bad) ? 1u : 0u;
      uint32_t mh = (uint32_t)(m >> 32), ml = (uint32_t)m;
      block_min_key<T>(mh, ml, rs, parity);
      k = ((unsigned long long)mh << 32) | ml;
      if (threadIdx.x == 0 && !bad && blockIdx.x != gs->withhold_cta) {
        if constexpr (PUB) __threadfence();
        st_relaxed_u64(&gs->bcast[b][0], tag | k);
      }
    }
    unpack_key(k, hi, lo);
    epoch += 1u;
    return bad == 0;
  }
}

template <int T, int MODE, bool PUB = false>
__device__ __forceinline__ bool reduce_min(uint32_t& hi, uint32_t& lo, RedSmem& rs, uint32_t& parity,
                                           GridSync* gs, uint32_t& epoch)
{
  return reduce_min<T, MODE, PUB>(hi, lo, rs, parity, gs, epoch, [] {});
}

// ---- operand staging: bulk copies (the TMA engine, cp.async.bulk) into shared memory
//
// Two staging buffers of STAGE_WORDS words each at a 16-byte-aligned shared address (the
// start of the dynamic shared memory), each with an mbarrier that the copy completes.  A
// bulk copy needs 16-byte-aligned addresses and a size that is a multiple of 16 bytes, so
// a tile [lo, hi) of an operand is widened to the 16-byte bounds around it (at most 3
// limbs each side) and read from its offset inside the buffer.  The widened copy stays
// inside the limb buffer: its base is 16-byte aligned (pool allocation) and the plan pads
// it by 16 bytes.  Every wait is bounded.
constexpr int STAGE_WORDS = CHUNK + 8;               // one tile widened to 16-byte bounds
constexpr int STAGE_SMEM_WORDS = 2 * STAGE_WORDS;    // two buffers (the next tile in flight)
constexpr unsigned long long STAGE_TIMEOUT_NS = 1000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

struct Stage {
  uint32_t* buf;                 // 2 x STAGE_WORDS words, 16-byte aligned, shared
  unsigned long long* mbar;      // 2 mbarriers in shared memory; nullptr: plain loads
  uint32_t* state;               // shared: bit b = parity of buffer b's next phase;
                                 // STAGE_BROKEN once a wait ran out
  uint32_t inject;               // test hook: report a failure after staging normally
  uint32_t coherent;             // plain loads that bypass the non-coherent caches (operands in
                                 // host memory that the host rewrites between requests)
};
constexpr uint32_t STAGE_BROKEN = 0x80000000u;

// Once per kernel, by every thread, before the first residues().
__device__ __forceinline__ void stage_init(Stage s)
{
  if (s.mbar != nullptr && threadIdx.x == 0) {
    for (int b = 0; b < 2; ++b)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(s.mbar + b)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    *s.state = 0u;
  }
  __syncthreads();
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* m, uint32_t parity)
{
  uint32_t ok;
  asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
               "selp.u32 %0, 1, 0, p;\n\t}"
               : "=r"(ok) : "r"(smem_u32(m)), "r"(parity) : "memory");
  return ok != 0u;
}

// Waits (bounded) until phase `parity` of the mbarrier has completed.
__device__ __forceinline__ bool mbar_wait(unsigned long long* m, uint32_t parity)
{
  if (mbar_try_wait(m, parity)) return true;
  const unsigned long long t0 = globaltimer_ns();
  while (!mbar_try_wait(m, parity))
    if (globaltimer_ns() - t0 > STAGE_TIMEOUT_NS) return false;
  return true;
}

// Tile t (most significant first) of an n-limb operand: [lo, hi).
__device__ __forceinline__ void stage_tile(int t, int n, int& lo, int& hi)
{
  hi = n - t * CHUNK;
  lo = hi > CHUNK ? hi - CHUNK : 0;
}

// Thread 0: bulk copy of tile [lo, hi) of x, widened to 16-byte bounds, into buffer b.
__device__ __forceinline__ void stage_issue(const uint32_t* x, int lo, int hi, Stage s, int b)
{
  const uintptr_t ga = (uintptr_t)(x + lo) & ~(uintptr_t)15;
  const uintptr_t gb = ((uintptr_t)(x + hi) + 15) & ~(uintptr_t)15;
  const uint32_t bytes = (uint32_t)(gb - ga);                  // <= 4 (CHUNK + 6), multiple of 16
  const uint32_t m = smem_u32(s.mbar + b);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(m), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               :: "r"(smem_u32(s.buf + b * STAGE_WORDS)), "l"(ga), "r"(bytes), "r"(m) : "memory");
}

// One tile of Horner steps z' = REDC(z * (2^64 mod q) + limb), most significant limb last
// in `chunk`.  narrow (moduli below 2^30): z stays lazily in [0, 2q) in 32-bit arithmetic
// (z * r2 + limb < 2q^2 + 2^32 < q 2^32, so REDC without the final subtraction is below 2q).
__device__ __forceinline__ uint32_t horner_tile(uint32_t z, const uint32_t* chunk, int len, const ModConst& c,
                                                bool narrow)
{
  if (narrow) {
    for (int i = len - 1; i >= 0; --i) {
      const uint64_t t = (uint64_t)z * c.r2 + chunk[i];
      const uint32_t lo = (uint32_t)t, hi = (uint32_t)(t >> 32);
      z = hi + __umulhi(lo * c.qinv, c.q) + (lo != 0u);
    }
  } else {
    for (int i = len - 1; i >= 0; --i) z = redc((uint64_t)z * c.r2 + chunk[i], c.q, c.qinv);
  }
  return z;
}

// x mod q_j for the nloc moduli mods[0..nloc), into acc[] (shared).  Limbs are staged
// most-significant tile first; Horner in Montgomery form keeps z = y * 2^-32 where y is the
// residue of the limbs consumed so far: z' = REDC(z * (2^64 mod q) + limb).  narrow: the
// moduli are below 2^30 (z lazy until the final conversion, which is canonical).  Returns
// false if a staging wait ran out (after waiting, bounded, for the copy still in flight).
template <int T>
__device__ bool residues(const uint32_t* __restrict__ x, uint32_t n, const ModConst* __restrict__ mods,
                         uint32_t nloc, uint32_t* __restrict__ acc, Stage stg, bool narrow)
{
  for (uint32_t j = threadIdx.x; j < nloc; j += T) acc[j] = 0u;
  int nt = ((int)n + CHUNK - 1) / CHUNK;
  bool ok = true;
  if (stg.mbar == nullptr) {
    uint32_t* const chunk = stg.buf;
    for (int t = 0; t < nt; ++t) {
      int lo, hi;
      stage_tile(t, (int)n, lo, hi);
      __syncthreads();
      if (stg.coherent) {
        const volatile uint32_t* xv = x;
        for (int i = lo + (int)threadIdx.x; i < hi; i += T) chunk[i - lo] = xv[i];
      } else {
        for (int i = lo + (int)threadIdx.x; i < hi; i += T) chunk[i - lo] = __ldg(x + i);
      }
      __syncthreads();
      const int len = hi - lo;
      for (uint32_t j = threadIdx.x; j < nloc; j += T) acc[j] = horner_tile(acc[j], chunk, len, mods[j], narrow);
    }
  } else {
    __syncthreads();                   // the state word of the previous call is written
    uint32_t phase = *stg.state;       // bit b: the parity of buffer b's next phase
    if (phase & STAGE_BROKEN) nt = 0, ok = false;
    __syncthreads();                   // every thread read it before thread 0 issues
    if (threadIdx.x == 0 && nt > 0) {
      int lo, hi;
      stage_tile(0, (int)n, lo, hi);
      stage_issue(x, lo, hi, stg, 0);
    }
    for (int t = 0; t < nt; ++t) {
      const int b = t & 1;
      int lo, hi;
      stage_tile(t, (int)n, lo, hi);
      if (threadIdx.x == 0 && t + 1 < nt) {          // the other buffer was released by the
        int lo1, hi1;                                // barrier that ended tile t - 1
        stage_tile(t + 1, (int)n, lo1, hi1);
        stage_issue(x, lo1, hi1, stg, b ^ 1);
      }
      const bool got = mbar_wait(stg.mbar + b, (phase >> b) & 1u);
      phase ^= 1u << b;
      if (!__syncthreads_and(got)) {
        // a copy did not complete: wait (bounded) for the one issued into the other buffer;
        // the mbarrier phases are no longer known, so later calls fail at once
        if (t + 1 < nt) mbar_wait(stg.mbar + (b ^ 1), (phase >> (b ^ 1)) & 1u);
        ok = false;
        phase = STAGE_BROKEN;
        break;
      }
      const uint32_t* const chunk =
          stg.buf + b * STAGE_WORDS + (uint32_t)(((uintptr_t)(x + lo) & 15) >> 2);
      const int len = hi - lo;
      for (uint32_t j = threadIdx.x; j < nloc; j += T) acc[j] = horner_tile(acc[j], chunk, len, mods[j], narrow);
      __syncthreads();                 // buffer b is free for tile t + 2
    }
    if (threadIdx.x == 0) *stg.state = phase;
  }
  if (stg.inject) ok = false;
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < nloc; j += T) {
    const ModConst c = mods[j];
    acc[j] = redc((uint64_t)acc[j] * c.r2, c.q, c.qinv);
  }
  __syncthreads();
  return ok;
}

template <int T, int MODE>
__device__ void finish_pair(const ModConst* __restrict__ mods, const PairDesc& d, int L, uint32_t j0, uint32_t nloc,
                            uint32_t* st, RedSmem& rs, uint32_t& parity, uint32_t& epoch, GridSync* gs,
                            const uint32_t* u0g, const uint32_t* v0g, const int2* hist, uint32_t iters, int remaining,
                            long long lu, long long lv, mgcd_pair* digits, uint32_t* count, int32_t* status,
                            InvTab inv, uint32_t* hbuf, uint32_t* ibuf, unsigned long long* prof_replay = nullptr);

// The whole gcd of one pair by this CTA (GRID = false) or by the cooperative grid, the
// calling CTA owning global moduli [j0, j0 + nloc).
//   st, acc2   shared arrays of nloc words; stg: the operand staging buffers (stage_init done)
//   u0g, v0g   this CTA's initial residues (global scratch, nloc words each)
//   hist       (p, b) history, one entry per reduction iteration (global scratch, nq entries)
// A CTA whose operands could not be staged contributes the key (0, 0), which no modulus
// produces (it would need q = 1): the first exchange then stops every CTA of the pair
// together and the pair is answered with ST_TIMEOUT.
template <int T, int MODE>
__device__ void run_pair(const uint32_t* __restrict__ limbs, const PairDesc& d, const ModConst* __restrict__ mods,
                         int L, uint32_t j0, uint32_t nloc, uint32_t* st, uint32_t* acc2, Stage stg,
                         RedSmem& rs, uint32_t* u0g, uint32_t* v0g, int2* hist, GridSync* gs,
                         mgcd_pair* digits, uint32_t* count, uint32_t* iters_out, int32_t* status,
                         InvTab inv)
{
  const bool writer = threadIdx.x == 0 && lead_cta<MODE>();
  const ModConst* __restrict__ my = mods + j0;
  uint32_t parity = 0, epoch = 0;

  // ---- MGCD2: residues
  const bool staged = residues<T>(limbs + d.u_off, d.u_len, my, nloc, st, stg, L <= 30);
  const bool ok = residues<T>(limbs + d.v_off, d.v_len, my, nloc, acc2, stg, L <= 30) && staged;

  uint32_t kh = 0xFFFFFFFFu, kl = 0xFFFFFFFFu;
  for (uint32_t j = threadIdx.x; j < nloc; j += T) {
    const ModConst c = my[j];
    const uint32_t u = st[j], v = acc2[j];
    u0g[j] = u;
    v0g[j] = v;
    const uint32_t t = t_init(u, v, c.q, c.qinv);
    st[j] = t;
    uint32_t h, l;
    t_key(t, c.q, h, l);
    if (key_less(h, l, kh, kl)) { kh = h; kl = l; }
  }
  if (!ok) kh = kl = 0u;
  if (!reduce_min<T, MODE>(kh, kl, rs, parity, gs, epoch)) {
    if (writer) *status = ST_TIMEOUT;
    return;
  }
  if (kh == 0u && kl == 0u) {
    if (writer) { *status = ST_TIMEOUT; *count = 0; }
    return;
  }
  uint32_t p;
  int32_t b;
  key_pair(kh, kl, p, b);

  // ---- MGCD3: reduction loop (GmpCudaDevice-getGcdKernel.cu:365-402)
  int remaining = (int)d.nq;
  int ubits = ((int)d.u_len + 1) * 32, vbits = ((int)d.v_len + 1) * 32;
  uint32_t iters = 0;
  // Certification bounds (BOUND_THREAD of each CTA; every CTA computes the same values),
  // stepped while the CTA waits in the exchange.
  long long lu = 0, lv = 0;
  if (threadIdx.x == BOUND_THREAD) {
    lu = bound_init(limbs + d.u_off, d.u_len);
    lv = bound_init(limbs + d.v_off, d.v_len);
  }
  while (b != MOD_INFINITY) {
    if (writer) hist[iters] = make_int2((int)p, b);
    ++iters;
    kh = 0xFFFFFFFFu;
    kl = 0xFFFFFFFFu;
    for (uint32_t j = threadIdx.x; j < nloc; j += T) {
      const ModConst c = my[j];
      const uint32_t t = t_update(st[j], c.q, c.qinv, p, b, L <= 30);
      st[j] = t;
      uint32_t h, l;
      t_key(t, c.q, h, l);
      if (key_less(h, l, kh, kl)) { kh = h; kl = l; }
    }
    remaining -= 1;
    const uint32_t absb = b < 0 ? 0u - (uint32_t)b : (uint32_t)b;
    const int tbits = ubits - (L - 1) + __ffs((int)absb);
    ubits = vbits;
    vbits = tbits;
    if (remaining * (L - 2) <= ubits) {
      if (writer) { *status = ST_REDUX; *count = 0; }
      return;
    }
    const uint32_t pp = p;
    const int32_t bb = b;
    if (!reduce_min<T, MODE>(kh, kl, rs, parity, gs, epoch, [&] {
          if (threadIdx.x == BOUND_THREAD) bound_step(lu, lv, pp, bb);
        })) {
      if (writer) *status = ST_TIMEOUT;
      return;
    }
    key_pair(kh, kl, p, b);
  }
  if (writer) *iters_out = iters;
  finish_pair<T, MODE>(mods, d, L, j0, nloc, st, rs, parity, epoch, gs, u0g, v0g, hist, iters, remaining, lu, lv,
                       digits, count, status, inv, stg.buf, acc2);
}

// Recovery (MGCD4, GmpCudaDevice-getGcdKernel.cu:404-443) for a pair spread over several
// CTAs, in panels of up to 32 digits instead of one cross-CTA exchange per digit.  The
// reference takes one digit per round -- the lowest-indexed surviving modulus with a
// nonzero value gives (p, g) and every surviving value becomes (u - g) / p -- and ends when
// no nonzero value is left (or, with a digit just taken, when no modulus is left).
//   1. one exchange finds the lowest remaining modulus (zero or not); its CTA holds the
//      lowest remaining moduli of the pair;
//   2. that CTA takes its first <= 32 remaining moduli as the panel, computes their pairwise
//      inverses once, and one warp produces digits inside the panel by the reference's
//      rule -- the lanes are the lowest remaining moduli overall, so the lowest nonzero lane
//      is the lowest nonzero modulus overall -- until no lane is nonzero, 32 digits, or no
//      modulus is left; it writes the digits and the running count before
//   3. one exchange (its release publishes them);
//   4. every other surviving modulus applies the panel as one composed map
//      u <- (u - S) / P, S = sum_i g_i prod_{l<i} p_l, P = prod_l p_l (one inverse);
//   5. a panel without digits (its lanes all zero) falls back to one reference round over
//      all CTAs, which also detects the end (no nonzero value left).
// Digits, their order and the end conditions are those of the per-digit loop.
template <int T, int MODE>
__device__ void recover_panels(const ModConst* __restrict__ mods, const PairDesc& d, uint32_t j0, uint32_t nloc,
                               uint32_t* st, RedSmem& rs, uint32_t& parity, uint32_t& epoch, GridSync* gs,
                               int remaining, mgcd_pair* digits, uint32_t* count, int32_t* status, InvTab inv)
{
  __shared__ uint32_t pidx[32];        // panel lanes: local moduli indices, ascending
  __shared__ uint32_t pinv[32][32];    // pinv[a][b] = R / q_a mod q_b (Montgomery)
  __shared__ mgcd_pair pdig[32];       // the panel's digits
  __shared__ uint32_t pn;              // panel size, then the digits it produced
  const bool writer = threadIdx.x == 0 && lead_cta<MODE>();
  const ModConst* __restrict__ my = mods + j0;
  const uint32_t lane = threadIdx.x & 31u;
  mgcd_pair* const out = digits + d.out_off;
  uint32_t ndig = 0;                   // digits emitted (the same in every CTA)
  uint32_t scan = 0;                   // local moduli below this are retired
  bool fail = false;                   // a bounded wait ran out
  __syncthreads();                     // the replayed values of every thread are in st
  for (;;) {
    // ---- 1. the lowest remaining modulus
    while (scan < nloc && st[scan] == U_RETIRED) ++scan;
    uint32_t kh = scan < nloc ? j0 + scan : 0xFFFFFFFFu, kl = scan < nloc ? 0u : 0xFFFFFFFFu;
    if (!reduce_min<T, MODE>(kh, kl, rs, parity, gs, epoch)) { fail = true; break; }
    if (kh == 0xFFFFFFFFu) break;      // no modulus left (not reached while remaining > 0)
    const bool front = kh >= j0 && kh < j0 + nloc;
    uint32_t np = 0;
    // ---- 2. the front CTA's panel
    if (front) {
      if (threadIdx.x < 32u) {
        uint32_t n = 0;
        for (uint32_t base = scan; n < 32u && base < nloc; base += 32u) {
          const uint32_t j = base + lane;
          const bool rem = j < nloc && st[j] != U_RETIRED;
          const uint32_t m = __ballot_sync(0xFFFFFFFFu, rem);
          const uint32_t pos = n + __popc(m & ((1u << lane) - 1u));
          if (rem && pos < 32u) pidx[pos] = j;
          n += __popc(m);
        }
        if (lane == 0) pn = n < 32u ? n : 32u;
      }
      __syncthreads();
      np = pn;
      for (uint32_t e = threadIdx.x; e < np * np; e += T) {
        const uint32_t a = e / np, bb = e % np;
        uint32_t v = 0u;
        if (a != bb) {
          const uint32_t ja = pidx[a], jb = pidx[bb];
          const ModConst cb = my[jb];
          const uint32_t qa = my[ja].q;
          v = (j0 + ja < inv.n && j0 + jb < inv.n)
                  ? __ldg(inv.tab + (size_t)(j0 + ja) * inv.n + (j0 + jb))
                  : inv_mod(redc((uint64_t)(qa > cb.q ? qa - cb.q : qa), cb.q, cb.qinv), cb.q, cb.qinv);
        }
        pinv[a][bb] = v;
      }
      __syncthreads();
      if (threadIdx.x < 32u) {
        const bool in = lane < np;
        const uint32_t j = in ? pidx[lane] : 0u;
        const ModConst c = my[in ? j : pidx[0]];
        uint32_t u = in ? st[j] : 0u;
        uint32_t live = __ballot_sync(0xFFFFFFFFu, in);
        uint32_t nd = 0;
        int rem = remaining;
        while (nd < 32u && rem > 0) {
          const uint32_t nz = __ballot_sync(0xFFFFFFFFu, ((live >> lane) & 1u) && u != 0u);
          if (!nz) break;
          const uint32_t src = __ffs((int)nz) - 1u;
          const int32_t g = __shfl_sync(0xFFFFFFFFu, to_signed(u, c.q), (int)src);
          const uint32_t p = __shfl_sync(0xFFFFFFFFu, c.q, (int)src);
          if (lane == 0) out[ndig + nd] = mgcd_pair{p, g};
          live &= ~(1u << src);
          if ((live >> lane) & 1u) u = mont_mul(mod_sub(u, from_signed(g, c.q), c.q), pinv[src][lane], c.q, c.qinv);
          ++nd;
          --rem;
        }
        if (in) st[j] = ((live >> lane) & 1u) ? u : U_RETIRED;
        if (lane == 0) {
          pn = nd;
          __threadfence();             // the digits before the count
          *count = ndig + nd;          // published by the exchange below
          __threadfence();
        }
      }
      __syncthreads();
    }
    // ---- 3. publish the panel (an exchange that orders the digits and the count before it)
    kh = 0xFFFFFFFFu;
    kl = 0xFFFFFFFFu;
    if (!reduce_min<T, MODE, true>(kh, kl, rs, parity, gs, epoch)) { fail = true; break; }
    if (threadIdx.x == 0) pn = *reinterpret_cast<volatile uint32_t*>(count) - ndig;
    __syncthreads();
    const uint32_t nd = pn;
    if (threadIdx.x < nd) {
      const volatile uint32_t* src = reinterpret_cast<const volatile uint32_t*>(out + ndig + threadIdx.x);
      pdig[threadIdx.x] = mgcd_pair{src[0], (int32_t)src[1]};
    }
    __syncthreads();
    if (nd == 0u) {
      // ---- 5. one reference round: the lowest nonzero modulus anywhere, or the end
      kh = 0xFFFFFFFFu;
      kl = 0xFFFFFFFFu;
      for (uint32_t j = threadIdx.x; j < nloc; j += T) {
        const uint32_t u = st[j];
        if (u != U_RETIRED && u != 0u) { kh = j0 + j; kl = (uint32_t)to_signed(u, my[j].q); break; }
      }
      if (!reduce_min<T, MODE>(kh, kl, rs, parity, gs, epoch)) { fail = true; break; }
      if (kh == 0xFFFFFFFFu) {         // no nonzero value left: done
        if (ndig == 0u) {              // u = 0: the per-digit loop emits one zero digit
          if (writer) out[0] = mgcd_pair{mods[0].q, 0};
          ndig = 1u;
        }
        break;
      }
      const uint32_t p = mods[kh].q;
      const int32_t g = (int32_t)kl;
      for (uint32_t j = threadIdx.x; j < nloc; j += T) {
        uint32_t u = st[j];
        if (u == U_RETIRED) continue;
        const ModConst c = my[j];
        if (c.q == p) { st[j] = U_RETIRED; continue; }
        const uint32_t jj = j0 + j;
        const uint32_t dinv = (kh < inv.n && jj < inv.n)
                                  ? __ldg(inv.tab + (size_t)kh * inv.n + jj)
                                  : inv_mod(redc((uint64_t)(p > c.q ? p - c.q : p), c.q, c.qinv), c.q, c.qinv);
        st[j] = mont_mul(mod_sub(u, from_signed(g, c.q), c.q), dinv, c.q, c.qinv);
      }
      if (writer) out[ndig] = mgcd_pair{p, g};
      ++ndig;
      remaining -= 1;
      __syncthreads();
      if (remaining <= 0) break;
      continue;
    }
    // ---- 4. the panel's digits on every other surviving modulus, as one composed map
    const uint32_t last = front ? pidx[np - 1u] : 0u;
    for (uint32_t j = threadIdx.x; j < nloc; j += T) {
      const uint32_t u = st[j];
      if (u == U_RETIRED || (front && j <= last)) continue;   // the panel lanes are done
      const ModConst c = my[j];
      const uint32_t q = c.q, qi = c.qinv;
      uint32_t accP = c.r1, S = 0u;                            // Montgomery forms of P and S
      for (uint32_t i = 0; i < nd; ++i) {
        const mgcd_pair dg = pdig[i];
        const uint32_t pR = mont_mul(dg.modulus > q ? dg.modulus - q : dg.modulus, c.r2, q, qi);
        const uint32_t gR = mont_mul(from_signed(dg.value, q), c.r2, q, qi);
        const uint32_t t = mont_mul(gR, accP, q, qi);
        S = S + t - ((S >= q - t) ? q : 0u);
        accP = mont_mul(accP, pR, q, qi);
      }
      const uint32_t uR = mont_mul(u, c.r2, q, qi);
      st[j] = mont_mul(mod_sub(uR, S, q), inv_mod(redc((uint64_t)accP, q, qi), q, qi), q, qi);
    }
    ndig += nd;
    remaining -= (int)nd;
    __syncthreads();
    if (remaining <= 0) break;
  }
  if (writer) {
    *status = fail ? ST_TIMEOUT : (remaining <= 0 ? ST_RECOVERY : ST_OK);
    *count = ndig;
  }
  __syncthreads();
}

// After the reduction loop of one pair: certification, replay and recovery (MGCD4).
// st holds the final t states of this CTA's moduli; `remaining` the surviving count;
// lu, lv (meaningful in BOUND_THREAD) the size bounds of the final u and v.
template <int T, int MODE>
__device__ void finish_pair(const ModConst* __restrict__ mods, const PairDesc& d, int L, uint32_t j0, uint32_t nloc,
                            uint32_t* st, RedSmem& rs, uint32_t& parity, uint32_t& epoch, GridSync* gs,
                            const uint32_t* u0g, const uint32_t* v0g, const int2* hist, uint32_t iters, int remaining,
                            long long lu, long long lv, mgcd_pair* digits, uint32_t* count, int32_t* status,
                            InvTab inv, uint32_t* hbuf, uint32_t* ibuf, unsigned long long* prof_replay)
{
  const bool writer = threadIdx.x == 0 && lead_cta<MODE>();
  const ModConst* __restrict__ my = mods + j0;
  uint32_t p, kh, kl;
  const long long t_begin = prof_replay ? clock64() : 0;   // phase accounting: certification + replay
  // Certify the result: all surviving residues of v are 0, so v = 0 if the surviving
  // moduli (each > 2^(L-1)) multiply to more than |v|; recovery is exact if they exceed
  // 2|u| (symmetric digits).  Otherwise report that more moduli are needed.
  if (threadIdx.x == BOUND_THREAD) rs.cert = bound_certified(remaining, L, lu, lv) ? 0u : 1u;
  if constexpr (MODE == SYNC_GRID) __threadfence();
  __syncthreads();
  if (rs.cert) {
    if (writer) { *status = ST_INSUFFICIENT; *count = 0; }
    __syncthreads();
    return;
  }
  if constexpr (MODE == SYNC_GRID) {
    // CTA 0's thread 0 wrote the (p, b) history during the loop, whose exchanges order
    // nothing but the keys: one fenced exchange publishes it to every CTA.
    uint32_t h = 0xFFFFFFFFu, l = 0xFFFFFFFFu;
    if (!reduce_min<T, MODE, true>(h, l, rs, parity, gs, epoch)) {
      if (writer) *status = ST_TIMEOUT;
      return;
    }
  }

  // ---- replay: u mod q of the surviving moduli from (u0, v0) and the (p, b) history.
  // Invariant (U, V) = s * (u_i, v_i) mod q; each step (U, V, s) <- (V p, U - b V, s p) / R.
  // Moduli below 2^30 keep U, V, s lazily in [0, 2q) (bn V + U < 2q^2 + 2q < q 2^32, so the
  // REDC without its final subtraction stays below 2q).  The surviving moduli are first
  // listed in ibuf (shared, nloc words), so that thread t replays survivors t, t + T, ...
  // with every lane busy; the history is read in chunks of REPLAY_CHUNK entries that the
  // whole CTA stages into shared memory (hbuf), so every step reads a broadcast from shared
  // memory instead of waiting on a global load.
  const bool narrow = L <= 30;
  uint32_t ns;                                         // survivors, listed in ibuf
  {
    __shared__ uint32_t nsurv;
    if (threadIdx.x == 0) nsurv = 0u;
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < nloc; j += T)
      if (st[j] != T_RETIRED) ibuf[atomicAdd(&nsurv, 1u)] = j;
    __syncthreads();
    ns = nsurv;
    int2* const hb = reinterpret_cast<int2*>(hbuf);
    for (uint32_t base = 0; base < ns; base += T) {
      const bool have = base + threadIdx.x < ns;
      const uint32_t j = have ? ibuf[base + threadIdx.x] : 0u;
      const ModConst c = my[j];
      const uint32_t q = c.q, qi = c.qinv;
      uint32_t U = have ? u0g[j] : 0u, V = have ? v0g[j] : 0u, sc = 1u;
      for (uint32_t c0 = 0; c0 < iters; c0 += REPLAY_CHUNK) {
        const uint32_t n = iters - c0 < REPLAY_CHUNK ? iters - c0 : REPLAY_CHUNK;
        __syncthreads();                               // the previous chunk is consumed
        for (uint32_t e = threadIdx.x; e < n; e += T) hb[e] = hist[c0 + e];
        __syncthreads();
        if (!have) continue;
        if (narrow) {
#pragma unroll 4
          for (uint32_t e = 0; e < n; ++e) {
            // lazy operands: p < 2^L <= 2q as it is, and |b| <= p/2 < q puts q - b in (0, 2q)
            const int2 h = hb[e];
            const uint32_t pm = (uint32_t)h.x;
            const uint32_t bn = q - (uint32_t)h.y;
            const uint64_t T2 = (uint64_t)bn * V + U;
            const uint32_t U2 = mont_mul_lazy(V, pm, q, qi);
            const uint32_t lo = (uint32_t)T2, hi = (uint32_t)(T2 >> 32);
            V = hi + __umulhi(lo * qi, q) + (lo != 0u);
            sc = mont_mul_lazy(sc, pm, q, qi);
            U = U2;
          }
        } else {
#pragma unroll 4
          for (uint32_t e = 0; e < n; ++e) {
            const int2 h = hb[e];
            const uint32_t pp = (uint32_t)h.x;
            const uint32_t pm = pp > q ? pp - q : pp;
            const uint32_t bn = from_signed(-h.y, q);               // -b mod q
            const uint32_t U2 = mont_mul(V, pm, q, qi);
            const uint32_t V2 = redc((uint64_t)bn * V + U, q, qi);
            sc = mont_mul(sc, pm, q, qi);
            U = U2;
            V = V2;
          }
        }
      }
      if (have) {
        if (narrow) {
          U = mod_canon(U, q);
          sc = mod_canon(sc, q);
        }
        st[j] = mont_mul(U, inv_mod(redc((uint64_t)sc, q, qi), q, qi), q, qi);   // U / s
      }
    }
    __syncthreads();                                   // hbuf, ibuf and the replayed values
    for (uint32_t j = threadIdx.x; j < nloc; j += T)
      if (st[j] == T_RETIRED) st[j] = U_RETIRED;
  }
  if (prof_replay) {                   // non-null in every thread of the CTA or in none
    __syncthreads();
    if (threadIdx.x == 0) *prof_replay += (unsigned long long)(clock64() - t_begin);
  }

  if constexpr (MODE != SYNC_CTA) {   // several CTAs: recovery in panels
    recover_panels<T, MODE>(mods, d, j0, nloc, st, rs, parity, epoch, gs, remaining, digits, count, status, inv);
    return;
  }

  // ---- MGCD4: recovery (GmpCudaDevice-getGcdKernel.cu:404-443), over the survivors listed
  // in ibuf (in no particular order: each thread keeps the lowest index among its own)
  kh = 0xFFFFFFFFu;
  kl = 0u;
  for (uint32_t i = threadIdx.x; i < ns; i += T) {
    const uint32_t j = ibuf[i], u = st[j];
    if (u != 0u && j0 + j < kh) { kh = j0 + j; kl = (uint32_t)to_signed(u, my[j].q); }
  }
  if (!reduce_min<T, MODE>(kh, kl, rs, parity, gs, epoch)) {
    if (writer) *status = ST_TIMEOUT;
    return;
  }
  uint32_t ndig = 0;
  int32_t g;
  uint32_t pidx = kh == 0xFFFFFFFFu ? 0u : kh;      // table index of the digit's modulus
  if (kh == 0xFFFFFFFFu) { p = mods[0].q; g = 0; } else { p = mods[kh].q; g = (int32_t)kl; }
  do {
    kh = 0xFFFFFFFFu;
    kl = 0u;
    for (uint32_t i = threadIdx.x; i < ns; i += T) {
      const uint32_t j = ibuf[i];
      uint32_t u = st[j];
      if (u == U_RETIRED) continue;
      const ModConst c = my[j];
      const uint32_t q = c.q, qi = c.qinv;
      if (q == p) { st[j] = U_RETIRED; continue; }
      const uint32_t jj = j0 + j;
      const uint32_t dinv = (pidx < inv.n && jj < inv.n)
                                ? __ldg(inv.tab + (size_t)pidx * inv.n + jj)            // R / p mod q
                                : inv_mod(redc((uint64_t)(p > q ? p - q : p), q, qi), q, qi);
      u = mont_mul(mod_sub(u, from_signed(g, q), q), dinv, q, qi);
      st[j] = u;
      if (u != 0u && jj < kh) { kh = jj; kl = (uint32_t)to_signed(u, q); }
    }
    if (writer) digits[d.out_off + ndig] = mgcd_pair{p, g};
    ++ndig;
    remaining -= 1;
    if (remaining <= 0) break;
    if (!reduce_min<T, MODE>(kh, kl, rs, parity, gs, epoch)) {
      if (writer) *status = ST_TIMEOUT;
      return;
    }
    pidx = kh == 0xFFFFFFFFu ? 0u : kh;
    if (kh == 0xFFFFFFFFu) { p = mods[0].q; g = 0; } else { p = mods[kh].q; g = (int32_t)kl; }
  } while (g != 0);
  if (writer) {
    *status = (g != 0) ? ST_RECOVERY : ST_OK;
    *count = ndig;
  }
  __syncthreads();
}


}  // namespace mgcd

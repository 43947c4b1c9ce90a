// mgcd_internal.h -- types shared by the host orchestration and the kernels.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/modgcd.h"

namespace mgcd {

struct ModConst;

// One gcd job.  u is the larger operand (u >= v > 0); both are little-endian 32-bit limbs
// in the batch's limb array, with no leading zero limbs.
struct PairDesc {
  uint64_t u_off, v_off;
  uint32_t u_len, v_len;
  uint32_t nq;       // moduli used (the reference's count, a multiple of 256, or a scaled
                     // count rounded up to a multiple of 32)
  uint32_t out_off;  // first digit slot in the digit array; nq + 1 slots are reserved
  uint64_t g_off;    // first limb of the binary gcd in the result-limb array
  uint32_t g_cap;    // limbs reserved there (the smaller operand's length)
  uint32_t nq_cap;   // moduli the pair may grow to during its reduction loop (the reference's
                     // count; <= nq: no growth)
};

// Device-side mixed-radix conversion (mgcd_radix_dev.cu): pairs with up to RADIX_MAX
// digits are converted on the GPU; glen = RADIX_HOST marks a pair left to the host
// (more digits, or a failed pair).
constexpr uint32_t RADIX_MAX = 4096;
constexpr uint32_t RADIX_HOST = 0xFFFFFFFFu;
size_t radix_smem_bytes();
cudaError_t launch_radix(const PairDesc* pairs, uint32_t npairs, const mgcd_pair* digits, const uint32_t* count,
                         const int32_t* status, uint32_t* glimbs, uint32_t* glen, int grid, cudaStream_t s);

// Per-pair results written by the kernels.
enum : int32_t {
  ST_OK = 0,
  ST_REDUX = 1,      // ran out of moduli in the reduction loop
  ST_RECOVERY = 2,   // ran out of moduli in the recovery loop
  ST_TIMEOUT = 3,    // a bounded cross-CTA wait expired
  ST_INSUFFICIENT = 4,  // result not certified: too few moduli survived the reduction loop
  ST_PENDING = -1
};

// Pairwise inverse table: invtab[i * invtab_n + j] = q_i^{-1} * 2^32 mod q_j for table
// moduli i, j < invtab_n (Montgomery form; the diagonal is unused).  Recovery divides by
// the digit's modulus with one load and one Montgomery product instead of an inverse.
struct InvTab {
  const uint32_t* tab;
  uint32_t n;
};

// Continuous serving: a lane's persistent K-slot kernel (batchk_kernel in ring mode) takes
// requests from this ring while it runs.  The ring lives in pinned, mapped host memory:
// the host writes an entry's descriptor, operands and digit slots there and publishes it
// by a release store of `tail`; a CTA with a free slot claims the next entry through the
// device counter `head` (compare-and-swap below the tail it acquired), computes it and
// writes its digits, count and status there, then releases done[i] = i + 1.
constexpr uint32_t STREAM_RING = 2048;
struct StreamRing {
  uint32_t tail;                     // entries published (host release store, kernel acquire load)
  uint32_t stop;                     // host: the lane's kernels leave as soon as they are idle
  uint32_t pad_[30];
  PairDesc desc[STREAM_RING];        // entry i at i % STREAM_RING
  uint32_t done[STREAM_RING];        // i + 1 once entry i's results are written (kernel release store)
  uint32_t count[STREAM_RING];
  int32_t status[STREAM_RING];
  uint32_t iters[STREAM_RING];
};

constexpr int PHASE_WORDS = 14;

struct BatchArgs {
  InvTab inv;
  const uint32_t* limbs;
  const PairDesc* pairs;
  const uint32_t* order;     // processing order (indices into pairs)
  uint32_t npairs;
  const ModConst* mods;
  int L;
  uint32_t* queue;           // work counter, zero before launch
  uint32_t* scratch;         // per-CTA scratch: u0[nq_max], v0[nq_max], hist[2*nq_max]
  size_t scratch_words;      // words per CTA
  uint32_t nq_max;
  mgcd_pair* digits;
  uint32_t* count;           // digits per pair
  uint32_t* iters;           // reduction iterations per pair (work accounting)
  int32_t* status;
  uint32_t stage_fail;       // test hook: this CTA reports an operand-staging failure (~0: none)
  unsigned long long* trace; // per CTA: start and end (globaltimer ns), SM id, pairs taken (null: off)
  unsigned long long* phases; // per CTA (K-slot kernel, PHASE_WORDS each): clock cycles of thread 0 in
                              // set-up, update, pivot choice and finish, reduction iterations, moduli
                              // rounds, pairs, cycles of certification and replay; over all threads:
                              // update rounds, rounds that needed an inverse, finite slot states (null: off)
  unsigned long long* span;  // the kernel's earliest CTA start and ~(latest CTA end), globaltimer ns,
                             // each lowered by atomicMin (null: off)
  uint32_t grow_permille;    // moduli added per growth step, thousandths of the pair's nq_cap
  uint32_t* nq_final;        // per pair: moduli in its set at the end (null: not recorded)
  unsigned long long* updates; // per pair: surviving moduli summed over its iterations (null: off)
  StreamRing* ring;          // ring mode (device view of the mapped ring)
  uint32_t* ring_head;       // entries claimed (device memory)
  unsigned long long idle_ns;  // ring mode: a CTA whose slots are all empty leaves after this long idle
};

// State of the cross-CTA reduction used by a single pair spread over a cooperative grid.
// Cooperative grid (leader exchange), exchange e: every CTA stores its minimum, tagged with
// bit (e / 2 + 1) & 1, into keys[e & 1][cta]; CTA 0 polls all slots until their tags
// match, reduces them and stores the tagged result into bcast[e & 1]; the other CTAs poll
// that word.  A slot read in exchange e holds the value of e or of e - 2 (no CTA can be two
// exchanges ahead of another), which the tag tells apart: no atomics and no fences.
// Cluster grid, exchange e: the leader thread of every cluster folds the cluster's minimum
// into slot[e % 3] (atomic min) and arrives on a monotonic counter; leaders wait (bounded)
// for e + 1 full rounds of arrivals, then read the slot.  Cluster 0 resets slot[(e + 1) % 3]
// before arriving: all leaders have read that slot (exchange e - 2) once it is past e - 1.
constexpr int MAX_GRID_CTAS = 1024;
struct GridSync {
  unsigned long long keys[2][MAX_GRID_CTAS];   // zero before use
  unsigned long long bcast[2][16];             // [b][0]; one 128-byte line each
  unsigned long long slot[3];                  // ~0 before use
  unsigned int arrive;
  unsigned int error;                          // set by the first CTA whose wait expired
  unsigned int withhold_cta;                   // test hook: this CTA never publishes (0xFFFFFFFF: none)
  unsigned long long timeout_ns;               // bound of every wait
};

struct GridArgs {
  InvTab inv;
  const uint32_t* limbs;
  PairDesc pair;
  const ModConst* mods;
  int L;
  uint32_t* scratch;         // u0[nq], v0[nq], hist[2*nq]
  GridSync* sync;
  uint32_t per_cta;          // moduli owned by each CTA (contiguous ranges)
  mgcd_pair* digits;
  uint32_t* count;
  uint32_t* iters;
  int32_t* status;
  uint32_t stage_fail;       // test hook: this CTA reports an operand-staging failure (~0: none)
};

// Launch helpers (mgcd_kernels.cu).
// k = pairs per CTA run in lockstep (1: batch_kernel; 2, 4: batchk_kernel).  Scratch per
// CTA: 4 * k * nq_max words.  Moduli below 2^30 (a.L <= 30; `narrow` for the occupancy
// query) select the kernels with lazily reduced Montgomery products.
size_t batch_smem_bytes(int threads, int k, uint32_t nq_max);
cudaError_t batch_max_blocks_per_sm(int threads, int k, bool narrow, size_t smem, int* blocks);
// after: a programmatic dependent launch -- the kernel may start once every CTA of the
// stream's previous kernel has started (the batch kernels trigger at their start).
cudaError_t launch_batch(const BatchArgs& a, int threads, int k, int grid, size_t smem, cudaStream_t s,
                         bool after = false);
// The same K-slot kernel in ring mode (continuous serving, a.ring set): threads 512 or 1024,
// k 2 or 4.
cudaError_t launch_ring(const BatchArgs& a, int threads, int k, int grid, size_t smem, cudaStream_t s);

// One pair on a cluster of `ctas` CTAs (<= 16) of `threads` threads; same arguments and
// shared-memory size as the grid path.
cudaError_t launch_cluster(const GridArgs& a, int threads, int ctas, size_t smem, cudaStream_t s);

// Persistent batched kernel for pairs larger than one CTA: `clusters` thread-block
// clusters of `csize` CTAs each pull pairs from the queue, k pairs per cluster in lockstep
// (k = 1: any CTA size; k = 2, 4: 256 or 512 threads).  a.scratch_words = 4 * k * nq_max.
size_t cluster_batch_smem_bytes(int csize, uint32_t nq_max, int k);
cudaError_t cluster_batch_max_clusters(int threads, int k, int csize, size_t smem, int* clusters);
cudaError_t launch_cluster_batch(const BatchArgs& a, int threads, int k, int csize, int clusters, size_t smem,
                                 cudaStream_t s, bool after = false);

// One pair on a cooperative grid of `clusters` clusters of `csize` CTAs (hierarchical
// exchange; a.sync is the global state, a.per_cta the moduli per CTA).
cudaError_t cgrid_max_clusters(int threads, int csize, size_t smem, int* clusters);
cudaError_t launch_cgrid(const GridArgs& a, int threads, int csize, int clusters, size_t smem, cudaStream_t s);

// Resets the grid exchange state on the device (capturable in a CUDA graph).
cudaError_t launch_gridsync_init(GridSync* gs, unsigned long long timeout_ns, uint32_t withhold, cudaStream_t s);

size_t grid_smem_bytes(uint32_t per_cta);
constexpr int GRID_THREADS = 1024;   // CTA size of the grid path (256 for the reference's shape)
constexpr int MAX_CLUSTER = 16;      // largest thread-block cluster (non-portable size)
cudaError_t grid_max_blocks_per_sm(int threads, size_t smem, int* blocks);
cudaError_t launch_grid(const GridArgs& a, int threads, int grid, size_t smem, cudaStream_t s);

// 256-thread blocks, 8 IMADs per thread per iteration.
cudaError_t launch_int_peak(uint32_t* out, int blocks, int iters, cudaStream_t s);

// Fills the n x n pairwise inverse table for the first n moduli.
cudaError_t launch_build_invtab(const ModConst* mods, uint32_t n, uint32_t* tab, cudaStream_t s);

}  // namespace mgcd

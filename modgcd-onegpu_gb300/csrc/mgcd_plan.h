// mgcd_plan.h -- host-side state of the library: the context (device, moduli table,
// inverse table, launch configuration) and plans (one batch's buffers, streams and
// schedule).  A context owns one plan for its own calls; the request server owns one plan
// per in-flight wave, all sharing the context's resident tables.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "../../include/modgcd.h"
#include "mgcd_internal.h"

namespace mgcd {

// Device buffer from the context's stream-ordered memory pool: growing it neither blocks
// the host nor serialises the other streams (plain cudaMalloc/cudaFree would).
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t grow(size_t want, cudaMemPool_t pool, cudaStream_t s);
  void release(cudaStream_t s);
  template <class T> T* as() const { return static_cast<T*>(p); }
};

// Pinned host buffer (grow-only, doubling).  A buffer it outgrows is kept until release():
// cudaFreeHost waits for all work on the device, which would stall a server behind every
// kernel in flight.
struct HostBuf {
  void* p = nullptr;
  size_t bytes = 0;
  std::vector<void*> retired;
  cudaError_t grow(size_t want);
  void release();
  template <class T> T* as() const { return static_cast<T*>(p); }
};

struct Bucket {
  int threads, k;      // CTA size, pairs per CTA in lockstep
  int csize;           // CTAs per thread-block cluster (0: one CTA per pair)
  int cls;             // size class
  uint32_t first, n, nq_max;
  int grid;            // CTAs (csize = 0) or clusters
  size_t smem;
  size_t scratch_off;  // words
};

// Size classes of the batched path, one persistent kernel each: pairs with at
// most 1,024 / 4,096 / 16,384 moduli run K per CTA (or K per small cluster, when the class
// or a serving lane asks for one); larger pairs K per thread-block cluster.
constexpr int NSTREAMS = MGCD_NUM_SIZE_CLASSES;
constexpr int CLUSTER_CLASS = 3;
constexpr uint32_t CTA_MAX_NQ = 16384;
constexpr size_t INVTAB_N = 16384;        // moduli covered by the pairwise inverse table

inline int size_class(uint32_t nq) { return nq <= 1024 ? 0 : nq <= 4096 ? 1 : nq <= CTA_MAX_NQ ? 2 : CLUSTER_CLASS; }

// Moduli a batched pair may grow to (mgcd_set_growth): a sixteenth more than the reference's
// count, so that a pair whose smaller sets took more iterations still ends in its own loop
// (with the growth policy's defaults no pair of the mixed 1k-64k-bit batches went past the
// reference's count in the oracle's runs), rounded up to a warp.  The cap sizes a bucket's
// shared memory and scratch: the mixed batch ran 73.9 ms with an eighth, 72.8 with this.
inline uint32_t grow_cap(uint32_t ref) { return std::min<uint32_t>(CTA_MAX_NQ, (ref + ref / 16 + 31u) / 32u * 32u); }

struct Plan {
  cudaStream_t stream = nullptr;       // every launch of the plan
  cudaEvent_t t_run0 = nullptr, t_run1 = nullptr;   // timing of the whole run

  size_t np = 0;                       // pairs in the plan
  std::vector<int32_t> status;         // per pair: MGCD_OK / error code / -1 = computed on the GPU
  std::vector<int> slot;               // per pair: index into GPU arrays, or -1
  std::vector<std::vector<uint32_t>> trivial;  // per pair: host-decided result (zero operand)
  std::vector<PairDesc> descs;         // GPU pairs
  std::vector<uint32_t> order;
  std::vector<Bucket> buckets;
  std::vector<uint32_t> grid_pairs;    // GPU indices run as single-pair launches
  std::vector<uint32_t> ref_nq, eff_nq; // per GPU pair: reference count, count of the final run
  size_t ndig = 0, scratch_words = 0, grid_scratch_off = 0;
  size_t nglimbs = 0;                  // result limbs reserved (sum of g_cap)
  // results planned in the caller's layout (mgcd_gcd_batch, slots contiguous): d_glimbs[x]
  // is the caller's g[direct_base + x], copied there in one piece; in_place: fetch did so
  bool direct = false, in_place = false;
  uint64_t direct_base = 0;
  bool plain = false;                  // single-pair latency policy
  bool graphable = true;               // may be recorded into a CUDA graph (context setting)
  int cluster_ctas = 0;                // CTAs per cluster of size class 3 (0: the context's setting)
  int small_cluster_ctas = 0;          // CTAs per cluster for pairs of size classes 1-2 (0: the
                                       // context's setting); serving waves favour latency
  int cluster_k = 0;                   // pairs per cluster of size class 3 (0: the context's setting)

  DevBuf d_limbs, d_pairs, d_order, d_digits, d_count, d_iters, d_status, d_queue, d_scratch, d_gsync, d_retry;
  DevBuf d_nqf, d_upd;                 // per pair (K-slot kernels): final moduli count, loop updates
  DevBuf d_span;                       // per bucket kernel: earliest CTA start, ~(latest CTA end), ns
  DevBuf d_glimbs, d_glen;             // binary gcds converted on the device
  DevBuf d_trace;                      // per-CTA occupancy trace of the bucket kernels (4 words each)
  DevBuf d_phases;                     // per-CTA phase accounting of the K-slot kernels (8 words each)
  std::vector<int> trace_cls;          // size class of each traced CTA (launch order)
  HostBuf h_count, h_iters, h_status, h_digits, h_glimbs, h_glen, h_nqf, h_upd;
  int launches = 0, retried = 0;
  bool ran = false, synced = false, bucket_timed = false;
  double work[4] = {0, 0, 0, 0};       // residue steps, loop updates, recovery updates, operand bytes
  double alg_bytes = 0;                // algorithmic bytes: operands + (prime, constant) per modulus + digits
  std::vector<double> bucket_work;     // the same per bucket kernel (4 per bucket)
  uint64_t h2d_bytes = 0, d2h_bytes = 0;

  // CUDA graph of the plan's GPU work; dropped whenever a buffer it uses moves
  cudaGraphExec_t graph = nullptr;
  int graph_kernels = 0;

  cudaError_t create(int priority = 0);   // the stream at this priority (lower = more urgent)
  void destroy(cudaMemPool_t pool);
  void drop_graph();
  size_t device_bytes() const;
};

}  // namespace mgcd

struct mgcd_context {
  int device = 0, L = 32, sms = 0;
  size_t smem_optin = 0;               // largest dynamic shared memory per CTA
  cudaMemPool_t pool = nullptr;
  std::vector<uint32_t> moduli;
  mgcd::DevBuf mods;
  mgcd::DevBuf d_invtab;               // pairwise inverse table (InvTab)
  uint32_t invtab_n = 0;
  mgcd::Plan main;                     // the plan of the context's own calls
  bool serving = false;                // a request server runs on this context

  // Per size class of the batched path: CTA size, pairs per CTA in lockstep, fraction of
  // the reference moduli count, CTAs per cluster (cluster class only).
  struct ClassCfg { int threads, k; float nq_scale; int csize; };
  ClassCfg cfg[mgcd::NSTREAMS] = {{256, 4, 1.0f, 0}, {512, 4, 1.0f, 0}, {1024, 2, 1.0f, 0}, {1024, 1, 1.0f, 8}};
  bool use_graph = false;
  int single_policy = MGCD_SINGLE_AUTO;  // launch shape of pairs that span several CTAs
  unsigned long long wait_timeout_ns = 2000000000ull;   // bound of every cross-CTA wait
  uint32_t withhold_cta = 0xFFFFFFFFu;                  // test hook (mgcd_test_withhold_cta)
  uint32_t stage_fail_cta = 0xFFFFFFFFu;                // test hook (mgcd_test_fail_staging)
  uint32_t force_nq = 0;                                // test hook (mgcd_test_force_moduli)
  bool trace = false;                                   // record per-CTA occupancy (mgcd_set_cta_trace)
  // Moduli grown on demand in the K-slot kernels (mgcd_set_growth): batched pairs start with
  // this fraction of the reference count (0: off) and grow by grow_permille thousandths of it
  // at a time, up to the reference count.
  float grow_start = 0.4f;
  uint32_t grow_permille = 50;
};

namespace mgcd {

// Plan operations (mgcd_capi.cpp).  All return MGCD_* codes.
//   plan_batch   validate, order and size the pairs on the host, copy the batch to the
//                device on P.stream (asynchronous when `limbs` is pinned); given the
//                caller's result layout (g_off, g_cap), results are planned in it when its
//                slots are contiguous (Plan::direct);
//   run_plan     launch the GPU work (asynchronous);
//   sync_plan    wait; rerun uncertified pairs of a scaled run with the reference count;
//   fetch        copy the results back (pinned; a direct plan's binary results straight
//                into `direct_g`, the caller's array) and account the work;
//   convert_all  digits -> binary gcds for every pair of the plan.
int plan_batch(mgcd_context* c, Plan& P, size_t np, const uint32_t* limbs, const uint64_t* u_off,
               const uint32_t* u_len, const uint64_t* v_off, const uint32_t* v_len, bool plain,
               const uint64_t* g_off = nullptr, const uint32_t* g_cap = nullptr);
int run_plan(mgcd_context* c, Plan& P);
int sync_plan(mgcd_context* c, Plan& P);
int fetch(mgcd_context* c, Plan& P, uint32_t* direct_g = nullptr);
int convert_all(mgcd_context* c, Plan& P, uint32_t* g, const uint64_t* g_off, const uint32_t* g_cap,
                uint32_t* g_len, int32_t* status, bool threaded);
int to_status(int32_t st);

}  // namespace mgcd

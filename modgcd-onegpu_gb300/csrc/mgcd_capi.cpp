// mgcd_capi.cpp -- the C ABI (include/modgcd.h): contexts, batch planning and launches,
// result conversion.
//
// Host flow of one batch (the reference's per-call flow, GmpCudaDevice-gcd.cu:59-132,
// generalised to many pairs):
//   upload    order each pair so that u >= v (the reference swaps its mpz operands,
//             :61-62), strip leading zero limbs, size the moduli (numModuliNeededFor,
//             :49-55) and reject pairs that need more moduli than the table holds (:76-78);
//             pairs with a zero operand are answered on the host (gcd(x, 0) = x);
//             group the rest by size into CTA-size buckets, largest first; copy the batch.
//   run       one persistent kernel per bucket, each on its own stream so buckets overlap;
//             pairs too large for one CTA run one at a time on a cooperative grid.
//   download  copy digits back and convert each pair's digits to binary.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/modgcd.h"
#include "mgcd_internal.h"
#include "mgcd_moduli.h"
#include "mgcd_radix.h"

using namespace mgcd;

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t grow(size_t want)
  {
    if (want <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    const size_t sz = std::max<size_t>(want + want / 4, 256);
    cudaError_t e = cudaMalloc(&p, sz);
    if (e == cudaSuccess) bytes = sz;
    return e;
  }
  void release()
  {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

struct HostBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t grow(size_t want)
  {
    if (want <= bytes) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    const size_t sz = std::max<size_t>(want + want / 4, 256);
    cudaError_t e = cudaHostAlloc(&p, sz, cudaHostAllocDefault);
    if (e == cudaSuccess) bytes = sz;
    return e;
  }
  void release()
  {
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
  }
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

// Size classes of the batched path, one persistent kernel (and stream) each: pairs with at
// most 1,024 / 4,096 / 16,384 moduli run one per CTA; larger pairs one per cluster.
constexpr int NSTREAMS = 4;
constexpr int CLUSTER_CLASS = 3;
constexpr uint32_t CTA_MAX_NQ = 16384;
constexpr size_t INVTAB_N = 16384;        // moduli covered by the pairwise inverse table

int env_int(const char* name, int dflt)
{
  const char* s = std::getenv(name);
  return s ? std::atoi(s) : dflt;
}

int to_status(int32_t st)
{
  switch (st) {
    case ST_OK: return MGCD_OK;
    case ST_REDUX: return MGCD_ERR_REDUX;
    case ST_RECOVERY: return MGCD_ERR_RECOVERY;
    case ST_TIMEOUT: return MGCD_ERR_TIMEOUT;
    case ST_INSUFFICIENT: return MGCD_ERR_REDUX;
    default: return MGCD_ERR_KERNEL;
  }
}

int size_class(uint32_t nq) { return nq <= 1024 ? 0 : nq <= 4096 ? 1 : nq <= CTA_MAX_NQ ? 2 : CLUSTER_CLASS; }

size_t strip(const uint32_t* x, size_t n)
{
  while (n && x[n - 1] == 0) --n;
  return n;
}

int cmp_mag(const uint32_t* a, size_t na, const uint32_t* b, size_t nb)
{
  if (na != nb) return na < nb ? -1 : 1;
  for (size_t i = na; i-- > 0;)
    if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
  return 0;
}

}  // namespace

struct mgcd_context {
  int device = 0, L = 32, sms = 0;
  size_t smem_optin = 0;               // largest dynamic shared memory per CTA
  cudaStream_t stream = nullptr;
  cudaStream_t bstream[NSTREAMS] = {};
  cudaEvent_t ev_start = nullptr, ev_b[NSTREAMS] = {};
  std::vector<uint32_t> moduli;
  DevBuf mods;

  // current plan
  size_t np = 0;                       // pairs in the plan
  std::vector<int32_t> status;         // per pair: MGCD_OK / error code / -1 = computed on the GPU
  std::vector<int> slot;               // per pair: index into GPU arrays, or -1
  std::vector<std::vector<uint32_t>> trivial;  // per pair: host-decided result (zero operand)
  std::vector<PairDesc> descs;         // GPU pairs
  std::vector<uint32_t> order;
  std::vector<Bucket> buckets;
  std::vector<uint32_t> grid_pairs;    // GPU indices run on the cooperative grid
  size_t ndig = 0, scratch_words = 0, grid_scratch_off = 0;
  bool plain = false;                  // single-pair latency policy

  DevBuf d_limbs, d_pairs, d_order, d_digits, d_count, d_iters, d_status, d_queue, d_scratch, d_gsync;
  HostBuf h_count, h_iters, h_status, h_digits;
  int launches = 0;
  bool ran = false;
  double work[4] = {0, 0, 0, 0};
  // Per size class of the batched path: CTA size, pairs per CTA in lockstep, fraction of
  // the reference moduli count, CTAs per cluster (cluster class only).
  struct { int threads, k; float nq_scale; int csize; } cfg[NSTREAMS] = {
      {256, 4, 1.0f, 0}, {512, 4, 1.0f, 0}, {1024, 2, 1.0f, 0}, {1024, 1, 1.0f, 8}};
  // CUDA graph of the plan's GPU work (mgcd_batch_use_graph); rebuilt after every upload
  bool use_graph = false, bucket_timed = false;
  cudaGraphExec_t graph = nullptr;
  int graph_kernels = 0;
  std::vector<uint32_t> ref_nq, eff_nq; // per GPU pair: reference count, count of the final run
  int retried = 0;
  bool synced = false;
  DevBuf d_retry;
  DevBuf d_invtab;                     // pairwise inverse table (InvTab)
  int single_policy = MGCD_SINGLE_AUTO;  // launch shape of pairs that span several CTAs
  unsigned long long wait_timeout_ns = 2000000000ull;   // bound of every cross-CTA wait
  uint32_t withhold_cta = 0xFFFFFFFFu;                  // test hook (mgcd_test_withhold_cta)
  uint32_t force_nq = 0;                                // test hook (mgcd_test_force_moduli)
  uint32_t invtab_n = 0;
  // timing: the whole run on `stream`, and each bucket launch on its stream
  cudaEvent_t t_run0 = nullptr, t_run1 = nullptr, t_b0[NSTREAMS] = {}, t_b1[NSTREAMS] = {};
  uint64_t h2d_bytes = 0, d2h_bytes = 0;
};

#define CK(call)                                     \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return MGCD_ERR_CUDA;     \
  } while (0)

// The recorded graph holds device pointers and launch parameters of the current plan:
// dropped whenever a buffer it uses moves or a captured parameter changes.
static void drop_graph(mgcd_context* c)
{
  if (c->graph) cudaGraphExecDestroy(c->graph);
  c->graph = nullptr;
  c->graph_kernels = 0;
}

extern "C" {

const char* mgcd_status_string(int s)
{
  switch (s) {
    case MGCD_OK: return "OK";
    case MGCD_ERR_INVALID_ARG: return "Invalid argument.";
    case MGCD_ERR_NO_DEVICE: return "Invalid device number.";
    case MGCD_ERR_CUDA: return "CUDA error.";
    case MGCD_ERR_NOT_ENOUGH_MODULI: return "Not enough moduli available for given input.";
    case MGCD_ERR_GRID: return "Cannot allocate enough threads to support computation.";
    case MGCD_ERR_REDUX: return "Ran out of moduli in the reduction loop.";
    case MGCD_ERR_RECOVERY: return "Ran out of moduli in the recovery loop.";
    case MGCD_ERR_KERNEL: return "Unknown error in the gcd kernel.";
    case MGCD_ERR_TIMEOUT: return "A device-side wait timed out.";
    case MGCD_ERR_CAPACITY: return "Output buffer too small.";
    case MGCD_ERR_BUDGET: return "Request exceeds the admission budget.";
    case MGCD_ERR_BUSY: return "Queue full.";
    default: return "Unknown status.";
  }
}

int mgcd_device_count(int* count)
{
  if (!count) return MGCD_ERR_INVALID_ARG;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) n = 0;
  *count = n;
  return MGCD_OK;
}

int mgcd_set_device(int devNo)
{
  int n = 0;
  mgcd_device_count(&n);
  if (devNo < 0 || devNo >= n) return MGCD_ERR_NO_DEVICE;
  CK(cudaSetDevice(devNo));
  return MGCD_OK;
}

size_t mgcd_gen_moduli(int L, uint32_t* out, size_t count) { return gen_moduli(L, out, count); }

int mgcd_moduli_needed(int L, size_t bits) { return moduli_needed(L, bits); }

int mgcd_create(int device, int L, mgcd_context** out)
{
  if (!out || (L != 22 && L != 27 && L != 32)) return MGCD_ERR_INVALID_ARG;
  *out = nullptr;
  int n = 0;
  mgcd_device_count(&n);
  if (device < 0) {
    if (n == 0 || cudaGetDevice(&device) != cudaSuccess) return MGCD_ERR_NO_DEVICE;
  }
  if (device >= n) return MGCD_ERR_NO_DEVICE;
  CK(cudaSetDevice(device));
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, device));
  if (prop.warpSize != 32) return MGCD_ERR_NO_DEVICE;

  auto* c = new mgcd_context();
  c->device = device;
  c->L = L;
  c->sms = prop.multiProcessorCount;
  c->smem_optin = prop.sharedMemPerBlockOptin;
  // Table size: enough moduli for ~1.2M-bit operands at every width (L = 22 is limited by
  // the 97,358 usable 22-bit primes).
  const size_t want = (L == 22) ? 97280 : 131072;
  c->moduli.resize(want);
  const size_t got = gen_moduli(L, c->moduli.data(), want);
  c->moduli.resize(got / 256 * 256);
  std::vector<ModConstHost> mc(c->moduli.size());
  mod_constants(c->moduli.data(), c->moduli.size(), mc.data());
  int rc = MGCD_OK;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) rc = MGCD_ERR_CUDA;
  for (int i = 0; i < NSTREAMS && rc == MGCD_OK; ++i)
    if (cudaStreamCreateWithFlags(&c->bstream[i], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_b[i], cudaEventDisableTiming) != cudaSuccess)
      rc = MGCD_ERR_CUDA;
  if (rc == MGCD_OK && cudaEventCreateWithFlags(&c->ev_start, cudaEventDisableTiming) != cudaSuccess) rc = MGCD_ERR_CUDA;
  if (rc == MGCD_OK && (cudaEventCreate(&c->t_run0) != cudaSuccess || cudaEventCreate(&c->t_run1) != cudaSuccess))
    rc = MGCD_ERR_CUDA;
  for (int i = 0; i < NSTREAMS && rc == MGCD_OK; ++i)
    if (cudaEventCreate(&c->t_b0[i]) != cudaSuccess || cudaEventCreate(&c->t_b1[i]) != cudaSuccess) rc = MGCD_ERR_CUDA;
  if (rc == MGCD_OK && c->mods.grow(mc.size() * sizeof(ModConstHost)) != cudaSuccess) rc = MGCD_ERR_CUDA;
  if (rc == MGCD_OK &&
      cudaMemcpy(c->mods.p, mc.data(), mc.size() * sizeof(ModConstHost), cudaMemcpyHostToDevice) != cudaSuccess)
    rc = MGCD_ERR_CUDA;
  // Pairwise inverses of the first INVTAB_N moduli (every pair of the batched path), for
  // recovery: 1 GiB at n = 16,384.
  c->invtab_n = (uint32_t)std::min<size_t>(INVTAB_N, c->moduli.size());
  if (rc == MGCD_OK && c->d_invtab.grow((size_t)c->invtab_n * c->invtab_n * sizeof(uint32_t)) != cudaSuccess)
    rc = MGCD_ERR_CUDA;
  if (rc == MGCD_OK && (launch_build_invtab(c->mods.as<ModConst>(), c->invtab_n, c->d_invtab.as<uint32_t>(),
                                            c->stream) != cudaSuccess ||
                        cudaStreamSynchronize(c->stream) != cudaSuccess))
    rc = MGCD_ERR_CUDA;
  if (rc != MGCD_OK) {
    mgcd_destroy(c);
    return rc;
  }
  *out = c;
  return MGCD_OK;
}

int mgcd_destroy(mgcd_context* c)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  drop_graph(c);
  for (DevBuf* b : {&c->mods, &c->d_limbs, &c->d_pairs, &c->d_order, &c->d_digits, &c->d_count, &c->d_iters,
                    &c->d_status, &c->d_queue, &c->d_scratch, &c->d_gsync, &c->d_retry, &c->d_invtab})
    b->release();
  for (HostBuf* b : {&c->h_count, &c->h_iters, &c->h_status, &c->h_digits}) b->release();
  for (int i = 0; i < NSTREAMS; ++i) {
    if (c->bstream[i]) cudaStreamDestroy(c->bstream[i]);
    if (c->ev_b[i]) cudaEventDestroy(c->ev_b[i]);
    if (c->t_b0[i]) cudaEventDestroy(c->t_b0[i]);
    if (c->t_b1[i]) cudaEventDestroy(c->t_b1[i]);
  }
  if (c->t_run0) cudaEventDestroy(c->t_run0);
  if (c->t_run1) cudaEventDestroy(c->t_run1);
  if (c->ev_start) cudaEventDestroy(c->ev_start);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return MGCD_OK;
}

int mgcd_max_grid_size(const mgcd_context* c, int* out)
{
  if (!c || !out) return MGCD_ERR_INVALID_ARG;
  *out = (int)(c->moduli.size() / 256);
  return MGCD_OK;
}

int mgcd_num_moduli(const mgcd_context* c, size_t* out)
{
  if (!c || !out) return MGCD_ERR_INVALID_ARG;
  *out = c->moduli.size();
  return MGCD_OK;
}

int mgcd_moduli(const mgcd_context* c, uint32_t* out, size_t n)
{
  if (!c || (!out && n) || n > c->moduli.size()) return MGCD_ERR_INVALID_ARG;
  std::memcpy(out, c->moduli.data(), n * sizeof(uint32_t));
  return MGCD_OK;
}

// ------------------------------------------------------------------------- batch ----

static int schedule(mgcd_context* c, const std::vector<PairDesc>& descs, const std::vector<uint32_t>& subset,
                    bool plain, std::vector<Bucket>& buckets, std::vector<uint32_t>& grid_pairs, size_t& scratch);

static int plan_batch(mgcd_context* c, size_t np, const uint32_t* limbs, const uint64_t* u_off,
                      const uint32_t* u_len, const uint64_t* v_off, const uint32_t* v_len, bool plain)
{
  if (!c || (np && (!limbs || !u_off || !u_len || !v_off || !v_len))) return MGCD_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));   // buffers below may be reallocated
  drop_graph(c);
  c->np = np;
  c->plain = plain;
  c->ran = false;
  c->status.assign(np, -1);
  c->slot.assign(np, -1);
  c->trivial.assign(np, {});
  c->descs.clear();
  c->ref_nq.clear();
  c->grid_pairs.clear();
  c->buckets.clear();
  uint64_t limb_end = 0;
  uint32_t out_off = 0;
  for (size_t i = 0; i < np; ++i) {
    const uint32_t* u = limbs + u_off[i];
    const uint32_t* v = limbs + v_off[i];
    size_t ul = strip(u, u_len[i]), vl = strip(v, v_len[i]);
    limb_end = std::max<uint64_t>(limb_end, std::max(u_off[i] + u_len[i], v_off[i] + v_len[i]));
    if (ul == 0 || vl == 0) {  // gcd(x, 0) = |x|: no modular work
      const uint32_t* x = ul ? u : v;
      c->trivial[i].assign(x, x + (ul ? ul : vl));
      c->status[i] = MGCD_OK;
      continue;
    }
    PairDesc d;
    if (cmp_mag(u, ul, v, vl) >= 0) {
      d.u_off = u_off[i]; d.u_len = (uint32_t)ul; d.v_off = v_off[i]; d.v_len = (uint32_t)vl;
    } else {
      d.u_off = v_off[i]; d.u_len = (uint32_t)vl; d.v_off = u_off[i]; d.v_len = (uint32_t)ul;
    }
    const uint32_t top = limbs[d.u_off + d.u_len - 1];
    const size_t ubits = (size_t)(d.u_len - 1) * 32 + (32 - __builtin_clz(top));
    const int ref_nq = c->force_nq ? (int)c->force_nq : moduli_needed(c->L, ubits);
    if ((size_t)ref_nq > c->moduli.size()) {
      c->status[i] = MGCD_ERR_NOT_ENOUGH_MODULI;
      continue;
    }
    // Batches may use fewer moduli than the reference formula (less work per iteration);
    // a pair whose result cannot then be certified is rerun with the reference count.
    int nq = ref_nq;
    const float scale = c->cfg[size_class(ref_nq)].nq_scale;
    if (!plain && scale < 1.0f)
      nq = std::min(ref_nq, std::max(256, ((int)std::ceil(scale * ref_nq) + 255) / 256 * 256));
    d.nq = (uint32_t)nq;
    d.out_off = out_off;
    out_off += (uint32_t)ref_nq + 1;
    c->slot[i] = (int)c->descs.size();
    c->descs.push_back(d);
    c->ref_nq.push_back((uint32_t)ref_nq);
  }
  c->ndig = out_off;
  const size_t ng = c->descs.size();
  c->order.clear();
  std::vector<uint32_t> all(ng);
  for (uint32_t k = 0; k < ng; ++k) all[k] = k;
  size_t scratch = 0;
  int rc = schedule(c, c->descs, all, plain, c->buckets, c->grid_pairs, scratch);
  if (rc != MGCD_OK) return rc;
  c->scratch_words = scratch;
  c->eff_nq.clear();
  for (const PairDesc& d : c->descs) c->eff_nq.push_back(d.nq);

  // Device buffers and upload.
  CK(c->d_limbs.grow(std::max<uint64_t>(limb_end, 1) * sizeof(uint32_t)));
  CK(c->d_pairs.grow(std::max<size_t>(ng, 1) * sizeof(PairDesc)));
  CK(c->d_order.grow(std::max<size_t>(c->order.size(), 1) * sizeof(uint32_t)));
  CK(c->d_digits.grow(std::max<size_t>(c->ndig, 1) * sizeof(mgcd_pair)));
  CK(c->d_count.grow(std::max<size_t>(ng, 1) * sizeof(uint32_t)));
  CK(c->d_iters.grow(std::max<size_t>(ng, 1) * sizeof(uint32_t)));
  CK(c->d_status.grow(std::max<size_t>(ng, 1) * sizeof(int32_t)));
  CK(c->d_queue.grow(2 * NSTREAMS * sizeof(uint32_t)));
  CK(c->d_scratch.grow(std::max<size_t>(scratch, 1) * sizeof(uint32_t)));
  CK(c->d_gsync.grow(sizeof(GridSync)));
  c->h2d_bytes = ng ? limb_end * sizeof(uint32_t) + ng * sizeof(PairDesc) + c->order.size() * sizeof(uint32_t) : 0;
  if (ng) {
    CK(cudaMemcpyAsync(c->d_limbs.p, limbs, limb_end * sizeof(uint32_t), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_pairs.p, c->descs.data(), ng * sizeof(PairDesc), cudaMemcpyHostToDevice, c->stream));
    if (!c->order.empty())
      CK(cudaMemcpyAsync(c->d_order.p, c->order.data(), c->order.size() * sizeof(uint32_t),
                         cudaMemcpyHostToDevice, c->stream));
  }
  return MGCD_OK;
}

// Groups the pairs `subset` (indices into descs) into size-class buckets (batches) or
// single-pair launches (plain); appends the processing order to c->order and returns the
// scratch words needed.
static int schedule(mgcd_context* c, const std::vector<PairDesc>& descs, const std::vector<uint32_t>& subset,
                    bool plain, std::vector<Bucket>& buckets, std::vector<uint32_t>& grid_pairs, size_t& scratch)
{
  buckets.clear();
  grid_pairs.clear();
  const uint32_t plain_cta_max = 256;   // single pairs: one CTA, else a cluster or a grid
  std::vector<uint32_t> byb[NSTREAMS];
  for (uint32_t k : subset) {
    const uint32_t nq = descs[k].nq;
    if (plain) {
      if (nq <= plain_cta_max) byb[0].push_back(k); else grid_pairs.push_back(k);
    } else {
      byb[size_class(nq)].push_back(k);
    }
  }
  int kThreads[NSTREAMS], kSlots[NSTREAMS];
  for (int b = 0; b < NSTREAMS; ++b) {
    kThreads[b] = c->cfg[b].threads;
    kSlots[b] = c->cfg[b].k;
  }
  for (int b = NSTREAMS - 1; b >= 0; --b) {  // largest CTA size first: its pairs are the longest
    auto& v = byb[b];
    if (v.empty()) continue;
    std::sort(v.begin(), v.end(), [&](uint32_t x, uint32_t y) {
      const PairDesc &a = descs[x], &bb = descs[y];
      if (a.nq != bb.nq) return a.nq > bb.nq;
      return a.u_len + a.v_len > bb.u_len + bb.v_len;
    });
    Bucket bk;
    bk.threads = plain ? 256 : kThreads[b];
    bk.k = plain ? 1 : kSlots[b];
    bk.csize = 0;
    bk.cls = b;
    bk.first = (uint32_t)c->order.size();
    bk.n = (uint32_t)v.size();
    bk.nq_max = descs[v[0]].nq;
    bk.scratch_off = scratch;
    if (b == CLUSTER_CLASS) {
      // one pair per cluster; more CTAs per cluster when a pair's share exceeds shared memory
      int cs = c->cfg[b].csize;
      while (cs < MAX_CLUSTER && cluster_batch_smem_bytes(cs, bk.nq_max) > c->smem_optin) cs *= 2;
      cs = std::min(cs, MAX_CLUSTER);
      bk.csize = cs;
      bk.k = 1;
      bk.smem = cluster_batch_smem_bytes(cs, bk.nq_max);
      int nc = 0;
      if (bk.smem > c->smem_optin || cluster_batch_max_clusters(bk.threads, cs, bk.smem, &nc) != cudaSuccess ||
          nc < 1)
        return MGCD_ERR_GRID;
      bk.grid = (int)std::min<size_t>(v.size(), (size_t)nc);
      scratch += (size_t)bk.grid * 4 * bk.nq_max;
    } else {
      bk.smem = batch_smem_bytes(bk.threads, bk.k, bk.nq_max);
      int bps = 0;
      if (batch_max_blocks_per_sm(bk.threads, bk.k, bk.smem, &bps) != cudaSuccess || bps < 1) return MGCD_ERR_GRID;
      bk.grid = (int)std::min<size_t>((v.size() + bk.k - 1) / bk.k, (size_t)c->sms * bps);
      scratch += (size_t)bk.grid * 4 * bk.k * bk.nq_max;
    }
    c->order.insert(c->order.end(), v.begin(), v.end());
    buckets.push_back(bk);
  }
  uint32_t grid_nq_max = 0;
  for (uint32_t k : grid_pairs) grid_nq_max = std::max(grid_nq_max, descs[k].nq);
  c->grid_scratch_off = scratch;
  scratch += 4 * (size_t)grid_nq_max;
  return MGCD_OK;
}

int mgcd_batch_upload(mgcd_context* c, size_t np, const uint32_t* limbs, const uint64_t* u_off,
                      const uint32_t* u_len, const uint64_t* v_off, const uint32_t* v_len)
{
  return plan_batch(c, np, limbs, u_off, u_len, v_off, v_len, false);
}

int mgcd_set_nq_scale(mgcd_context* c, float scale)
{
  if (!c || !(scale >= 0.5f && scale <= 1.0f)) return MGCD_ERR_INVALID_ARG;
  for (auto& b : c->cfg) b.nq_scale = scale;
  return MGCD_OK;
}

int mgcd_set_size_class(mgcd_context* c, int cls, int threads, int k, float nq_scale)
{
  if (!c || cls < 0 || cls >= NSTREAMS || !(nq_scale >= 0.5f && nq_scale <= 1.0f)) return MGCD_ERR_INVALID_ARG;
  if (threads != 256 && threads != 512 && threads != 1024) return MGCD_ERR_INVALID_ARG;
  if (k != 1 && k != 2 && !(k == 4 && threads <= 512)) return MGCD_ERR_INVALID_ARG;
  if (cls == CLUSTER_CLASS && k != 1) return MGCD_ERR_INVALID_ARG;
  c->cfg[cls].threads = threads;
  c->cfg[cls].k = k;
  c->cfg[cls].nq_scale = nq_scale;
  return MGCD_OK;
}

int mgcd_set_cluster_size(mgcd_context* c, int ctas)
{
  if (!c || ctas < 2 || ctas > MAX_CLUSTER) return MGCD_ERR_INVALID_ARG;
  c->cfg[CLUSTER_CLASS].csize = ctas;
  return MGCD_OK;
}

int mgcd_get_cluster_size(const mgcd_context* c, int* ctas)
{
  if (!c || !ctas) return MGCD_ERR_INVALID_ARG;
  *ctas = c->cfg[CLUSTER_CLASS].csize;
  return MGCD_OK;
}

int mgcd_batch_use_graph(mgcd_context* c, int enable)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  c->use_graph = enable != 0;
  if (!c->use_graph) {
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    drop_graph(c);
  }
  return MGCD_OK;
}

int mgcd_set_single_pair_policy(mgcd_context* c, int policy)
{
  if (!c || (policy != MGCD_SINGLE_AUTO && policy != MGCD_SINGLE_REFERENCE_SHAPE)) return MGCD_ERR_INVALID_ARG;
  c->single_policy = policy;
  return MGCD_OK;
}

int mgcd_set_wait_timeout_ms(mgcd_context* c, unsigned ms)
{
  if (!c || ms == 0) return MGCD_ERR_INVALID_ARG;
  c->wait_timeout_ns = (unsigned long long)ms * 1000000ull;
  cudaStreamSynchronize(c->stream);
  drop_graph(c);
  return MGCD_OK;
}

int mgcd_test_force_moduli(mgcd_context* c, unsigned nq)
{
  if (!c || nq % 256 || nq > c->moduli.size()) return MGCD_ERR_INVALID_ARG;
  c->force_nq = nq;
  return MGCD_OK;
}

int mgcd_test_withhold_cta(mgcd_context* c, int cta)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  c->withhold_cta = cta < 0 ? 0xFFFFFFFFu : (uint32_t)cta;
  cudaStreamSynchronize(c->stream);
  drop_graph(c);
  return MGCD_OK;
}

int mgcd_get_size_class(const mgcd_context* c, int cls, int* threads, int* k, float* nq_scale)
{
  if (!c || cls < 0 || cls >= NSTREAMS) return MGCD_ERR_INVALID_ARG;
  if (threads) *threads = c->cfg[cls].threads;
  if (k) *k = c->cfg[cls].k;
  if (nq_scale) *nq_scale = c->cfg[cls].nq_scale;
  return MGCD_OK;
}

int mgcd_batch_kernel_stats(const mgcd_context* c, int i, int* cls, int* pairs, float* ms)
{
  if (!c || !c->ran || !c->bucket_timed || i < 0 || i >= (int)c->buckets.size()) return MGCD_ERR_INVALID_ARG;
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, c->t_b0[i], c->t_b1[i]));
  if (cls) *cls = c->buckets[i].cls;
  if (pairs) *pairs = (int)c->buckets[i].n;
  if (ms) *ms = t;
  return MGCD_OK;
}

// Launches the buckets (one stream each, joined back into c->stream) and then the
// cooperative-grid pairs.  `pairs` is the descriptor array on the device, `queue_base`
// the first of the bucket work counters (zeroed here).
static int launch_set(mgcd_context* c, const std::vector<Bucket>& buckets, const std::vector<uint32_t>& grid_pairs,
                      const std::vector<PairDesc>& descs, PairDesc* pairs, uint32_t* queue_base, bool time_buckets)
{
  CK(cudaMemsetAsync(queue_base, 0, NSTREAMS * sizeof(uint32_t), c->stream));
  CK(cudaEventRecord(c->ev_start, c->stream));
  for (size_t b = 0; b < buckets.size(); ++b) {
    const Bucket& bk = buckets[b];
    BatchArgs a;
    a.inv = InvTab{c->d_invtab.as<uint32_t>(), c->invtab_n};
    a.limbs = c->d_limbs.as<uint32_t>();
    a.pairs = pairs;
    a.order = c->d_order.as<uint32_t>() + bk.first;
    a.npairs = bk.n;
    a.mods = c->mods.as<ModConst>();
    a.L = c->L;
    a.queue = queue_base + b;
    a.scratch = c->d_scratch.as<uint32_t>() + bk.scratch_off;
    a.scratch_words = 4 * (size_t)bk.k * bk.nq_max;
    a.nq_max = bk.nq_max;
    a.digits = c->d_digits.as<mgcd_pair>();
    a.count = c->d_count.as<uint32_t>();
    a.iters = c->d_iters.as<uint32_t>();
    a.status = c->d_status.as<int32_t>();
    CK(cudaStreamWaitEvent(c->bstream[b], c->ev_start, 0));
    if (time_buckets) CK(cudaEventRecord(c->t_b0[b], c->bstream[b]));
    if (bk.csize)
      CK(launch_cluster_batch(a, bk.threads, bk.csize, bk.grid, bk.smem, c->bstream[b]));
    else
      CK(launch_batch(a, bk.threads, bk.k, bk.grid, bk.smem, c->bstream[b]));
    if (time_buckets) CK(cudaEventRecord(c->t_b1[b], c->bstream[b]));
    CK(cudaEventRecord(c->ev_b[b], c->bstream[b]));
    ++c->launches;
  }
  for (size_t b = 0; b < buckets.size(); ++b) CK(cudaStreamWaitEvent(c->stream, c->ev_b[b], 0));

  if (!grid_pairs.empty()) {
    for (uint32_t k : grid_pairs) {
      const PairDesc& d = descs[k];
      GridArgs g;
      g.inv = InvTab{c->d_invtab.as<uint32_t>(), c->invtab_n};
      g.limbs = c->d_limbs.as<uint32_t>();
      g.pair = d;
      g.mods = c->mods.as<ModConst>();
      g.L = c->L;
      g.scratch = c->d_scratch.as<uint32_t>() + c->grid_scratch_off;
      g.digits = c->d_digits.as<mgcd_pair>();
      g.count = c->d_count.as<uint32_t>() + k;
      g.iters = c->d_iters.as<uint32_t>() + k;
      g.status = c->d_status.as<int32_t>() + k;
      const bool ref_shape = c->single_policy == MGCD_SINGLE_REFERENCE_SHAPE;
      if (!ref_shape && d.nq <= (uint32_t)MAX_CLUSTER * 1024) {
        // thread-block cluster: as many CTAs (<= 16) as keep one modulus per thread
        const int ctas = (int)std::min<uint32_t>(MAX_CLUSTER, (d.nq + 255) / 256);
        const uint32_t per = (d.nq + ctas - 1) / ctas;
        const int threads = per <= 256 ? 256 : per <= 512 ? 512 : 1024;
        g.per_cta = per;
        g.sync = nullptr;
        if (launch_cluster(g, threads, ctas, grid_smem_bytes(per), c->stream) != cudaSuccess) return MGCD_ERR_GRID;
        ++c->launches;
        continue;
      }
      // cooperative grid: one CTA per SM (or the reference's shape: 256-thread CTAs, 256 moduli)
      uint32_t per = ref_shape ? 256u : std::max<uint32_t>(32, (d.nq + c->sms - 1) / c->sms);
      const int threads = (ref_shape || per <= 256) ? 256 : per <= 512 ? 512 : GRID_THREADS;
      int bps = 0;
      if (grid_max_blocks_per_sm(threads, grid_smem_bytes(per), &bps) != cudaSuccess || bps < 1) return MGCD_ERR_GRID;
      uint32_t grid = (d.nq + per - 1) / per;
      if (grid > (uint32_t)(c->sms * bps)) {
        per = (d.nq + c->sms * bps - 1) / (c->sms * bps);
        grid = (d.nq + per - 1) / per;
        if (grid_max_blocks_per_sm(threads, grid_smem_bytes(per), &bps) != cudaSuccess ||
            grid > (uint32_t)(c->sms * bps))
          return MGCD_ERR_GRID;
      }
      g.per_cta = per;
      g.sync = c->d_gsync.as<GridSync>();
      CK(launch_gridsync_init(g.sync, c->wait_timeout_ns, c->withhold_cta, c->stream));
      ++c->launches;
      cudaError_t e = launch_grid(g, threads, (int)grid, grid_smem_bytes(per), c->stream);
      if (e == cudaErrorCooperativeLaunchTooLarge) return MGCD_ERR_GRID;
      if (e != cudaSuccess) return MGCD_ERR_CUDA;
      ++c->launches;
    }
  }
  return MGCD_OK;
}

static int run_plan(mgcd_context* c)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  c->launches = 0;
  c->retried = 0;
  const size_t ng = c->descs.size();
  if (ng == 0) {
    c->ran = true;
    return MGCD_OK;
  }
  if (c->use_graph && !c->plain) {
    if (!c->graph) {
      // Record the run once (status reset, queue reset, every bucket kernel on its stream,
      // joined back into c->stream); each later run is a single graph launch.
      CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      int rc = MGCD_OK;
      if (cudaMemsetAsync(c->d_status.p, 0xFF, ng * sizeof(int32_t), c->stream) != cudaSuccess) rc = MGCD_ERR_CUDA;
      if (rc == MGCD_OK)
        rc = launch_set(c, c->buckets, c->grid_pairs, c->descs, c->d_pairs.as<PairDesc>(), c->d_queue.as<uint32_t>(),
                        false);
      cudaGraph_t g = nullptr;
      const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
      if (rc == MGCD_OK && e != cudaSuccess) rc = MGCD_ERR_CUDA;
      if (rc == MGCD_OK && cudaGraphInstantiate(&c->graph, g, 0) != cudaSuccess) {
        c->graph = nullptr;
        rc = MGCD_ERR_CUDA;
      }
      if (g) cudaGraphDestroy(g);
      if (rc != MGCD_OK) return rc;
      c->graph_kernels = c->launches;
    }
    CK(cudaEventRecord(c->t_run0, c->stream));
    CK(cudaGraphLaunch(c->graph, c->stream));
    c->launches = c->graph_kernels;
    c->bucket_timed = false;
  } else {
    CK(cudaEventRecord(c->t_run0, c->stream));
    CK(cudaMemsetAsync(c->d_status.p, 0xFF, ng * sizeof(int32_t), c->stream));
    int rc = launch_set(c, c->buckets, c->grid_pairs, c->descs, c->d_pairs.as<PairDesc>(), c->d_queue.as<uint32_t>(),
                        true);
    if (rc != MGCD_OK) return rc;
    c->bucket_timed = true;
  }
  CK(cudaEventRecord(c->t_run1, c->stream));
  c->ran = true;
  c->synced = false;
  return MGCD_OK;
}

// Waits for the run; pairs that ran with fewer moduli than the reference count and could
// not be certified are rerun once with the reference count (same digit slots).
static int sync_plan(mgcd_context* c)
{
  if (!c || !c->ran) return MGCD_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  if (c->synced) return MGCD_OK;
  c->synced = true;
  const size_t ng = c->descs.size();
  bool scaled = false;
  for (size_t k = 0; k < ng && !scaled; ++k) scaled = c->descs[k].nq < c->ref_nq[k];
  if (!scaled) return MGCD_OK;
  CK(c->h_status.grow(ng * sizeof(int32_t)));
  CK(cudaMemcpy(c->h_status.p, c->d_status.p, ng * sizeof(int32_t), cudaMemcpyDeviceToHost));
  const int32_t* st = c->h_status.as<int32_t>();
  std::vector<uint32_t> redo;
  for (uint32_t k = 0; k < ng; ++k)
    if (st[k] != ST_OK && st[k] != ST_TIMEOUT && c->descs[k].nq < c->ref_nq[k]) redo.push_back(k);
  if (redo.empty()) return MGCD_OK;
  std::vector<PairDesc> rd = c->descs;
  for (uint32_t k : redo) rd[k].nq = c->ref_nq[k];
  const size_t main_order = c->order.size();
  std::vector<Bucket> bks;
  std::vector<uint32_t> gp;
  size_t scratch = 0;
  const size_t keep_grid_off = c->grid_scratch_off;
  int rc = schedule(c, rd, redo, false, bks, gp, scratch);
  if (rc != MGCD_OK) return rc;
  // device buffers: retry descriptors after the main ones, retry order after the main order
  CK(c->d_retry.grow(ng * sizeof(PairDesc)));
  if (c->order.size() * sizeof(uint32_t) > c->d_order.bytes) {
    // keep the main order: grow by copying
    DevBuf nb;
    CK(nb.grow(c->order.size() * sizeof(uint32_t)));
    CK(cudaMemcpy(nb.p, c->d_order.p, main_order * sizeof(uint32_t), cudaMemcpyDeviceToDevice));
    drop_graph(c);
    c->d_order.release();
    c->d_order = nb;
  }
  if (scratch > c->d_scratch.bytes / sizeof(uint32_t)) {
    drop_graph(c);
    c->d_scratch.release();
    CK(c->d_scratch.grow(scratch * sizeof(uint32_t)));
  }
  CK(cudaMemcpyAsync(c->d_retry.p, rd.data(), ng * sizeof(PairDesc), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->d_order.as<uint32_t>() + main_order, c->order.data() + main_order,
                     (c->order.size() - main_order) * sizeof(uint32_t), cudaMemcpyHostToDevice, c->stream));
  rc = launch_set(c, bks, gp, rd, c->d_retry.as<PairDesc>(), c->d_queue.as<uint32_t>() + NSTREAMS, false);
  c->order.resize(main_order);               // the plan itself is unchanged for later runs
  c->grid_scratch_off = keep_grid_off;
  if (rc != MGCD_OK) return rc;
  CK(cudaEventRecord(c->t_run1, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->retried = (int)redo.size();
  return MGCD_OK;
}

int mgcd_batch_elapsed_ms(const mgcd_context* c, float* run_ms, float* dominant_ms, int* dominant_threads)
{
  if (!c || !c->ran) return MGCD_ERR_INVALID_ARG;
  float r = 0.f, best = 0.f;
  int bt = 0;
  if (!c->descs.empty()) {
    CK(cudaEventElapsedTime(&r, c->t_run0, c->t_run1));
    for (size_t b = 0; b < c->buckets.size(); ++b) {
      float t = 0.f;
      CK(cudaEventElapsedTime(&t, c->t_b0[b], c->t_b1[b]));
      if (t > best) { best = t; bt = c->buckets[b].threads; }
    }
  }
  if (run_ms) *run_ms = r;
  if (dominant_ms) *dominant_ms = best;
  if (dominant_threads) *dominant_threads = bt;
  return MGCD_OK;
}

int mgcd_batch_transfer_bytes(const mgcd_context* c, uint64_t* h2d, uint64_t* d2h)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  if (h2d) *h2d = c->h2d_bytes;
  if (d2h) *d2h = c->d2h_bytes;
  return MGCD_OK;
}

int mgcd_int_peak(mgcd_context* c, double* ops)
{
  if (!c || !ops) return MGCD_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  uint32_t* sink = nullptr;
  CK(cudaMalloc(&sink, sizeof(uint32_t)));
  const int blocks = c->sms * 8, iters = 1 << 16;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  int rc = MGCD_OK;
  for (int rep = 0; rep < 4 && rc == MGCD_OK; ++rep) {
    cudaEventRecord(a, c->stream);
    if (launch_int_peak(sink, blocks, iters, c->stream) != cudaSuccess) rc = MGCD_ERR_CUDA;
    cudaEventRecord(b, c->stream);
    if (cudaEventSynchronize(b) != cudaSuccess) rc = MGCD_ERR_CUDA;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (rep > 0) best = std::min(best, ms);   // first launch is a warm-up
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(sink);
  if (rc != MGCD_OK) return rc;
  *ops = (double)blocks * 256.0 * iters * 8.0 / (best * 1e-3);
  return MGCD_OK;
}

int mgcd_batch_run(mgcd_context* c) { return run_plan(c); }

int mgcd_batch_sync(mgcd_context* c) { return sync_plan(c); }

int mgcd_batch_retried(const mgcd_context* c, int* pairs)
{
  if (!c || !pairs) return MGCD_ERR_INVALID_ARG;
  *pairs = c->retried;
  return MGCD_OK;
}

int mgcd_batch_launches(const mgcd_context* c, int* launches)
{
  if (!c || !launches) return MGCD_ERR_INVALID_ARG;
  *launches = c->launches;
  return MGCD_OK;
}

// Copies the GPU results of the plan to pinned host memory.
static int fetch(mgcd_context* c)
{
  const size_t ng = c->descs.size();
  CK(cudaSetDevice(c->device));
  if (ng == 0) return MGCD_OK;
  CK(c->h_count.grow(ng * sizeof(uint32_t)));
  CK(c->h_iters.grow(ng * sizeof(uint32_t)));
  CK(c->h_status.grow(ng * sizeof(int32_t)));
  CK(c->h_digits.grow(std::max<size_t>(c->ndig, 1) * sizeof(mgcd_pair)));
  CK(cudaMemcpyAsync(c->h_count.p, c->d_count.p, ng * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(c->h_iters.p, c->d_iters.p, ng * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(c->h_status.p, c->d_status.p, ng * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(c->h_digits.p, c->d_digits.p, c->ndig * sizeof(mgcd_pair), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->d2h_bytes = ng * (2 * sizeof(uint32_t) + sizeof(int32_t)) + c->ndig * sizeof(mgcd_pair);
  // work by the cost model
  const uint32_t* it = c->h_iters.as<uint32_t>();
  const uint32_t* cnt = c->h_count.as<uint32_t>();
  const int32_t* st = c->h_status.as<int32_t>();
  double R = 0, E = 0, M = 0, B = 0;
  for (size_t k = 0; k < ng; ++k) {
    const PairDesc& d = c->descs[k];
    R += (double)d.nq * (d.u_len + d.v_len);
    B += 4.0 * (d.u_len + d.v_len);
    if (st[k] != ST_OK) continue;
    const double I = it[k], K = cnt[k], N = c->eff_nq[k];
    E += I * N - I * (I + 1) / 2;
    M += K * (N - I) - K * (K + 1) / 2;
  }
  c->work[0] = R; c->work[1] = E; c->work[2] = M; c->work[3] = B;
  return MGCD_OK;
}

int mgcd_batch_work(const mgcd_context* c, double* r, double* e, double* m, double* b)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  if (r) *r = c->work[0];
  if (e) *e = c->work[1];
  if (m) *m = c->work[2];
  if (b) *b = c->work[3];
  return MGCD_OK;
}

static int convert_all(mgcd_context* c, uint32_t* g, const uint64_t* g_off, const uint32_t* g_cap,
                       uint32_t* g_len, int32_t* status)
{
  const size_t np = c->np;
  const mgcd_pair* dig = c->h_digits.as<mgcd_pair>();
  const uint32_t* cnt = c->h_count.as<uint32_t>();
  const int32_t* st = c->h_status.as<int32_t>();
  std::atomic<size_t> next{0};
  auto work = [&]() {
    for (;;) {
      const size_t i = next.fetch_add(1);
      if (i >= np) break;
      int s = c->status[i];
      size_t len = 0;
      if (c->slot[i] >= 0) {
        const int k = c->slot[i];
        s = to_status(st[k]);
        if (s == MGCD_OK && mixed_radix_to_limbs(dig + c->descs[k].out_off, cnt[k], g + g_off[i], g_cap[i], &len))
          s = MGCD_ERR_CAPACITY;
      } else if (s == MGCD_OK) {
        len = c->trivial[i].size();
        if (len > g_cap[i]) { s = MGCD_ERR_CAPACITY; len = 0; }
        else if (len) std::memcpy(g + g_off[i], c->trivial[i].data(), len * sizeof(uint32_t));
      }
      g_len[i] = (uint32_t)len;
      if (status) status[i] = s;
    }
  };
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = std::min<size_t>(hw, (np + 15) / 16);
  if (nt <= 1) {
    work();
  } else {
    std::vector<std::thread> th;
    for (size_t t = 0; t < nt; ++t) th.emplace_back(work);
    for (auto& t : th) t.join();
  }
  int rc = MGCD_OK;
  for (size_t i = 0; i < np && rc == MGCD_OK; ++i) {
    if (status) { if (status[i] != MGCD_OK) rc = status[i]; }
  }
  return rc;
}

int mgcd_batch_download(mgcd_context* c, uint32_t* g, const uint64_t* g_off, const uint32_t* g_cap,
                        uint32_t* g_len, int32_t* status)
{
  if (!c || !c->ran || (c->np && (!g || !g_off || !g_cap || !g_len || !status))) return MGCD_ERR_INVALID_ARG;
  int rc = sync_plan(c);
  if (rc != MGCD_OK) return rc;
  rc = fetch(c);
  if (rc != MGCD_OK) return rc;
  return convert_all(c, g, g_off, g_cap, g_len, status);
}

int mgcd_gcd_batch(mgcd_context* c, size_t np, const uint32_t* limbs, const uint64_t* u_off,
                   const uint32_t* u_len, const uint64_t* v_off, const uint32_t* v_len, uint32_t* g,
                   const uint64_t* g_off, const uint32_t* g_cap, uint32_t* g_len, int32_t* status)
{
  int rc = plan_batch(c, np, limbs, u_off, u_len, v_off, v_len, false);
  if (rc != MGCD_OK) return rc;
  rc = run_plan(c);
  if (rc != MGCD_OK) return rc;
  return mgcd_batch_download(c, g, g_off, g_cap, g_len, status);
}

// ------------------------------------------------------------------ single pair ----

static int single(mgcd_context* c, const uint32_t* u, size_t uSz, const uint32_t* v, size_t vSz)
{
  if (!c || (uSz && !u) || (vSz && !v)) return MGCD_ERR_INVALID_ARG;
  // Pack both operands contiguously (the plan reads one limb array).
  static thread_local std::vector<uint32_t> buf;
  buf.resize(uSz + vSz);
  if (uSz) std::memcpy(buf.data(), u, uSz * sizeof(uint32_t));
  if (vSz) std::memcpy(buf.data() + uSz, v, vSz * sizeof(uint32_t));
  const uint64_t uo = 0, vo = uSz;
  const uint32_t ul = (uint32_t)uSz, vl = (uint32_t)vSz;
  int rc = plan_batch(c, 1, buf.data(), &uo, &ul, &vo, &vl, true);
  if (rc != MGCD_OK) return rc;
  rc = run_plan(c);
  if (rc != MGCD_OK) return rc;
  rc = sync_plan(c);
  if (rc != MGCD_OK) return rc;
  return fetch(c);
}

int mgcd_gcd_digits(mgcd_context* c, const uint32_t* u, size_t uSz, const uint32_t* v, size_t vSz,
                    mgcd_pair* digits, size_t cap, size_t* count)
{
  if (!count || (cap && !digits)) return MGCD_ERR_INVALID_ARG;
  *count = 0;
  if (strip(u, uSz) == 0 || strip(v, vSz) == 0) return MGCD_ERR_INVALID_ARG;
  int rc = single(c, u, uSz, v, vSz);
  if (rc != MGCD_OK) return rc;
  if (c->slot[0] < 0) return c->status[0];
  const int32_t st = c->h_status.as<int32_t>()[0];
  if (st != ST_OK) return to_status(st);
  const uint32_t n = c->h_count.as<uint32_t>()[0];
  if (n > cap) return MGCD_ERR_CAPACITY;
  std::memcpy(digits, c->h_digits.as<mgcd_pair>() + c->descs[0].out_off, n * sizeof(mgcd_pair));
  *count = n;
  return MGCD_OK;
}

int mgcd_gcd(mgcd_context* c, const uint32_t* u, size_t uSz, const uint32_t* v, size_t vSz, uint32_t* g,
             size_t g_cap, size_t* g_len)
{
  if (!g_len || (g_cap && !g)) return MGCD_ERR_INVALID_ARG;
  *g_len = 0;
  int rc = single(c, u, uSz, v, vSz);
  if (rc != MGCD_OK) return rc;
  const uint64_t off = 0;
  const uint32_t cap = (uint32_t)std::min<size_t>(g_cap, 0xFFFFFFFFu);
  uint32_t len = 0;
  int32_t st = 0;
  rc = convert_all(c, g, &off, &cap, &len, &st);
  *g_len = len;
  return rc;
}

}  // extern "C"

// mgcd_capi.cpp -- the C ABI (include/modgcd.h): contexts, batch planning and launches,
// result conversion.
//
// Host flow of one batch (the reference's per-call flow, GmpCudaDevice-gcd.cu:59-132,
// generalised to many pairs):
//   upload    order each pair so that u >= v (the reference swaps its mpz operands,
//             :61-62), strip leading zero limbs, size the moduli (numModuliNeededFor,
//             :49-55) and reject pairs that need more moduli than the table holds (:76-78);
//             pairs with a zero operand are answered on the host (gcd(x, 0) = x);
//             group the rest by size into size-class buckets, largest first; copy the batch.
//   run       one persistent kernel per bucket, chained on one stream by programmatic
//             dependent launches so that the buckets overlap, largest class placed first;
//             single pairs too large for one CTA run on a cluster or a cooperative grid.
//   download  copy digits back and convert each pair's digits to binary.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/modgcd.h"
#include "mgcd_internal.h"
#include "mgcd_moduli.h"
#include "mgcd_plan.h"
#include "mgcd_radix.h"

using namespace mgcd;

#define CK(call)                                     \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return MGCD_ERR_CUDA;     \
  } while (0)

namespace mgcd {

cudaError_t DevBuf::grow(size_t want, cudaMemPool_t pool, cudaStream_t s)
{
  if (want <= bytes) return cudaSuccess;
  if (p) cudaFreeAsync(p, s);
  p = nullptr;
  bytes = 0;
  const size_t sz = std::max<size_t>(want + want / 4, 256);
  cudaError_t e = cudaMallocFromPoolAsync(&p, sz, pool, s);
  if (e == cudaSuccess) bytes = sz;
  return e;
}

void DevBuf::release(cudaStream_t s)
{
  if (p) cudaFreeAsync(p, s);
  p = nullptr;
  bytes = 0;
}

cudaError_t HostBuf::grow(size_t want)
{
  if (want <= bytes) return cudaSuccess;
  if (p) retired.push_back(p);
  p = nullptr;
  const size_t sz = std::max<size_t>(std::max(want, 2 * bytes), 4096);
  bytes = 0;
  cudaError_t e = cudaHostAlloc(&p, sz, cudaHostAllocDefault);
  if (e == cudaSuccess) bytes = sz;
  return e;
}

void HostBuf::release()
{
  for (void* q : retired) cudaFreeHost(q);
  retired.clear();
  if (p) cudaFreeHost(p);
  p = nullptr;
  bytes = 0;
}

cudaError_t Plan::create(int priority)
{
  if (cudaStreamCreateWithPriority(&stream, cudaStreamNonBlocking, priority) != cudaSuccess ||
      cudaEventCreate(&t_run0) != cudaSuccess || cudaEventCreate(&t_run1) != cudaSuccess)
    return cudaErrorUnknown;
  return cudaSuccess;
}

void Plan::drop_graph()
{
  if (graph) cudaGraphExecDestroy(graph);
  graph = nullptr;
  graph_kernels = 0;
}

void Plan::destroy(cudaMemPool_t)
{
  if (stream) cudaStreamSynchronize(stream);
  drop_graph();
  for (DevBuf* b : {&d_limbs, &d_pairs, &d_order, &d_digits, &d_count, &d_iters, &d_status, &d_queue, &d_scratch,
                    &d_gsync, &d_retry, &d_glimbs, &d_glen, &d_nqf, &d_upd, &d_span})
    b->release(stream);
  if (stream) cudaStreamSynchronize(stream);
  for (HostBuf* b : {&h_count, &h_iters, &h_status, &h_digits, &h_glimbs, &h_glen, &h_nqf, &h_upd}) b->release();
  if (t_run0) cudaEventDestroy(t_run0);
  if (t_run1) cudaEventDestroy(t_run1);
  if (stream) cudaStreamDestroy(stream);
  t_run0 = t_run1 = nullptr;
  stream = nullptr;
}

size_t Plan::device_bytes() const
{
  size_t s = 0;
  for (const DevBuf* b : {&d_limbs, &d_pairs, &d_order, &d_digits, &d_count, &d_iters, &d_status, &d_queue,
                          &d_scratch, &d_gsync, &d_retry, &d_glimbs, &d_glen, &d_nqf, &d_upd, &d_span})
    s += b->bytes;
  return s;
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

}  // namespace mgcd

namespace {

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

bool busy(const mgcd_context* c) { return c->serving; }

}  // namespace

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
  // Batches and servers keep many streams busy at once; with the default 8 hardware
  // connections unrelated streams share queues and wait on each other.  Only takes effect
  // if the process has not created its CUDA context yet; a caller's setting is kept.
  setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
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
  // A private stream-ordered pool that keeps freed memory for reuse.
  cudaMemPoolProps pp = {};
  pp.allocType = cudaMemAllocationTypePinned;
  pp.location.type = cudaMemLocationTypeDevice;
  pp.location.id = device;
  if (cudaMemPoolCreate(&c->pool, &pp) != cudaSuccess) {
    c->pool = nullptr;
    rc = MGCD_ERR_CUDA;
  }
  if (rc == MGCD_OK) {
    uint64_t keep = ~0ull;
    cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  if (rc == MGCD_OK && c->main.create() != cudaSuccess) rc = MGCD_ERR_CUDA;
  cudaStream_t s = c->main.stream;
  if (rc == MGCD_OK && c->mods.grow(mc.size() * sizeof(ModConstHost), c->pool, s) != cudaSuccess) rc = MGCD_ERR_CUDA;
  if (rc == MGCD_OK &&
      cudaMemcpyAsync(c->mods.p, mc.data(), mc.size() * sizeof(ModConstHost), cudaMemcpyHostToDevice, s) != cudaSuccess)
    rc = MGCD_ERR_CUDA;
  // Pairwise inverses of the first INVTAB_N moduli (every pair of the CTA classes), for
  // recovery: 1 GiB at n = 16,384.
  c->invtab_n = (uint32_t)std::min<size_t>(INVTAB_N, c->moduli.size());
  if (rc == MGCD_OK && c->d_invtab.grow((size_t)c->invtab_n * c->invtab_n * sizeof(uint32_t), c->pool, s) != cudaSuccess)
    rc = MGCD_ERR_CUDA;
  if (rc == MGCD_OK && (launch_build_invtab(c->mods.as<ModConst>(), c->invtab_n, c->d_invtab.as<uint32_t>(), s) !=
                            cudaSuccess ||
                        cudaStreamSynchronize(s) != cudaSuccess))
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
  if (busy(c)) return MGCD_ERR_BUSY;
  cudaSetDevice(c->device);
  cudaStream_t s = c->main.stream;
  if (s) {
    cudaStreamSynchronize(s);
    c->mods.release(s);
    c->d_invtab.release(s);
  }
  c->main.destroy(c->pool);
  if (c->pool) cudaMemPoolDestroy(c->pool);
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

}  // extern "C"

// ------------------------------------------------------------------------- batch ----

static int schedule(mgcd_context* c, Plan& P, std::vector<PairDesc>& descs, const std::vector<uint32_t>& subset,
                    bool plain, std::vector<Bucket>& buckets, std::vector<uint32_t>& grid_pairs, size_t& scratch,
                    bool latency = false);

int mgcd::plan_batch(mgcd_context* c, Plan& P, size_t np, const uint32_t* limbs, const uint64_t* u_off,
                     const uint32_t* u_len, const uint64_t* v_off, const uint32_t* v_len, bool plain,
                     const uint64_t* g_off, const uint32_t* g_cap)
{
  if (!c || (np && (!limbs || !u_off || !u_len || !v_off || !v_len))) return MGCD_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(P.stream));   // buffers below may be reallocated
  P.drop_graph();
  P.np = np;
  P.plain = plain;
  P.ran = false;
  P.status.assign(np, -1);
  P.slot.assign(np, -1);
  P.trivial.assign(np, {});
  P.descs.clear();
  P.ref_nq.clear();
  P.grid_pairs.clear();
  P.buckets.clear();
  uint64_t limb_end = 0;
  uint32_t out_off = 0;
  uint64_t glimbs = 0;
  for (size_t i = 0; i < np; ++i) {
    const uint32_t* u = limbs + u_off[i];
    const uint32_t* v = limbs + v_off[i];
    size_t ul = strip(u, u_len[i]), vl = strip(v, v_len[i]);
    limb_end = std::max<uint64_t>(limb_end, std::max(u_off[i] + u_len[i], v_off[i] + v_len[i]));
    if (ul == 0 || vl == 0) {  // gcd(x, 0) = |x|: no modular work
      const uint32_t* x = ul ? u : v;
      P.trivial[i].assign(x, x + (ul ? ul : vl));
      P.status[i] = MGCD_OK;
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
      P.status[i] = MGCD_ERR_NOT_ENOUGH_MODULI;
      continue;
    }
    // Batches may use fewer moduli than the reference formula (less work per iteration);
    // a pair whose result cannot then be certified is rerun with the reference count.  The
    // scaled count is rounded up to a warp (32): rounding to the reference's 256 undid the
    // scale for pairs below ~16k bits (reference counts of 512-2,048).
    int nq = ref_nq;
    const float scale = c->cfg[size_class(ref_nq)].nq_scale;
    if (!plain && scale < 1.0f)
      nq = std::min(ref_nq, std::max(256, ((int)std::ceil(scale * ref_nq) + 31) / 32 * 32));
    d.nq = (uint32_t)nq;
    d.out_off = out_off;
    // digit slots: up to the moduli the pair may end with (a grown set: grow_cap)
    const uint32_t slots = (!plain && c->grow_start > 0.0f) ? std::max((uint32_t)ref_nq, grow_cap(ref_nq)) : ref_nq;
    if ((uint64_t)out_off + (uint64_t)slots + 1 > 0xFFFFFFFFull) return MGCD_ERR_CAPACITY;   // digit slots of one batch
    out_off += slots + 1;
    d.g_off = glimbs;                 // gcd <= the smaller operand
    d.g_cap = d.v_len;
    d.nq_cap = 0;
    glimbs += d.g_cap;
    P.slot[i] = (int)P.descs.size();
    P.descs.push_back(d);
    P.ref_nq.push_back((uint32_t)ref_nq);
  }
  P.ndig = out_off;
  P.nglimbs = glimbs;
  P.direct = false;
  P.in_place = false;
  P.direct_base = 0;
  if (g_off && g_cap && np) {
    // The caller's result slots in place of the compact layout when they are contiguous
    // (g_off[i + 1] = g_off[i] + g_cap[i]) and not much larger than it: the device writes
    // each gcd where the caller wants it and one copy brings back the whole span.  A slot
    // smaller than the gcd is left to the host conversion, which reports it as before.
    bool tiled = true;
    for (size_t i = 0; i + 1 < np && tiled; ++i) tiled = g_off[i + 1] == g_off[i] + g_cap[i];
    const uint64_t span = tiled ? g_off[np - 1] + g_cap[np - 1] - g_off[0] : 0;
    if (tiled && span <= 2 * glimbs + 4096) {
      P.direct = true;
      P.direct_base = g_off[0];
      P.nglimbs = span;
      for (size_t i = 0; i < np; ++i) {
        if (P.slot[i] < 0) continue;
        PairDesc& d = P.descs[P.slot[i]];
        d.g_off = g_off[i] - g_off[0];
        d.g_cap = std::min(d.v_len, g_cap[i]);
      }
    }
  }
  const size_t ng = P.descs.size();
  P.order.clear();
  std::vector<uint32_t> all(ng);
  for (uint32_t k = 0; k < ng; ++k) all[k] = k;
  size_t scratch = 0;
  int rc = schedule(c, P, P.descs, all, plain, P.buckets, P.grid_pairs, scratch);
  if (rc != MGCD_OK) return rc;
  P.scratch_words = scratch;
  P.eff_nq.clear();
  for (const PairDesc& d : P.descs) P.eff_nq.push_back(d.nq);

  // Device buffers and upload.
  cudaStream_t s = P.stream;
  // + 4 limbs: the kernels stage operand tiles by bulk copies widened to 16-byte bounds
  CK(P.d_limbs.grow((std::max<uint64_t>(limb_end, 1) + 4) * sizeof(uint32_t), c->pool, s));
  if (reinterpret_cast<uintptr_t>(P.d_limbs.p) % 16 != 0) return MGCD_ERR_CUDA;   // pool blocks are 256-aligned
  CK(P.d_pairs.grow(std::max<size_t>(ng, 1) * sizeof(PairDesc), c->pool, s));
  CK(P.d_order.grow(std::max<size_t>(P.order.size(), 1) * sizeof(uint32_t), c->pool, s));
  CK(P.d_digits.grow(std::max<size_t>(P.ndig, 1) * sizeof(mgcd_pair), c->pool, s));
  CK(P.d_count.grow(std::max<size_t>(ng, 1) * sizeof(uint32_t), c->pool, s));
  CK(P.d_iters.grow(std::max<size_t>(ng, 1) * sizeof(uint32_t), c->pool, s));
  CK(P.d_status.grow(std::max<size_t>(ng, 1) * sizeof(int32_t), c->pool, s));
  CK(P.d_nqf.grow(std::max<size_t>(ng, 1) * sizeof(uint32_t), c->pool, s));
  CK(P.d_span.grow(2 * NSTREAMS * sizeof(unsigned long long), c->pool, s));
  CK(P.d_upd.grow(std::max<size_t>(ng, 1) * sizeof(unsigned long long), c->pool, s));
  CK(P.d_queue.grow(2 * NSTREAMS * sizeof(uint32_t), c->pool, s));
  CK(P.d_scratch.grow(std::max<size_t>(scratch, 1) * sizeof(uint32_t), c->pool, s));
  CK(P.d_gsync.grow(sizeof(GridSync), c->pool, s));
  CK(P.d_glimbs.grow(std::max<size_t>(P.nglimbs, 1) * sizeof(uint32_t), c->pool, s));
  CK(P.d_glen.grow(std::max<size_t>(ng, 1) * sizeof(uint32_t), c->pool, s));
  P.h2d_bytes = ng ? limb_end * sizeof(uint32_t) + ng * sizeof(PairDesc) + P.order.size() * sizeof(uint32_t) : 0;
  if (ng) {
    CK(cudaMemcpyAsync(P.d_limbs.p, limbs, limb_end * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(P.d_pairs.p, P.descs.data(), ng * sizeof(PairDesc), cudaMemcpyHostToDevice, s));
    if (!P.order.empty())
      CK(cudaMemcpyAsync(P.d_order.p, P.order.data(), P.order.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
  }
  return MGCD_OK;
}

// Groups the pairs `subset` (indices into descs) into size-class buckets (batches) or
// single-pair launches (plain); appends the processing order to P.order and returns the
// scratch words needed.  `latency`: the few pairs rerun after a scaled batch -- one
// launch in which every pair has a thread-block cluster of its own (about 512 moduli per
// CTA), so that they run side by side across the GPU instead of one CTA each.
static int schedule(mgcd_context* c, Plan& P, std::vector<PairDesc>& descs, const std::vector<uint32_t>& subset,
                    bool plain, std::vector<Bucket>& buckets, std::vector<uint32_t>& grid_pairs, size_t& scratch,
                    bool latency)
{
  buckets.clear();
  grid_pairs.clear();
  if (latency && !subset.empty()) {
    std::vector<uint32_t> v(subset);
    std::sort(v.begin(), v.end(), [&](uint32_t x, uint32_t y) { return descs[x].nq > descs[y].nq; });
    Bucket bk;
    bk.threads = 512;
    bk.k = 1;
    bk.cls = CLUSTER_CLASS;
    bk.first = (uint32_t)P.order.size();
    bk.n = (uint32_t)v.size();
    bk.nq_max = descs[v[0]].nq;
    bk.scratch_off = scratch;
    int cs = 2;
    while (cs < MAX_CLUSTER && (bk.nq_max + cs - 1) / cs > 512u) cs *= 2;
    const size_t room = c->smem_optin - 24576;
    while (cs < MAX_CLUSTER && cluster_batch_smem_bytes(cs, bk.nq_max, 1) > room) cs *= 2;
    bk.csize = cs;
    bk.smem = cluster_batch_smem_bytes(cs, bk.nq_max, 1);
    int nc = 0;
    if (bk.smem > room || cluster_batch_max_clusters(bk.threads, 1, cs, bk.smem, &nc) != cudaSuccess || nc < 1)
      return MGCD_ERR_GRID;
    bk.grid = (int)std::min<size_t>(v.size(), (size_t)nc);
    scratch += (size_t)bk.grid * 4 * bk.nq_max;
    P.order.insert(P.order.end(), v.begin(), v.end());
    buckets.push_back(bk);
    P.grid_scratch_off = scratch;
    return MGCD_OK;
  }
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
  for (int b = NSTREAMS - 1; b >= 0; --b) {  // largest class first: its pairs are the longest
    auto& v = byb[b];
    if (v.empty()) continue;
    // longest pairs first: by moduli count, then operand length, both descending (ties by
    // index); the keys are gathered once, which halves the sort's time against a comparator
    // that loads two descriptors per comparison
    {
      std::vector<std::pair<uint64_t, uint32_t>> key(v.size());
      for (size_t i = 0; i < v.size(); ++i) {
        const PairDesc& a = descs[v[i]];
        key[i] = {(uint64_t)a.nq << 32 | (uint32_t)(a.u_len + a.v_len), v[i]};
      }
      std::sort(key.begin(), key.end(), [](const std::pair<uint64_t, uint32_t>& x, const std::pair<uint64_t, uint32_t>& y) {
        return x.first > y.first || (x.first == y.first && x.second < y.second);
      });
      for (size_t i = 0; i < v.size(); ++i) v[i] = key[i].second;
    }
    Bucket bk;
    bk.threads = plain ? 256 : c->cfg[b].threads;
    bk.k = plain ? 1 : c->cfg[b].k;
    bk.csize = 0;
    bk.cls = b;
    bk.first = (uint32_t)P.order.size();
    bk.n = (uint32_t)v.size();
    bk.nq_max = descs[v[0]].nq;
    bk.scratch_off = scratch;
    const int small_cs = (b > 0 && b < CLUSTER_CLASS) ? P.small_cluster_ctas : 0;
    if (!plain && (b == CLUSTER_CLASS || c->cfg[b].csize > 0 || small_cs > 0)) {
      // k pairs per cluster; more CTAs per cluster when a CTA's share of the moduli would
      // not fit its shared memory (24 KB kept for the kernel's static shared memory, which
      // holds the cluster keys and the recovery panel)
      if (b == CLUSTER_CLASS && P.cluster_k) bk.k = P.cluster_k;
      if (bk.k > 4) bk.k = 4;
      int cs = (b == CLUSTER_CLASS && P.cluster_ctas) ? P.cluster_ctas : small_cs > 0 ? small_cs : c->cfg[b].csize;
      const size_t room = c->smem_optin - 24576;
      while (cs < MAX_CLUSTER && cluster_batch_smem_bytes(cs, bk.nq_max, bk.k) > room) cs *= 2;
      cs = std::min(cs, MAX_CLUSTER);
      bk.csize = cs;
      bk.smem = cluster_batch_smem_bytes(cs, bk.nq_max, bk.k);
      int nc = 0;
      if (bk.smem > room || cluster_batch_max_clusters(bk.threads, bk.k, cs, bk.smem, &nc) != cudaSuccess || nc < 1)
        return MGCD_ERR_GRID;
      bk.grid = (int)std::min<size_t>((v.size() + bk.k - 1) / bk.k, (size_t)nc);
      scratch += (size_t)bk.grid * 4 * bk.k * bk.nq_max;
    } else {
      // Moduli grown on demand (K-slot kernels, k >= 2): the bucket's pairs start with the
      // growth fraction of the reference count and may grow up to it, so shared memory and
      // scratch are sized for the bucket's largest reference count.  Pairs of a bucket that
      // would drop to one pair per CTA keep the class's fixed count.
      if (!plain && c->grow_start > 0.0f) {
        uint32_t cap_max = 0;
        for (uint32_t k : v) cap_max = std::max(cap_max, std::max(P.ref_nq[k], grow_cap(P.ref_nq[k])));
        int kk = bk.k;
        while (kk > 1 && batch_smem_bytes(bk.threads, kk, cap_max) > c->smem_optin - 16384) kk /= 2;
        if (kk >= 2 && cap_max <= CTA_MAX_NQ && cap_max <= c->moduli.size()) {
          bk.k = kk;
          bk.nq_max = cap_max;
          for (uint32_t k : v) {
            const uint32_t ref = P.ref_nq[k];
            const uint32_t n0 = ((uint32_t)std::ceil(c->grow_start * (float)ref) + 31u) / 32u * 32u;
            descs[k].nq = std::min(ref, std::max(64u, n0));
            descs[k].nq_cap = std::max(ref, grow_cap(ref));
          }
        }
      }
      // fewer pairs per CTA when k of the bucket's largest pairs would not fit shared memory
      // (16 KB kept for the kernel's static shared memory)
      while (bk.k > 1 && batch_smem_bytes(bk.threads, bk.k, bk.nq_max) > c->smem_optin - 16384) bk.k /= 2;
      bk.smem = batch_smem_bytes(bk.threads, bk.k, bk.nq_max);
      int bps = 0;
      if (batch_max_blocks_per_sm(bk.threads, bk.k, c->L <= 30, bk.smem, &bps) != cudaSuccess || bps < 1)
        return MGCD_ERR_GRID;
      bk.grid = (int)std::min<size_t>((v.size() + bk.k - 1) / bk.k, (size_t)c->sms * bps);
      scratch += (size_t)bk.grid * 4 * bk.k * bk.nq_max;
    }
    P.order.insert(P.order.end(), v.begin(), v.end());
    buckets.push_back(bk);
  }
  uint32_t grid_nq_max = 0;
  for (uint32_t k : grid_pairs) grid_nq_max = std::max(grid_nq_max, descs[k].nq);
  P.grid_scratch_off = scratch;
  scratch += 4 * (size_t)grid_nq_max;
  return MGCD_OK;
}

// Launches the buckets (one stream each, joined back into P.stream) and then the
// single-pair launches.  `pairs` is the descriptor array on the device, `queue_base` the
// first of the bucket work counters (zeroed here).
static int launch_set(mgcd_context* c, Plan& P, const std::vector<Bucket>& buckets,
                      const std::vector<uint32_t>& grid_pairs, const std::vector<PairDesc>& descs, PairDesc* pairs,
                      uint32_t* queue_base, bool time_buckets, bool traced = true)
{
  CK(cudaMemsetAsync(queue_base, 0, NSTREAMS * sizeof(uint32_t), P.stream));
  unsigned long long* trace = nullptr;
  unsigned long long* phases = nullptr;
  if (c->trace && traced) {
    size_t ctas = 0;
    for (const Bucket& bk : buckets) ctas += (size_t)bk.grid * (bk.csize ? bk.csize : 1);
    if (P.d_trace.bytes < std::max<size_t>(ctas, 1) * 4 * sizeof(unsigned long long) ||
        P.d_phases.bytes < std::max<size_t>(ctas, 1) * PHASE_WORDS * sizeof(unsigned long long)) {
      P.drop_graph();
      P.d_trace.release(P.stream);
      P.d_phases.release(P.stream);
      CK(P.d_trace.grow(std::max<size_t>(ctas, 1) * 4 * sizeof(unsigned long long), c->pool, P.stream));
      CK(P.d_phases.grow(std::max<size_t>(ctas, 1) * PHASE_WORDS * sizeof(unsigned long long), c->pool, P.stream));
    }
    CK(cudaMemsetAsync(P.d_trace.p, 0, ctas * 4 * sizeof(unsigned long long), P.stream));
    CK(cudaMemsetAsync(P.d_phases.p, 0, ctas * PHASE_WORDS * sizeof(unsigned long long), P.stream));
    trace = P.d_trace.as<unsigned long long>();
    phases = P.d_phases.as<unsigned long long>();
    P.trace_cls.clear();
  }
  // every bucket kernel on P.stream, largest class first, each after the first a
  // programmatic dependent of the one before (it starts once all CTAs of that one have
  // started, cta_begin): the kernels run side by side, the larger classes' persistent CTAs
  // placed first.  The span of each (earliest CTA start, latest CTA end) is its time.
  if (time_buckets) CK(cudaMemsetAsync(P.d_span.p, 0xFF, 2 * NSTREAMS * sizeof(unsigned long long), P.stream));
  for (size_t b = 0; b < buckets.size(); ++b) {
    const Bucket& bk = buckets[b];
    BatchArgs a{};
    a.trace = trace;
    a.phases = phases;
    a.span = time_buckets ? P.d_span.as<unsigned long long>() + 2 * b : nullptr;
    if (trace) {
      const int n = bk.grid * (bk.csize ? bk.csize : 1);
      trace += 4 * (size_t)n;
      phases += PHASE_WORDS * (size_t)n;
      P.trace_cls.insert(P.trace_cls.end(), n, bk.cls);
    }
    a.stage_fail = c->stage_fail_cta;
    a.inv = InvTab{c->d_invtab.as<uint32_t>(), c->invtab_n};
    a.limbs = P.d_limbs.as<uint32_t>();
    a.pairs = pairs;
    a.order = P.d_order.as<uint32_t>() + bk.first;
    a.npairs = bk.n;
    a.mods = c->mods.as<ModConst>();
    a.L = c->L;
    a.queue = queue_base + b;
    a.scratch = P.d_scratch.as<uint32_t>() + bk.scratch_off;
    a.scratch_words = 4 * (size_t)bk.k * bk.nq_max;
    a.nq_max = bk.nq_max;
    a.digits = P.d_digits.as<mgcd_pair>();
    a.count = P.d_count.as<uint32_t>();
    a.iters = P.d_iters.as<uint32_t>();
    a.status = P.d_status.as<int32_t>();
    a.grow_permille = c->grow_permille;
    a.nq_final = P.d_nqf.as<uint32_t>();
    a.updates = P.d_upd.as<unsigned long long>();
    if (bk.csize)
      CK(launch_cluster_batch(a, bk.threads, bk.k, bk.csize, bk.grid, bk.smem, P.stream, b > 0));
    else
      CK(launch_batch(a, bk.threads, bk.k, bk.grid, bk.smem, P.stream, b > 0));
    ++P.launches;
  }

  for (uint32_t k : grid_pairs) {
    const PairDesc& d = descs[k];
    GridArgs g;
    g.stage_fail = c->stage_fail_cta;
    g.inv = InvTab{c->d_invtab.as<uint32_t>(), c->invtab_n};
    g.limbs = P.d_limbs.as<uint32_t>();
    g.pair = d;
    g.mods = c->mods.as<ModConst>();
    g.L = c->L;
    g.scratch = P.d_scratch.as<uint32_t>() + P.grid_scratch_off;
    g.digits = P.d_digits.as<mgcd_pair>();
    g.count = P.d_count.as<uint32_t>() + k;
    g.iters = P.d_iters.as<uint32_t>() + k;
    g.status = P.d_status.as<int32_t>() + k;
    const bool ref_shape = c->single_policy == MGCD_SINGLE_REFERENCE_SHAPE;
    if (!ref_shape && d.nq <= (uint32_t)MAX_CLUSTER * 512) {
      // thread-block cluster: as many CTAs (<= 16) as keep one modulus per thread, up to 512
      // threads per CTA (with 1024-thread CTAs the cluster's two-level exchange measured
      // slower than the grid's leader exchange: 16.8 vs 16.5 ms at 9,728 moduli, 20.8 vs
      // 19.0 ms at 11,264; at 8,192 moduli the 512-thread cluster wins, 13.0 vs 14.0 ms)
      const int ctas = (int)std::min<uint32_t>(MAX_CLUSTER, (d.nq + 255) / 256);
      const uint32_t per = (d.nq + ctas - 1) / ctas;
      const int threads = per <= 256 ? 256 : per <= 512 ? 512 : 1024;
      g.per_cta = per;
      g.sync = nullptr;
      if (launch_cluster(g, threads, ctas, grid_smem_bytes(per), P.stream) != cudaSuccess) return MGCD_ERR_GRID;
      ++P.launches;
      continue;
    }
    if (c->single_policy == MGCD_SINGLE_CLUSTER_GRID) {
      // cooperative grid of 8-CTA clusters, at most one CTA per SM
      constexpr int CS = 8;
      int nclu = c->sms / CS;
      uint32_t per = std::max<uint32_t>(32, (d.nq + nclu * CS - 1) / (nclu * CS));
      const int threads = per <= 256 ? 256 : per <= 512 ? 512 : 1024;
      int maxc = 0;
      if (cgrid_max_clusters(threads, CS, grid_smem_bytes(per), &maxc) != cudaSuccess || maxc < 1) return MGCD_ERR_GRID;
      if (maxc < nclu) {
        nclu = maxc;
        per = (d.nq + nclu * CS - 1) / (nclu * CS);
        if (per > 1024 * 4) return MGCD_ERR_GRID;
      }
      nclu = (int)((d.nq + per * CS - 1) / (per * CS));
      g.per_cta = per;
      g.sync = P.d_gsync.as<GridSync>();
      CK(launch_gridsync_init(g.sync, c->wait_timeout_ns, c->withhold_cta, P.stream));
      ++P.launches;
      const int thr = per <= 256 ? 256 : per <= 512 ? 512 : 1024;
      cudaError_t e = launch_cgrid(g, thr, CS, nclu, grid_smem_bytes(per), P.stream);
      if (e == cudaErrorCooperativeLaunchTooLarge) return MGCD_ERR_GRID;
      if (e != cudaSuccess) return MGCD_ERR_CUDA;
      ++P.launches;
      continue;
    }
    // cooperative grid: at most one CTA per SM and at least 256 moduli per CTA (fewer CTAs in
    // each exchange); or the reference's shape: 256-thread CTAs, 256 moduli
    uint32_t per = ref_shape ? 256u : std::max<uint32_t>(256, (d.nq + c->sms - 1) / c->sms);
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
    if (grid > (uint32_t)MAX_GRID_CTAS) return MGCD_ERR_GRID;   // one exchange slot per CTA
    g.per_cta = per;
    g.sync = P.d_gsync.as<GridSync>();
    CK(launch_gridsync_init(g.sync, c->wait_timeout_ns, c->withhold_cta, P.stream));
    ++P.launches;
    cudaError_t e = launch_grid(g, threads, (int)grid, grid_smem_bytes(per), P.stream);
    if (e == cudaErrorCooperativeLaunchTooLarge) return MGCD_ERR_GRID;
    if (e != cudaSuccess) return MGCD_ERR_CUDA;
    ++P.launches;
  }
  return MGCD_OK;
}

// Converts every GPU pair's digits to binary limbs on P.stream (after the gcd kernels).
static int launch_convert(mgcd_context* c, Plan& P)
{
  const uint32_t ng = (uint32_t)P.descs.size();
  const int grid = (int)std::min<uint32_t>(ng, (uint32_t)c->sms * 2);
  CK(launch_radix(P.d_pairs.as<PairDesc>(), ng, P.d_digits.as<mgcd_pair>(), P.d_count.as<uint32_t>(),
                  P.d_status.as<int32_t>(), P.d_glimbs.as<uint32_t>(), P.d_glen.as<uint32_t>(), grid, P.stream));
  ++P.launches;
  return MGCD_OK;
}

int mgcd::run_plan(mgcd_context* c, Plan& P)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  P.launches = 0;
  P.retried = 0;
  const size_t ng = P.descs.size();
  if (ng == 0) {
    P.ran = true;
    P.synced = true;
    return MGCD_OK;
  }
  for (size_t k = 0; k < ng; ++k) P.eff_nq[k] = P.descs[k].nq;
  if (c->use_graph && P.graphable && !P.plain) {
    if (!P.graph) {
      // Record the run once (status reset, queue reset, the chained bucket kernels, the
      // conversion); each later run is a single graph launch.
      CK(cudaStreamBeginCapture(P.stream, cudaStreamCaptureModeThreadLocal));
      int rc = MGCD_OK;
      if (cudaMemsetAsync(P.d_status.p, 0xFF, ng * sizeof(int32_t), P.stream) != cudaSuccess ||
          cudaMemsetAsync(P.d_nqf.p, 0, ng * sizeof(uint32_t), P.stream) != cudaSuccess ||
          cudaMemsetAsync(P.d_upd.p, 0, ng * sizeof(unsigned long long), P.stream) != cudaSuccess)
        rc = MGCD_ERR_CUDA;
      if (rc == MGCD_OK)
        rc = launch_set(c, P, P.buckets, P.grid_pairs, P.descs, P.d_pairs.as<PairDesc>(), P.d_queue.as<uint32_t>(),
                        true);
      if (rc == MGCD_OK) rc = launch_convert(c, P);
      cudaGraph_t g = nullptr;
      const cudaError_t e = cudaStreamEndCapture(P.stream, &g);
      if (rc == MGCD_OK && e != cudaSuccess) rc = MGCD_ERR_CUDA;
      if (rc == MGCD_OK && cudaGraphInstantiate(&P.graph, g, 0) != cudaSuccess) {
        P.graph = nullptr;
        rc = MGCD_ERR_CUDA;
      }
      if (g) cudaGraphDestroy(g);
      if (rc != MGCD_OK) return rc;
      P.graph_kernels = P.launches;
    }
    CK(cudaEventRecord(P.t_run0, P.stream));
    CK(cudaGraphLaunch(P.graph, P.stream));
    P.launches = P.graph_kernels;
    P.bucket_timed = true;
  } else {
    CK(cudaEventRecord(P.t_run0, P.stream));
    CK(cudaMemsetAsync(P.d_status.p, 0xFF, ng * sizeof(int32_t), P.stream));
    CK(cudaMemsetAsync(P.d_nqf.p, 0, ng * sizeof(uint32_t), P.stream));
    CK(cudaMemsetAsync(P.d_upd.p, 0, ng * sizeof(unsigned long long), P.stream));
    int rc = launch_set(c, P, P.buckets, P.grid_pairs, P.descs, P.d_pairs.as<PairDesc>(), P.d_queue.as<uint32_t>(),
                        true);
    if (rc == MGCD_OK) rc = launch_convert(c, P);
    if (rc != MGCD_OK) return rc;
    P.bucket_timed = true;
  }
  CK(cudaEventRecord(P.t_run1, P.stream));
  P.ran = true;
  P.synced = false;
  return MGCD_OK;
}

// Waits for the run; pairs that ran with fewer moduli than the reference count and could
// not be certified are rerun once with the reference count (same digit slots).
int mgcd::sync_plan(mgcd_context* c, Plan& P)
{
  if (!c || !P.ran) return MGCD_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(P.stream));
  if (P.synced) return MGCD_OK;
  P.synced = true;
  const size_t ng = P.descs.size();
  bool scaled = false;
  for (size_t k = 0; k < ng && !scaled; ++k) scaled = P.descs[k].nq < P.ref_nq[k];
  if (!scaled) return MGCD_OK;
  CK(P.h_status.grow(ng * sizeof(int32_t)));
  CK(cudaMemcpyAsync(P.h_status.p, P.d_status.p, ng * sizeof(int32_t), cudaMemcpyDeviceToHost, P.stream));
  CK(cudaStreamSynchronize(P.stream));
  const int32_t* st = P.h_status.as<int32_t>();
  std::vector<uint32_t> redo;
  for (uint32_t k = 0; k < ng; ++k)
    if (st[k] != ST_OK && st[k] != ST_TIMEOUT && P.descs[k].nq < P.ref_nq[k]) redo.push_back(k);
  if (redo.empty()) return MGCD_OK;
  std::vector<PairDesc> rd = P.descs;
  for (uint32_t k : redo) {
    rd[k].nq = P.ref_nq[k];
    rd[k].nq_cap = 0;
    P.eff_nq[k] = P.ref_nq[k];
  }
  const size_t main_order = P.order.size();
  std::vector<Bucket> bks;
  std::vector<uint32_t> gp;
  size_t scratch = 0;
  const size_t keep_grid_off = P.grid_scratch_off;
  int rc = schedule(c, P, rd, redo, false, bks, gp, scratch, true);
  if (rc != MGCD_OK) return rc;
  // device buffers: retry descriptors after the main ones, retry order after the main order
  cudaStream_t s = P.stream;
  CK(P.d_retry.grow(ng * sizeof(PairDesc), c->pool, s));
  if (P.order.size() * sizeof(uint32_t) > P.d_order.bytes) {
    // keep the main order: grow by copying
    DevBuf nb;
    CK(nb.grow(P.order.size() * sizeof(uint32_t), c->pool, s));
    CK(cudaMemcpyAsync(nb.p, P.d_order.p, main_order * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    P.drop_graph();
    P.d_order.release(s);
    P.d_order = nb;
  }
  if (scratch > P.d_scratch.bytes / sizeof(uint32_t)) {
    P.drop_graph();
    P.d_scratch.release(s);
    CK(P.d_scratch.grow(scratch * sizeof(uint32_t), c->pool, s));
  }
  CK(cudaMemcpyAsync(P.d_retry.p, rd.data(), ng * sizeof(PairDesc), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(P.d_order.as<uint32_t>() + main_order, P.order.data() + main_order,
                     (P.order.size() - main_order) * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
  rc = launch_set(c, P, bks, gp, rd, P.d_retry.as<PairDesc>(), P.d_queue.as<uint32_t>() + NSTREAMS, false,
                  false);                   // the trace keeps the main run
  P.order.resize(main_order);               // the plan itself is unchanged for later runs
  P.grid_scratch_off = keep_grid_off;
  if (rc == MGCD_OK) rc = launch_convert(c, P);   // same digit and limb slots: convert again
  if (rc != MGCD_OK) return rc;
  CK(cudaEventRecord(P.t_run1, s));
  CK(cudaStreamSynchronize(s));
  P.retried = (int)redo.size();
  return MGCD_OK;
}

// Copies the GPU results of the plan to pinned host memory.
int mgcd::fetch(mgcd_context* c, Plan& P, uint32_t* direct_g)
{
  const size_t ng = P.descs.size();
  CK(cudaSetDevice(c->device));
  if (ng == 0) return MGCD_OK;
  CK(P.h_count.grow(ng * sizeof(uint32_t)));
  CK(P.h_iters.grow(ng * sizeof(uint32_t)));
  CK(P.h_status.grow(ng * sizeof(int32_t)));
  CK(P.h_glen.grow(ng * sizeof(uint32_t)));
  P.in_place = P.direct && direct_g != nullptr;
  if (!P.in_place) CK(P.h_glimbs.grow(std::max<size_t>(P.nglimbs, 1) * sizeof(uint32_t)));
  CK(P.h_nqf.grow(ng * sizeof(uint32_t)));
  CK(P.h_upd.grow(ng * sizeof(unsigned long long)));
  if (P.plain) CK(P.h_digits.grow(std::max<size_t>(P.ndig, 1) * sizeof(mgcd_pair)));
  cudaStream_t s = P.stream;
  // Results as binary limbs (converted on the device); digits only where the caller wants
  // them (single pairs) or the host converts (very long gcds).
  CK(cudaMemcpyAsync(P.h_count.p, P.d_count.p, ng * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(P.h_iters.p, P.d_iters.p, ng * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(P.h_status.p, P.d_status.p, ng * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(P.h_glen.p, P.d_glen.p, ng * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(P.in_place ? (void*)(direct_g + P.direct_base) : P.h_glimbs.p, P.d_glimbs.p,
                     P.nglimbs * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(P.h_nqf.p, P.d_nqf.p, ng * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(P.h_upd.p, P.d_upd.p, ng * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  uint64_t d2h = ng * (5 * sizeof(uint32_t) + sizeof(unsigned long long)) + P.nglimbs * sizeof(uint32_t);
  if (P.plain) {
    CK(cudaMemcpyAsync(P.h_digits.p, P.d_digits.p, P.ndig * sizeof(mgcd_pair), cudaMemcpyDeviceToHost, s));
    d2h += P.ndig * sizeof(mgcd_pair);
  }
  CK(cudaStreamSynchronize(s));
  if (!P.plain) {
    const uint32_t* gl = P.h_glen.as<uint32_t>();
    const int32_t* st0 = P.h_status.as<int32_t>();
    bool any = false;
    for (size_t k = 0; k < ng && !any; ++k) any = gl[k] == RADIX_HOST && st0[k] == ST_OK;
    if (any) CK(P.h_digits.grow(std::max<size_t>(P.ndig, 1) * sizeof(mgcd_pair)));
    any = false;
    for (size_t k = 0; k < ng; ++k) {
      if (gl[k] != RADIX_HOST || st0[k] != ST_OK) continue;
      const PairDesc& d = P.descs[k];
      const size_t n = P.h_count.as<uint32_t>()[k];
      CK(cudaMemcpyAsync(P.h_digits.as<mgcd_pair>() + d.out_off, P.d_digits.as<mgcd_pair>() + d.out_off,
                         n * sizeof(mgcd_pair), cudaMemcpyDeviceToHost, s));
      d2h += n * sizeof(mgcd_pair);
      any = true;
    }
    if (any) CK(cudaStreamSynchronize(s));
  }
  P.d2h_bytes = d2h;
  // work by the cost model
  const uint32_t* it = P.h_iters.as<uint32_t>();
  const uint32_t* cnt = P.h_count.as<uint32_t>();
  const int32_t* st = P.h_status.as<int32_t>();
  double R = 0, E = 0, M = 0, B = 0, AB = 0;
  std::vector<double> pw(4 * ng, 0.0);    // per pair: R, E, M, B
  const uint32_t* nqf = P.h_nqf.as<uint32_t>();
  const unsigned long long* upd = P.h_upd.as<unsigned long long>();
  for (size_t k = 0; k < ng; ++k) {
    const PairDesc& d = P.descs[k];
    double* w = &pw[4 * k];
    // the K-slot kernels record the final moduli count and the loop's updates (a pair's set
    // may have grown); a rerun pair, or one of another kernel, ran with eff_nq throughout
    const bool rec = nqf[k] != 0u && P.eff_nq[k] == d.nq;
    const double N = rec ? (double)nqf[k] : (double)P.eff_nq[k];
    w[0] = N * (d.u_len + d.v_len);
    w[3] = 4.0 * (d.u_len + d.v_len);
    if (st[k] == ST_OK) {
      const double I = it[k], K = cnt[k];
      w[1] = rec ? (double)upd[k] : I * N - I * (I + 1) / 2;
      w[2] = K * (N - I) - K * (K + 1) / 2;
      AB += 12.0 * N + 8.0 * (K + 1);      // a prime and its 8-byte constant per modulus, digits
    }
    R += w[0]; E += w[1]; M += w[2]; B += w[3];
  }
  P.work[0] = R; P.work[1] = E; P.work[2] = M; P.work[3] = B;
  P.alg_bytes = B + AB;
  P.bucket_work.assign(4 * P.buckets.size(), 0.0);
  for (size_t b = 0; b < P.buckets.size(); ++b)
    for (uint32_t i = 0; i < P.buckets[b].n; ++i) {
      const uint32_t k = P.order[P.buckets[b].first + i];
      for (int x = 0; x < 4; ++x) P.bucket_work[4 * b + x] += pw[4 * k + x];
    }
  return MGCD_OK;
}

int mgcd::convert_all(mgcd_context* c, Plan& P, uint32_t* g, const uint64_t* g_off, const uint32_t* g_cap,
                      uint32_t* g_len, int32_t* status, bool threaded)
{
  (void)c;
  const size_t np = P.np;
  const mgcd_pair* dig = P.h_digits.as<mgcd_pair>();
  const uint32_t* cnt = P.h_count.as<uint32_t>();
  const int32_t* st = P.h_status.as<int32_t>();
  const uint32_t* gl = P.h_glen.as<uint32_t>();
  const uint32_t* gv = P.h_glimbs.as<uint32_t>();
  std::atomic<size_t> next{0};
  auto work = [&]() {
    for (;;) {
      const size_t i = next.fetch_add(1);
      if (i >= np) break;
      int s = P.status[i];
      size_t len = 0;
      if (P.slot[i] >= 0) {
        const int k = P.slot[i];
        s = to_status(st[k]);
        if (s != MGCD_OK) {
        } else if (gl[k] != RADIX_HOST) {           // converted on the device
          len = gl[k];
          if (len > g_cap[i]) { s = MGCD_ERR_CAPACITY; len = 0; }
          else if (len && !P.in_place) std::memcpy(g + g_off[i], gv + P.descs[k].g_off, len * sizeof(uint32_t));
        } else if (mixed_radix_to_limbs(dig + P.descs[k].out_off, cnt[k], g + g_off[i], g_cap[i], &len)) {
          s = MGCD_ERR_CAPACITY;
        }
      } else if (s == MGCD_OK) {
        len = P.trivial[i].size();
        if (len > g_cap[i]) { s = MGCD_ERR_CAPACITY; len = 0; }
        else if (len) std::memcpy(g + g_off[i], P.trivial[i].data(), len * sizeof(uint32_t));
      }
      g_len[i] = (uint32_t)len;
      if (status) status[i] = s;
    }
  };
  // Threads only where the work outweighs starting them (tens of microseconds each): one core
  // copies the device-converted results at ~18 GB/s (8 MB of a 4,096-pair batch: 0.45 ms on
  // one thread, 0.65 ms on 4, 1.15 ms on 16), so one thread per 32 MiB; results converted
  // here from their digits (RADIX_HOST, quadratic in the length) take a thread per 16 pairs.
  size_t copy_bytes = 0;
  bool host_radix = false;
  for (size_t k = 0; k < P.descs.size(); ++k) {
    if (st[k] != ST_OK) continue;
    if (gl[k] == RADIX_HOST) host_radix = true;
    else if (!P.in_place) copy_bytes += (size_t)gl[k] * sizeof(uint32_t);
  }
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t want = host_radix ? (np + 15) / 16 : 1 + copy_bytes / (32u << 20);
  const size_t nt = threaded ? std::min<size_t>(hw, want) : 1;
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

extern "C" {

int mgcd_batch_upload(mgcd_context* c, size_t np, const uint32_t* limbs, const uint64_t* u_off,
                      const uint32_t* u_len, const uint64_t* v_off, const uint32_t* v_len)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  if (busy(c)) return MGCD_ERR_BUSY;
  return plan_batch(c, c->main, np, limbs, u_off, u_len, v_off, v_len, false);
}

int mgcd_set_nq_scale(mgcd_context* c, float scale)
{
  if (!c || !(scale >= 0.5f && scale <= 1.0f)) return MGCD_ERR_INVALID_ARG;
  for (auto& b : c->cfg) b.nq_scale = scale;
  return MGCD_OK;
}

static bool valid_growth(float start, unsigned step_permille)
{
  return start == 0.0f || (start >= 0.1f && start <= 1.0f && step_permille >= 10u && step_permille <= 500u);
}

int mgcd_set_growth(mgcd_context* c, float start, unsigned step_permille)
{
  if (!c || !valid_growth(start, step_permille)) return MGCD_ERR_INVALID_ARG;
  c->grow_start = start;
  c->grow_permille = step_permille;
  return MGCD_OK;
}

int mgcd_get_growth(const mgcd_context* c, float* start, unsigned* step_permille)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  if (start) *start = c->grow_start;
  if (step_permille) *step_permille = c->grow_permille;
  return MGCD_OK;
}

// Launch configurations that exist: CTA size 256/512/1024 with k = 1, 2, 4, or k = 8 with
// 512 threads (not in the cluster class).
static bool valid_class_cfg(int cls, int threads, int k, float nq_scale)
{
  if (cls < 0 || cls >= NSTREAMS || !(nq_scale >= 0.5f && nq_scale <= 1.0f)) return false;
  if (threads != 256 && threads != 512 && threads != 1024) return false;
  if (k == 8) return (threads == 512 || threads == 1024) && cls != CLUSTER_CLASS;
  return k == 1 || k == 2 || k == 4;
}

int mgcd_set_size_class(mgcd_context* c, int cls, int threads, int k, float nq_scale)
{
  if (!c || !valid_class_cfg(cls, threads, k, nq_scale)) return MGCD_ERR_INVALID_ARG;
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

int mgcd_set_class_cluster(mgcd_context* c, int cls, int ctas)
{
  if (!c || cls < 0 || cls >= NSTREAMS || ctas > MAX_CLUSTER || ctas < 0 || ctas == 1 ||
      (cls == CLUSTER_CLASS && ctas == 0))
    return MGCD_ERR_INVALID_ARG;
  c->cfg[cls].csize = ctas;
  return MGCD_OK;
}

int mgcd_get_class_cluster(const mgcd_context* c, int cls, int* ctas)
{
  if (!c || !ctas || cls < 0 || cls >= NSTREAMS) return MGCD_ERR_INVALID_ARG;
  *ctas = c->cfg[cls].csize;
  return MGCD_OK;
}

// Tuning table: one line per size class, "class threads k nq_scale cluster_ctas", and
// optionally "grow start step_permille" (moduli grown on demand, mgcd_set_growth; '#' starts
// a comment).  All lines are checked before any is applied.
int mgcd_load_tuning(mgcd_context* c, const char* path)
{
  if (!c || !path) return MGCD_ERR_INVALID_ARG;
  FILE* f = std::fopen(path, "r");
  if (!f) return MGCD_ERR_INVALID_ARG;
  mgcd_context::ClassCfg cfg[NSTREAMS];
  static_assert(sizeof(cfg) == sizeof(c->cfg), "copy of the whole table");
  std::memcpy(cfg, c->cfg, sizeof(cfg));
  char line[256];
  int rc = MGCD_OK;
  float g_start = c->grow_start;
  unsigned g_step = c->grow_permille;
  while (rc == MGCD_OK && std::fgets(line, sizeof line, f)) {
    const char* s = line;
    while (*s == ' ' || *s == '\t') ++s;
    if (*s == '#' || *s == '\n' || *s == '\r' || *s == 0) continue;
    if (std::strncmp(s, "grow", 4) == 0) {
      if (std::sscanf(s + 4, "%f %u", &g_start, &g_step) != 2 || !valid_growth(g_start, g_step)) rc = MGCD_ERR_INVALID_ARG;
      continue;
    }
    int cls, threads, k, cs;
    float sc;
    if (std::sscanf(s, "%d %d %d %f %d", &cls, &threads, &k, &sc, &cs) != 5 || !valid_class_cfg(cls, threads, k, sc) ||
        cs < 0 || cs == 1 || cs > MAX_CLUSTER || (cls == CLUSTER_CLASS && cs == 0) || (cs > 0 && k > 4)) {
      rc = MGCD_ERR_INVALID_ARG;
      break;
    }
    cfg[cls].threads = threads;
    cfg[cls].k = k;
    cfg[cls].nq_scale = sc;
    cfg[cls].csize = cs;
  }
  std::fclose(f);
  if (rc == MGCD_OK) {
    std::memcpy(c->cfg, cfg, sizeof(cfg));
    c->grow_start = g_start;
    c->grow_permille = g_step;
  }
  return rc;
}

int mgcd_save_tuning(const mgcd_context* c, const char* path)
{
  if (!c || !path) return MGCD_ERR_INVALID_ARG;
  FILE* f = std::fopen(path, "w");
  if (!f) return MGCD_ERR_INVALID_ARG;
  std::fprintf(f, "# modgcd tuning table (modulus width %d): class threads k nq_scale cluster_ctas\n", c->L);
  for (int i = 0; i < NSTREAMS; ++i)
    std::fprintf(f, "%d %d %d %.3f %d\n", i, c->cfg[i].threads, c->cfg[i].k, c->cfg[i].nq_scale, c->cfg[i].csize);
  std::fprintf(f, "grow %.3f %u\n", c->grow_start, c->grow_permille);
  return std::fclose(f) == 0 ? MGCD_OK : MGCD_ERR_INVALID_ARG;
}

int mgcd_batch_use_graph(mgcd_context* c, int enable)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  c->use_graph = enable != 0;
  if (!c->use_graph) {
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->main.stream);
    c->main.drop_graph();
  }
  return MGCD_OK;
}

int mgcd_set_single_pair_policy(mgcd_context* c, int policy)
{
  if (!c || (policy != MGCD_SINGLE_AUTO && policy != MGCD_SINGLE_REFERENCE_SHAPE &&
             policy != MGCD_SINGLE_CLUSTER_GRID))
    return MGCD_ERR_INVALID_ARG;
  c->single_policy = policy;
  return MGCD_OK;
}

int mgcd_set_wait_timeout_ms(mgcd_context* c, unsigned ms)
{
  if (!c || ms == 0) return MGCD_ERR_INVALID_ARG;
  c->wait_timeout_ns = (unsigned long long)ms * 1000000ull;
  cudaStreamSynchronize(c->main.stream);
  c->main.drop_graph();
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
  cudaStreamSynchronize(c->main.stream);
  c->main.drop_graph();
  return MGCD_OK;
}

int mgcd_test_fail_staging(mgcd_context* c, int cta)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  c->stage_fail_cta = cta < 0 ? 0xFFFFFFFFu : (uint32_t)cta;
  cudaStreamSynchronize(c->main.stream);
  c->main.drop_graph();
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

// Bucket kernel i's time in the last run: its CTAs' earliest start to latest end (the span
// the kernels record with the global timer).
static int bucket_span_ms(const mgcd_context* c, int i, float* ms)
{
  unsigned long long sp[2] = {0, 0};
  CK(cudaSetDevice(c->device));
  CK(cudaMemcpy(sp, c->main.d_span.as<unsigned long long>() + 2 * i, sizeof sp, cudaMemcpyDeviceToHost));
  const unsigned long long t0 = sp[0], t1 = ~sp[1];
  *ms = (sp[0] != ~0ull && sp[1] != ~0ull && t1 >= t0) ? (float)((double)(t1 - t0) * 1e-6) : 0.f;
  return MGCD_OK;
}

int mgcd_batch_kernel_stats(const mgcd_context* c, int i, int* cls, int* pairs, float* ms)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  const Plan& P = c->main;
  if (!P.ran || !P.bucket_timed || i < 0 || i >= (int)P.buckets.size()) return MGCD_ERR_INVALID_ARG;
  float t = 0.f;
  int rc = bucket_span_ms(c, i, &t);
  if (rc != MGCD_OK) return rc;
  if (cls) *cls = P.buckets[i].cls;
  if (pairs) *pairs = (int)P.buckets[i].n;
  if (ms) *ms = t;
  return MGCD_OK;
}

int mgcd_batch_kernel_work(const mgcd_context* c, int i, double* residue_steps, double* euclid_updates,
                           double* recovery_updates, double* operand_bytes)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  const Plan& P = c->main;
  if (i < 0 || 4 * (size_t)i + 3 >= P.bucket_work.size()) return MGCD_ERR_INVALID_ARG;
  const double* w = &P.bucket_work[4 * (size_t)i];
  if (residue_steps) *residue_steps = w[0];
  if (euclid_updates) *euclid_updates = w[1];
  if (recovery_updates) *recovery_updates = w[2];
  if (operand_bytes) *operand_bytes = w[3];
  return MGCD_OK;
}

int mgcd_batch_elapsed_ms(const mgcd_context* c, float* run_ms, float* dominant_ms, int* dominant_threads)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  const Plan& P = c->main;
  if (!P.ran) return MGCD_ERR_INVALID_ARG;
  float r = 0.f, best = 0.f;
  int bt = 0;
  if (!P.descs.empty()) {
    CK(cudaEventElapsedTime(&r, P.t_run0, P.t_run1));
    if (P.bucket_timed)
      for (size_t b = 0; b < P.buckets.size(); ++b) {
        float t = 0.f;
        const int rc = bucket_span_ms(c, (int)b, &t);
        if (rc != MGCD_OK) return rc;
        if (t > best) { best = t; bt = P.buckets[b].threads; }
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
  if (h2d) *h2d = c->main.h2d_bytes;
  if (d2h) *d2h = c->main.d2h_bytes;
  return MGCD_OK;
}

int mgcd_int_peak(mgcd_context* c, double* ops)
{
  if (!c || !ops) return MGCD_ERR_INVALID_ARG;
  if (busy(c)) return MGCD_ERR_BUSY;
  CK(cudaSetDevice(c->device));
  cudaStream_t s = c->main.stream;
  DevBuf sink;
  CK(sink.grow(sizeof(uint32_t), c->pool, s));
  const int blocks = c->sms * 8, iters = 1 << 16;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  int rc = MGCD_OK;
  for (int rep = 0; rep < 4 && rc == MGCD_OK; ++rep) {
    cudaEventRecord(a, s);
    if (launch_int_peak(sink.as<uint32_t>(), blocks, iters, s) != cudaSuccess) rc = MGCD_ERR_CUDA;
    cudaEventRecord(b, s);
    if (cudaEventSynchronize(b) != cudaSuccess) rc = MGCD_ERR_CUDA;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (rep > 0) best = std::min(best, ms);   // first launch is a warm-up
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  sink.release(s);
  if (rc != MGCD_OK) return rc;
  *ops = (double)blocks * 256.0 * iters * 8.0 / (best * 1e-3);
  return MGCD_OK;
}

int mgcd_batch_run(mgcd_context* c)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  if (busy(c)) return MGCD_ERR_BUSY;
  return run_plan(c, c->main);
}

int mgcd_batch_sync(mgcd_context* c)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  return sync_plan(c, c->main);
}

int mgcd_batch_retried(const mgcd_context* c, int* pairs)
{
  if (!c || !pairs) return MGCD_ERR_INVALID_ARG;
  *pairs = c->main.retried;
  return MGCD_OK;
}

int mgcd_batch_launches(const mgcd_context* c, int* launches)
{
  if (!c || !launches) return MGCD_ERR_INVALID_ARG;
  *launches = c->main.launches;
  return MGCD_OK;
}

int mgcd_batch_work(const mgcd_context* c, double* r, double* e, double* m, double* b)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  const double* w = c->main.work;
  if (r) *r = w[0];
  if (e) *e = w[1];
  if (m) *m = w[2];
  if (b) *b = w[3];
  return MGCD_OK;
}

int mgcd_batch_alg_bytes(const mgcd_context* c, double* alg_bytes)
{
  if (!c || !alg_bytes) return MGCD_ERR_INVALID_ARG;
  *alg_bytes = c->main.alg_bytes;
  return MGCD_OK;
}

int mgcd_set_cta_trace(mgcd_context* c, int enable)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  if (c->trace != (enable != 0)) c->main.drop_graph();
  c->trace = enable != 0;
  return MGCD_OK;
}

int mgcd_batch_cta_trace(mgcd_context* c, mgcd_cta_record* out, size_t cap, size_t* n)
{
  if (!c || !n || (cap && !out)) return MGCD_ERR_INVALID_ARG;
  Plan& P = c->main;
  const size_t ctas = c->trace ? P.trace_cls.size() : 0;
  *n = ctas;
  if (!ctas || !cap) return MGCD_OK;
  if (!P.ran) return MGCD_ERR_INVALID_ARG;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(P.stream));
  std::vector<unsigned long long> raw(4 * ctas), ph(PHASE_WORDS * ctas);
  CK(cudaMemcpy(raw.data(), P.d_trace.p, raw.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(ph.data(), P.d_phases.p, ph.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  unsigned long long t0 = ~0ull;
  for (size_t i = 0; i < ctas; ++i)
    if (raw[4 * i]) t0 = std::min(t0, raw[4 * i]);
  for (size_t i = 0; i < ctas && i < cap; ++i) {
    mgcd_cta_record& r = out[i];
    r.size_class = P.trace_cls[i];
    r.sm = (uint32_t)raw[4 * i + 2];
    r.pairs = (uint32_t)raw[4 * i + 3];
    r.ran = raw[4 * i] != 0 && raw[4 * i + 1] != 0;
    r.t_start_ms = r.ran ? (double)(raw[4 * i] - t0) * 1e-6 : 0.0;
    r.t_end_ms = r.ran ? (double)(raw[4 * i + 1] - t0) * 1e-6 : 0.0;
    r.cycles_setup = ph[PHASE_WORDS * i];
    r.cycles_update = ph[PHASE_WORDS * i + 1];
    r.cycles_pivot = ph[PHASE_WORDS * i + 2];
    r.cycles_finish = ph[PHASE_WORDS * i + 3];
    r.iterations = ph[PHASE_WORDS * i + 4];
    r.rounds = ph[PHASE_WORDS * i + 5];
    r.cycles_replay = ph[PHASE_WORDS * i + 7];
    r.update_rounds = ph[PHASE_WORDS * i + 8];
    r.rounds_with_inverse = ph[PHASE_WORDS * i + 9];
    r.finite_slot_updates = ph[PHASE_WORDS * i + 10];
    r.cycles_layout = ph[PHASE_WORDS * i + 11];
    r.cycles_grow = ph[PHASE_WORDS * i + 12];
    r.grow_steps = ph[PHASE_WORDS * i + 13];
  }
  return MGCD_OK;
}

int mgcd_batch_pair_digits(mgcd_context* c, size_t i, mgcd_pair* out, size_t cap, size_t* n, uint32_t* nq_final)
{
  if (!c || !n) return MGCD_ERR_INVALID_ARG;
  Plan& P = c->main;
  if (!P.synced || i >= P.np) return MGCD_ERR_INVALID_ARG;
  const int k = P.slot[i];
  if (k < 0 || P.h_count.p == nullptr) return MGCD_ERR_INVALID_ARG;
  const size_t cnt = P.h_count.as<uint32_t>()[k];
  *n = cnt;
  if (nq_final) {
    const uint32_t f = P.h_nqf.p ? P.h_nqf.as<uint32_t>()[k] : 0u;
    *nq_final = (f != 0u && P.eff_nq[k] == P.descs[k].nq) ? f : P.eff_nq[k];
  }
  if (cnt > cap) return MGCD_ERR_CAPACITY;
  CK(cudaSetDevice(c->device));
  if (cnt)
    CK(cudaMemcpy(out, P.d_digits.as<mgcd_pair>() + P.descs[k].out_off, cnt * sizeof(mgcd_pair),
                  cudaMemcpyDeviceToHost));
  return MGCD_OK;
}

int mgcd_batch_download(mgcd_context* c, uint32_t* g, const uint64_t* g_off, const uint32_t* g_cap,
                        uint32_t* g_len, int32_t* status)
{
  if (!c) return MGCD_ERR_INVALID_ARG;
  Plan& P = c->main;
  if (!P.ran || (P.np && (!g || !g_off || !g_cap || !g_len || !status))) return MGCD_ERR_INVALID_ARG;
  int rc = sync_plan(c, P);
  if (rc != MGCD_OK) return rc;
  rc = fetch(c, P);
  if (rc != MGCD_OK) return rc;
  return convert_all(c, P, g, g_off, g_cap, g_len, status, true);
}

int mgcd_gcd_batch(mgcd_context* c, size_t np, const uint32_t* limbs, const uint64_t* u_off,
                   const uint32_t* u_len, const uint64_t* v_off, const uint32_t* v_len, uint32_t* g,
                   const uint64_t* g_off, const uint32_t* g_cap, uint32_t* g_len, int32_t* status)
{
  if (!c || (np && (!g || !g_off || !g_cap || !g_len || !status))) return MGCD_ERR_INVALID_ARG;
  if (busy(c)) return MGCD_ERR_BUSY;
  Plan& P = c->main;
  // results planned in the caller's layout where it allows: one device-to-host copy puts them
  // in place, with no pass over them on the host
  int rc = plan_batch(c, P, np, limbs, u_off, u_len, v_off, v_len, false, g_off, g_cap);
  if (rc != MGCD_OK) return rc;
  rc = run_plan(c, P);
  if (rc != MGCD_OK) return rc;
  rc = sync_plan(c, P);
  if (rc != MGCD_OK) return rc;
  rc = fetch(c, P, g);
  if (rc != MGCD_OK) return rc;
  return convert_all(c, P, g, g_off, g_cap, g_len, status, true);
}

// ------------------------------------------------------------------ single pair ----

static int single(mgcd_context* c, const uint32_t* u, size_t uSz, const uint32_t* v, size_t vSz)
{
  if (!c || (uSz && !u) || (vSz && !v)) return MGCD_ERR_INVALID_ARG;
  if (busy(c)) return MGCD_ERR_BUSY;
  // Pack both operands contiguously (the plan reads one limb array).
  static thread_local std::vector<uint32_t> buf;
  buf.resize(uSz + vSz);
  if (uSz) std::memcpy(buf.data(), u, uSz * sizeof(uint32_t));
  if (vSz) std::memcpy(buf.data() + uSz, v, vSz * sizeof(uint32_t));
  const uint64_t uo = 0, vo = uSz;
  const uint32_t ul = (uint32_t)uSz, vl = (uint32_t)vSz;
  Plan& P = c->main;
  int rc = plan_batch(c, P, 1, buf.data(), &uo, &ul, &vo, &vl, true);
  if (rc != MGCD_OK) return rc;
  rc = run_plan(c, P);
  if (rc != MGCD_OK) return rc;
  rc = sync_plan(c, P);
  if (rc != MGCD_OK) return rc;
  return fetch(c, P);
}

int mgcd_gcd_digits(mgcd_context* c, const uint32_t* u, size_t uSz, const uint32_t* v, size_t vSz,
                    mgcd_pair* digits, size_t cap, size_t* count)
{
  if (!count || (cap && !digits)) return MGCD_ERR_INVALID_ARG;
  *count = 0;
  if (strip(u, uSz) == 0 || strip(v, vSz) == 0) return MGCD_ERR_INVALID_ARG;
  int rc = single(c, u, uSz, v, vSz);
  if (rc != MGCD_OK) return rc;
  const Plan& P = c->main;
  if (P.slot[0] < 0) return P.status[0];
  const int32_t st = P.h_status.as<int32_t>()[0];
  if (st != ST_OK) return to_status(st);
  const uint32_t n = P.h_count.as<uint32_t>()[0];
  if (n > cap) return MGCD_ERR_CAPACITY;
  std::memcpy(digits, P.h_digits.as<mgcd_pair>() + P.descs[0].out_off, n * sizeof(mgcd_pair));
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
  rc = convert_all(c, c->main, g, &off, &cap, &len, &st, false);
  *g_len = len;
  return rc;
}

}  // extern "C"

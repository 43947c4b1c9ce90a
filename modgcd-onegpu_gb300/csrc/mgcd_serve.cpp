// mgcd_serve.cpp -- request server: continuous batching of single gcd requests on one GPU.
// No counterpart in the reference (its GmpCudaDevice::gcd is one blocking call per pair).
//
// Requests are queued per lane (the batched path's size class of the pair).
//
// Continuous lanes (size classes 0-1, the default): each lane has a ring in pinned, mapped
// host memory and persistent K-slot kernels (batchk_kernel in ring mode) that take entries
// from it while they run.  The server thread admits a request by writing its operands and
// descriptor into a free ring entry and publishing it (a release store of the tail); a CTA
// whose slot frees up claims it at the next iteration of its reduction loop, so a request
// joins kernels that are already running instead of waiting for a batch to form or to
// drain.  A CTA releases done[i] once the entry's digits are written (to host memory); the
// server converts them and answers.  A lane launches more CTAs while its requests in
// flight and queued outnumber its running slots; CTAs whose slots stay empty leave after a
// short idle time, so idle lanes hold no SMs.
//
// Waves (size classes 2-3, requests beyond a continuous lane's limits, and every lane when
// continuous lanes are switched off): the server thread turns the queued requests of a
// lane into a wave -- one plan of the batched path with its own streams and buffers -- as
// soon as that lane has a free wave slot and the HBM admission budget allows, and launches
// it without waiting for the waves already on the GPU.  When a wave's completion event
// fires, its digits are copied back and converted and every request of the wave is
// answered.
//
// The moduli table, its Montgomery constants and the pairwise inverse table stay resident
// in the context for both.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/modgcd.h"
#include "mgcd_moduli.h"
#include "mgcd_plan.h"
#include "mgcd_radix.h"

using namespace mgcd;

namespace {

using Clock = std::chrono::steady_clock;

double now_s() { return std::chrono::duration<double>(Clock::now().time_since_epoch()).count(); }

constexpr int NLANES = NSTREAMS;       // one lane per size class
// Waves of one lane that may be in flight at once.  Pairs of the cluster lane take seconds
// each and a wave is answered only when all of its pairs are done, so later arrivals there
// get waves of their own instead of waiting for a slot.
constexpr int LANE_SLOTS[NLANES] = {2, 2, 2, 8};
// Requests per wave: a wave is answered when its slowest pair is done, so the cluster lane
// (one thread-block cluster per pair anyway) gives every request a wave of its own.
constexpr size_t LANE_MAX_WAVE[NLANES] = {16384, 16384, 4096, 1};
constexpr size_t POOL_RESERVE = size_t(2) << 30;   // device memory reserved at start
constexpr size_t MAX_QUEUED = size_t(1) << 22;

struct Request {
  uint64_t ticket = 0;
  std::vector<uint32_t> limbs;         // u then v
  uint32_t ul = 0, vl = 0;
  int lane = 0;
  int ref_nq = 0;                      // the reference's moduli count
  bool stream = false;                 // served by the lane's continuous kernels
  bool full = false;                   // (continuous) runs with the reference count
  uint32_t seq = 0;                    // (continuous) ring entry number
  size_t bytes = 0;                    // device bytes while admitted
  double t_submit = 0, t_done = 0;
  std::vector<uint32_t> g;
  int status = -1;
  bool done = false;
};

// ---- continuous lanes
// Size classes 0-1.  Class 2 (4,096-16,384 moduli) stays on waves: its pairs take ~100 ms on
// one CTA of a K-slot kernel, ~45 ms on the 4-CTA clusters its waves use, and that latency,
// not the wait for a slot, dominates its requests (measured: p99 of requests below 1M bits
// 124-156 ms with class 2 continuous, against 82 ms with waves for every class).
constexpr int STREAM_LANES = 2;
constexpr uint32_t STREAM_NQ_CAP[STREAM_LANES] = {1024, 4096};   // largest reference count taken
constexpr int STREAM_MAX_CTAS[STREAM_LANES] = {48, 112};         // CTAs a lane may run at once
constexpr int STREAM_LANE_STREAMS = 8;                                 // instances of a lane in flight
constexpr unsigned long long STREAM_IDLE_NS = 300000;                  // an idle CTA leaves after 0.3 ms

struct StreamInstance {
  cudaEvent_t done = nullptr;
  int first = 0, ctas = 0;             // its CTAs' scratch slots
  int stream = 0;                      // index into the lane's streams
};

struct StreamLane {
  int lane = 0, k = 4, threads = 1024;
  uint32_t nq_cap = 0, limb_cap = 0;   // per ring entry: moduli, operand limbs (u + v)
  size_t smem = 0, scratch_words = 0;  // per CTA
  StreamRing* ring_h = nullptr;        // pinned, mapped: host and device views
  StreamRing* ring_d = nullptr;
  uint32_t* limbs_h = nullptr;
  uint32_t* limbs_d = nullptr;
  mgcd_pair* dig_h = nullptr;
  mgcd_pair* dig_d = nullptr;
  uint32_t* d_head = nullptr;          // entries claimed (device counter)
  uint32_t* d_scratch = nullptr;       // STREAM_MAX_CTAS slots of scratch_words
  cudaStream_t streams[STREAM_LANE_STREAMS] = {};   // one per instance in flight: a launch on a
  bool stream_busy[STREAM_LANE_STREAMS] = {};       // busy stream would queue behind it
  uint32_t tail = 0;                   // entries published
  std::vector<Request*> entry;         // by ring slot: the request in flight there
  std::vector<uint32_t> live;          // entry numbers in flight
  std::vector<char> slot_used;         // scratch slots held by running instances
  std::vector<StreamInstance> inst;    // launched, not yet seen complete
  int ctas = 0;                        // CTAs of those instances
};

struct Wave {
  Plan plan;
  int lane = 0;
  bool busy = false;
  std::vector<Request*> reqs;
  size_t bytes = 0;
  cudaEvent_t done = nullptr;
  HostBuf staging;                     // pinned operand limbs of the wave
  std::vector<uint64_t> uo, vo, goff;
  std::vector<uint32_t> ul, vl, gcap, glen, gbuf;
  std::vector<int32_t> st;
  size_t trace = 0;                    // index of this wave's record in the server trace
};

constexpr size_t MAX_TRACE = size_t(1) << 20;   // wave records kept
constexpr int SERVE_CLUSTER_CTAS = 8;            // CTAs per cluster for class-3 requests
// CTAs per cluster for the waves of lanes 1-2 (0: the batch table's one CTA per K pairs).
// Measured on 1,000 mixed requests with 1 % at 1M bits, 10k / 100k req/s: table p50 6.1 /
// 6.6 ms, p99 242 / 204 ms; lane 2 on 4-CTA clusters p50 6.3 / 6.6, p99 149 / 165; lanes 1
// and 2 on 2- and 4-CTA clusters p99 104 / 135 but p50 up to 50 ms at 50k-100k req/s (lane 1
// carries a third of the requests and loses throughput on clusters).  Applied to waves
// whose clusters fit the GPU at once (start_wave); larger waves use the batch table.
constexpr int SERVE_LANE_CLUSTER[NLANES] = {0, 0, 4, 0};

size_t strip(const uint32_t* x, size_t n)
{
  while (n && x[n - 1] == 0) --n;
  return n;
}

}  // namespace

struct mgcd_server {
  mgcd_context* c = nullptr;
  size_t budget = 0, in_flight = 0, peak_bytes = 0;
  std::mutex mu;
  std::condition_variable cv_done, cv_work;
  std::deque<Request*> pending[NLANES];
  bool continuous = true;              // continuous lanes for size classes 0-1
  StreamLane sl[STREAM_LANES];
  std::deque<Request*> spending[STREAM_LANES];   // queued for the continuous lanes
  std::deque<Request*> retry[STREAM_LANES];      // uncertified with a scaled count: rerun in full
  size_t stream_live = 0;
  size_t queued = 0;
  std::unordered_map<uint64_t, Request*> table;
  uint64_t next_ticket = 1;
  std::vector<Wave> waves;
  std::thread th;
  bool stop = false;
  uint64_t n_waves = 0, n_launches = 0, n_done = 0;
  double t0 = 0;                       // server start (trace clock origin)
  std::vector<mgcd_wave_trace> trace;
};

namespace {

// Packs the wave's operands into pinned memory, plans and launches it (no waiting).
int start_wave(mgcd_server* S, Wave& w)
{
  mgcd_context* c = S->c;
  const size_t n = w.reqs.size();
  size_t tot = 0;
  for (const Request* r : w.reqs) tot += r->ul + r->vl;
  if (w.staging.grow(std::max<size_t>(tot, 1) * sizeof(uint32_t)) != cudaSuccess) return MGCD_ERR_CUDA;
  uint32_t* h = w.staging.as<uint32_t>();
  w.uo.resize(n); w.vo.resize(n); w.ul.resize(n); w.vl.resize(n);
  size_t off = 0;
  for (size_t i = 0; i < n; ++i) {
    const Request* r = w.reqs[i];
    if (r->ul + r->vl) std::memcpy(h + off, r->limbs.data(), (r->ul + r->vl) * sizeof(uint32_t));
    w.uo[i] = off;
    w.ul[i] = r->ul;
    w.vo[i] = off + r->ul;
    w.vl[i] = r->vl;
    off += r->ul + r->vl;
  }
  // Small clusters (latency) for a wave whose clusters fit the GPU in one round; a larger
  // wave is throughput bound and takes the batch table's one CTA per K pairs.
  const int lc = SERVE_LANE_CLUSTER[w.lane];
  w.plan.small_cluster_ctas = (lc > 0 && n * (size_t)lc <= (size_t)c->sms * (size_t)c->cfg[w.lane].k) ? lc : 0;
  int rc = plan_batch(c, w.plan, n, h, w.uo.data(), w.ul.data(), w.vo.data(), w.vl.data(), false);
  if (rc == MGCD_OK) rc = run_plan(c, w.plan);
  if (rc == MGCD_OK && cudaEventRecord(w.done, w.plan.stream) != cudaSuccess) rc = MGCD_ERR_CUDA;
  return rc;
}

// After the wave's event: reruns of uncertified pairs, digits back, conversion.
int finish_wave(mgcd_server* S, Wave& w)
{
  mgcd_context* c = S->c;
  const size_t n = w.reqs.size();
  int rc = sync_plan(c, w.plan);
  if (rc == MGCD_OK) rc = fetch(c, w.plan);
  if (rc != MGCD_OK) return rc;
  w.goff.resize(n); w.gcap.resize(n); w.glen.resize(n); w.st.resize(n);
  size_t tot = 0;
  for (size_t i = 0; i < n; ++i) {
    w.goff[i] = tot;
    w.gcap[i] = std::max<uint32_t>(1u, std::max(w.ul[i], w.vl[i]));
    tot += w.gcap[i];
  }
  w.gbuf.resize(std::max<size_t>(tot, 1));
  convert_all(c, w.plan, w.gbuf.data(), w.goff.data(), w.gcap.data(), w.glen.data(), w.st.data(), n >= 256);
  return MGCD_OK;
}

// ---- continuous lanes

int cmp_limbs(const uint32_t* a, size_t an, const uint32_t* b, size_t bn)
{
  if (an != bn) return an < bn ? -1 : 1;
  for (size_t i = an; i-- > 0;)
    if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
  return 0;
}

// Ring, operand and digit areas (pinned, mapped), the claim counter and scratch of lane l.
int lane_init(mgcd_server* S, StreamLane& L, int l, int priority)
{
  mgcd_context* c = S->c;
  L.lane = l;
  // 1,024-thread CTAs with K = 4 slots, whatever the batch table says: a lane's CTAs are
  // capped (STREAM_MAX_CTAS) and share the GPU with the other lanes, so its concurrency is
  // its CTAs x K; the batch table's two-per-SM 512 x 2 shape for class 1 halved it (the
  // saturation replay served 21.1k instead of 25.0k GCDs/s)
  L.threads = 1024;
  L.k = 4;
  L.nq_cap = STREAM_NQ_CAP[l];
  while (L.k > 2 && batch_smem_bytes(L.threads, L.k, L.nq_cap) > c->smem_optin - 16384) L.k /= 2;
  L.smem = batch_smem_bytes(L.threads, L.k, L.nq_cap);
  if (L.smem > c->smem_optin - 16384) return MGCD_ERR_GRID;
  // operand limbs of the largest pair whose reference count fits the cap
  size_t lo = 2, hi = (size_t)32 * L.nq_cap * 4;
  while (lo < hi) {
    const size_t mid = (lo + hi + 1) / 2;
    if (moduli_needed(c->L, mid) <= (int)L.nq_cap) lo = mid; else hi = mid - 1;
  }
  L.limb_cap = 2 * (uint32_t)((lo + 31) / 32);
  L.scratch_words = 4 * (size_t)L.k * L.nq_cap;
  L.entry.assign(STREAM_RING, nullptr);
  L.slot_used.assign(STREAM_MAX_CTAS[l], 0);
  const unsigned flags = cudaHostAllocMapped | cudaHostAllocPortable;
  void* p = nullptr;
  if (cudaHostAlloc(&p, sizeof(StreamRing), flags) != cudaSuccess) return MGCD_ERR_CUDA;
  L.ring_h = static_cast<StreamRing*>(p);
  std::memset(L.ring_h, 0, sizeof(StreamRing));
  if (cudaHostAlloc(&p, (size_t)STREAM_RING * L.limb_cap * sizeof(uint32_t), flags) != cudaSuccess)
    return MGCD_ERR_CUDA;
  L.limbs_h = static_cast<uint32_t*>(p);
  if (cudaHostAlloc(&p, (size_t)STREAM_RING * (L.nq_cap + 1) * sizeof(mgcd_pair), flags) != cudaSuccess)
    return MGCD_ERR_CUDA;
  L.dig_h = static_cast<mgcd_pair*>(p);
  if (cudaHostGetDevicePointer(reinterpret_cast<void**>(&L.ring_d), L.ring_h, 0) != cudaSuccess ||
      cudaHostGetDevicePointer(reinterpret_cast<void**>(&L.limbs_d), L.limbs_h, 0) != cudaSuccess ||
      cudaHostGetDevicePointer(reinterpret_cast<void**>(&L.dig_d), L.dig_h, 0) != cudaSuccess)
    return MGCD_ERR_CUDA;
  if (cudaMalloc(reinterpret_cast<void**>(&L.d_head), sizeof(uint32_t)) != cudaSuccess ||
      cudaMemset(L.d_head, 0, sizeof(uint32_t)) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void**>(&L.d_scratch),
                 (size_t)STREAM_MAX_CTAS[l] * L.scratch_words * sizeof(uint32_t)) != cudaSuccess)
    return MGCD_ERR_CUDA;
  for (cudaStream_t& st : L.streams)
    if (cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, priority) != cudaSuccess) return MGCD_ERR_CUDA;
  return MGCD_OK;
}

void lane_free(StreamLane& L)
{
  for (cudaStream_t st : L.streams)
    if (st) cudaStreamSynchronize(st);
  for (StreamInstance& x : L.inst)
    if (x.done) cudaEventDestroy(x.done);
  L.inst.clear();
  for (cudaStream_t st : L.streams)
    if (st) cudaStreamDestroy(st);
  if (L.d_scratch) cudaFree(L.d_scratch);
  if (L.d_head) cudaFree(L.d_head);
  if (L.dig_h) cudaFreeHost(L.dig_h);
  if (L.limbs_h) cudaFreeHost(L.limbs_h);
  if (L.ring_h) cudaFreeHost(L.ring_h);
  L = StreamLane();
}

bool lane_fits(const StreamLane& L, const Request* r)
{
  return L.ring_h && r->ul && r->vl && (uint32_t)r->ref_nq <= L.nq_cap && r->ul + r->vl <= L.limb_cap;
}

// Writes r into the next ring entry and publishes it; false if that entry is still in use.
bool lane_publish(mgcd_server* S, StreamLane& L, Request* r)
{
  const uint32_t slot = L.tail % STREAM_RING;
  if (L.entry[slot]) return false;
  const uint32_t* u = r->limbs.data();
  const uint32_t* v = u + r->ul;
  uint32_t* dst = L.limbs_h + (size_t)slot * L.limb_cap;
  PairDesc d;
  const bool u_big = cmp_limbs(u, r->ul, v, r->vl) >= 0;
  d.u_len = u_big ? r->ul : r->vl;
  d.v_len = u_big ? r->vl : r->ul;
  std::memcpy(dst, u_big ? u : v, d.u_len * sizeof(uint32_t));
  std::memcpy(dst + d.u_len, u_big ? v : u, d.v_len * sizeof(uint32_t));
  d.u_off = (uint64_t)slot * L.limb_cap;
  d.v_off = d.u_off + d.u_len;
  int nq = r->ref_nq;
  const float scale = S->c->cfg[L.lane].nq_scale;
  if (!r->full && scale < 1.0f) nq = std::min(nq, std::max(256, ((int)std::ceil(scale * nq) + 31) / 32 * 32));
  d.nq = (uint32_t)nq;
  d.out_off = slot * (L.nq_cap + 1);
  d.g_off = 0;
  d.g_cap = 0;
  d.nq_cap = 0;
  L.ring_h->desc[slot] = d;
  L.ring_h->done[slot] = 0u;
  r->seq = L.tail;
  r->full = r->full || nq == r->ref_nq;
  L.entry[slot] = r;
  L.live.push_back(L.tail);
  ++L.tail;
  __atomic_store_n(&L.ring_h->tail, L.tail, __ATOMIC_RELEASE);   // orders the entry before it
  ++S->stream_live;
  return true;
}

// Answers the lane's completed entries (called with the server lock held).
bool lane_poll(mgcd_server* S, StreamLane& L)
{
  bool any = false;
  for (size_t i = 0; i < L.live.size();) {
    const uint32_t seq = L.live[i];
    const uint32_t slot = seq % STREAM_RING;
    if (__atomic_load_n(&L.ring_h->done[slot], __ATOMIC_ACQUIRE) != seq + 1u) {
      ++i;
      continue;
    }
    Request* r = L.entry[slot];
    const int32_t st = L.ring_h->status[slot];
    L.entry[slot] = nullptr;
    L.live[i] = L.live.back();
    L.live.pop_back();
    --S->stream_live;
    any = true;
    if ((st == ST_INSUFFICIENT || st == ST_REDUX) && !r->full) {
      r->full = true;                  // rerun with the reference count (as a batch does)
      S->retry[L.lane].push_back(r);
      continue;
    }
    int rc = to_status(st);
    if (rc == MGCD_OK) {
      const size_t cap = std::max<size_t>(1, std::max(r->ul, r->vl));
      r->g.resize(cap);
      size_t len = 0;
      if (mixed_radix_to_limbs(L.dig_h + (size_t)slot * (L.nq_cap + 1), L.ring_h->count[slot], r->g.data(), cap, &len))
        rc = MGCD_ERR_CAPACITY;
      r->g.resize(rc == MGCD_OK ? len : 0);
    }
    r->status = rc;
    r->t_done = now_s();
    r->done = true;
    r->limbs.clear();
    r->limbs.shrink_to_fit();
    S->n_done += 1;
    S->in_flight -= r->bytes;
  }
  return any;
}

// Instances whose CTAs have all left give back their scratch slots and stream.
void lane_reap(StreamLane& L)
{
  for (size_t i = 0; i < L.inst.size();) {
    StreamInstance& x = L.inst[i];
    if (cudaEventQuery(x.done) != cudaSuccess) {
      ++i;
      continue;
    }
    for (int j = 0; j < x.ctas; ++j) L.slot_used[x.first + j] = 0;
    L.ctas -= x.ctas;
    L.stream_busy[x.stream] = false;
    cudaEventDestroy(x.done);
    L.inst[i] = L.inst.back();
    L.inst.pop_back();
  }
}

// More CTAs while the entries in flight and queued outnumber the running slots.  An added
// instance is at least as large as the CTAs already running (capped by the lane's share),
// so a lane reaches its full size in a few launches even when its load grows slowly; the
// instances stay resident while they find work.
bool lane_launch(mgcd_server* S, StreamLane& L, size_t queued)
{
  const int cap = STREAM_MAX_CTAS[L.lane];
  const size_t want = std::min<size_t>((L.live.size() + queued + L.k - 1) / L.k, (size_t)cap);
  if (L.live.empty() || want <= (size_t)L.ctas) return false;
  const int need = std::min(cap - L.ctas, std::max((int)want - L.ctas, L.ctas));
  if (need <= 0) return false;
  int si = 0;
  while (si < STREAM_LANE_STREAMS && L.stream_busy[si]) ++si;
  if (si == STREAM_LANE_STREAMS) return false;
  // the longest run of free scratch slots, up to `need`
  int best = -1, best_len = 0;
  for (int j = 0; j < cap;) {
    if (L.slot_used[j]) { ++j; continue; }
    int e = j;
    while (e < cap && !L.slot_used[e] && e - j < need) ++e;
    if (e - j > best_len) { best = j; best_len = e - j; }
    j = e + 1;
  }
  if (best < 0) return false;
  mgcd_context* c = S->c;
  BatchArgs a{};
  a.inv = InvTab{c->d_invtab.as<uint32_t>(), c->invtab_n};
  a.limbs = L.limbs_d;
  a.pairs = L.ring_d->desc;
  a.mods = c->mods.as<ModConst>();
  a.L = c->L;
  a.scratch = L.d_scratch + (size_t)best * L.scratch_words;
  a.scratch_words = L.scratch_words;
  a.nq_max = L.nq_cap;
  a.digits = L.dig_d;
  a.count = L.ring_d->count;
  a.iters = L.ring_d->iters;
  a.status = L.ring_d->status;
  a.stage_fail = 0xFFFFFFFFu;
  a.ring = L.ring_d;
  a.ring_head = L.d_head;
  a.idle_ns = STREAM_IDLE_NS;
  StreamInstance x;
  x.first = best;
  x.ctas = best_len;
  x.stream = si;
  if (cudaEventCreateWithFlags(&x.done, cudaEventDisableTiming) != cudaSuccess) return false;
  if (launch_ring(a, L.threads, L.k, best_len, L.smem, L.streams[si]) != cudaSuccess ||
      cudaEventRecord(x.done, L.streams[si]) != cudaSuccess) {
    cudaEventDestroy(x.done);
    return false;
  }
  L.stream_busy[si] = true;
  for (int j = 0; j < best_len; ++j) L.slot_used[best + j] = 1;
  L.ctas += best_len;
  L.inst.push_back(x);
  ++S->n_launches;
  return true;
}

void serve_loop(mgcd_server* S)
{
  cudaSetDevice(S->c->device);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    bool progressed = false;
    // ---- continuous lanes: answer completed entries, admit queued requests into free
    // ring entries (reruns first), add CTAs while entries outnumber running slots
    for (int l = 0; l < STREAM_LANES; ++l) {
      StreamLane& L = S->sl[l];
      if (!L.ring_h) continue;
      if (lane_poll(S, L)) { progressed = true; S->cv_done.notify_all(); }
      lane_reap(L);
      while (!S->retry[l].empty() && lane_publish(S, L, S->retry[l].front())) S->retry[l].pop_front();
      auto& q = S->spending[l];
      while (!q.empty() && S->retry[l].empty() && S->in_flight + q.front()->bytes <= S->budget) {
        Request* r = q.front();
        if (!lane_publish(S, L, r)) break;
        q.pop_front();
        --S->queued;
        S->in_flight += r->bytes;
        S->peak_bytes = std::max(S->peak_bytes, S->in_flight);
        progressed = true;
      }
      while (lane_launch(S, L, q.size() + S->retry[l].size())) progressed = true;
    }
    // ---- completed waves: answer their requests
    for (Wave& w : S->waves) {
      if (!w.busy) continue;
      const cudaError_t q = cudaEventQuery(w.done);
      if (q == cudaErrorNotReady) continue;
      const double t_gpu = now_s();
      lk.unlock();
      const int rc = q == cudaSuccess ? finish_wave(S, w) : MGCD_ERR_CUDA;
      const double t = now_s();
      lk.lock();
      if (w.trace < S->trace.size()) {
        S->trace[w.trace].t_gpu_done = t_gpu - S->t0;
        S->trace[w.trace].t_answered = t - S->t0;
      }
      for (size_t i = 0; i < w.reqs.size(); ++i) {
        Request* r = w.reqs[i];
        if (rc == MGCD_OK) {
          r->status = w.st[i];
          r->g.assign(w.gbuf.begin() + w.goff[i], w.gbuf.begin() + w.goff[i] + w.glen[i]);
        } else {
          r->status = rc;
        }
        r->t_done = t;
        r->done = true;
        r->limbs.clear();
        r->limbs.shrink_to_fit();
      }
      S->n_done += w.reqs.size();
      S->in_flight -= w.bytes;
      w.reqs.clear();
      w.busy = false;
      S->cv_done.notify_all();
      progressed = true;
    }
    // ---- admit queued requests into free wave slots, smallest lanes first
    for (int lane = 0; lane < NLANES; ++lane) {
      auto& q = S->pending[lane];
      if (q.empty()) continue;
      Wave* w = nullptr;
      for (Wave& x : S->waves)
        if (x.lane == lane && !x.busy) { w = &x; break; }
      if (!w) continue;
      size_t bytes = 0;
      while (!q.empty() && w->reqs.size() < LANE_MAX_WAVE[lane] &&
             S->in_flight + bytes + q.front()->bytes <= S->budget) {
        bytes += q.front()->bytes;
        w->reqs.push_back(q.front());
        q.pop_front();
      }
      if (w->reqs.empty()) continue;
      S->queued -= w->reqs.size();
      S->in_flight += bytes;
      S->peak_bytes = std::max(S->peak_bytes, S->in_flight);
      w->bytes = bytes;
      w->busy = true;
      const double t_admit = now_s() - S->t0;
      lk.unlock();
      const int rc = start_wave(S, *w);
      const double t_launched = now_s() - S->t0;
      lk.lock();
      ++S->n_waves;
      S->n_launches += (uint64_t)w->plan.launches;
      w->trace = S->trace.size();
      if (S->trace.size() < MAX_TRACE)
        S->trace.push_back(mgcd_wave_trace{lane, (uint32_t)w->reqs.size(), t_admit, t_launched, 0.0, 0.0});
      if (rc != MGCD_OK) {   // answer the wave's requests with the failure
        cudaStreamSynchronize(w->plan.stream);
        const double t = now_s();
        for (Request* r : w->reqs) {
          r->status = rc;
          r->t_done = t;
          r->done = true;
        }
        S->n_done += w->reqs.size();
        S->in_flight -= w->bytes;
        w->reqs.clear();
        w->busy = false;
        S->cv_done.notify_all();
      }
      progressed = true;
    }
    bool any_busy = S->stream_live > 0;
    for (int l = 0; l < STREAM_LANES; ++l) any_busy = any_busy || !S->retry[l].empty();
    for (const Wave& w : S->waves) any_busy = any_busy || w.busy;
    if (S->stop && S->queued == 0 && !any_busy) break;
    if (!progressed) S->cv_work.wait_for(lk, std::chrono::microseconds(any_busy ? 20 : 500));
  }
}

int submit_at(mgcd_server* S, const uint32_t* u, size_t uSz, const uint32_t* v, size_t vSz, double t_submit,
              uint64_t* ticket)
{
  if (!S || !ticket || (uSz && !u) || (vSz && !v)) return MGCD_ERR_INVALID_ARG;
  mgcd_context* c = S->c;
  const size_t ul = strip(u, uSz), vl = strip(v, vSz);
  const bool u_big = ul > vl || (ul == vl && ul && u[ul - 1] >= v[vl - 1]);
  const uint32_t* big = u_big ? u : v;
  const size_t bl = u_big ? ul : vl;
  int nq = 0;
  if (ul && vl) {
    const size_t bits = (bl - 1) * 32 + (32 - __builtin_clz(big[bl - 1]));
    nq = c->force_nq ? (int)c->force_nq : moduli_needed(c->L, bits);
    if ((size_t)nq > c->moduli.size()) return MGCD_ERR_NOT_ENOUGH_MODULI;
  }
  auto* r = new Request();
  r->limbs.resize(ul + vl);
  if (ul) std::memcpy(r->limbs.data(), u, ul * sizeof(uint32_t));
  if (vl) std::memcpy(r->limbs.data() + ul, v, vl * sizeof(uint32_t));
  r->ul = (uint32_t)ul;
  r->vl = (uint32_t)vl;
  r->lane = size_class((uint32_t)nq);
  r->ref_nq = nq;
  // device bytes while admitted: operands, descriptor and order entry, digit slots, status
  // words, and the pair's share of the reduction scratch (u0, v0, (p, b) history)
  r->bytes = 4 * (ul + vl) + sizeof(PairDesc) + 4 + 8 * ((size_t)nq + 1) + 12 + 16 * (size_t)nq;
  if (r->bytes > S->budget) {
    delete r;
    return MGCD_ERR_BUDGET;
  }
  {
    std::lock_guard<std::mutex> g(S->mu);
    if (S->stop) {
      delete r;
      return MGCD_ERR_INVALID_ARG;
    }
    if (S->queued >= MAX_QUEUED) {
      delete r;
      return MGCD_ERR_BUSY;
    }
    r->ticket = S->next_ticket++;
    r->t_submit = t_submit > 0 ? t_submit : now_s();
    S->table[r->ticket] = r;
    r->stream = S->continuous && r->lane < STREAM_LANES && lane_fits(S->sl[r->lane], r);
    if (r->stream) S->spending[r->lane].push_back(r);
    else S->pending[r->lane].push_back(r);
    ++S->queued;
    *ticket = r->ticket;
  }
  S->cv_work.notify_one();
  return MGCD_OK;
}

// Waits (up to timeout_ms; 0 = no limit) for the ticket; on completion copies the result,
// releases the ticket and returns the request's status.
int take(mgcd_server* S, uint64_t ticket, unsigned timeout_ms, uint32_t* g, size_t g_cap, size_t* g_len,
         double* latency_s)
{
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->table.find(ticket);
  if (it == S->table.end()) return MGCD_ERR_INVALID_ARG;
  Request* r = it->second;
  const auto pred = [&] { return r->done; };
  if (timeout_ms == 0) S->cv_done.wait(lk, pred);
  else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) return MGCD_ERR_TIMEOUT;
  int rc = r->status;
  if (g_len) *g_len = r->g.size();
  if (latency_s) *latency_s = r->t_done - r->t_submit;
  if (rc == MGCD_OK) {
    if (r->g.size() > g_cap) rc = MGCD_ERR_CAPACITY;
    else if (!r->g.empty()) std::memcpy(g, r->g.data(), r->g.size() * sizeof(uint32_t));
  }
  S->table.erase(it);
  delete r;
  return rc;
}

}  // namespace

extern "C" {

int mgcd_serve_start(mgcd_context* c, size_t budget_bytes, mgcd_server** out)
{
  if (!c || !out || budget_bytes == 0) return MGCD_ERR_INVALID_ARG;
  *out = nullptr;
  if (c->serving) return MGCD_ERR_BUSY;
  if (cudaSetDevice(c->device) != cudaSuccess) return MGCD_ERR_CUDA;
  cudaStreamSynchronize(c->main.stream);
  auto* S = new mgcd_server();
  S->c = c;
  S->budget = budget_bytes;
  S->t0 = now_s();
  std::vector<int> lanes;
  for (int l = 0; l < NLANES; ++l) lanes.insert(lanes.end(), LANE_SLOTS[l], l);
  S->waves.resize(lanes.size());
  // The short requests' lanes get the most urgent stream priority, so that CTAs of their
  // waves are scheduled first whenever SMs free up; class-3 requests (seconds each) the least.
  int least = 0, greatest = 0;
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  int rc = MGCD_OK;
  for (size_t i = 0; i < S->waves.size() && rc == MGCD_OK; ++i) {
    Wave& w = S->waves[i];
    w.lane = lanes[i];
    w.plan.graphable = false;
    if (w.lane == CLUSTER_CLASS) {   // one request per wave: one pair per cluster
      w.plan.cluster_ctas = SERVE_CLUSTER_CTAS;
      w.plan.cluster_k = 1;
    }
    if (w.plan.create(w.lane == CLUSTER_CLASS ? least : greatest) != cudaSuccess ||
        cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming) != cudaSuccess)
      rc = MGCD_ERR_CUDA;
  }
  if (rc != MGCD_OK) {
    for (Wave& w : S->waves) {
      w.plan.destroy(c->pool);
      if (w.done) cudaEventDestroy(w.done);
    }
    delete S;
    return rc;
  }
  for (int l = 0; l < STREAM_LANES && rc == MGCD_OK; ++l) rc = lane_init(S, S->sl[l], l, greatest);
  if (rc != MGCD_OK) {
    for (int l = 0; l < STREAM_LANES; ++l) lane_free(S->sl[l]);
    for (Wave& w : S->waves) {
      w.plan.destroy(c->pool);
      if (w.done) cudaEventDestroy(w.done);
    }
    delete S;
    return rc;
  }
  // Reserve pool memory up front so that waves allocate from it without the driver mapping
  // new memory while kernels run (the pool keeps freed memory).
  {
    void* p = nullptr;
    cudaStream_t s = S->waves[0].plan.stream;
    if (cudaMallocFromPoolAsync(&p, std::min(budget_bytes, POOL_RESERVE), c->pool, s) == cudaSuccess)
      cudaFreeAsync(p, s);
    cudaStreamSynchronize(s);
  }
  c->serving = true;
  S->th = std::thread(serve_loop, S);
  *out = S;
  return MGCD_OK;
}

int mgcd_serve_stop(mgcd_server* S)
{
  if (!S) return MGCD_ERR_INVALID_ARG;
  {
    std::lock_guard<std::mutex> g(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  if (S->th.joinable()) S->th.join();
  cudaSetDevice(S->c->device);
  for (int l = 0; l < STREAM_LANES; ++l) {
    if (S->sl[l].ring_h) __atomic_store_n(&S->sl[l].ring_h->stop, 1u, __ATOMIC_RELEASE);   // idle CTAs leave
    lane_free(S->sl[l]);
  }
  for (Wave& w : S->waves) {
    w.plan.destroy(S->c->pool);
    w.staging.release();
    if (w.done) cudaEventDestroy(w.done);
  }
  for (auto& kv : S->table) delete kv.second;
  S->c->serving = false;
  delete S;
  return MGCD_OK;
}

int mgcd_serve_submit(mgcd_server* S, const uint32_t* u, size_t uSz, const uint32_t* v, size_t vSz,
                      uint64_t* ticket)
{
  return submit_at(S, u, uSz, v, vSz, 0.0, ticket);
}

int mgcd_serve_set_continuous(mgcd_server* S, int enable)
{
  if (!S) return MGCD_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(S->mu);
  if (!S->table.empty()) return MGCD_ERR_BUSY;
  S->continuous = enable != 0;
  return MGCD_OK;
}

int mgcd_serve_poll(mgcd_server* S, uint64_t ticket, int* done)
{
  if (!S || !done) return MGCD_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(S->mu);
  auto it = S->table.find(ticket);
  if (it == S->table.end()) return MGCD_ERR_INVALID_ARG;
  *done = it->second->done ? 1 : 0;
  return MGCD_OK;
}

int mgcd_serve_take(mgcd_server* S, uint64_t ticket, unsigned timeout_ms, uint32_t* g, size_t g_cap,
                    size_t* g_len, double* latency_s)
{
  if (!S || (g_cap && !g)) return MGCD_ERR_INVALID_ARG;
  return take(S, ticket, timeout_ms, g, g_cap, g_len, latency_s);
}

int mgcd_serve_replay(mgcd_server* S, size_t n, const uint32_t* limbs, const uint64_t* u_off,
                      const uint32_t* u_len, const uint64_t* v_off, const uint32_t* v_len, const double* arrival_s,
                      uint32_t* g, const uint64_t* g_off, const uint32_t* g_cap, uint32_t* g_len, int32_t* status,
                      double* latency_s, double* makespan_s)
{
  if (!S || (n && (!limbs || !u_off || !u_len || !v_off || !v_len || !arrival_s || !g || !g_off || !g_cap ||
                   !g_len || !status || !latency_s)))
    return MGCD_ERR_INVALID_ARG;
  std::vector<size_t> idx(n);
  for (size_t i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return arrival_s[a] < arrival_s[b]; });
  std::vector<uint64_t> tk(n, 0);
  std::vector<int> sub(n, MGCD_OK);
  const double t0 = now_s();
  for (size_t k = 0; k < n; ++k) {
    const size_t i = idx[k];
    const double due = t0 + arrival_s[i];
    for (;;) {   // open loop: submit at the scheduled arrival time
      const double left = due - now_s();
      if (left <= 0) break;
      if (left > 200e-6) std::this_thread::sleep_for(std::chrono::duration<double>(left - 100e-6));
    }
    sub[i] = submit_at(S, limbs + u_off[i], u_len[i], limbs + v_off[i], v_len[i], due, &tk[i]);
  }
  double last = t0;
  int rc = MGCD_OK;
  for (size_t i = 0; i < n; ++i) {
    size_t len = 0;
    double lat = 0;
    int s = sub[i];
    if (s == MGCD_OK) {
      s = take(S, tk[i], 0, g + g_off[i], g_cap[i], &len, &lat);
      last = std::max(last, t0 + arrival_s[i] + lat);
    }
    status[i] = s;
    g_len[i] = (uint32_t)len;
    latency_s[i] = lat;
    if (s != MGCD_OK && rc == MGCD_OK) rc = s;
  }
  if (makespan_s) *makespan_s = last - t0;
  return rc;
}

int mgcd_serve_trace(mgcd_server* S, mgcd_wave_trace* out, size_t cap, size_t* n)
{
  if (!S || !n || (cap && !out)) return MGCD_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(S->mu);
  *n = S->trace.size();
  const size_t k = std::min(cap, S->trace.size());
  if (k) std::memcpy(out, S->trace.data(), k * sizeof(mgcd_wave_trace));
  return MGCD_OK;
}

int mgcd_serve_stats(mgcd_server* S, uint64_t* waves, uint64_t* launches, uint64_t* peak_bytes,
                     uint64_t* completed)
{
  if (!S) return MGCD_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(S->mu);
  if (waves) *waves = S->n_waves;
  if (launches) *launches = S->n_launches;
  if (peak_bytes) *peak_bytes = S->peak_bytes;
  if (completed) *completed = S->n_done;
  return MGCD_OK;
}

}  // extern "C"

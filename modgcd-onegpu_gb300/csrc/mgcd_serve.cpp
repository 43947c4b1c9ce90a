// mgcd_serve.cpp -- request server: continuous batching of single gcd requests on one GPU.
// No counterpart in the reference (its GmpCudaDevice::gcd is one blocking call per pair).
//
// Requests are queued per lane (the batched path's size class of the pair).  A server
// thread turns the queued requests of a lane into a wave -- one plan of the batched path
// with its own streams and buffers -- as soon as that lane has a free wave slot and the
// HBM admission budget allows, and launches it without waiting for the waves already on
// the GPU: their persistent kernels are still draining while the new wave's CTAs take the
// SMs they free, so the work of requests that arrived later overlaps with the earlier
// ones'.  The moduli table, its Montgomery constants and the pairwise inverse table stay
// resident in the context; a wave holds only its operands, residues, scratch and digits.
// When a wave's completion event fires, its digits are copied back and converted and
// every request of the wave is answered.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
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
  size_t bytes = 0;                    // device bytes while admitted
  double t_submit = 0, t_done = 0;
  std::vector<uint32_t> g;
  int status = -1;
  bool done = false;
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

void serve_loop(mgcd_server* S)
{
  cudaSetDevice(S->c->device);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    bool progressed = false;
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
    bool any_busy = false;
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
    S->pending[r->lane].push_back(r);
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

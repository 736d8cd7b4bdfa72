// Serving loop: pricing, Greeks and LSMC requests with continuous batching on
// one GPU.  (The reference has no serving layer; each request is one of its
// calls: a European price or greeks_fd(all five Greeks) on gbm / heston /
// merton (greeks.rs:322-358), or lsmc_american_option (lsmc.rs:25-115).)
//
//  * Requests are submitted from any thread (submit/poll/wait) or replayed
//    from an arrival schedule; one dispatcher thread owns the device work.
//  * Admission is by device memory: every admitted job takes its bytes (the
//    instance table with its RNG stream descriptors, partial sums, LSMC path
//    array and sweep scratch) from one pre-allocated arena of the configured
//    budget; a request waits until its bytes are free.  Nothing is allocated
//    with cudaMalloc while serving.
//  * Continuous batching: whenever a lane (a CUDA stream) is free, the
//    dispatcher admits what has arrived.  Small pricing/Greeks requests that
//    arrived since the last dispatch go out as ONE launch (one block per
//    256-path chunk of any of them) on a highest-priority stream; LSMC
//    requests (chains of short dependent passes, one CUDA graph launch for
//    the large ones) on middle-priority streams; large pricing and Greeks
//    requests as their own launches on lowest-priority streams.
//    Launches on different lanes run concurrently; kernels are sized so that
//    blocks retire after one chunk (pricing/Greeks) or one step (LSMC), so the
//    block scheduler gives the SMs to high-priority work as blocks retire.
//  * A request's result depends only on the request: its paths' streams are
//    its own, its chunk partials are added in chunk order, and the LSMC
//    launch shape depends only on (n_paths, steps).  The same request gives
//    the same bits alone and in any mix.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "greeks_kernels.h"
#include "host_common.h"
#include "lsmc_kernels.h"

namespace stocha {

// First-fit allocator over the offsets of one device slab; free blocks are
// coalesced with their neighbours.  Host-only bookkeeping.
class Arena {
 public:
  static constexpr uint64_t kAlign = 256;
  explicit Arena(uint64_t cap) : cap_(cap & ~(kAlign - 1)) {
    if (cap_) free_[0] = cap_;
  }
  static uint64_t round(uint64_t b) { return (b + kAlign - 1) & ~(kAlign - 1); }
  bool alloc(uint64_t bytes, uint64_t* off) {
    bytes = round(bytes ? bytes : 1);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < bytes) continue;
      const uint64_t o = it->first, rest = it->second - bytes;
      free_.erase(it);
      if (rest) free_[o + bytes] = rest;
      live_[o] = bytes;
      used_ += bytes;
      peak_ = std::max(peak_, used_);
      *off = o;
      return true;
    }
    return false;
  }
  void release(uint64_t off) {
    auto it = live_.find(off);
    if (it == live_.end()) return;
    uint64_t o = it->first, b = it->second;
    live_.erase(it);
    used_ -= b;
    auto next = free_.lower_bound(o);
    if (next != free_.end() && o + b == next->first) {
      b += next->second;
      free_.erase(next);
    }
    auto prev = free_.lower_bound(o);
    if (prev != free_.begin()) {
      --prev;
      if (prev->first + prev->second == o) {
        o = prev->first;
        b += prev->second;
        free_.erase(prev);
      }
    }
    free_[o] = b;
  }
  uint64_t capacity() const { return cap_; }
  uint64_t used() const { return used_; }
  uint64_t peak() const { return peak_; }
  uint64_t largest_free() const {
    uint64_t m = 0;
    for (auto& f : free_) m = std::max(m, f.second);
    return m;
  }
  size_t free_blocks() const { return free_.size(); }

 private:
  uint64_t cap_, used_ = 0, peak_ = 0;
  std::map<uint64_t, uint64_t> free_, live_;
};

}  // namespace stocha

using namespace stocha;

namespace {

constexpr uint64_t kChunk = 256;           // paths per block of a pricing/Greeks launch
constexpr uint64_t kSmallPaths = 100000;   // requests up to this size go to high-priority lanes
constexpr size_t kBatchMaxInst = 64;       // instances per batched launch
constexpr uint64_t kBatchMaxItems = 1u << 16;
constexpr size_t kPinnedBytes = 1u << 20;  // staging per lane (>= the largest batch's table and sums)

double now_s(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// Where a request is: queued (submitted, not admitted), admitted (its job is
// on a lane or done) or cancelled before admission.
enum : uint8_t { kQueued = 0, kAdmitted = 1, kCancelled = 2 };

struct Req {
  stocha_request r;
  stocha_result res;
  uint64_t bytes = 0;  // arena bytes of its job when run alone
  bool small = false;
  bool lsmc = false;
  uint8_t phase = kQueued;  // under the server's lock
};

// A request as the dispatcher sees it (its own copy, taken under the lock).
struct Pending {
  uint64_t ticket;
  Req q;
};

// Lane classes, by stream priority: small pricing/Greeks batches, small LSMC
// jobs, everything large.
enum LaneClass : int { kHigh = 0, kMid = 1, kLow = 2 };

struct Lane {
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  int cls = kLow;
  bool busy = false;
  char* pin = nullptr;  // pinned staging: instance table in, sums and status out
  // the job in flight
  bool lsmc = false;
  std::vector<uint64_t> tickets;
  std::vector<int> kinds;
  std::vector<stocha_model> models;
  std::vector<double> bumps;
  uint64_t off = 0;
  size_t out_pin = 0;  // offset of the results in pin
  LsmcJob lj;
  LsmcGraphs* graphs = nullptr;  // this stream's LSMC sweep graphs
};

}  // namespace

struct stocha_server {
  int device = 0;
  int sms = 152;
  stocha_ctx* ctx = nullptr;  // ziggurat tables, error reporting
  char* slab = nullptr;
  Arena arena{0};
  std::vector<Lane> lanes;
  std::chrono::steady_clock::time_point t0;

  std::mutex mu;
  std::condition_variable cv_in, cv_done;
  std::deque<Req> reqs;          // by ticket
  std::deque<uint64_t> inbox;    // submitted, not yet seen by the dispatcher
  bool stop = false;
  std::thread thread;

  // dispatcher-only state
  std::deque<Pending> pending;  // seen, not admitted (submission order)
  uint64_t jobs = 0, batched = 0, completed = 0, failed = 0;
  uint64_t cancelled = 0;  // under the lock

  void loop();
  bool poll_lanes();
  bool dispatch();
  bool launch_batch(Lane& L, const std::vector<const Pending*>& t, uint64_t off, uint64_t items);
  bool launch_lsmc(Lane& L, const Pending& p, uint64_t off);
  void fail(const std::vector<uint64_t>& t, int code, const std::string& msg);
  std::vector<const Pending*> claim(const std::vector<const Pending*>& t);
};

namespace {

// Device bytes of a pricing/Greeks job: instance table (with the paths' RNG
// stream descriptors), chunk partials, instance sums, status word.
uint64_t batch_bytes(size_t n_inst, uint64_t items) {
  return Arena::round(n_inst * sizeof(GInst)) + Arena::round(items * kGreekAcc * 8) +
         Arena::round(n_inst * kGreekAcc * 8) + 256;
}
// Pinned staging of a pricing/Greeks job: the table in, the sums and the
// status word out.
size_t batch_pinned(size_t n_inst) { return Arena::round(n_inst * sizeof(GInst)) + n_inst * kGreekAcc * 8 + 16; }

uint64_t items_of(const Req& q) { return (q.r.inst.n_paths + kChunk - 1) / kChunk; }

LsmcJob lsmc_job(const stocha_request& r) {
  const stocha_greeks_instance& x = r.inst;
  LsmcJob j;
  j.s0 = x.s0;
  j.k = x.strike;
  j.r = x.r;
  j.sigma = x.sigma;
  j.t = x.t;
  j.steps = x.steps;
  j.n_paths = x.n_paths;
  j.deg = (uint64_t)r.poly_degree;
  j.seed = x.seed;
  j.is_put = x.payoff == STOCHA_PAYOFF_PUT;
  j.precision = STOCHA_FP32;
  return j;
}

int validate(const stocha_request& r) {
  const stocha_greeks_instance& x = r.inst;
  if (r.kind == STOCHA_REQ_LSMC) return lsmc_validate(lsmc_job(r));
  if (r.kind != STOCHA_REQ_PRICE && r.kind != STOCHA_REQ_GREEKS)
    return set_error(STOCHA_ERR_VALUE, "request kind must be price, greeks or lsmc");
  if (x.model != STOCHA_MODEL_GBM && x.model != STOCHA_MODEL_HESTON && x.model != STOCHA_MODEL_MERTON)
    return set_error(STOCHA_ERR_VALUE, "model must be gbm, heston or merton");
  if (x.model == STOCHA_MODEL_HESTON && x.scheme != 0)
    return set_error(STOCHA_ERR_VALUE, "served Heston requests use the euler scheme (the batched serving kernel implements Euler only)");
  if (x.payoff != STOCHA_PAYOFF_CALL && x.payoff != STOCHA_PAYOFF_PUT)
    return set_error(STOCHA_ERR_VALUE, "payoff must be call or put");
  if (x.n_paths == 0 || x.steps == 0) return set_error(STOCHA_ERR_VALUE, "steps and n_paths must be positive");
  // the FP32 kernels count a path's normals in 32 bits
  if (x.steps >= (1ull << 32)) return set_error(STOCHA_ERR_VALUE, "steps must be below 2^32");
  return STOCHA_OK;
}


}  // namespace

void stocha_server::fail(const std::vector<uint64_t>& t, int code, const std::string& msg) {
  std::lock_guard<std::mutex> lk(mu);
  const double now = now_s(t0);
  for (uint64_t k : t) {
    reqs[k].res.status = -code;
    reqs[k].res.t_done = now;
    ++failed;
  }
  set_error(code, msg);
  cv_done.notify_all();
}

bool stocha_server::launch_batch(Lane& L, const std::vector<const Pending*>& t, uint64_t off, uint64_t items) {
  const size_t n = t.size();
  char* base = slab + off;
  const uint64_t o_part = Arena::round(n * sizeof(GInst));
  const uint64_t o_sums = o_part + Arena::round(items * kGreekAcc * 8);
  const uint64_t o_err = o_sums + Arena::round(n * kGreekAcc * 8);
  GInst* inst = (GInst*)L.pin;
  L.models.resize(n);
  L.bumps.resize(n);
  L.tickets.resize(n);
  L.kinds.resize(n);
  uint64_t it = 0;
  for (size_t i = 0; i < n; ++i) {
    const Req& q = t[i]->q;
    const stocha_model m = greeks_model_of(q.r.inst);
    L.models[i] = m;
    L.bumps[i] = q.r.inst.bump_size;
    L.tickets[i] = t[i]->ticket;
    L.kinds[i] = q.r.kind;
    greeks_make_inst(m, q.r.inst.payoff, q.r.inst.strike, q.r.inst.bump_size, q.r.inst.seed,
                     q.r.kind == STOCHA_REQ_PRICE, &inst[i]);
    inst[i].chunk = kChunk;
    inst[i].item_begin = it;
    it += items_of(q);
  }
  L.out_pin = o_part;  // results are staged after the table
  GreeksLaunch g;
  std::memset(&g, 0, sizeof g);
  g.inst = (const GInst*)base;
  g.item_inst = nullptr;  // blocks find their instance from item_begin
  g.total_items = items;
  g.counter = nullptr;
  g.direct = 1;
  g.item_part = (double*)(base + o_part);
  g.inst_sums = (double*)(base + o_sums);
  g.n_inst = (int)n;
  g.tabs = ctx->d_tabs;
  g.err = (unsigned*)(base + o_err);
  cudaError_t e;
  if ((e = cudaMemcpyAsync(base, L.pin, n * sizeof(GInst), cudaMemcpyHostToDevice, L.st)) ||
      (e = cudaMemsetAsync(g.err, 0, sizeof(unsigned), L.st))) {
    fail(L.tickets, STOCHA_ERR_CUDA, std::string("serving: ") + cudaGetErrorString(e));
    return false;
  }
  launch_greeks_batch(g, L.st);
  if ((e = cudaGetLastError()) ||
      (e = cudaMemcpyAsync(L.pin + L.out_pin, g.inst_sums, n * kGreekAcc * 8, cudaMemcpyDeviceToHost, L.st)) ||
      (e = cudaMemcpyAsync(L.pin + L.out_pin + n * kGreekAcc * 8, g.err, sizeof(unsigned), cudaMemcpyDeviceToHost,
                           L.st)) ||
      (e = cudaEventRecord(L.ev, L.st))) {
    fail(L.tickets, STOCHA_ERR_CUDA, std::string("serving: ") + cudaGetErrorString(e));
    return false;
  }
  L.lsmc = false;
  L.off = off;
  L.busy = true;
  return true;
}

bool stocha_server::launch_lsmc(Lane& L, const Pending& p, uint64_t off) {
  const uint64_t ticket = p.ticket;
  const LsmcJob j = lsmc_job(p.q.r);
  size_t pb = 0, sb = 0;
  lsmc_footprint(j, sms, &pb, &sb);
  char* base = slab + off;
  unsigned* err = (unsigned*)(base + pb + Arena::round(sb));
  cudaError_t e;
  if ((e = cudaMemsetAsync(err, 0, sizeof(unsigned), L.st))) {
    fail({ticket}, STOCHA_ERR_CUDA, std::string("serving: ") + cudaGetErrorString(e));
    return false;
  }
  const double* res = nullptr;
  int rc = lsmc_enqueue(j, sms, base, base + pb, ctx->d_tabs, err, true, L.st, L.graphs, &res);
  if (rc) {
    fail({ticket}, rc, stocha_last_error());
    return false;
  }
  L.out_pin = 0;
  if ((e = cudaMemcpyAsync(L.pin, res, 2 * sizeof(double), cudaMemcpyDeviceToHost, L.st)) ||
      (e = cudaMemcpyAsync(L.pin + 16, err, sizeof(unsigned), cudaMemcpyDeviceToHost, L.st)) ||
      (e = cudaEventRecord(L.ev, L.st))) {
    fail({ticket}, STOCHA_ERR_CUDA, std::string("serving: ") + cudaGetErrorString(e));
    return false;
  }
  L.lsmc = true;
  L.lj = j;
  L.tickets = {ticket};
  L.off = off;
  L.busy = true;
  return true;
}

// Finalises the jobs whose launches have completed; true if any did.
bool stocha_server::poll_lanes() {
  bool any = false;
  for (Lane& L : lanes) {
    if (!L.busy) continue;
    const cudaError_t q = cudaEventQuery(L.ev);
    if (q == cudaErrorNotReady) continue;
    any = true;
    L.busy = false;
    arena.release(L.off);
    ++jobs;
    if (q != cudaSuccess) {
      fail(L.tickets, STOCHA_ERR_CUDA, std::string("serving: ") + cudaGetErrorString(q));
      continue;
    }
    std::lock_guard<std::mutex> lk(mu);
    const double now = now_s(t0);
    if (L.lsmc) {
      const double* r2 = (const double*)L.pin;
      const unsigned err = *(const unsigned*)(L.pin + 16);
      stocha_result& res = reqs[L.tickets[0]].res;
      res.t_done = now;
      if (err) {
        res.status = -STOCHA_ERR_DEVICE;
        ++failed;
      } else {
        lsmc_estimate(L.lj, r2, &res.price, &res.std_err);
        res.status = 1;
        ++completed;
      }
    } else {
      const size_t n = L.tickets.size();
      const double* sums = (const double*)(L.pin + L.out_pin);
      const unsigned err = *(const unsigned*)(L.pin + L.out_pin + n * kGreekAcc * 8);
      for (size_t i = 0; i < n; ++i) {
        stocha_result& res = reqs[L.tickets[i]].res;
        res.t_done = now;
        if (err) {
          res.status = -STOCHA_ERR_DEVICE;
          ++failed;
          continue;
        }
        double g[5];
        greeks_from_sums(L.models[i], L.bumps[i], sums + i * kGreekAcc, &res.price, &res.std_err, g);
        for (int j = 0; j < 5; ++j) res.greeks[j] = L.kinds[i] == STOCHA_REQ_GREEKS ? g[j] : 0.0;
        res.status = 1;
        ++completed;
      }
    }
    cv_done.notify_all();
  }
  return any;
}

// Admits pending requests onto free lanes while their bytes fit; true if
// anything was launched.
// Admits the requests of t that were not cancelled: under the lock, so that a
// cancel either comes first (the request is dropped here) or finds it
// admitted.  Stamps their admission time.
std::vector<const Pending*> stocha_server::claim(const std::vector<const Pending*>& t) {
  std::vector<const Pending*> out;
  std::lock_guard<std::mutex> lk(mu);
  const double now = now_s(t0);
  for (const Pending* p : t) {
    Req& r = reqs[p->ticket];
    if (r.phase == kCancelled) continue;
    r.phase = kAdmitted;
    r.res.t_admit = now;
    out.push_back(p);
  }
  return out;
}

bool stocha_server::dispatch() {
  if (pending.empty()) return false;
  bool progress = false;
  {  // requests cancelled while queued leave the queue
    std::lock_guard<std::mutex> lk(mu);
    std::deque<Pending> keep;
    for (Pending& p : pending)
      if (reqs[p.ticket].phase != kCancelled) keep.push_back(p);
    if (keep.size() != pending.size()) {
      pending.swap(keep);
      progress = true;
    }
  }
  if (pending.empty()) return progress;
  auto free_lane = [&](int cls) -> Lane* {
    for (Lane& L : lanes)
      if (!L.busy && L.cls == cls) return &L;
    return nullptr;
  };
  // small work never runs at the lowest priority: it waits for a lane of
  // its own class or the other small class
  auto lane_for = [&](bool small, bool lsmc) -> Lane* {
    // large LSMC jobs are chains of short dependent passes: middle priority
    if (!small) return free_lane(lsmc ? kMid : kLow);
    Lane* L = free_lane(lsmc ? kMid : kHigh);
    return L ? L : free_lane(lsmc ? kHigh : kMid);
  };
  std::vector<bool> taken(pending.size(), false);
  // 1. one batch of the small pricing/Greeks requests (highest priority; a
  //    middle lane if every highest one is busy)
  {
    std::vector<const Pending*> t;
    std::vector<size_t> idx;
    uint64_t items = 0;
    for (size_t i = 0; i < pending.size() && t.size() < kBatchMaxInst; ++i) {
      const Req& q = pending[i].q;
      if (!q.small || q.lsmc) continue;
      const uint64_t k = items_of(q);
      if (items + k > kBatchMaxItems || batch_bytes(t.size() + 1, items + k) > arena.capacity() ||
          batch_pinned(t.size() + 1) > kPinnedBytes)
        break;
      t.push_back(&pending[i]);
      idx.push_back(i);
      items += k;
    }
    Lane* L = t.empty() ? nullptr : lane_for(true, false);
    uint64_t off = 0;
    if (L && arena.alloc(batch_bytes(t.size(), items), &off)) {
      const std::vector<const Pending*> c = claim(t);
      uint64_t citems = 0;
      for (const Pending* p : c) citems += items_of(p->q);
      if (c.empty() || !launch_batch(*L, c, off, citems)) arena.release(off);
      for (size_t i : idx) taken[i] = true;
      batched += c.size();
      progress = true;
    }
  }
  // 2. the rest one job each, in submission order: small LSMC on middle
  //    lanes, large requests on low lanes; a request whose bytes do not fit yet
  //    waits without holding back smaller ones behind it
  for (size_t i = 0; i < pending.size(); ++i) {
    if (taken[i]) continue;
    const Pending& p = pending[i];
    const Req& q = p.q;
    if (q.small && !q.lsmc) continue;  // waits for the next batch
    Lane* L = lane_for(q.small, q.lsmc);
    if (!L) continue;
    uint64_t off = 0;
    if (!arena.alloc(q.bytes, &off)) continue;
    const bool admitted = !claim({&p}).empty();
    const bool ok = admitted && (q.lsmc ? launch_lsmc(*L, p, off) : launch_batch(*L, {&p}, off, items_of(q)));
    if (!ok) arena.release(off);
    taken[i] = true;
    progress = true;
  }
  if (progress) {
    std::deque<Pending> rest;
    for (size_t i = 0; i < pending.size(); ++i)
      if (!taken[i]) rest.push_back(pending[i]);
    pending.swap(rest);
  }
  return progress;
}

void stocha_server::loop() {
  cudaSetDevice(device);
  for (;;) {
    bool busy = false;
    for (Lane& L : lanes) busy |= L.busy;
    {
      std::unique_lock<std::mutex> lk(mu);
      if (!busy && pending.empty() && inbox.empty()) {
        if (stop) break;
        cv_in.wait(lk, [&] { return stop || !inbox.empty(); });
      }
      while (!inbox.empty()) {
        const uint64_t k = inbox.front();
        pending.push_back(Pending{k, reqs[k]});
        inbox.pop_front();
      }
      if (stop && !busy && pending.empty()) break;
    }
    bool progress = poll_lanes();
    progress |= dispatch();
    if (!progress) std::this_thread::yield();
  }
}

extern "C" {

int stocha_server_create(int32_t device, uint64_t budget_bytes, int32_t lanes, stocha_server** out) {
  if (!out) return set_error(STOCHA_ERR_VALUE, "out must not be NULL");
  *out = nullptr;
  if (lanes < 3 || lanes > 64) return set_error(STOCHA_ERR_VALUE, "lanes must be in [3, 64]");
  if (budget_bytes < (1u << 20)) return set_error(STOCHA_ERR_VALUE, "budget_bytes must be at least 1 MiB");
  stocha_server* s = new stocha_server();
  s->device = device;
  s->t0 = std::chrono::steady_clock::now();
  int rc = stocha_ctx_create(device, &s->ctx);
  if (rc) {
    delete s;
    return rc;
  }
  cudaSetDevice(device);
  cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, device);
  cudaError_t e = cudaMalloc((void**)&s->slab, budget_bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    stocha_ctx_destroy(s->ctx);
    delete s;
    return set_error(STOCHA_ERR_NOMEM, "device allocation of the serving budget (" + std::to_string(budget_bytes) +
                                           " bytes) failed: " + cudaGetErrorString(e));
  }
  s->arena = Arena(budget_bytes);
  int lo = 0, hi = 0;
  cudaDeviceGetStreamPriorityRange(&lo, &hi);  // hi: numerically smallest = highest priority
  const int prio[3] = {hi, (lo + hi) / 2, lo};
  s->lanes.resize(lanes);
  // small batches finish in well under a millisecond: few lanes; LSMC jobs
  // are longer chains; large pricing/Greeks jobs need the most lanes
  const int n_high = std::max(1, lanes / 8), n_mid = std::max(1, lanes / 4);
  for (int i = 0; i < lanes; ++i) {
    Lane& L = s->lanes[i];
    L.cls = i < n_high ? kHigh : i < n_high + n_mid ? kMid : kLow;
    if ((e = cudaStreamCreateWithPriority(&L.st, cudaStreamNonBlocking, prio[L.cls])) ||
        (e = cudaEventCreateWithFlags(&L.ev, cudaEventDisableTiming)) ||
        (e = cudaMallocHost((void**)&L.pin, kPinnedBytes)) || (e = lsmc_graphs_create(&L.graphs))) {
      cudaGetLastError();
      stocha_server_destroy(s);
      return set_error(STOCHA_ERR_CUDA, std::string("serving lanes: ") + cudaGetErrorString(e));
    }
  }
  s->thread = std::thread([s] { s->loop(); });
  *out = s;
  return STOCHA_OK;
}

int stocha_server_destroy(stocha_server* s) {
  if (!s) return STOCHA_OK;
  if (s->thread.joinable()) {
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
    }
    s->cv_in.notify_all();
    s->thread.join();
  }
  cudaSetDevice(s->device);
  for (Lane& L : s->lanes) {
    if (L.st) cudaStreamSynchronize(L.st);
    if (L.ev) cudaEventDestroy(L.ev);
    if (L.st) cudaStreamDestroy(L.st);
    if (L.pin) cudaFreeHost(L.pin);
    lsmc_graphs_release(L.graphs);
  }
  if (s->slab) cudaFree(s->slab);
  if (s->ctx) stocha_ctx_destroy(s->ctx);
  delete s;
  return STOCHA_OK;
}

int stocha_server_submit(stocha_server* s, const stocha_request* req, uint64_t* ticket) {
  if (!s || !req || !ticket) return set_error(STOCHA_ERR_VALUE, "server, request and ticket must not be NULL");
  int rc = validate(*req);
  if (rc) return rc;
  Req q;
  q.r = *req;
  std::memset(&q.res, 0, sizeof q.res);
  q.lsmc = req->kind == STOCHA_REQ_LSMC;
  q.small = req->inst.n_paths <= kSmallPaths;
  if (q.lsmc) {
    size_t pb = 0, sb = 0;
    lsmc_footprint(lsmc_job(*req), s->sms, &pb, &sb);
    q.bytes = pb + Arena::round(sb) + 256;
  } else {
    q.bytes = batch_bytes(1, items_of(q));
  }
  if (q.bytes > s->arena.capacity())
    return set_error(STOCHA_ERR_NOMEM, "request needs " + std::to_string(q.bytes) +
                                           " bytes of device memory; the serving budget is " +
                                           std::to_string(s->arena.capacity()));
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return set_error(STOCHA_ERR_VALUE, "server is stopping");
    q.res.t_submit = now_s(s->t0);
    *ticket = s->reqs.size();
    s->reqs.push_back(q);
    s->inbox.push_back(*ticket);
  }
  s->cv_in.notify_one();
  return STOCHA_OK;
}

int stocha_server_poll(stocha_server* s, uint64_t ticket, stocha_result* out) {
  if (!s || !out) return set_error(STOCHA_ERR_VALUE, "server and out must not be NULL");
  std::lock_guard<std::mutex> lk(s->mu);
  if (ticket >= s->reqs.size()) return set_error(STOCHA_ERR_VALUE, "unknown ticket");
  *out = s->reqs[ticket].res;
  return STOCHA_OK;
}

int stocha_server_cancel(stocha_server* s, uint64_t ticket, int32_t* cancelled) {
  if (!s || !cancelled) return set_error(STOCHA_ERR_VALUE, "server and cancelled must not be NULL");
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (ticket >= s->reqs.size()) return set_error(STOCHA_ERR_VALUE, "unknown ticket");
    Req& r = s->reqs[ticket];
    if (r.phase == kAdmitted) {
      *cancelled = 0;  // on a lane or done: it runs to completion
      return STOCHA_OK;
    }
    *cancelled = 1;
    if (r.phase == kCancelled) return STOCHA_OK;
    r.phase = kCancelled;
    r.res.status = -STOCHA_ERR_CANCELLED;
    r.res.t_done = now_s(s->t0);
    ++s->cancelled;
  }
  s->cv_done.notify_all();
  s->cv_in.notify_one();  // the dispatcher drops it from its queue
  return STOCHA_OK;
}

int stocha_server_wait(stocha_server* s, uint64_t ticket, double timeout_s, stocha_result* out) {
  if (!s || !out) return set_error(STOCHA_ERR_VALUE, "server and out must not be NULL");
  std::unique_lock<std::mutex> lk(s->mu);
  if (ticket >= s->reqs.size()) return set_error(STOCHA_ERR_VALUE, "unknown ticket");
  auto done = [&] { return s->reqs[ticket].res.status != 0; };
  if (timeout_s < 0) {
    s->cv_done.wait(lk, done);
  } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) {
    *out = s->reqs[ticket].res;
    return set_error(STOCHA_ERR_TIMEOUT, "request not finished within the timeout");
  }
  *out = s->reqs[ticket].res;
  return STOCHA_OK;
}

int stocha_server_replay(stocha_server* s, const stocha_request* reqs, const double* arrival_s, uint64_t n,
                         stocha_result* out) {
  if (!s || (n && (!reqs || !arrival_s || !out)))
    return set_error(STOCHA_ERR_VALUE, "server, requests, arrivals and out must not be NULL");
  for (uint64_t i = 0; i < n; ++i) {
    int rc = validate(reqs[i]);
    if (rc) return set_error(rc, "request " + std::to_string(i) + ": " + stocha_last_error());
  }
  std::vector<uint64_t> tickets(n);
  const auto t0 = std::chrono::steady_clock::now();
  for (uint64_t i = 0; i < n; ++i) {
    const auto due = t0 + std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                              std::chrono::duration<double>(arrival_s[i]));
    for (;;) {  // sleep until shortly before the arrival, then yield to it
      const auto left = due - std::chrono::steady_clock::now();
      if (left <= std::chrono::steady_clock::duration::zero()) break;
      if (left > std::chrono::microseconds(300))
        std::this_thread::sleep_for(left - std::chrono::microseconds(200));
      else
        std::this_thread::yield();
    }
    int rc = stocha_server_submit(s, &reqs[i], &tickets[i]);
    if (rc) return rc;
  }
  for (uint64_t i = 0; i < n; ++i) {
    int rc = stocha_server_wait(s, tickets[i], -1.0, &out[i]);
    if (rc) return rc;
  }
  return STOCHA_OK;
}

int stocha_server_stats(stocha_server* s, stocha_server_counters* out) {
  if (!s || !out) return set_error(STOCHA_ERR_VALUE, "server and out must not be NULL");
  std::memset(out, 0, sizeof *out);
  std::lock_guard<std::mutex> lk(s->mu);
  out->submitted = s->reqs.size();
  out->completed = s->completed;
  out->failed = s->failed;
  out->cancelled = s->cancelled;
  out->jobs = s->jobs;
  out->batched_requests = s->batched;
  out->budget_bytes = s->arena.capacity();
  out->peak_bytes = s->arena.peak();
  out->in_use_bytes = s->arena.used();
  out->lanes = (int32_t)s->lanes.size();
  int h = 0;
  for (const Lane& L : s->lanes) h += L.cls != kLow;
  out->high_lanes = h;
  return STOCHA_OK;
}

// Diagnostic: runs the arena on a host-only script.  ops[i] > 0: allocate
// that many bytes (offset or -1 into res[i]); ops[i] <= 0: release the block
// of allocation number -ops[i] (res[i] = 0).  res[n] = used, res[n+1] = peak,
// res[n+2] = largest free block, res[n+3] = number of free blocks.
int stocha_debug_arena(uint64_t capacity, const int64_t* ops, uint64_t n, int64_t* res) {
  Arena a(capacity);
  std::vector<uint64_t> offs(n, 0);
  for (uint64_t i = 0; i < n; ++i) {
    if (ops[i] > 0) {
      uint64_t off = 0;
      if (a.alloc((uint64_t)ops[i], &off)) {
        offs[i] = off;
        res[i] = (int64_t)off;
      } else {
        res[i] = -1;
      }
    } else {
      const uint64_t k = (uint64_t)(-ops[i]);
      if (k < i && res[k] >= 0 && ops[k] > 0) a.release(offs[k]);
      res[i] = 0;
    }
  }
  res[n] = (int64_t)a.used();
  res[n + 1] = (int64_t)a.peak();
  res[n + 2] = (int64_t)a.largest_free();
  res[n + 3] = (int64_t)a.free_blocks();
  return STOCHA_OK;
}

}  // extern "C"

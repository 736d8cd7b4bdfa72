// Device -> host delivery of large results into pageable memory (the NumPy
// arrays the reference's functions return).
//
// On a Grace host, a copy into host pages that already exist runs at the
// chip-to-chip link's rate (~190 GB/s measured on GB300, the same as pinned
// memory), but fresh memory is untouched virtual memory: the first write to
// each page faults it in and the kernel zero-fills it, which a
// single-threaded copy does at ~30 GB/s.  Two remedies:
//   * the result cache (stocha_host_buffer_acquire/release) keeps released
//     result buffers, whose pages exist, for later results of a similar size;
//   * into fresh memory, the destination's pages are populated by a small
//     pool of host threads (one write per page) and the copy is issued chunk
//     by chunk as chunks become ready.
// A cached buffer is also registered with the driver (cudaHostRegister) when
// it is first reused.  Copies into unregistered pageable memory pin its pages
// on the fly, and the driver drops those pins now and then: measured on
// GB300, one copy of a 6 GB result in five or six took 165-255 ms instead of
// 34 ms.  Registered once, the buffer keeps its pins while it stays cached.
#include <atomic>
#include <condition_variable>
#include <cstdlib>
#include <deque>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include <sys/mman.h>
#include <unistd.h>

#include "host_common.h"

namespace stocha {
namespace {

constexpr size_t kChunk = 8u << 20;          // bytes per copy
constexpr size_t kParallelMin = 16u << 20;   // below this: one plain copy

// Fixed set of worker threads; run() hands every worker the same task and
// wait() blocks until all have returned.  One task at a time (guarded by
// the caller's lock on `use`).
class HostPool {
 public:
  static HostPool& get() {
    static HostPool p;
    return p;
  }
  int size() const { return (int)threads_.size(); }
  std::mutex use;

  void run(std::function<void(int)> fn) {
    std::lock_guard<std::mutex> lk(mu_);
    task_ = std::move(fn);
    pending_ = (int)threads_.size();
    ++gen_;
    cv_.notify_all();
  }
  void wait() {
    std::unique_lock<std::mutex> lk(mu_);
    done_.wait(lk, [&] { return pending_ == 0; });
  }

 private:
  HostPool() {
    unsigned hw = std::thread::hardware_concurrency();
    int n = (int)(hw / 2);
    if (n < 2) n = 2;
    if (n > 8) n = 8;
    for (int i = 0; i < n; ++i) threads_.emplace_back([this, i] { loop(i); });
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
      ++gen_;
    }
    cv_.notify_all();
    for (auto& t : threads_) t.join();
  }
  void loop(int idx) {
    uint64_t seen = 0;
    for (;;) {
      std::function<void(int)> fn;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
        if (stop_) return;
        fn = task_;
      }
      fn(idx);
      std::lock_guard<std::mutex> lk(mu_);
      if (--pending_ == 0) done_.notify_all();
    }
  }
  std::vector<std::thread> threads_;
  std::mutex mu_;
  std::condition_variable cv_, done_;
  std::function<void(int)> task_;
  uint64_t gen_ = 0;
  int pending_ = 0;
  bool stop_ = false;
};

// Released result buffers, kept mapped (their pages exist) for reuse.
class HostCache {
 public:
  static HostCache& get() {
    static HostCache c;
    return c;
  }

  void* acquire(size_t bytes) {
    const size_t want = round_up(bytes ? bytes : 1);
    {
      std::lock_guard<std::mutex> lk(mu_);
      // best fit among the cached buffers of capacity want .. want * 5/4
      size_t best = free_.size();
      for (size_t i = 0; i < free_.size(); ++i) {
        const size_t c = free_[i].cap;
        if (c >= want && c - want <= want / 4 && (best == free_.size() || c < free_[best].cap)) best = i;
      }
      if (best != free_.size()) {
        const Buf b = free_[best];
        free_.erase(free_.begin() + (std::ptrdiff_t)best);
        cached_ -= b.cap;
        live_[b.p] = Live{b.cap, true, b.registered};
        return b.p;
      }
    }
    void* p = mmap(nullptr, want, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    if (p == MAP_FAILED) return nullptr;
    std::lock_guard<std::mutex> lk(mu_);
    live_[p] = Live{want, false, false};
    return p;
  }

  // false: not a buffer from acquire (or released twice)
  bool release(void* p) {
    std::vector<Buf> drop;
    {
      std::lock_guard<std::mutex> lk(mu_);
      auto it = live_.find(p);
      if (it == live_.end()) return false;
      const Buf b{p, it->second.cap, it->second.registered};
      const bool keep = it->second.populated && b.cap <= cap_;
      live_.erase(it);
      if (keep) {
        free_.push_back(b);
        cached_ += b.cap;
        while (cached_ > cap_) {  // the oldest go first
          drop.push_back(free_.front());
          cached_ -= free_.front().cap;
          free_.pop_front();
        }
      } else {
        drop.push_back(b);
      }
    }
    for (const Buf& b : drop) {
      if (b.registered) cudaHostUnregister(b.p);
      munmap(b.p, b.cap);
    }
    return true;
  }

  // Registers [dst, dst + cap) with the driver if dst is a handed-out buffer
  // whose pages exist and that is not registered yet; true when it is
  // registered afterwards.
  bool register_populated(const void* dst) {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = live_.find(const_cast<void*>(dst));
    if (it == live_.end() || !it->second.populated) return false;
    if (!it->second.registered) {
      if (cudaHostRegister(it->first, it->second.cap, cudaHostRegisterPortable) != cudaSuccess) {
        cudaGetLastError();  // not fatal: the copy still works into pageable memory
        return false;
      }
      it->second.registered = true;
    }
    return true;
  }

  // Whether [dst, dst + bytes) lies in a handed-out buffer whose pages exist.
  bool populated(const void* dst, size_t bytes) {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = live_.find(const_cast<void*>(dst));
    return it != live_.end() && it->second.populated && bytes <= it->second.cap;
  }
  void mark_populated(const void* dst, size_t bytes) {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = live_.find(const_cast<void*>(dst));
    if (it != live_.end() && round_up(bytes) >= it->second.cap) it->second.populated = true;
  }
  void stats(size_t* cached, size_t* cap) {
    std::lock_guard<std::mutex> lk(mu_);
    if (cached) *cached = cached_;
    if (cap) *cap = cap_;
  }

 private:
  struct Buf {
    void* p;
    size_t cap;
    bool registered;
  };
  struct Live {
    size_t cap;
    bool populated;
    bool registered;  // cudaHostRegister'ed (pins kept while cached)
  };
  HostCache() {
    page_ = (size_t)sysconf(_SC_PAGESIZE);
    const char* env = std::getenv("STOCHA_HOST_CACHE_BYTES");
    if (env && *env) {
      cap_ = (size_t)std::strtoull(env, nullptr, 10);
    } else {
      const size_t phys = (size_t)sysconf(_SC_PHYS_PAGES) * page_;
      cap_ = phys / 8;
      if (cap_ > (64ull << 30)) cap_ = 64ull << 30;
    }
  }
  size_t round_up(size_t n) const { return (n + page_ - 1) / page_ * page_; }

  std::mutex mu_;
  std::deque<Buf> free_;
  std::unordered_map<void*, Live> live_;
  size_t cached_ = 0, cap_ = 0, page_ = 4096;
};

}  // namespace

bool host_dst_cached(const void* dst, size_t bytes) {
  HostCache& c = HostCache::get();
  if (!c.populated(dst, bytes)) return false;
  c.register_populated(dst);
  return true;
}

int copy_to_host_populated(cudaStream_t st, void* dst, const void* src, size_t bytes) {
  HostCache& cache = HostCache::get();
  if (bytes < kParallelMin || cache.populated(dst, bytes)) {
    if (bytes >= kParallelMin) cache.register_populated(dst);
    STOCHA_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
    cache.mark_populated(dst, bytes);
    return STOCHA_OK;
  }
  HostPool& pool = HostPool::get();
  std::lock_guard<std::mutex> use(pool.use);
  const size_t page = (size_t)sysconf(_SC_PAGESIZE);
  const size_t nch = (bytes + kChunk - 1) / kChunk;
  std::unique_ptr<std::atomic<int>[]> ready(new std::atomic<int>[nch]);
  for (size_t i = 0; i < nch; ++i) ready[i].store(0, std::memory_order_relaxed);
  std::atomic<size_t> next{0};
  char* d = (char*)dst;
  pool.run([&](int) {
    for (;;) {
      const size_t i = next.fetch_add(1);
      if (i >= nch) return;
      const size_t a = i * kChunk, b = a + kChunk < bytes ? a + kChunk : bytes;
      // one write per page (the bytes are overwritten by the copy)
      volatile char* p = d;
      for (size_t o = a; o < b; o = (o / page + 1) * page) p[o] = 0;
      ready[i].store(1, std::memory_order_release);
    }
  });
  int rc = STOCHA_OK;
  for (size_t i = 0; i < nch && rc == STOCHA_OK; ++i) {
    while (!ready[i].load(std::memory_order_acquire)) std::this_thread::yield();
    const size_t a = i * kChunk, len = (a + kChunk < bytes ? kChunk : bytes - a);
    const cudaError_t e = cudaMemcpyAsync(d + a, (const char*)src + a, len, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) rc = cuda_error(e, "cudaMemcpyAsync (device to host)");
  }
  pool.wait();  // the task's captures live on this frame
  if (rc == STOCHA_OK) cache.mark_populated(dst, bytes);
  return rc;
}

}  // namespace stocha

extern "C" {

int stocha_host_buffer_acquire(size_t bytes, void** out) {
  if (!out) return stocha::set_error(STOCHA_ERR_VALUE, "out must not be NULL");
  *out = stocha::HostCache::get().acquire(bytes);
  if (!*out) return stocha::set_error(STOCHA_ERR_NOMEM, "host buffer allocation failed");
  return STOCHA_OK;
}

int stocha_host_buffer_release(void* ptr) {
  if (!stocha::HostCache::get().release(ptr))
    return stocha::set_error(STOCHA_ERR_VALUE, "not a buffer from stocha_host_buffer_acquire");
  return STOCHA_OK;
}

int stocha_host_cache_stats(size_t* cached_bytes, size_t* cap_bytes) {
  stocha::HostCache::get().stats(cached_bytes, cap_bytes);
  return STOCHA_OK;
}

}  // extern "C"

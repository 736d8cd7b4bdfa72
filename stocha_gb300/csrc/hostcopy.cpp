// Device -> host delivery of large results into fresh pageable memory (the
// NumPy arrays the reference's functions return).
//
// On a Grace host, a copy into host pages that already exist runs at the
// chip-to-chip link's rate (~170 GB/s measured on GB300), but NumPy hands us
// untouched virtual memory: the first write to each page faults it in and the
// kernel zero-fills it, which a single-threaded copy does at 10-30 GB/s.  So
// the destination's pages are populated by a small pool of host threads
// (one write per page) while the GPU computes, and the copy is issued chunk
// by chunk as chunks become ready.
#include <atomic>
#include <condition_variable>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

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

}  // namespace

int copy_to_host_populated(cudaStream_t st, void* dst, const void* src, size_t bytes) {
  if (bytes < kParallelMin) {
    STOCHA_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
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
  return rc;
}

}  // namespace stocha

// host_pool.h -- a small fixed pool of host threads for independent per-run
// work (a batch's per-run chunk preparation: step records, laser source
// values and the moving-window injection drawn from each run's own KISS
// stream).  run(n, fn) calls fn(i) once for every i in [0, n), on the pool
// and on the calling thread, and returns when all calls have returned.
#pragma once

#include <condition_variable>
#include <cstdint>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace cyl {

class HostPool {
 public:
  explicit HostPool(int nthreads) {
    for (int i = 0; i < nthreads; ++i) threads_.emplace_back([this] { loop(); });
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> lock(mu_);
      quit_ = true;
    }
    cv_.notify_all();
    for (auto& t : threads_) t.join();
  }
  HostPool(const HostPool&) = delete;
  HostPool& operator=(const HostPool&) = delete;

  void run(int n, const std::function<void(int)>& fn) {
    if (threads_.empty() || n <= 1) {
      for (int i = 0; i < n; ++i) fn(i);
      return;
    }
    {
      std::lock_guard<std::mutex> lock(mu_);
      fn_ = &fn;
      n_ = n;
      next_ = 0;
      pending_ = n;
      ++gen_;
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> lock(mu_);
    cv_done_.wait(lock, [&] { return pending_ == 0; });
    fn_ = nullptr;
  }

 private:
  // take items until none is left; a thread that wakes after the call has
  // ended finds fn_ cleared (or the next call's items) and is still correct
  void work() {
    for (;;) {
      int i;
      const std::function<void(int)>* f;
      {
        std::lock_guard<std::mutex> lock(mu_);
        if (!fn_ || next_ >= n_) return;
        i = next_++;
        f = fn_;
      }
      (*f)(i);
      std::lock_guard<std::mutex> lock(mu_);
      if (--pending_ == 0) cv_done_.notify_all();
    }
  }
  void loop() {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lock(mu_);
        cv_.wait(lock, [&] { return quit_ || gen_ != seen; });
        if (quit_) return;
        seen = gen_;
      }
      work();
    }
  }

  std::vector<std::thread> threads_;
  std::mutex mu_;
  std::condition_variable cv_, cv_done_;
  const std::function<void(int)>* fn_ = nullptr;
  int n_ = 0, next_ = 0, pending_ = 0;
  uint64_t gen_ = 0;
  bool quit_ = false;
};

}  // namespace cyl

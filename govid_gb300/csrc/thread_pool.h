// A fixed worker pool for host-side fan-out (tile encoding, packet planning).
// run(count, fn) hands out indices 0..count-1 and blocks until every call has
// returned; a single item runs inline on the caller, as ebiv/pool.go:58-72
// does for the untiled frame.
#pragma once

#include <condition_variable>
#include <cstdint>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace ebiv {

class WorkerPool {
 public:
  explicit WorkerPool(int n) {
    for (int i = 0; i < n; i++) workers_.emplace_back([this] { loop(); });
  }
  ~WorkerPool() {
    {
      std::lock_guard<std::mutex> g(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
  }
  WorkerPool(const WorkerPool&) = delete;
  WorkerPool& operator=(const WorkerPool&) = delete;

  int size() const { return (int)workers_.size(); }

  void run(int count, const std::function<void(int)>& fn) {
    if (count <= 0) return;
    if (count == 1 || workers_.empty()) {
      for (int i = 0; i < count; i++) fn(i);
      return;
    }
    std::unique_lock<std::mutex> lk(mu_);
    job_ = &fn;
    next_ = 0;
    count_ = count;
    done_ = 0;
    gen_++;
    cv_.notify_all();
    done_cv_.wait(lk, [&] { return done_ == count_; });
    job_ = nullptr;
  }

 private:
  void loop() {
    uint64_t seen = 0;
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
      cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
      if (stop_) return;
      seen = gen_;
      while (job_ && next_ < count_) {
        const int i = next_++;
        const std::function<void(int)>* f = job_;
        lk.unlock();
        (*f)(i);
        lk.lock();
        if (++done_ == count_) done_cv_.notify_all();
      }
    }
  }

  std::vector<std::thread> workers_;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(int)>* job_ = nullptr;
  int next_ = 0, count_ = 0, done_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

}  // namespace ebiv

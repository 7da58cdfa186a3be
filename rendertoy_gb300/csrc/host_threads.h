// host_threads.h — a small thread pool for the library's host work (the BVH
// builder, the batch scene builds).
#pragma once
#include <atomic>
#include <cstddef>
#include <exception>
#include <mutex>
#include <system_error>
#include <thread>
#include <vector>

namespace rtx {

// Runs fn(k) for k = 0 .. n-1 on up to n_threads threads, the calling thread
// among them (it takes whatever threads that could not be started leave).
// An exception (an allocation that failed) stops the remaining work and is
// rethrown on the calling thread once every thread has joined.
template <class F>
void run_parallel(size_t n, unsigned n_threads, F&& fn) {
  std::atomic<size_t> next{0};
  std::exception_ptr err;
  std::mutex mu;
  auto work = [&] {
    try {
      for (size_t k; (k = next.fetch_add(1)) < n;) fn(k);
    } catch (...) {
      next = n;
      std::lock_guard<std::mutex> lock(mu);
      if (!err) err = std::current_exception();
    }
  };
  std::vector<std::thread> pool;
  for (unsigned t = 1; t < n_threads && t < n; ++t) {
    try {
      pool.emplace_back(work);
    } catch (const std::system_error&) {
      break;
    }
  }
  work();
  for (auto& th : pool) th.join();
  if (err) std::rethrow_exception(err);
}

}  // namespace rtx

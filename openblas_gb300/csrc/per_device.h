// One-time setup per CUDA device, shared by every host thread.
//
// Kernel attributes (the dynamic shared-memory limit, non-portable cluster
// sizes) and occupancy figures belong to a device, and several host threads
// may reach the first launch on a device at the same time.  PerDeviceOnce
// runs a setup step once per device ordinal under a lock and publishes its
// completion with release/acquire ordering, so no thread goes on before the
// step has finished.  PerDeviceValue caches a value computed the same way.
// This header needs no CUDA headers: the caller passes the ordinal.
#pragma once

#include <stdint.h>

#include <atomic>
#include <mutex>

namespace gb {

class PerDeviceOnce {
 public:
  static constexpr int kMaxDevices = 64;

  // Runs `step` (which returns 0 on success) unless it has already
  // succeeded for `dev`.  A failed step is tried again by the next caller.
  // Ordinals outside 0..63 run the step on every call.
  template <typename F>
  int run(int dev, F &&step) {
    if (dev < 0 || dev >= kMaxDevices) return step();
    const uint64_t bit = 1ull << dev;
    if (done_.load(std::memory_order_acquire) & bit) return 0;
    std::lock_guard<std::mutex> lk(mu_);
    if (done_.load(std::memory_order_relaxed) & bit) return 0;
    const int st = step();
    if (st == 0) done_.fetch_or(bit, std::memory_order_release);
    return st;
  }

 private:
  std::atomic<uint64_t> done_{0};
  std::mutex mu_;
};

template <typename T>
class PerDeviceValue {
 public:
  // The value that `compute()` returned the first time it ran for `dev`.
  template <typename F>
  T get(int dev, F &&compute) {
    if (dev < 0 || dev >= PerDeviceOnce::kMaxDevices) return compute();
    once_.run(dev, [&] {
      vals_[dev] = compute();
      return 0;
    });
    return vals_[dev];  // written before the release that run() observed or made
  }

 private:
  PerDeviceOnce once_;
  T vals_[PerDeviceOnce::kMaxDevices] = {};
};

}  // namespace gb

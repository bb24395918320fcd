// rvh_optin.hpp — which kernels have been opted into large dynamic shared
// memory, per device.  cudaFuncSetAttribute applies to the current device's
// context only, so one process that drives several GPUs must opt each kernel
// in once on every device it launches on: the record is keyed by (device,
// kernel).  Host-only C++ (tests/test_abi.py compiles it alone with g++).
#pragma once

#include <mutex>
#include <set>
#include <utility>

namespace rvh {

class OptInRecord {
public:
    // Runs opt_in() unless (dev, fn) is already recorded; records it when
    // opt_in() succeeds.  Returns whether (dev, fn) is opted in afterwards.
    template <class F>
    bool ensure(int dev, const void* fn, F&& opt_in) {
        std::lock_guard<std::mutex> g(mu_);
        const std::pair<int, const void*> key{dev, fn};
        if (done_.count(key)) return true;
        if (!opt_in()) return false;
        done_.insert(key);
        return true;
    }
    size_t size() {
        std::lock_guard<std::mutex> g(mu_);
        return done_.size();
    }

private:
    std::mutex mu_;
    std::set<std::pair<int, const void*>> done_;
};

}  // namespace rvh

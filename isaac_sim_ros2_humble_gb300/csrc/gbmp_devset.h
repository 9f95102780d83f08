// gbmp_devset.h -- set of (device, kernel) pairs, for once-per-device kernel set-up.
//
// Kernel attributes such as the dynamic shared-memory limit belong to a function on one
// device: a kernel configured while device 0 was current is not configured on device 1.
// The library records which pairs it has configured so that every (device, kernel)
// pair is configured once, from whichever host thread gets there first.  Plain C++ (no
// CUDA types), so that the keying can be tested on a machine without a GPU.
#pragma once

#include <mutex>
#include <set>
#include <utility>

namespace gbmp {

class DeviceKernelSet {
  public:
    bool contains(int device, const void *fn) {
        std::lock_guard<std::mutex> lock(mu_);
        return set_.count(std::make_pair(device, fn)) != 0;
    }
    // Returns true when the pair was not recorded before.
    bool insert(int device, const void *fn) {
        std::lock_guard<std::mutex> lock(mu_);
        return set_.insert(std::make_pair(device, fn)).second;
    }
    size_t size() {
        std::lock_guard<std::mutex> lock(mu_);
        return set_.size();
    }

  private:
    std::mutex mu_;
    std::set<std::pair<int, const void *>> set_;
};

}  // namespace gbmp

// ledger.h -- device-memory accounting of one context (plain C++, no CUDA).
//
// Every device buffer a context allocates -- its tables, the CRS and Galois
// key tables, resident databases, per-client key tables, serving-loop slots
// and staging buffers -- reserves its bytes here before cudaMalloc and
// returns them when freed.  With a budget set, a reservation that would
// exceed it is refused, so the caller fails with INSPIRE_ERR_OUT_OF_MEMORY
// before the device runs out (admission by device memory).  Buffers that
// outlive the context (a database destroyed after it) keep the ledger alive
// through shared ownership.
#pragma once
#include <cstdint>
#include <mutex>

namespace ighost {

class Ledger {
 public:
  // Reserve `bytes`; false, with nothing reserved, if the budget would be exceeded.
  bool reserve(uint64_t bytes) {
    std::lock_guard<std::mutex> lk(m_);
    if (budget_ && (bytes > budget_ || used_ > budget_ - bytes)) return false;
    used_ += bytes;
    return true;
  }
  void release(uint64_t bytes) {
    std::lock_guard<std::mutex> lk(m_);
    used_ = bytes > used_ ? 0 : used_ - bytes;
  }
  // 0: no limit.  A budget below the bytes already reserved is refused.
  bool set_budget(uint64_t budget) {
    std::lock_guard<std::mutex> lk(m_);
    if (budget && budget < used_) return false;
    budget_ = budget;
    return true;
  }
  uint64_t used() const {
    std::lock_guard<std::mutex> lk(m_);
    return used_;
  }
  uint64_t budget() const {
    std::lock_guard<std::mutex> lk(m_);
    return budget_;
  }

 private:
  mutable std::mutex m_;
  uint64_t used_ = 0, budget_ = 0;
};

}  // namespace ighost

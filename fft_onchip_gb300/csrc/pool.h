// fftoc — byte-range allocator for the serving loop's fixed device pool.
//
// Host-only bookkeeping over [0, capacity): first-fit allocation of aligned
// ranges, frees in any order, adjacent free ranges coalesced.  The server
// admits a request only when its bytes fit in one free range, so device
// memory use never exceeds the pool it allocated at start-up.
#pragma once
#include <cstdint>
#include <iterator>
#include <map>

namespace fftoc {

class RangePool {
 public:
  explicit RangePool(int64_t capacity, int64_t align = 256) : cap_(capacity), align_(align) {
    if (capacity > 0) free_[0] = capacity;
  }

  // Offset of a free range of `bytes` (rounded up to the alignment), or -1.
  int64_t alloc(int64_t bytes) {
    if (bytes <= 0) return -1;
    const int64_t need = (bytes + align_ - 1) / align_ * align_;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < need) continue;
      const int64_t off = it->first, len = it->second;
      free_.erase(it);
      if (len > need) free_[off + need] = len - need;
      used_ += need;
      live_[off] = need;
      return off;
    }
    return -1;
  }

  // Return a range obtained from alloc(); false if `off` is not live.
  bool release(int64_t off) {
    auto l = live_.find(off);
    if (l == live_.end()) return false;
    int64_t start = off, len = l->second;
    live_.erase(l);
    used_ -= len;
    auto next = free_.lower_bound(start);
    if (next != free_.end() && next->first == start + len) {
      len += next->second;
      next = free_.erase(next);
    }
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == start) {
        prev->second += len;
        return true;
      }
    }
    free_[start] = len;
    return true;
  }

  int64_t capacity() const { return cap_; }
  int64_t used() const { return used_; }
  int64_t largest_free() const {
    int64_t m = 0;
    for (const auto& f : free_) m = f.second > m ? f.second : m;
    return m;
  }
  size_t free_ranges() const { return free_.size(); }
  size_t live_ranges() const { return live_.size(); }

 private:
  int64_t cap_, align_;
  int64_t used_ = 0;
  std::map<int64_t, int64_t> free_;  // offset -> length
  std::map<int64_t, int64_t> live_;  // offset -> length
};

}  // namespace fftoc

// First-fit range allocator over [0, capacity) with coalescing free list.
// Pure host code (offsets only), used to carve the server's HBM arena.
#pragma once
#include <cstddef>
#include <cstdint>
#include <iterator>
#include <map>

namespace yell_gb300 {

class RangeAllocator {
 public:
  static constexpr size_t kAlign = 256;

  explicit RangeAllocator(size_t capacity = 0) { reset(capacity); }

  void reset(size_t capacity) {
    capacity_ = capacity - capacity % kAlign;
    free_.clear();
    if (capacity_) free_[0] = capacity_;
    in_use_ = peak_ = 0;
  }

  static size_t round(size_t bytes) { return (bytes + kAlign - 1) / kAlign * kAlign; }

  // First fit; false when no free range is large enough.
  bool alloc(size_t bytes, size_t* off) {
    const size_t need = round(bytes ? bytes : 1);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= need) {
        *off = it->first;
        const size_t rest = it->second - need;
        const size_t start = it->first + need;
        free_.erase(it);
        if (rest) free_[start] = rest;
        in_use_ += need;
        if (in_use_ > peak_) peak_ = in_use_;
        return true;
      }
    }
    return false;
  }

  void free(size_t off, size_t bytes) {
    const size_t len = round(bytes ? bytes : 1);
    in_use_ -= len;
    auto next = free_.lower_bound(off);
    size_t start = off, size = len;
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == off) {
        start = prev->first;
        size += prev->second;
        free_.erase(prev);
      }
    }
    if (next != free_.end() && off + len == next->first) {
      size += next->second;
      free_.erase(next);
    }
    free_[start] = size;
  }

  size_t capacity() const { return capacity_; }
  size_t in_use() const { return in_use_; }
  size_t peak() const { return peak_; }
  size_t free_ranges() const { return free_.size(); }
  size_t largest_free() const {
    size_t m = 0;
    for (const auto& kv : free_) m = kv.second > m ? kv.second : m;
    return m;
  }

 private:
  size_t capacity_ = 0, in_use_ = 0, peak_ = 0;
  std::map<size_t, size_t> free_;
};

}  // namespace yell_gb300

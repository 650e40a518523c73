// pn_arena.h -- best-fit sub-allocator over one device range (host bookkeeping only).
//
// The server takes its whole memory budget with one cudaMalloc when it starts and hands pieces
// of it to the waves it admits.  Giving a piece back is a host operation: no cudaFree, so a
// finishing wave never synchronises the device while other waves are still running.  A piece
// is returned only after the host has seen the wave that used it complete.
#pragma once

#include <cstddef>
#include <map>
#include <mutex>
#include <unordered_map>

namespace pn {

class Arena {
 public:
  static constexpr size_t kAlign = 256;

  Arena(char* base, size_t size) : base_(base), size_(size & ~(kAlign - 1)) {
    if (size_ > 0) insert_free(0, size_);
  }

  // nullptr when no free range is large enough
  void* alloc(size_t bytes) {
    const size_t b = round_up(bytes == 0 ? 1 : bytes);
    std::lock_guard<std::mutex> lk(mu_);
    auto it = by_size_.lower_bound(b);
    if (it == by_size_.end()) return nullptr;
    const size_t sz = it->first, off = it->second;
    erase_free(off, sz);
    if (sz > b) insert_free(off + b, sz - b);
    live_[off] = b;
    used_ += b;
    if (used_ > peak_) peak_ = used_;
    return base_ + off;
  }

  // false when p was not handed out by this arena (or was returned already)
  bool free(void* p) {
    if (!p) return true;
    std::lock_guard<std::mutex> lk(mu_);
    const size_t off = (size_t)((char*)p - base_);
    auto it = live_.find(off);
    if ((char*)p < base_ || it == live_.end()) return false;
    size_t start = off, sz = it->second;
    live_.erase(it);
    used_ -= sz;
    // merge with the free neighbours
    auto nx = free_.lower_bound(off);
    if (nx != free_.end() && nx->first == off + sz) {
      const size_t nsz = nx->second;
      erase_free(nx->first, nsz);
      sz += nsz;
    }
    auto pv = free_.lower_bound(start);
    if (pv != free_.begin()) {
      --pv;
      if (pv->first + pv->second == start) {
        const size_t po = pv->first, psz = pv->second;
        erase_free(po, psz);
        start = po;
        sz += psz;
      }
    }
    insert_free(start, sz);
    return true;
  }

  size_t size() const { return size_; }
  size_t used() const {
    std::lock_guard<std::mutex> lk(mu_);
    return used_;
  }
  size_t peak() const {
    std::lock_guard<std::mutex> lk(mu_);
    return peak_;
  }
  size_t free_bytes() const {
    std::lock_guard<std::mutex> lk(mu_);
    return size_ - used_;
  }
  size_t largest_free() const {
    std::lock_guard<std::mutex> lk(mu_);
    return by_size_.empty() ? 0 : by_size_.rbegin()->first;
  }
  size_t n_free_ranges() const {
    std::lock_guard<std::mutex> lk(mu_);
    return free_.size();
  }
  static size_t round_up(size_t b) { return (b + kAlign - 1) & ~(kAlign - 1); }

 private:
  void insert_free(size_t off, size_t sz) {
    free_[off] = sz;
    by_size_.emplace(sz, off);
  }
  void erase_free(size_t off, size_t sz) {
    free_.erase(off);
    auto r = by_size_.equal_range(sz);
    for (auto it = r.first; it != r.second; ++it)
      if (it->second == off) {
        by_size_.erase(it);
        break;
      }
  }

  char* base_;
  size_t size_;
  mutable std::mutex mu_;
  std::map<size_t, size_t> free_;            // offset -> size
  std::multimap<size_t, size_t> by_size_;    // size -> offset
  std::unordered_map<size_t, size_t> live_;  // offset -> size
  size_t used_ = 0, peak_ = 0;
};

}  // namespace pn

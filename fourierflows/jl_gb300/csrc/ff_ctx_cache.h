// A small thread-safe cache of one device address per CUDA context, keyed by the
// context's unique ID (cuCtxGetId: IDs are never reused within a process).  A device
// reset, or a primary context that is destroyed and re-created, gives the device a new
// context with a new ID, so the next lookup fetches the address again instead of
// returning one that belonged to the old context's module.  Plain C++ (no CUDA), so the
// cache logic is unit-tested on the CPU.
#pragma once

#include <mutex>

namespace ff {

template <int N> class CtxAddressCache {
 public:
  // The address cached for context `id`; on a miss, fetch(&addr) looks it up (returns
  // 0 on success) and the result is cached.  When all N slots are taken, the oldest
  // entry is replaced.
  template <class Fetch> int get(unsigned long long id, void** out, Fetch fetch) {
    std::lock_guard<std::mutex> lk(mu_);
    for (int i = 0; i < n_; ++i)
      if (ids_[i] == id) {
        *out = addr_[i];
        return 0;
      }
    void* p = nullptr;
    const int st = fetch(&p);
    if (st) return st;
    const int slot = n_ < N ? n_++ : (int)(next_++ % N);
    ids_[slot] = id;
    addr_[slot] = p;
    *out = p;
    return 0;
  }

  int size() {
    std::lock_guard<std::mutex> lk(mu_);
    return n_;
  }

 private:
  std::mutex mu_;
  unsigned long long ids_[N] = {};
  void* addr_[N] = {};
  int n_ = 0;
  unsigned next_ = 0;
};

}  // namespace ff

// Randomised check of pn::Arena against a shadow model: alignment, no overlap between live
// ranges, byte accounting, failure only when no free range is large enough, and full
// coalescing back to one range once everything is returned.
#include <cstdio>
#include <cstdlib>
#include <map>
#include <random>
#include <vector>

#include "pn_arena.h"

static int fail(const char* what, long long a, long long b) {
  std::printf("FAIL %s %lld %lld\n", what, a, b);
  return 1;
}

int main() {
  const size_t size = (size_t)64 << 20;
  std::vector<char> backing(size + 256);
  char* base = (char*)(((uintptr_t)backing.data() + 255) & ~(uintptr_t)255);
  pn::Arena a(base, size);
  std::mt19937_64 rng(12345);
  std::map<char*, size_t> live;   // start -> rounded size
  size_t used = 0;
  for (int it = 0; it < 200000; ++it) {
    const bool do_alloc = live.empty() || (rng() % 100) < 55;
    if (do_alloc) {
      size_t want = (rng() % 4 == 0) ? (rng() % (4u << 20)) : (rng() % 4096);
      const size_t largest = a.largest_free();
      char* p = (char*)a.alloc(want);
      const size_t r = pn::Arena::round_up(want == 0 ? 1 : want);
      if (!p) {
        if (r <= largest) return fail("refused although a range fits", (long long)r, (long long)largest);
        continue;
      }
      if (((uintptr_t)p & 255) != 0) return fail("misaligned", (long long)(p - base), 0);
      if (p < base || p + r > base + size) return fail("out of range", (long long)(p - base), (long long)r);
      auto nx = live.lower_bound(p);
      if (nx != live.end() && nx->first < p + r) return fail("overlap (next)", (long long)(p - base), 0);
      if (nx != live.begin()) {
        auto pv = std::prev(nx);
        if (pv->first + pv->second > p) return fail("overlap (prev)", (long long)(p - base), 0);
      }
      live[p] = r;
      used += r;
    } else {
      auto itl = live.begin();
      std::advance(itl, (long)(rng() % live.size()));
      if (!a.free(itl->first)) return fail("free refused", (long long)(itl->first - base), 0);
      used -= itl->second;
      live.erase(itl);
    }
    if (a.used() != used) return fail("used", (long long)a.used(), (long long)used);
  }
  for (auto& kv : live)
    if (!a.free(kv.first)) return fail("final free", 0, 0);
  if (a.used() != 0) return fail("not empty", (long long)a.used(), 0);
  if (a.n_free_ranges() != 1 || a.largest_free() != size) return fail("not coalesced", (long long)a.n_free_ranges(), 0);
  if (a.free(base + 256)) return fail("double free accepted", 0, 0);
  if (a.peak() == 0 || a.peak() > size) return fail("peak", (long long)a.peak(), 0);
  std::printf("ok\n");
  return 0;
}

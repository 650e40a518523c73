// Host-side invariants of the two-threads-per-cell split of the plain path's kernels
// (pn_device.cuh), for every compiled order and class: the lower half starts at moment 0 (which
// carries the intensity partials and the adjoint source), the split sits at a degree boundary, and
// the degree masks of the two halves are disjoint and together the class's mask.  Prints "ok".
#include <cstdio>

#include "generated/pn_orders.h"
#include "pn_device.cuh"

static int failures = 0;

template <int N, int C>
void check_class() {
  constexpr int n = pn::Ord<N>::n(C);
  if constexpr (n > 0) {
    constexpr int ms = pn::split_moment<N, C>();
    constexpr unsigned lo = pn::range_deg_mask<N, C, 0, ms>();
    constexpr unsigned hi = pn::range_deg_mask<N, C, ms, n>();
    bool ok = ms >= 1 && ms <= n;
    if (ms < n) ok = ok && pn::degree_of<N, C>(ms - 1) != pn::degree_of<N, C>(ms);
    ok = ok && (lo & hi) == 0u && (lo | hi) == pn::Ord<N>::deg_mask(C);
    if (!ok) {
      std::printf("N=%d class %d: split %d of %d, masks %x %x\n", N, C, ms, n, lo, hi);
      ++failures;
    }
  }
}

template <int N>
void check_order() {
  check_class<N, 0>(); check_class<N, 1>(); check_class<N, 2>(); check_class<N, 3>();
  check_class<N, 4>(); check_class<N, 5>(); check_class<N, 6>(); check_class<N, 7>();
}

int main() {
#define PN_CHECK(N) check_order<N>();
  PN_FOR_EACH_ORDER(PN_CHECK)
#undef PN_CHECK
  double f = 1.0;
  for (int k = 1; k <= 16; ++k) {
    f *= k;
    if (pn::inv_fact(k) != 1.0 / f) {
      std::printf("inv_fact(%d)\n", k);
      ++failures;
    }
  }
  if (failures == 0) std::printf("ok\n");
  return failures == 0 ? 0 : 1;
}

// pn_order_batch.cu -- instantiates the batched groups for one P_N order (compiled once per order
// with -DPN_ORDER=N, separately from pn_order.cu so the two halves build in parallel).
#include "pn_batch.cuh"

#ifndef PN_ORDER
#error "compile with -DPN_ORDER=<order>"
#endif

#define PN_CAT2(a, b) a##b
#define PN_CAT(a, b) PN_CAT2(a, b)

namespace pn {
// dims: bit mask of the active axes shared by every solve of the group.  FP32 groups of the common
// shapes (x; x,y; x,y,z) get kernels specialised on the mask; the rest check the axes at run time.
BatchGroupBase* PN_CAT(make_batch_group_, PN_ORDER)(int precision, int dims) {
  if (precision == PN_FP32) {
    switch (dims) {
      case 1: return new BatchGroup<float, PN_ORDER, 1>();
      case 3: return new BatchGroup<float, PN_ORDER, 3>();
      case 7: return new BatchGroup<float, PN_ORDER, 7>();
      default: return new BatchGroup<float, PN_ORDER, 0>();
    }
  }
  return new BatchGroup<double, PN_ORDER, 0>();
}

}  // namespace pn

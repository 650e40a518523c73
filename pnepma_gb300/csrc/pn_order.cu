// pn_order.cu -- instantiates the solver for one P_N order (compiled once per order with
// -DPN_ORDER=N so the orders build in parallel).
#include "pn_noalloc.cuh"
#include "pn_solver.cuh"

#ifndef PN_ORDER
#error "compile with -DPN_ORDER=<order>"
#endif

#define PN_CAT2(a, b) a##b
#define PN_CAT(a, b) PN_CAT2(a, b)

namespace pn {
SolverBase* PN_CAT(make_solver_, PN_ORDER)(int precision) {
  if (precision == PN_FP32) return new Solver<float, PN_ORDER>();
  return new Solver<double, PN_ORDER>();
}

int PN_CAT(noalloc_forward_, PN_ORDER)(const pn_desc* d, unsigned char* scratch, size_t cap, const double* rho,
                                         const double* noa, const double* acs, double* intensities, cudaStream_t s,
                                         std::string& err) {
  return noalloc_forward<PN_ORDER>(d, scratch, cap, rho, noa, acs, intensities, s, err);
}
}  // namespace pn

// pn_capi.cu -- the extern "C" entry points declared in include/pnepma.h.
// No C++ exception and no abort crosses this boundary: every entry point returns a pn_status.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <map>
#include <mutex>
#include <new>
#include <string>

#include "../../include/pnepma.h"
#include "generated/pn_orders.h"
#include "pn_layout.h"
#include "pn_solver_base.h"
#include "pn_tape_pool.h"
#include "pn_trace.h"

namespace pn {

#define PN_DECL(N) SolverBase* make_solver_##N(int precision);
PN_FOR_EACH_ORDER(PN_DECL)
#undef PN_DECL

static SolverBase* make_solver(int N, int precision) {
  switch (N) {
#define PN_CASE(K) \
  case K:          \
    return make_solver_##K(precision);
    PN_FOR_EACH_ORDER(PN_CASE)
#undef PN_CASE
    default:
      return nullptr;
  }
}

static long long orders_mask() {
  long long m = 0;
#define PN_BIT(K) m |= (1LL << K);
  PN_FOR_EACH_ORDER(PN_BIT)
#undef PN_BIT
  return m;
}
}  // namespace pn

struct pn_handle {
  pn::SolverBase* s = nullptr;
};

static thread_local std::string g_last_error;

namespace pn {
void set_last_error(const std::string& msg) { g_last_error = msg; }

TapePool& tape_pool(int device) {
  static std::mutex mu;
  static std::map<int, TapePool*> pools;
  std::lock_guard<std::mutex> lk(mu);
  TapePool*& p = pools[device];
  if (!p) p = new TapePool;   // lives until the process exits
  return *p;
}

unsigned long long next_handle_id() {
  static std::atomic<unsigned long long> id{0};
  return ++id;
}
}  // namespace pn

static int fail(const std::string& msg, int code) {
  g_last_error = msg;
  return code;
}

#define PN_GUARD(expr)                                   \
  try {                                                  \
    return (expr);                                       \
  } catch (const std::bad_alloc&) {                      \
    if (h && h->s) h->s->err = "host allocation failed"; \
    return PN_ERR_NO_MEMORY;                             \
  } catch (...) {                                        \
    if (h && h->s) h->s->err = "internal error";         \
    return PN_ERR_INVALID;                               \
  }

extern "C" {

int32_t pn_abi_version(void) { return PN_ABI_VERSION; }

int64_t pn_compiled_orders(void) { return pn::orders_mask(); }

int pn_query_sizes(const pn_desc* desc, pn_sizes* sizes) {
  try {
    if (!sizes) return fail("sizes is NULL", PN_ERR_INVALID);
    pn::Layout L;
    std::string err;
    int rc = L.init(desc, err);
    if (rc) return fail(err, rc);
    for (int c = 0; c < 8; ++c) {
      sizes->n_moments[c] = L.nm[c];
      for (int k = 0; k < 3; ++k) sizes->shape[c][k] = L.shape[c][k];
    }
    sizes->n_rho = L.n_rho;
    sizes->n_eee_cells = L.n_eee_cells;
    sizes->n_noa = L.n_eee_cells * L.ne;
    sizes->n_acs = L.n_eee_cells * L.nr;
    sizes->n_state = L.n_state;
    sizes->n_beam_face = L.n_beam;
    sizes->n_advection = L.n_adv;
    sizes->n_boundary = L.n_bnd;
    const long long esize = desc->precision == PN_FP32 ? 4 : 8;
    const long long slot = L.slot_elems * esize;
    int K = desc->checkpoint_stride;
    if (K <= 0) K = ((long long)(L.ns + 1) * slot <= (2LL << 30)) ? 1 : (int)std::ceil(std::sqrt((double)L.ns));
    if (K > L.ns) K = L.ns;
    const long long nck = L.ns / K + 1 + ((L.ns % K) ? 1 : 0);
    const long long nwork = K - 1 > 2 ? K - 1 : 2;
    sizes->device_bytes = (nck + nwork + 2) * slot + L.rho_elems * (esize + 8) +
                          L.n_eee_cells * (L.ne + L.nr) * 8 * 3 + (long long)(L.ns + 1) * (L.nr + 1) * 8 * 3 +
                          L.n_bnd * 16 + L.n_beam * 8 + (L.n_rho > L.n_state ? L.n_rho : L.n_state) * 8;
    return PN_OK;
  } catch (...) {
    return fail("internal error", PN_ERR_INVALID);
  }
}

int pn_create(const pn_desc* desc, pn_handle** out) {
  if (!out) return fail("out is NULL", PN_ERR_INVALID);
  *out = nullptr;
  try {
    pn::Layout L;
    std::string err;
    int rc = L.init(desc, err);
    if (rc) return fail(err, rc);
    if (desc->precision != PN_FP64 && desc->precision != PN_FP32) return fail("unknown precision", PN_ERR_INVALID);
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev < 1) {
      cudaGetLastError();
      return fail("no CUDA device is available", PN_ERR_NO_DEVICE);
    }
    pn::SolverBase* s = pn::make_solver(desc->order, desc->precision);
    if (!s) return fail("P_N order " + std::to_string(desc->order) + " is not compiled into the library", PN_ERR_UNSUPPORTED);
    rc = s->create(desc);
    if (rc) {
      std::string m = s->err;
      delete s;
      return fail(m, rc);
    }
    pn_handle* h = new pn_handle;
    h->s = s;
    *out = h;
    return PN_OK;
  } catch (const std::bad_alloc&) {
    return fail("host allocation failed", PN_ERR_NO_MEMORY);
  } catch (...) {
    return fail("internal error", PN_ERR_INVALID);
  }
}

int pn_forward(pn_handle* h, const double* rho, const double* noa, const double* acs, double* intensities) {
  if (!h || !h->s) return fail("handle is NULL", PN_ERR_INVALID);
  pn::TraceRange trace("pn_forward");
  PN_GUARD(h->s->forward(rho, noa, acs, intensities, nullptr, false))
}

int pn_adjoint(pn_handle* h, const double* intensities_bar, double* rho_bar, double* noa_bar, double* acs_bar) {
  if (!h || !h->s) return fail("handle is NULL", PN_ERR_INVALID);
  pn::TraceRange trace("pn_adjoint");
  PN_GUARD(h->s->adjoint(intensities_bar, rho_bar, noa_bar, acs_bar, nullptr, false))
}

// The stream argument of the device-pointer calls: NULL names the legacy default stream (the
// solver's own non-blocking stream, which does not synchronise with it, serves the host-pointer
// calls only).
static cudaStream_t caller_stream(void* stream) { return stream ? (cudaStream_t)stream : cudaStreamLegacy; }

int pn_forward_device(pn_handle* h, const double* rho, const double* noa, const double* acs, double* intensities,
                      void* stream) {
  if (!h || !h->s) return fail("handle is NULL", PN_ERR_INVALID);
  pn::TraceRange trace("pn_forward_device");
  PN_GUARD(h->s->forward(rho, noa, acs, intensities, caller_stream(stream), true))
}

int pn_adjoint_device(pn_handle* h, const double* intensities_bar, double* rho_bar, double* noa_bar,
                      double* acs_bar, void* stream) {
  if (!h || !h->s) return fail("handle is NULL", PN_ERR_INVALID);
  pn::TraceRange trace("pn_adjoint_device");
  PN_GUARD(h->s->adjoint(intensities_bar, rho_bar, noa_bar, acs_bar, caller_stream(stream), true))
}

int pn_generation_field(pn_handle* h, const double* rho, double* field) {
  if (!h || !h->s) return fail("handle is NULL", PN_ERR_INVALID);
  pn::TraceRange trace("pn_generation_field");
  PN_GUARD(h->s->generation_field(rho, field))
}

int pn_set_state(pn_handle* h, const double* rho, const double* state) {
  if (!h || !h->s) return fail("handle is NULL", PN_ERR_INVALID);
  PN_GUARD(h->s->set_state(rho, state))
}

int pn_step(pn_handle* h, int32_t step) {
  if (!h || !h->s) return fail("handle is NULL", PN_ERR_INVALID);
  PN_GUARD(h->s->step(step))
}

int pn_get_state(pn_handle* h, double* state) {
  if (!h || !h->s) return fail("handle is NULL", PN_ERR_INVALID);
  PN_GUARD(h->s->get_state(state))
}

int pn_query_handle(const pn_handle* h, pn_handle_info* info) {
  if (!h || !h->s || !info) return fail("handle or info is NULL", PN_ERR_INVALID);
  h->s->info(info);
  return PN_OK;
}

void pn_destroy(pn_handle* h) {
  if (!h) return;
  try {
    delete h->s;
  } catch (...) {
  }
  delete h;
}

const char* pn_last_error(const pn_handle* h) {
  if (h && h->s) return h->s->err.c_str();
  return g_last_error.c_str();
}

}  // extern "C"

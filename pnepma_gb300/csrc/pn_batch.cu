// pn_batch.cu -- the pn_batch_* entry points: solves grouped by order, one group per stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "../../include/pnepma.h"
#include "generated/pn_orders.h"
#include "pn_layout.h"

#include "pn_batch_base.h"
#include "pn_batch_impl.h"
#include "pn_trace.h"

namespace pn {
#define PN_DECL(N) BatchGroupBase* make_batch_group_##N(int precision, int dims);
PN_FOR_EACH_ORDER(PN_DECL)
#undef PN_DECL
void set_last_error(const std::string& msg);
}  // namespace pn

struct pn_batch {
  int n = 0;
  int precision = 0;
  std::vector<pn::BatchGroupBase*> groups;
  std::vector<cudaStream_t> streams;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  std::vector<pn::BIo> io;
  ~pn_batch() {
    for (auto* g : groups) delete g;
    for (auto s : streams) cudaStreamDestroy(s);
    for (auto e : joins) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
  }
};

static int batch_fail(const std::string& m, int code) {
  pn::set_last_error(m);
  return code;
}

static pn::BatchGroupBase* make_group(int N, int precision, int dims) {
  switch (N) {
#define PN_CASE(K) \
  case K:          \
    return pn::make_batch_group_##K(precision, dims);
    PN_FOR_EACH_ORDER(PN_CASE)
#undef PN_CASE
    default:
      return nullptr;
  }
}

// run fn(group, stream) on every group, each on its own stream forked from and joined to `s`
template <class F>
static int run_groups(pn_batch* b, cudaStream_t s, F fn) {
  if (cudaEventRecord(b->fork, s) != cudaSuccess) return batch_fail("cudaEventRecord failed", PN_ERR_CUDA);
  for (size_t g = 0; g < b->groups.size(); ++g) {
    if (cudaStreamWaitEvent(b->streams[g], b->fork, 0) != cudaSuccess) return batch_fail("cudaStreamWaitEvent failed", PN_ERR_CUDA);
    int rc = fn(b->groups[g], b->streams[g]);
    if (rc) return batch_fail(b->groups[g]->err, rc);
    if (cudaEventRecord(b->joins[g], b->streams[g]) != cudaSuccess) return batch_fail("cudaEventRecord failed", PN_ERR_CUDA);
    if (cudaStreamWaitEvent(s, b->joins[g], 0) != cudaSuccess) return batch_fail("cudaStreamWaitEvent failed", PN_ERR_CUDA);
  }
  return PN_OK;
}

namespace pn {

int batch_create(const pn_desc* const* descs, int n, long long budget, int K, int flags, Arena* arena, pn_batch** out,
                 std::string& err) {
  *out = nullptr;
  if (!descs || n < 1) { err = "empty batch"; return PN_ERR_INVALID; }
  pn_batch* b = nullptr;
  try {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
      cudaGetLastError();
      err = "no CUDA device is available";
      return PN_ERR_NO_DEVICE;
    }
    const int precision = descs[0] ? descs[0]->precision : 0;
    // groups: same order and same set of active axes
    std::map<std::pair<int, int>, std::vector<int>> by_order;
    for (int i = 0; i < n; ++i) {
      if (!descs[i]) { err = "descriptor is NULL"; return PN_ERR_INVALID; }
      if (descs[i]->precision != precision) { err = "all descriptors of a batch share one precision"; return PN_ERR_INVALID; }
      int dims = 0;
      for (int k = 0; k < 3; ++k) dims |= (descs[i]->n_points[k] > 1 ? 1 : 0) << k;
      by_order[{descs[i]->order, dims}].push_back(i);
    }
    b = new pn_batch;
    b->n = n;
    b->precision = precision;
    b->io.resize(n);
    // share the budget between the groups in proportion to their solve counts
    for (auto& kv : by_order) {
      BatchGroupBase* g = make_group(kv.first.first, precision, kv.first.second);
      if (!g) {
        delete b;
        err = "P_N order " + std::to_string(kv.first.first) + " is not compiled into the library";
        return PN_ERR_UNSUPPORTED;
      }
      g->arena = arena;
      b->groups.push_back(g);
      const long long share = budget * (long long)kv.second.size() / n;
      int rc = g->create(descs, kv.second.data(), (int)kv.second.size(), share, K, flags);
      if (rc) {
        err = g->err;
        delete b;
        return rc;
      }
      cudaStream_t st;
      cudaEvent_t ev;
      if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
        delete b;
        err = "stream creation failed";
        return PN_ERR_CUDA;
      }
      b->streams.push_back(st);
      b->joins.push_back(ev);
    }
    if (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) {
      delete b;
      err = "event creation failed";
      return PN_ERR_CUDA;
    }
    // the uploads ran on each group's own stream: wait for those, not for the whole device
    for (auto* g : b->groups)
      if (int rc = g->wait_created()) {
        err = "device error during batch creation: " + g->err;
        delete b;
        return rc;
      }
    *out = b;
    return PN_OK;
  } catch (const std::bad_alloc&) {
    delete b;
    err = "host allocation failed";
    return PN_ERR_NO_MEMORY;
  } catch (...) {
    delete b;
    err = "internal error";
    return PN_ERR_INVALID;
  }
}

int batch_status(pn_batch* b) {
  for (auto* g : b->groups) {
    const int s = g->device_status();
    if (s != PN_OK) return s;
  }
  return PN_OK;
}

long long batch_device_bytes(const pn_batch* b) {
  long long s = 0;
  for (auto* g : b->groups) s += g->device_bytes();
  return s;
}

}  // namespace pn

extern "C" {

int pn_batch_create(const pn_desc* const* descs, int32_t n, const pn_batch_options* options, pn_batch** out) {
  if (!out) return batch_fail("out is NULL", PN_ERR_INVALID);
  *out = nullptr;
  std::string err;
  long long budget = options ? options->memory_budget : 0;
  const int K = options ? options->checkpoint_stride : 0;
  try {
    if (budget <= 0) {
      int ndev = 0;
      if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return batch_fail("no CUDA device is available", PN_ERR_NO_DEVICE);
      }
      size_t fr = 0, tot = 0;
      if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return batch_fail("cudaMemGetInfo failed", PN_ERR_CUDA);
      budget = (long long)(fr / 2);
    }
  } catch (...) {
    return batch_fail("internal error", PN_ERR_INVALID);
  }
  int rc = pn::batch_create(descs, n, budget, K, options ? options->flags : 0, nullptr, out, err);
  if (rc) return batch_fail(err, rc);
  return PN_OK;
}

int pn_batch_forward(pn_batch* b, const double* const* rho, const double* const* noa, const double* const* acs,
                     double* const* intensities, void* stream) {
  if (!b || !rho || !noa || !acs || !intensities) return batch_fail("NULL argument", PN_ERR_INVALID);
  try {
    for (int i = 0; i < b->n; ++i) {
      if (!rho[i] || !noa[i] || !acs[i] || !intensities[i]) return batch_fail("NULL buffer", PN_ERR_INVALID);
      b->io[i].rho = rho[i];
      b->io[i].noa = noa[i];
      b->io[i].acs = acs[i];
      b->io[i].I = intensities[i];
    }
    pn::TraceRange trace("pn_batch_forward");
    return run_groups(b, (cudaStream_t)stream,
                      [&](pn::BatchGroupBase* g, cudaStream_t s) { return g->forward(b->io.data(), s); });
  } catch (...) {
    return batch_fail("internal error", PN_ERR_INVALID);
  }
}

int pn_batch_adjoint(pn_batch* b, const double* const* intensities_bar, double* const* rho_bar,
                     double* const* noa_bar, double* const* acs_bar, void* stream) {
  if (!b || !intensities_bar || !rho_bar || !noa_bar || !acs_bar) return batch_fail("NULL argument", PN_ERR_INVALID);
  try {
    for (int i = 0; i < b->n; ++i) {
      if (!intensities_bar[i] || !rho_bar[i] || !noa_bar[i] || !acs_bar[i]) return batch_fail("NULL buffer", PN_ERR_INVALID);
      b->io[i].ibar = intensities_bar[i];
      b->io[i].rho_bar = rho_bar[i];
      b->io[i].noa_bar = noa_bar[i];
      b->io[i].acs_bar = acs_bar[i];
    }
    pn::TraceRange trace("pn_batch_adjoint");
    return run_groups(b, (cudaStream_t)stream,
                      [&](pn::BatchGroupBase* g, cudaStream_t s) { return g->adjoint(b->io.data(), s); });
  } catch (...) {
    return batch_fail("internal error", PN_ERR_INVALID);
  }
}

int pn_batch_query(const pn_batch* b, pn_batch_info* info) {
  if (!b || !info) return batch_fail("NULL argument", PN_ERR_INVALID);
  info->n_solves = b->n;
  info->n_groups = (int32_t)b->groups.size();
  info->checkpoint_stride = 0;
  info->tma_groups = 0;
  info->device_bytes = 0;
  info->forward_kernels = 0;
  info->adjoint_kernels = 0;
  info->recomputed_steps = 0;
  for (auto* g : b->groups) {
    info->checkpoint_stride = std::max(info->checkpoint_stride, g->stride());
    info->tma_groups += g->tma() ? 1 : 0;
    info->device_bytes += g->device_bytes();
    info->forward_kernels += g->launches_forward();
    info->adjoint_kernels += g->launches_adjoint();
    info->recomputed_steps += g->recomputed_steps();
  }
  try {
    const int st = pn::batch_status(const_cast<pn_batch*>(b));
    if (st != PN_OK) return batch_fail("a bounded device-side wait ran out", st);
  } catch (...) {
    return batch_fail("internal error", PN_ERR_INVALID);
  }
  return PN_OK;
}

void pn_batch_destroy(pn_batch* b) {
  try {
    delete b;
  } catch (...) {
  }
}

}  // extern "C"

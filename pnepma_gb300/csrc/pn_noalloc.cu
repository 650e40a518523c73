// pn_noalloc.cu -- pn_forward_noalloc: the FP64 forward intensity march with all of its device
// scratch in one fixed array that belongs to the library.
//
// Some callers cannot allocate device memory while they solve: a process whose GPU memory is
// reserved by another allocator (for example a Julia session whose CUDA pool owns the device, or
// a framework that has pre-reserved its memory budget), or a latency-bound loop where cudaMalloc
// and cudaFree would synchronise the device.  This entry point serves them: it calls no
// cudaMalloc, cudaFree, graph instantiation or stream creation, and takes its state, densities,
// tables and partial sums from g_pn_scratch below.
//
// The array is PN_NOALLOC_SCRATCH_BYTES (64 MiB) per GPU and every GPU that loads this code keeps
// it until the process exits.  All calls share it and it keeps the contents of the last call, so
// each call re-copies its tables and zeroes the state and the sums before it uses them; calls
// whose work overlaps on the GPU (two streams, or two host threads) race on it and must be
// serialised by the caller.  In host code `g_pn_scratch` names a host-side stand-in, not device
// memory: its device address is looked up with cudaGetSymbolAddress, once per device, on the first
// call made with that device current.  That first call should therefore come before any stream
// capture.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/pnepma.h"
#include "generated/pn_orders.h"
#include "pn_layout.h"

static __device__ __align__(256) unsigned char g_pn_scratch[PN_NOALLOC_SCRATCH_BYTES];

namespace pn {
#define PN_DECL(N)                                                                                            \
  int noalloc_forward_##N(const pn_desc* d, unsigned char* scratch, size_t cap, const double* rho,            \
                          const double* noa, const double* acs, double* intensities, cudaStream_t s,          \
                          std::string& err);
PN_FOR_EACH_ORDER(PN_DECL)
#undef PN_DECL
void set_last_error(const std::string& msg);  // pn_capi.cu: the message pn_last_error(NULL) returns
}  // namespace pn

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (looked up once per device).
int scratch_address(void** out, std::string& err) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0) {
    cudaGetLastError();
    err = "no CUDA device is available";
    return PN_ERR_NO_DEVICE;
  }
  if (dev >= kMaxDevices) {
    err = "device ordinal beyond the supported range";
    return PN_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_pn_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      err = std::string("cudaGetSymbolAddress of the scratch array failed: ") + cudaGetErrorString(e);
      return PN_ERR_CUDA;
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return PN_OK;
}

}  // namespace

extern "C" int pn_forward_noalloc(const pn_desc* desc, const double* rho, const double* noa, const double* acs,
                                  double* intensities, void* stream) {
  try {
    std::string err;
    if (!desc) {
      pn::set_last_error("descriptor is NULL");
      return PN_ERR_INVALID;
    }
    void* base = nullptr;
    int rc = scratch_address(&base, err);
    if (rc) {
      pn::set_last_error(err);
      return rc;
    }
    switch (desc->order) {
#define PN_CASE(K)                                                                                          \
  case K:                                                                                                   \
    rc = pn::noalloc_forward_##K(desc, (unsigned char*)base, (size_t)PN_NOALLOC_SCRATCH_BYTES, rho, noa, acs, \
                                 intensities, (cudaStream_t)stream, err);                                   \
    break;
      PN_FOR_EACH_ORDER(PN_CASE)
#undef PN_CASE
      default:
        rc = PN_ERR_UNSUPPORTED;
        err = "P_N order not compiled into the library";
    }
    if (rc) pn::set_last_error(err);
    return rc;
  } catch (...) {
    pn::set_last_error("internal error");
    return PN_ERR_INVALID;
  }
}

// pn_selftest.cu -- device self-tests of the library's own numerical helpers.
#include <cuda_runtime.h>

#include <string>

#include "../../include/pnepma.h"
#include "generated/pn_orders.h"
#include "pn_device.cuh"

namespace pn {
void set_last_error(const std::string& msg);
}

static __global__ void phi1_kernel(const float* x, float* fast, float* ref, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    fast[i] = pn::phi1(x[i]);
    ref[i] = pn::phi1_ref(x[i]);
  }
}

extern "C" int pn_selftest_phi1(int32_t n, const float* x, float* phi1_fast, float* phi1_ref) {
  if (n < 0 || (n > 0 && (!x || !phi1_fast || !phi1_ref))) {
    pn::set_last_error("NULL argument");
    return PN_ERR_INVALID;
  }
  if (n == 0) return PN_OK;
  float* d = nullptr;
  if (cudaMalloc(&d, sizeof(float) * 3 * (size_t)n) != cudaSuccess) {
    cudaGetLastError();
    pn::set_last_error("device allocation failed");
    return PN_ERR_NO_MEMORY;
  }
  cudaError_t e = cudaMemcpy(d, x, sizeof(float) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    phi1_kernel<<<(n + 255) / 256, 256>>>(d, d + n, d + 2 * (size_t)n, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(phi1_fast, d + n, sizeof(float) * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(phi1_ref, d + 2 * (size_t)n, sizeof(float) * n, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) {
    pn::set_last_error(std::string("self-test failed: ") + cudaGetErrorString(e));
    return PN_ERR_CUDA;
  }
  return PN_OK;
}

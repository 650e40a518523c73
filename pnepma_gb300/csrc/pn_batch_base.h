// pn_batch_base.h -- the interface of a group of batched solves (one order, one element type).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/pnepma.h"
#include "pn_arena.h"

namespace pn {

// device pointers of one solve's inputs and outputs, in the caller's layouts
struct BIo {
  const double* rho;
  const double* noa;
  const double* acs;
  const double* ibar;
  double* I;
  double* rho_bar;
  double* noa_bar;
  double* acs_bar;
};

class BatchGroupBase {
 public:
  virtual ~BatchGroupBase() {}
  virtual int create(const pn_desc* const* d, const int* idx, int n, long long budget, int K, int flags) = 0;
  virtual int forward(const BIo* io_host, cudaStream_t s) = 0;
  virtual int adjoint(const BIo* io_host, cudaStream_t s) = 0;
  virtual long long device_bytes() const = 0;
  virtual long long launches_forward() const = 0;
  virtual long long launches_adjoint() const = 0;
  virtual int stride() const = 0;
  virtual long long recomputed_steps() const { return 0; }
  // wait for the uploads create() issued on the group's own stream
  virtual int wait_created() = 0;
  // true when the group's sub-steps run through the TMA tile kernel
  virtual bool tma() const { return false; }
  // status word of the group's kernels (PN_OK, or PN_ERR_TIMEOUT after a wait ran out); read it
  // once the group's work has completed
  virtual int device_status() { return PN_OK; }
  // device ranges come from this arena when set (returned to it, never cudaFree'd), else cudaMalloc
  Arena* arena = nullptr;
  std::string err;
  std::vector<int> members;   // indices into the caller's descriptor array, in group order
};

}  // namespace pn

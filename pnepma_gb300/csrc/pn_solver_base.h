// pn_solver_base.h -- the interface every compiled (order, precision) solver implements.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "../../include/pnepma.h"

namespace pn {

class SolverBase {
 public:
  virtual ~SolverBase() {}
  virtual int create(const pn_desc* d) = 0;
  virtual int forward(const double* rho, const double* noa, const double* acs, double* I, cudaStream_t st,
                      bool device_ptrs) = 0;
  virtual int adjoint(const double* ibar, double* rho_bar, double* noa_bar, double* acs_bar, cudaStream_t st,
                      bool device_ptrs) = 0;
  virtual int generation_field(const double* rho, double* field) = 0;
  virtual int set_state(const double* rho, const double* state) = 0;
  virtual int step(int i) = 0;
  virtual int get_state(double* state) = 0;
  virtual long long device_bytes() const = 0;
  virtual void info(pn_handle_info* out) const = 0;
  std::string err;
};

}  // namespace pn

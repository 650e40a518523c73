// pn_tape_pool.h -- one shared full-tape buffer per device for the plain (one solve per handle)
// path.
//
// A handle whose full forward tape (every state of the march) exceeds the 2 GiB it may keep for
// itself would otherwise checkpoint and recompute most of the march in the adjoint sweep.  With
// HBM for one full tape but not one per handle, such handles share this buffer: a forward march
// records its tape here, and the following adjoint sweep of the same handle reads it.  The
// buffer grows to the largest tape asked for (while that fits in 80 % of the free memory; the
// handle checkpoints otherwise).  Users are ordered on the GPU by an event recorded after each
// use; an adjoint whose tape was overwritten by another handle's forward re-runs its own forward
// first.  Freed when the last handle that may use it is destroyed.
#pragma once

#include <cuda_runtime.h>

#include <mutex>

namespace pn {

struct TapePool {
  std::mutex mu;
  char* base = nullptr;
  size_t bytes = 0;
  unsigned long long epoch = 0;   // changes whenever base changes (graphs hold the address)
  unsigned long long owner = 0;   // id of the handle whose tape the buffer holds (0: none)
  unsigned long long gen = 0;     // incremented by every forward recorded into the buffer
  cudaEvent_t last = nullptr;     // recorded after every use
  int users = 0;                  // live handles that may use the buffer
};

// the pool of `device` (created on first use, never destroyed)
TapePool& tape_pool(int device);
// process-unique handle ids (never reused, unlike addresses)
unsigned long long next_handle_id();

}  // namespace pn

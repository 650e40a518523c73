// pn_batch_impl.h -- library-internal construction of a pn_batch (used by pn_batch_create and
// by the server, which places every wave's device memory in its own arena).
#pragma once

#include <string>

#include "../../include/pnepma.h"
#include "pn_arena.h"

namespace pn {

// Group the solves by (order, active axes), build each group's tables, tiles and graphs.  With
// an arena every device range is taken from it; without one, from cudaMalloc.  Waits only for
// the group streams' own uploads.  budget: device bytes the checkpoint tapes may take.
int batch_create(const pn_desc* const* descs, int n, long long budget, int K, int flags, Arena* arena, pn_batch** out,
                 std::string& err);

// PN_OK, or the first error status a group's kernels recorded (read after the work completed)
int batch_status(pn_batch* b);

long long batch_device_bytes(const pn_batch* b);

}  // namespace pn

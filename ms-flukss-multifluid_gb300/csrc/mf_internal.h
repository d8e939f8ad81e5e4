// mf_internal.h - declarations shared by the library's translation units
// (not part of the public C ABI).
#pragma once

#include "mf_device.cuh"

namespace mf {

struct CtxView {
  const mf_params* p;
  const DevParams* dp;
  int ng, nc;
};

// Parameters, device parameters, ghost width and component count of a context.
CtxView ctx_view(const mf_ctx* c);

}  // namespace mf

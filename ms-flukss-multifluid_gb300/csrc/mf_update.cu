// mf_update.cu - update kernel with the fast physics (contraction allowed,
// reciprocals reused): the mixed-precision path and the fast FP64 path.
#define MF_PHYS fast
#include "mf_sources.cuh"
#include "mf_update_kernel.cuh"

namespace mf {

template <typename R>
cudaError_t launch_update_fast(const DevParams& P, const StageBuffers& B, const StageDesc* d_desc,
                               int ndesc, long long max_v, int flags, double dt_scale,
                               StepState* state, DtPartial* partials, int* nblocks_v,
                               cudaStream_t s) {
  const dim3 gv((unsigned)((max_v + kBlock - 1) / kBlock), (unsigned)ndesc);
  if (nblocks_v) *nblocks_v = (int)(gv.x * gv.y);
#define MF_UPD(G, FL) k_update<R, G, FL><<<gv, kBlock, 0, s>>>(P, B, d_desc, state, dt_scale, partials)
  if (P.glm) {
    if (flags == 0) MF_UPD(1, 0);
    else if (flags == kStageDt) MF_UPD(1, kStageDt);
    else MF_UPD(1, kStageAverage | kStageDt);
  } else {
    if (flags == 0) MF_UPD(0, 0);
    else if (flags == kStageDt) MF_UPD(0, kStageDt);
    else MF_UPD(0, kStageAverage | kStageDt);
  }
#undef MF_UPD
  return cudaGetLastError();
}

template cudaError_t launch_update_fast<double>(const DevParams&, const StageBuffers&,
                                                const StageDesc*, int, long long, int, double,
                                                StepState*, DtPartial*, int*, cudaStream_t);
template cudaError_t launch_update_fast<float>(const DevParams&, const StageBuffers&,
                                               const StageDesc*, int, long long, int, double,
                                               StepState*, DtPartial*, int*, cudaStream_t);

}  // namespace mf

// mf_stage.cu - one explicit stage of every patch of a batch: primitive
// variables, face fluxes in each direction, update (host-side composition).
#include "mf_kernels.cuh"

namespace mf {

cudaError_t launch_stage(const DevParams& P, int precision, const StageBuffers& B,
                         const Batch& b, int flags, double dt_scale, StepState* state,
                         DtPartial* partials, int* nblocks_v, cudaStream_t s) {
  int ne = 0;
  cudaError_t e = launch_prim(P, B.uin, B.w, b, s, precision == MF_PREC_MIXED ? B.wf : nullptr);
  if (e != cudaSuccess) return e;
  if (B.ev) cudaEventRecord(B.ev[ne++], s);
  for (int d = 0; d < P.sd; ++d) {
    if (precision == MF_PREC_MIXED)
      e = launch_flux_fast<float>(P, d, B.w, B.f[d], B.bn[d], b, state, s, B.wf);
    else if (precision == MF_PREC_FP64_FAST)
      e = launch_flux_fast<double>(P, d, B.w, B.f[d], B.bn[d], b, state, s);
    else
      e = launch_flux_exact(P, d, B.w, B.f[d], B.bn[d], b, state, s);
    if (e != cudaSuccess) return e;
    if (B.ev) cudaEventRecord(B.ev[ne++], s);
  }
  if (precision == MF_PREC_MIXED)
    e = launch_update_fast<float>(P, B, b, flags, dt_scale, state, partials, nblocks_v, s);
  else if (precision == MF_PREC_FP64_FAST)
    e = launch_update_fast<double>(P, B, b, flags, dt_scale, state, partials, nblocks_v, s);
  else
    e = launch_update_exact(P, B, b, flags, dt_scale, state, partials, nblocks_v, s);
  if (e != cudaSuccess) return e;
  if (B.ev) cudaEventRecord(B.ev[ne++], s);
  return cudaSuccess;
}

}  // namespace mf

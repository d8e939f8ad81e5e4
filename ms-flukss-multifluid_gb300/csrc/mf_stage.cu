// mf_stage.cu - one explicit stage of every patch of a batch: primitive
// variables, face fluxes in each direction, update (host-side composition).
#include "mf_kernels.cuh"

namespace mf {

cudaError_t launch_stage(const DevParams& P, int precision, const StageBuffers& B,
                         const Batch& b, int flags, double dt_scale, StepState* state,
                         DtPartial* partials, int* nblocks_v, cudaStream_t s) {
  int ne = 0;
  float* wf = (precision == MF_PREC_MIXED) ? B.wf : nullptr;
  cudaError_t e;
  if (B.lean) {
    // primitive state of the valid cells, the siblings' copies into the
    // ghost layers, then the far-field ghosts (which read the copies)
    const LeanPrim& L = *B.lean;
    e = launch_prim(P, B.uin, B.w, *L.prim, s, wf);
    if (e != cudaSuccess) return e;
    if (B.ev) cudaEventRecord(B.ev[ne++], s);
    if (L.nregs && L.exchange_w) {
      e = launch_exchange(B.w, L.regs, L.nregs, P.nc, s);
      if (e != cudaSuccess) return e;
      if (B.ev) cudaEventRecord(B.ev[ne++], s);
    }
    if (L.nregs && wf) {
      e = launch_exchange_f(wf, L.regs, L.nregs, P.nc, s);
      if (e != cudaSuccess) return e;
      if (B.ev) cudaEventRecord(B.ev[ne++], s);
    }
    if (L.nfar) {
      e = launch_farfield(P, B.uin, B.w, wf, L.far, L.nfar, b.runs, L.exchange_w, s);
      if (e != cudaSuccess) return e;
      if (B.ev) cudaEventRecord(B.ev[ne++], s);
    }
  } else {
    e = launch_prim(P, B.uin, B.w, b, s, wf);
    if (e != cudaSuccess) return e;
    if (B.ev) cudaEventRecord(B.ev[ne++], s);
  }
  if (B.fused && precision == MF_PREC_MIXED) {
    e = launch_fused(P, B, b, B.fused->tiles, B.fused->ntiles, B.fused->tile, flags, dt_scale,
                     state, partials, s);
    if (e != cudaSuccess) return e;
    if (nblocks_v) *nblocks_v = B.fused->ntiles;
    if (B.ev) cudaEventRecord(B.ev[ne++], s);
    return cudaSuccess;
  }
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

// mf_update.cu - update kernel with the fast physics (contraction allowed,
// reciprocals reused): the mixed-precision path and the fast FP64 path.
#define MF_PHYS fast
#include "mf_sources.cuh"
#include "mf_update_kernel.cuh"

namespace mf {

template <typename R>
cudaError_t launch_update_fast(const DevParams& P, const StageBuffers& B, const Batch& b,
                               int flags, double dt_scale, StepState* state,
                               DtPartial* partials, int* nblocks_v, cudaStream_t s, int first,
                               int end) {
  const int nt = b.nt[2];
  if (end < 0) end = b.tot_v;
  if (nblocks_v) *nblocks_v = (int)flat_blocks(b.tot_v, nt);
  if (first % nt != 0) return cudaErrorInvalidValue;
  if (end - first <= 0) return cudaSuccess;
  const unsigned gv = flat_blocks(end - first, nt);
  // charge-exchange rates: FP64, or FP32 in the opt-in MF_PREC_MIXED_CE32 form
#define MF_UPD(G, FL, CE)                                                                    \
  k_update<R, G, FL, CE><<<gv, nt, 0, s>>>(P, B, b.desc, b.ndesc, first, end, b.runs, state, \
                                           dt_scale, partials)
#define MF_UPD_CE(G, FL)                      \
  do {                                        \
    if constexpr (sizeof(R) == 4) {           \
      if (P.ce32) {                           \
        MF_UPD(G, FL, float);                 \
        break;                                \
      }                                       \
    }                                         \
    MF_UPD(G, FL, double);                    \
  } while (0)
  if (P.glm) {
    if (flags == 0) MF_UPD_CE(1, 0);
    else if (flags == kStageDt) MF_UPD_CE(1, kStageDt);
    else MF_UPD_CE(1, kStageAverage | kStageDt);
  } else {
    if (flags == 0) MF_UPD_CE(0, 0);
    else if (flags == kStageDt) MF_UPD_CE(0, kStageDt);
    else MF_UPD_CE(0, kStageAverage | kStageDt);
  }
#undef MF_UPD_CE
#undef MF_UPD
  return cudaGetLastError();
}

template cudaError_t launch_update_fast<double>(const DevParams&, const StageBuffers&,
                                                const Batch&, int, double, StepState*,
                                                DtPartial*, int*, cudaStream_t, int, int);
template cudaError_t launch_update_fast<float>(const DevParams&, const StageBuffers&,
                                               const Batch&, int, double, StepState*,
                                               DtPartial*, int*, cudaStream_t, int, int);

}  // namespace mf

// mf_flux.cu - face-flux kernel with the fast physics (contraction allowed,
// reciprocals reused): FP32 for the mixed-precision path, FP64 for the fast
// FP64 path.
#define MF_PHYS fast
#include "mf_riemann.cuh"
#include "mf_flux_kernel.cuh"

namespace mf {

template <typename R>
cudaError_t launch_flux_fast(const DevParams& P, int dir, const double* w, void* f, void* bn,
                             const StageDesc* d_desc, int ndesc, long long max_f,
                             const StepState* state, cudaStream_t s) {
  const dim3 gf((unsigned)((max_f + kBlock - 1) / kBlock), (unsigned)ndesc);
  R* F = (R*)f;
  R* Bn = (R*)bn;
  if (dir == 0) k_flux<R, 0><<<gf, kBlock, 0, s>>>(P, w, F, Bn, d_desc, state);
  if (dir == 1) k_flux<R, 1><<<gf, kBlock, 0, s>>>(P, w, F, Bn, d_desc, state);
  if (dir == 2) k_flux<R, 2><<<gf, kBlock, 0, s>>>(P, w, F, Bn, d_desc, state);
  return cudaGetLastError();
}

template cudaError_t launch_flux_fast<double>(const DevParams&, int, const double*, void*, void*,
                                              const StageDesc*, int, long long, const StepState*,
                                              cudaStream_t);
template cudaError_t launch_flux_fast<float>(const DevParams&, int, const double*, void*, void*,
                                             const StageDesc*, int, long long, const StepState*,
                                             cudaStream_t);

}  // namespace mf
